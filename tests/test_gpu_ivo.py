"""IVO on the device (dcg_ivo: the virtual-space Fock matrix and its per-irrep ZHEEV-algorithm
eigenvectors) against the reference's reference.DFPCMONEW of its three runnable IVO cases at
the reference test's tolerance (1e-13), and the whole driver (C++ readers, device MDCINT
canonicalisation, dcg_ivo, DFPCMONEW writer) on run directories rebuilt from the fixtures."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from test_ivo import IVO_CASES, load_ivo_fixture  # noqa: E402


def _system_input(s, totsym=33):
    from dirac_caspt2_gb300 import api
    return api.SystemInput(ninact=s.ninact, nact=s.nact, nsec=s.nsec, nelec=s.nelec, nmo=s.nmo, nsymrpa=s.nsymrpa,
                           multb=s.multb, irpamo=s.irpamo, h=s.h, ecore=s.ecore, rec_idx=s.rec_idx,
                           rec_val=s.rec_val, realonly=s.realonly, totsym=totsym, selectroot=1)


@pytest.mark.parametrize("case", IVO_CASES)
def test_device_ivo_matches_reference(gpu_lib, case):
    from dirac_caspt2_gb300 import api, ivo
    from oracle import caspt2_oracle as O
    s, me, inp, d, ref, _ = load_ivo_fixture(case)
    with api.Caspt2Session(0) as ses:
        ses.set_system(_system_input(s))
        eps, U, bsym, numh = ses.ivo(d.nfsym, me, inp.nhomo)
    assert numh == 6
    new = ivo.rotate_dfpcmo(d, inp, U, bsym, s.nsymrpa)
    assert np.abs(new.coef - ref).max() <= 1e-13
    _, ev, _ = O.ivo(s, O.Integrals(s), me, d, inp.nhomo, inp.occ_mo_num, inp.vcut_mo_num, lartg="old")
    for isym, w in ev.items():
        if len(w):
            assert np.abs(eps[bsym == isym] - w).max() <= 1e-12


@pytest.mark.parametrize("case", IVO_CASES[::2])
def test_run_ivo_end_to_end(gpu_lib, tmp_path, case):
    from dirac_caspt2_gb300 import ivo, synth
    s, me, inp, d, ref, text = load_ivo_fixture(case)
    dd = str(tmp_path)
    synth.write_mrconee(os.path.join(dd, "MRCONEE"), s.nmo, s.ecore, s.h, me, inp.diracver, s.nsymrpa, s.multb,
                        s.irpamo)
    synth.write_mdcint(os.path.join(dd, "MDCINT"), s.nmo, s.rec_idx, s.rec_val, s.realonly)
    open(os.path.join(dd, "DFPCMO"), "w").write(text)
    occ, vc = inp.occ_mo_num, inp.vcut_mo_num
    keys = [".ninact", "0", ".nact", str(s.nact), ".nsec", str(s.nsec), ".nelec", str(s.nelec),
            ".caspt2_ciroots", "33 1", ".diracver", str(inp.diracver), ".scheme", "6",
            ".noccg", str(occ[0]), ".noccu", str(occ[1]), ".nvcutg", str(vc[0]), ".nvcutu", str(vc[1]),
            ".subprograms", "IVO", ".end"]
    open(os.path.join(dd, "active.ivo.inp"), "w").write("\n".join(keys) + "\n")
    res = ivo.run_ivo(dd)
    assert res.numh == 6 and os.path.exists(os.path.join(dd, "DFPCMONEW"))
    from dirac_caspt2_gb300 import dirac_io
    back = dirac_io.read_dfpcmo(os.path.join(dd, "DFPCMONEW"), inp.diracver >= 21)
    assert np.abs(back.coef - ref).max() <= 1e-13
    assert np.array_equal(back.evals, d.evals) and np.array_equal(back.supersym, d.supersym)


def test_ivo_errors(gpu_lib):
    from dirac_caspt2_gb300 import api
    s, me, inp, d, ref, _ = load_ivo_fixture(IVO_CASES[0])
    with api.Caspt2Session(0) as ses:
        ses.system = _system_input(s)
        with pytest.raises(api.DcgError) as ei:
            ses.ivo(d.nfsym, me, 0)
        assert ei.value.code == -3
        ses.set_system(_system_input(s))
        with pytest.raises(api.DcgError) as ei:
            ses.ivo(3, me, 0)
        assert ei.value.code == -1
        with pytest.raises(api.DcgError) as ei:
            ses.ivo(d.nfsym, me, s.nact + 2)
        assert ei.value.code == -1
        eps, U, bsym, numh = ses.ivo(d.nfsym, me, 0)   # the context stays usable
        assert numh == 6
