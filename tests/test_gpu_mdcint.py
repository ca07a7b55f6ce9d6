"""The MDCINT canonicalisation on the device (dcg_mdcint_canonicalize, replacing
create_newmdcint) against the host restatement, record for record and bit for bit: on the raw
MDCINT records of two reference test cases and on synthetic MDCINT files (complex and real,
scheme 6).  Through dcg_set_system_mdcint the reference cases then reproduce their printed
energies (1e-10 Eh) and the synthetic systems the energies of the MDCINTNEW path exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from test_mdcint import RAW_CASES, load_raw  # noqa: E402


def _same_stream(a, b):
    assert a.idx.shape == b.idx.shape
    assert np.array_equal(a.idx, b.idx)
    assert np.array_equal(a.val.real, b.val.real)
    if not a.realonly:
        assert np.array_equal(a.val.imag, b.val.imag)


@pytest.mark.parametrize("case", RAW_CASES)
def test_device_canonicalisation_golden(gpu_lib, case):
    import os
    from conftest import GOLDEN_DIR
    from dirac_caspt2_gb300 import api, dirac_io
    raw = load_raw(case)
    with api.Caspt2Session(0) as ses:
        dev = ses.mdcint_canonicalize(raw)
        _same_stream(dev, dirac_io.canonicalize_mdcint(raw))
        s = api.SystemInput.from_npz(os.path.join(GOLDEN_DIR, f"{case}.npz"))
        ses.set_system_mdcint(s, raw)
        eig, _ = ses.casci(max(1, s.selectroot))
        e2, sc, e0, et = ses.caspt2()
    g = np.load(os.path.join(GOLDEN_DIR, f"{case}.npz"))
    assert abs(eig[s.selectroot - 1] - float(g["ref_casci"])) <= 1e-10
    assert abs(et - float(g["ref_total"])) <= 1e-10


@pytest.mark.parametrize("realonly", [False, True])
def test_device_canonicalisation_synthetic(gpu_lib, tmp_path, realonly):
    from dirac_caspt2_gb300 import api, dirac_io, synth
    S = synth.make_system(synth.SynthConfig(4, 6, 16, 3, seed=12, realonly=realonly))
    synth.write_case_files(S, str(tmp_path))
    inp = dirac_io.read_active_inp(str(tmp_path / "active.inp"))
    mrc = dirac_io.read_mrconee(str(tmp_path / "MRCONEE"), inp)
    raw = dirac_io.read_mdcint_raw(str(tmp_path), mrc, inp)
    host = dirac_io.canonicalize_mdcint(raw)
    s = api.SystemInput.from_files(str(tmp_path))
    with api.Caspt2Session(0) as ses:
        _same_stream(ses.mdcint_canonicalize(raw), host)
        ref = ses.solve(s)
        ses.set_system_mdcint(s, raw)
        eig, _ = ses.casci(1)
        e2, sc, e0, et = ses.caspt2()
    assert eig[0] == ref.casci_energies[0]
    assert et == ref.total_energy


@pytest.mark.parametrize("pinned", [False, True])
def test_native_files_to_device(gpu_lib, tmp_path, pinned):
    """A run directory read by the library's C++ readers (MDCINT split over two files, entry
    arrays optionally page-locked) and canonicalised on the device gives the energies of the
    Python reader path exactly."""
    from dirac_caspt2_gb300 import api, dirac_io, synth
    S = synth.make_system(synth.SynthConfig(4, 6, 16, 3, seed=13))
    d = str(tmp_path)
    synth.write_case_files(S, d)
    recs = dirac_io.read_fortran_records(str(tmp_path / "MDCINT"))
    half = (len(recs) - 2) // 2
    dirac_io.write_fortran_records(str(tmp_path / "MDCINT"), recs[:1 + half] + recs[-1:])
    dirac_io.write_fortran_records(str(tmp_path / "MDCINXXXX1"), recs[:1] + recs[1 + half:])
    s = api.SystemInput.from_files(d)
    inp = dirac_io.read_active_inp(str(tmp_path / "active.inp"))
    with api.Caspt2Session(0) as ses:
        ref = ses.solve(s)
        with api.NativeFiles(d, inp, pinned=pinned) as nf:
            ses.set_system_mdcint(nf.system_input(), nf)
            eig, _ = ses.casci(1)
            e2, sc, e0, et = ses.caspt2()
    assert eig[0] == ref.casci_energies[0]
    assert et == ref.total_energy
