"""The library's C++ readers of MRCONEE and MDCINT (dcg_read_mrconee / dcg_read_mdcint)
against the Python restatement of the reference readers, on synthetic run directories and
(when mounted) the reference's own test inputs.  File parsing only: no GPU."""
import os
import struct

import numpy as np
import pytest

REF_DEV = "/root/reference/test/dev"


def _lib_or_skip():
    from dirac_caspt2_gb300 import api
    try:
        return api.load_library()
    except (ImportError, OSError) as e:   # library not built in this checkout
        pytest.skip(f"library not loadable: {e}")


def _compare(d, inp):
    from dirac_caspt2_gb300 import api, dirac_io
    py_m = dirac_io.read_mrconee(os.path.join(d, "MRCONEE"), inp)
    py_r = dirac_io.read_mdcint_raw(d, py_m, inp)
    with api.NativeFiles(d, inp) as nf:
        m = nf.mrconee()
        r = nf.raw()
    assert m.nmo == py_m.nmo and m.nsymrpa == py_m.nsymrpa and m.dirac_32bit == py_m.dirac_32bit
    assert m.ecore == py_m.ecore and m.hf_energy == py_m.hf_energy
    assert np.array_equal(m.multb, py_m.multb)
    assert np.array_equal(m.irpamo, py_m.irpamo)
    assert np.array_equal(m.mo_energy, py_m.mo_energy)
    assert np.array_equal(m.dirac_to_cas[1:], py_m.dirac_to_cas[1:])
    assert np.array_equal(m.cas_to_dirac[1:], py_m.cas_to_dirac[1:])
    assert np.array_equal(m.h, py_m.h)
    for f in ("rec_ikr", "rec_jkr", "rec_off", "indk", "indl", "re", "im", "kr"):
        assert np.array_equal(getattr(r, f), getattr(py_r, f)), f
    assert np.array_equal(r.dirac_to_cas[1:], py_r.dirac_to_cas[1:])
    assert (r.nmo, r.scheme, r.realonly) == (py_r.nmo, py_r.scheme, py_r.realonly)
    return r


@pytest.mark.parametrize("realonly", [False, True])
def test_native_matches_python_synthetic(tmp_path, realonly):
    _lib_or_skip()
    from dirac_caspt2_gb300 import dirac_io, synth
    S = synth.make_system(synth.SynthConfig(4, 6, 8, 3, seed=11, realonly=realonly))
    d = str(tmp_path / "case")
    synth.write_case_files(S, d)
    inp = dirac_io.read_active_inp(os.path.join(d, "active.inp"))
    r = _compare(d, inp)
    assert r.realonly == realonly and len(r.re) > 0


def test_native_multi_file_and_ras(tmp_path):
    """Records spread over MDCINT and MDCINXXXX1 (each with its header and end record), read
    with a RAS partition of the active spinors."""
    _lib_or_skip()
    from dirac_caspt2_gb300 import dirac_io, synth
    S = synth.make_system(synth.SynthConfig(2, 6, 6, 3, seed=4))
    d = str(tmp_path / "case")
    synth.write_case_files(S, d)
    recs = dirac_io.read_fortran_records(os.path.join(d, "MDCINT"))
    hdr, body, end = recs[0], recs[1:-1], recs[-1]
    half = len(body) // 2
    dirac_io.write_fortran_records(os.path.join(d, "MDCINT"), [hdr] + body[:half] + [end])
    dirac_io.write_fortran_records(os.path.join(d, "MDCINXXXX1"), [hdr] + body[half:] + [end])
    inp = dirac_io.read_active_inp(os.path.join(d, "active.inp"))
    r = _compare(d, inp)
    assert len(r.rec_ikr) == len(body)
    ras = dirac_io.ActiveInput(ninact=2, nact=6, nsec=6, nelec=3, ciroots=[(1, 1)], eshift=0.0, diracver=21,
                               scheme=6, ras1=[3, 4], ras2=[5, 6], ras3=[9, 10], ras1_max_hole=1, ras3_max_elec=1)
    _compare(d, ras)


def test_native_subrecords(tmp_path):
    """A record stored as two sub-records (negative markers on the continued part) reads
    back whole."""
    _lib_or_skip()
    from dirac_caspt2_gb300 import dirac_io, synth
    S = synth.make_system(synth.SynthConfig(2, 2, 4, 1, seed=2))
    d = str(tmp_path / "case")
    synth.write_case_files(S, d)
    p = os.path.join(d, "MRCONEE")
    recs = dirac_io.read_fortran_records(p)
    with open(p, "wb") as f:
        for k, rec in enumerate(recs):
            if k == 5:
                a, b = rec[:40], rec[40:]
                f.write(struct.pack("<i", -len(a)) + a + struct.pack("<i", -len(a)))
                f.write(struct.pack("<i", len(b)) + b + struct.pack("<i", len(b)))
            else:
                f.write(struct.pack("<i", len(rec)) + rec + struct.pack("<i", len(rec)))
    inp = dirac_io.read_active_inp(os.path.join(d, "active.inp"))
    _compare(d, inp)


def test_native_errors(tmp_path):
    _lib_or_skip()
    from dirac_caspt2_gb300 import api, dirac_io, synth
    inp = dirac_io.ActiveInput(ninact=2, nact=2, nsec=4, nelec=1, ciroots=[(1, 1)], eshift=0.0, diracver=21)
    with pytest.raises(api.DcgError) as ei:
        api.NativeFiles(str(tmp_path / "missing"), inp)
    assert ei.value.code == -7 and "cannot open" in str(ei.value)
    S = synth.make_system(synth.SynthConfig(2, 2, 4, 1, seed=2))
    d = str(tmp_path / "case")
    synth.write_case_files(S, d)
    p = os.path.join(d, "MDCINT")
    data = open(p, "rb").read()
    open(p, "wb").write(data[:-7])
    with pytest.raises(api.DcgError) as ei:
        api.NativeFiles(d, inp)
    assert ei.value.code == -7 and "truncated" in str(ei.value)
    big = dirac_io.ActiveInput(ninact=2, nact=2, nsec=40, nelec=1, ciroots=[(1, 1)], eshift=0.0, diracver=21)
    with pytest.raises(api.DcgError) as ei:
        api.NativeFiles(d, big)
    assert ei.value.code == -1


def _ref_cases():
    if not os.path.isdir(REF_DEV):
        return []
    out = []
    for c in sorted(os.listdir(REF_DEV)):
        d = os.path.join(REF_DEV, c)
        inp = next((f for f in ("active.inp", "active.ivo.inp") if os.path.exists(os.path.join(d, f))), None)
        if inp and all(os.path.exists(os.path.join(d, f)) for f in ("MRCONEE", "MDCINT")):
            out.append((c, inp))
    return out


@pytest.mark.skipif(not os.path.isdir(REF_DEV), reason="reference test tree not mounted")
@pytest.mark.parametrize("case,inpname", _ref_cases())
def test_native_matches_python_reference_inputs(case, inpname):
    _lib_or_skip()
    from dirac_caspt2_gb300 import dirac_io
    d = os.path.join(REF_DEV, case)
    inp = dirac_io.read_active_inp(os.path.join(d, inpname))
    _compare(d, inp)


def _mrconee_cases():
    out = []
    for top in ("dev", "slow", "unmarked"):
        base = os.path.join(os.path.dirname(REF_DEV), top)
        if not os.path.isdir(base):
            continue
        for c in sorted(os.listdir(base)):
            d = os.path.join(base, c)
            inp = next((f for f in ("active.inp", "active.ivo.inp") if os.path.exists(os.path.join(d, f))), None)
            if inp and os.path.exists(os.path.join(d, "MRCONEE")):
                out.append((top + "/" + c, inp))
    return out


@pytest.mark.skipif(not os.path.isdir(REF_DEV), reason="reference test tree not mounted")
@pytest.mark.parametrize("case,inpname", _mrconee_cases())
def test_native_mrconee_reference_inputs(case, inpname):
    """Every MRCONEE of the reference's tests (32- and 64-bit DIRAC builds, symmetry and C1,
    RAS inputs) reads the same through both readers."""
    _lib_or_skip()
    from dirac_caspt2_gb300 import api, dirac_io
    d = os.path.join(os.path.dirname(REF_DEV), case)
    inp = dirac_io.read_active_inp(os.path.join(d, inpname))
    py_m = dirac_io.read_mrconee(os.path.join(d, "MRCONEE"), inp)
    with api.NativeFiles(d, inp, mdcint=False) as nf:
        m = nf.mrconee()
    assert m.dirac_32bit == py_m.dirac_32bit and m.nmo == py_m.nmo and m.ecore == py_m.ecore
    for f in ("multb", "irpamo", "mo_energy", "h"):
        assert np.array_equal(getattr(m, f), getattr(py_m, f)), f
    assert np.array_equal(m.cas_to_dirac[1:], py_m.cas_to_dirac[1:])
