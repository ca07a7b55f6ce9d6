"""DIRAC readers: MRCONEE/MDCINT -> MDCINTNEW restatement, active.inp parser, Fortran
record layout, against synthetic files and (when present) the reference's test inputs."""
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN_DIR

REF_DEV = "/root/reference/test/dev"


def test_fortran_records_roundtrip(tmp_path):
    from dirac_caspt2_gb300 import dirac_io
    recs = [b"abc", b"", bytes(range(256)) * 10]
    p = str(tmp_path / "f.bin")
    dirac_io.write_fortran_records(p, recs)
    assert dirac_io.read_fortran_records(p) == recs


def test_active_inp_parser():
    from dirac_caspt2_gb300 import dirac_io
    txt = ".ninact\n6\n.nact\n6\n.nsec\n2\n.nelec\n2\n.caspt2_ciroots\n33 1 2\n.subprograms\nCASCI\nCASPT2\n" \
          ".diracver\n23\n.ras1\n3..4\n2\n.ras2\n9..10\n.ras3\n11..12\n2\n.minelecras3\n1\n.end\n"
    a = dirac_io.read_active_inp(txt)
    assert (a.ninact, a.nact, a.nsec, a.nelec) == (6, 6, 2, 2)
    assert a.ciroots == [(33, 1), (33, 2)]
    assert a.ras1 == [3, 4] and a.ras1_max_hole == 2 and a.ras3 == [11, 12] and a.ras3_max_elec == 2
    assert a.min_elec_ras3 == 1 and a.mdcint_scheme == 4   # DIRAC >= 23 default scheme
    b = dirac_io.read_active_inp(a.to_text())
    assert b.ras2 == [9, 10] and b.ciroots == a.ciroots


@pytest.mark.parametrize("realonly", [False, True])
def test_synthetic_files_roundtrip(tmp_path, realonly):
    """Files written for a synthetic system read back to the same MDCINTNEW records
    (records whose value is exactly zero are dropped by the 0.25e-12 write cutoff)."""
    from dirac_caspt2_gb300 import dirac_io, synth
    S = synth.make_system(synth.SynthConfig(4, 4, 6, 2, seed=3, realonly=realonly))
    d = str(tmp_path / "case")
    synth.write_case_files(S, d)
    inp = dirac_io.read_active_inp(os.path.join(d, "active.inp"))
    mrc = dirac_io.read_mrconee(os.path.join(d, "MRCONEE"), inp)
    new = dirac_io.read_mdcint_new(d, mrc, inp)
    assert new.realonly == realonly
    assert np.abs(mrc.h - S.h).max() == 0.0
    a = {tuple(r): v for r, v in zip(S.rec_idx.tolist(), S.rec_val) if abs(v) > 0.25e-12}
    b = {tuple(r): v for r, v in zip(new.idx.tolist(), new.val)}
    assert set(a) == set(b)
    assert max(abs(a[k] - b[k]) for k in a) == 0.0


@pytest.mark.skipif(not os.path.isdir(REF_DEV), reason="reference test tree not mounted")
@pytest.mark.parametrize("case", ["c2_h2o_dev", "check_minelecras3_dev", "ninact_0_h2_dev"])
def test_readers_match_fixture(case):
    """The committed fixtures are what the readers produce from the reference's inputs."""
    from dirac_caspt2_gb300 import dirac_io
    d = os.path.join(REF_DEV, case)
    inp = dirac_io.read_active_inp(os.path.join(d, "active.inp"))
    mrc = dirac_io.read_mrconee(os.path.join(d, "MRCONEE"), inp)
    new = dirac_io.read_mdcint_new(d, mrc, inp)
    z = np.load(os.path.join(GOLDEN_DIR, f"{case}.npz"))
    assert np.array_equal(new.idx, z["rec_idx"].astype(np.int32))
    assert np.array_equal(new.val.real, z["rec_re"])
    assert np.array_equal(mrc.irpamo, z["irpamo"])
