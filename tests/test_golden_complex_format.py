"""The reference's runnable golden cases are all real-only (MDCINT realonly = T).  Their MDCINT
records rewritten in the complex record layout, with zero imaginary parts, make the reader
report a complex system (module_realonly.F90:29-77 decides by whether the first record parses
with imaginary parts).  On the host: the Python readers then see the same records with
realonly False, and the canonical MDCINTNEW stream (create_newmdcint.F90:171-321) carries the
golden values with zero imaginary parts; the real layout written back reproduces the fixture
exactly.  The GPU counterpart, tests/test_gpu_golden_complex.py, runs these directories through
the library's C++ readers and the full path."""
import os

import numpy as np
import pytest

from conftest import GOLDEN_CASES, GOLDEN_DIR
from test_mdcint import load_raw, write_case_dir


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_complex_layout_reads_as_complex(case, tmp_path):
    from dirac_caspt2_gb300 import dirac_io
    inp = write_case_dir(case, str(tmp_path), complex_layout=True)
    mrc = dirac_io.read_mrconee(str(tmp_path / "MRCONEE"), inp)
    raw = dirac_io.read_mdcint_raw(str(tmp_path), mrc, inp)
    ref = load_raw(case)
    assert ref.realonly and not raw.realonly
    for f in ("rec_ikr", "rec_jkr", "rec_off", "indk", "indl", "re", "kr", "dirac_to_cas"):
        assert np.array_equal(getattr(raw, f), getattr(ref, f)), f
    assert not np.any(raw.im)
    new = dirac_io.canonicalize_mdcint(raw)
    g = np.load(os.path.join(GOLDEN_DIR, f"{case}.npz"))
    assert np.array_equal(new.idx, g["rec_idx"].astype(np.int32))
    assert np.array_equal(new.val.real, g["rec_re"])
    assert not np.any(new.val.imag)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_real_layout_round_trip(case, tmp_path):
    from dirac_caspt2_gb300 import dirac_io
    inp = write_case_dir(case, str(tmp_path), complex_layout=False)
    mrc = dirac_io.read_mrconee(str(tmp_path / "MRCONEE"), inp)
    raw = dirac_io.read_mdcint_raw(str(tmp_path), mrc, inp)
    ref = load_raw(case)
    assert raw.realonly
    for f in ("rec_ikr", "rec_jkr", "rec_off", "indk", "indl", "re", "kr", "dirac_to_cas"):
        assert np.array_equal(getattr(raw, f), getattr(ref, f)), f
    assert raw.scheme == ref.scheme
