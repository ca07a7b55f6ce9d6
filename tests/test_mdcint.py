"""MDCINT -> MDCINTNEW on the host (dirac_io.canonicalize_mdcint, the restatement of
create_newmdcint.F90:171-321): on the raw MDCINT records of two reference test cases
(tests/golden/*_mdcint_raw.npz: a scheme other than 6, with the bra/ket-exchanged copies;
ninact = 0) it reproduces the MDCINTNEW stream stored with their golden energies, exactly; and
the ABI layout of dcg_mdcint_raw matches the C header."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN_DIR, ROOT

RAW_CASES = ["check_minelecras3_dev", "ninact_0_h2_dev"]


def load_raw(case):
    from dirac_caspt2_gb300 import dirac_io
    z = np.load(os.path.join(GOLDEN_DIR, f"{case}_mdcint_raw.npz"))
    return dirac_io.MdcintRaw(rec_ikr=z["rec_ikr"], rec_jkr=z["rec_jkr"], rec_off=z["rec_off"], indk=z["indk"],
                              indl=z["indl"], re=z["re"], im=z["im"], kr=z["kr"], nmo=int(z["nmo"]),
                              dirac_to_cas=z["dirac_to_cas"], scheme=int(z["scheme"]), realonly=bool(z["realonly"]))


def write_case_dir(case, directory, complex_layout):
    """The case's run directory rebuilt from its fixture: MRCONEE and active.inp as the reference
    ships them, MDCINT rewritten as one file in the real-only or the complex record layout."""
    from dirac_caspt2_gb300 import dirac_io
    z = np.load(os.path.join(GOLDEN_DIR, f"{case}_mdcint_raw.npz"))
    os.makedirs(directory, exist_ok=True)
    open(os.path.join(directory, "MRCONEE"), "wb").write(z["mrconee"].tobytes())
    open(os.path.join(directory, "active.inp"), "w").write(str(z["active_inp"]))
    dirac_io.write_mdcint_raw(os.path.join(directory, "MDCINT"), load_raw(case), bool(z["dirac_32bit"]),
                              realonly=not complex_layout)
    return dirac_io.read_active_inp(os.path.join(directory, "active.inp"))


@pytest.mark.parametrize("case", RAW_CASES)
def test_host_canonicalisation_reproduces_golden_stream(case):
    from dirac_caspt2_gb300 import dirac_io
    raw = load_raw(case)
    new = dirac_io.canonicalize_mdcint(raw)
    g = np.load(os.path.join(GOLDEN_DIR, f"{case}.npz"))
    assert np.array_equal(new.idx, g["rec_idx"].astype(np.int32))
    assert np.array_equal(new.val.real, g["rec_re"])
    if "rec_im" in g.files:
        assert np.array_equal(new.val.imag, g["rec_im"])
    assert raw.scheme != 6 or case == "ninact_0_h2_dev"


def test_mdcint_raw_layout(tmp_path):
    from dirac_caspt2_gb300 import api
    src = tmp_path / "l.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "dcaspt2_gb300.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu\\n", sizeof(dcg_mdcint_raw), '
                   'offsetof(dcg_mdcint_raw, nkr), offsetof(dcg_mdcint_raw, kr), '
                   'offsetof(dcg_mdcint_raw, scheme), offsetof(dcg_mdcint_raw, realonly));return 0;}\n')
    exe = tmp_path / "l"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    T = api._MdcintRaw
    assert got == [ctypes.sizeof(T), T.nkr.offset, T.kr.offset, T.scheme.offset, T.realonly.offset]
