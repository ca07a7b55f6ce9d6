"""C ABI: the library builds for sm_103a, loads, and exports every entry point the public
header declares (no compute calls: this runs without a GPU)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "dcaspt2_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dcg_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from dirac_caspt2_gb300 import build, api
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (dcg_\w+)", out))
    declared = _declared()
    assert declared, "no declarations found"
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    L = api.load_library()
    for s in declared:
        assert hasattr(L, s)
    assert set(api.EXPORTED_SYMBOLS) <= set(declared)


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    from dirac_caspt2_gb300 import api
    monkeypatch.setattr(api, "_lib", None)
    with pytest.raises(ImportError):
        api.load_library(str(tmp_path / "nope.so"))


def test_version_string_without_gpu():
    from dirac_caspt2_gb300 import api
    assert b"sm_103a" in api.load_library().dcg_version()


def test_autotune_table_without_gpu():
    """The tuner's mode and table are host state: readable without a device."""
    from dirac_caspt2_gb300 import api
    prev = api.autotune_mode(-1)
    assert prev in (0, 1)
    assert api.autotune_mode(0) == prev
    assert api.autotune_mode(-1) == 0
    api.autotune_mode(prev)
    assert isinstance(api.autotune_entries(), list)


def test_autotune_table_file_is_read(tmp_path, monkeypatch):
    """DCG_TUNE_FILE entries are loaded at the first lookup (in a fresh process)."""
    import subprocess
    import sys
    f = tmp_path / "tune.txt"
    f.write_text("1 0 792 300 1728 2 5 18 3.19 4.36\n2 1 43200 300 300 0 3 4 0.52 0.58\n")
    code = ("from dirac_caspt2_gb300 import api; e = api.autotune_entries(); "
            "print(len(e), sorted((x['kind'], x['m'], x['choice']) for x in e))")
    env = dict(os.environ, DCG_TUNE_FILE=str(f), PYTHONPATH=ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "2 [('fp64_gemm_tile_ksplit', 792, 5), ('split_gemm_kernel_raster', 43200, 3)]"
