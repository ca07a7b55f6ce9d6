"""bench.py reads DRAM traffic figures from the ncu summaries under profiles/ (the
`traffic_bytes_per_launch = N` lines) for its roofline objects: each summary it names must
exist and carry that line."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_split_family_traffic_is_recorded():
    b = _bench()
    t = b._traffic("split_mma", b.CONFIG)
    assert isinstance(t, int) and t > 0


def test_dominant_kernel_traffic_is_recorded():
    b = _bench()
    for fam in ("eig_tri", "eig_back"):
        t = b._dominant_traffic(fam)
        assert isinstance(t, int) and t > 0, fam
    assert b._dominant_traffic("hstream") is None
