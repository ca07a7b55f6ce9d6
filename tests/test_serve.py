"""Host logic of the serving path without a GPU: Poisson arrivals and latency summaries, the
stream driver against a simulated single-slot server, the stream's size distribution, the
device generator's record set (run on the CPU) against the host generator, the ABI layout of
dcg_request_result / dcg_system against the C header, and the library's behaviour with no
GPU (errors, no crash)."""
import ctypes
import os
import subprocess
import threading
import time

import numpy as np
import pytest

from conftest import ROOT


def test_poisson_arrivals():
    from dirac_caspt2_gb300 import serve
    t = serve.poisson_arrivals(20000, 20.0, seed=3)
    assert t[0] == 0.0 and np.all(np.diff(t) >= 0)
    gaps = np.diff(t)
    assert abs(gaps.mean() - 0.05) < 0.05 * 0.03
    assert abs(gaps.std() - 0.05) < 0.05 * 0.05          # exponential: std = mean
    assert np.array_equal(t, serve.poisson_arrivals(20000, 20.0, seed=3))
    assert serve.poisson_arrivals(0, 20.0).size == 0


def test_latency_summary():
    from dirac_caspt2_gb300 import serve
    s = serve.latency_summary(np.arange(1, 101) / 1000.0)
    assert s["p50_ms"] == pytest.approx(50.5)
    assert s["p99_ms"] == pytest.approx(99.01)
    assert s["max_ms"] == pytest.approx(100.0)
    assert np.isnan(serve.latency_summary([])["p50_ms"])


class _FakeServer:
    """One slot, FIFO, fixed service time; results become pollable when their simulated end
    time has passed (the poll/pending contract of Caspt2Server)."""

    def __init__(self, service_s):
        self.svc = service_s
        self.lock = threading.Lock()
        self.end = 0.0
        self.out = []

    def clock(self):
        return time.perf_counter()

    def submit(self, rid, sysm):
        with self.lock:
            t = time.perf_counter()
            start = max(t, self.end)
            self.end = start + self.svc
            self.out.append((rid, t, start, self.end))

    def _ready(self):
        now = time.perf_counter()
        return [o for o in self.out if o[3] <= now]

    def poll(self, timeout_ms=0):
        from dirac_caspt2_gb300 import api
        deadline = time.perf_counter() + timeout_ms / 1000.0
        while True:
            with self.lock:
                ready = self._ready()
                if ready:
                    rid, ts, t0, t1 = ready[0]
                    self.out.remove(ready[0])
                    z = {k: 0.0 for k in api.SUBSPACES}
                    return api.ServedResult(rid, 0, 1, -1.0, dict(z), dict(z), 0.0, -1.0, ts, t0, t1, 0, 1)
            if time.perf_counter() >= deadline:
                return None
            time.sleep(0.001)

    def pending(self):
        with self.lock:
            now = time.perf_counter()
            q = sum(1 for o in self.out if o[2] > now)
            r = sum(1 for o in self.out if o[2] <= now < o[3])
            return q, r


def test_run_stream_with_simulated_server():
    from dirac_caspt2_gb300 import serve
    srv = _FakeServer(0.01)
    arr = serve.poisson_arrivals(30, 200.0, seed=1)
    rep = serve.run_stream(srv, [(k, None) for k in range(30)], arr, timeout_s=30)
    assert rep.requests == 30 and rep.failed == 0 and len(rep.results) == 30
    assert rep.service["p50_ms"] == pytest.approx(10.0, abs=1e-6)
    assert rep.latency["p50_ms"] >= 10.0 - 1e-6
    # a single 10 ms slot cannot exceed 100 solves/s, and the stream keeps it busy most of the time
    assert 30.0 < rep.solves_per_s <= 100.0 + 1e-6
    assert rep.max_running == 1


def test_max_concurrency():
    from dirac_caspt2_gb300 import serve
    assert serve.max_concurrency([]) == 0
    assert serve.max_concurrency([(0, 1), (1, 2), (2, 3)]) == 1      # touching intervals do not overlap
    assert serve.max_concurrency([(0, 3), (1, 2), (1.5, 4), (3.5, 5)]) == 3


def test_stream_configs():
    from dirac_caspt2_gb300 import synth_device as sd
    cfgs = sd.stream_configs(256, seed=0)
    assert len(cfgs) == 256
    assert {c.nact for c in cfgs} == {4, 6, 8, 10, 12}
    for c in cfgs:
        assert c.nelec == c.nact // 2
        assert 4 <= c.ninact <= 24 and c.ninact % 2 == 0
        assert 60 <= c.nsec <= 400 and c.nsec % 2 == 0
    assert len({c.seed for c in cfgs}) == 256
    assert [c.seed for c in cfgs] == [c.seed for c in sd.stream_configs(256, seed=0)]


@pytest.mark.parametrize("dims,realonly", [((4, 4, 10, 2), False), ((2, 6, 8, 3), False), ((4, 2, 6, 1), True)])
def test_device_generator_record_set(dims, realonly):
    """Same canonical record set as the host generator; values = sum_L B^L_pq B^L_rs of the
    generator's own factors; Hermitian, time-reversal-symmetric one-electron matrix."""
    import torch
    from dirac_caspt2_gb300 import synth, synth_device as sd
    cfg = synth.SynthConfig(*dims, realonly=realonly, seed=5)
    d = sd.make_system_device(cfg, "cpu", keep_factors=True)
    h = synth.make_system(cfg)
    assert np.array_equal(d.rec_idx.numpy(), h.rec_idx)
    B = d.B.numpy()
    g = np.einsum("Lpq,Lrs->pqrs", B, B)
    ix = d.rec_idx.numpy() - 1
    val = d.rec_re.numpy() + (0 if d.rec_im is None else 1j * d.rec_im.numpy())
    assert np.abs(val - g[ix[:, 0], ix[:, 1], ix[:, 2], ix[:, 3]]).max() < 1e-15
    assert (d.rec_im is None) == realonly
    assert np.abs(d.h - d.h.conj().T).max() == 0.0
    n = d.nmo
    t = np.array([(-1) ** (x + y) for x in range(1, n + 1) for y in range(1, n + 1)]).reshape(n, n)
    p = np.arange(n) ^ 1
    assert np.abs(d.h[np.ix_(p, p)] - t * d.h.conj()).max() < 1e-15
    assert d.rec_idx.dtype == torch.int32 and d.rec_idx.is_contiguous()


def test_device_generator_chunking(monkeypatch):
    """Contracting the blocks in first-index chunks gives the same records in the same order."""
    from dirac_caspt2_gb300 import synth, synth_device as sd
    cfg = synth.SynthConfig(6, 4, 12, 2, seed=2)
    a = sd.make_system_device(cfg, "cpu")
    monkeypatch.setattr(sd, "CHUNK_ELEMENTS", 100)
    b = sd.make_system_device(cfg, "cpu")
    assert a.nrec == b.nrec > 0
    assert np.array_equal(a.rec_idx.numpy(), b.rec_idx.numpy())
    assert np.array_equal(a.rec_re.numpy(), b.rec_re.numpy())
    assert np.array_equal(a.rec_im.numpy(), b.rec_im.numpy())


_LAYOUT_C = r"""
#include <stddef.h>
#include <stdio.h>
#include "dcaspt2_gb300.h"
#define P(T, f) printf(#T " " #f " %zu\n", offsetof(T, f))
int main(void) {
    printf("dcg_request_result size %zu\n", sizeof(dcg_request_result));
    P(dcg_request_result, request_id); P(dcg_request_result, status); P(dcg_request_result, ndet);
    P(dcg_request_result, casci_energy); P(dcg_request_result, e2); P(dcg_request_result, sumc2);
    P(dcg_request_result, e0); P(dcg_request_result, etotal); P(dcg_request_result, t_submit);
    P(dcg_request_result, t_start); P(dcg_request_result, t_end); P(dcg_request_result, slot);
    P(dcg_request_result, attempts); P(dcg_request_result, error);
    printf("dcg_system size %zu\n", sizeof(dcg_system));
    P(dcg_system, eshift); P(dcg_system, multb); P(dcg_system, nrec); P(dcg_system, rec_im);
    P(dcg_system, ras1_size); P(dcg_system, rec_on_device);
    return 0;
}
"""


def test_abi_layout_matches_header(tmp_path):
    """ctypes mirrors of dcg_request_result and dcg_system have the C layout of the header."""
    from dirac_caspt2_gb300 import api
    src = tmp_path / "layout.c"
    src.write_text(_LAYOUT_C)
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    types = {"dcg_request_result": api._RequestResult, "dcg_system": api._System}
    checked = 0
    for line in filter(None, out):
        t, f, v = line.split()
        if f == "size":
            assert ctypes.sizeof(types[t]) == int(v), line
        else:
            assert getattr(types[t], f).offset == int(v), line
        checked += 1
    assert checked == 22


def test_footprint_estimate_host_only():
    """dcg_footprint_estimate needs no GPU: positive and growing with each dimension."""
    from dirac_caspt2_gb300 import api, synth
    lib = api.load_library()
    base = api.SystemInput.from_synth(synth.make_system(synth.SynthConfig(4, 4, 10, 2, seed=0)))

    def est(**kw):
        b = api.HostBuffers(base)
        for k, v in kw.items():
            setattr(b.struct, k, v)
        return api.footprint_estimate(b)

    e0 = est()
    assert e0 > 0
    assert est(nsec=300) > e0 and est(ninact=20) > e0 and est(nact=10, nelec=5) > e0 and est(nrec=10**8) > e0
    assert lib.dcg_footprint_estimate(None) == -1


def test_server_without_gpu_fails_cleanly():
    """With no usable CUDA device the server is not created and says so (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from dirac_caspt2_gb300 import api
    with pytest.raises(api.DcgError):
        api.Caspt2Server(0, api.DCG_PREC_FP64, slots=2)
    lib = api.load_library()
    assert lib.dcg_server_create(0, 0, 0, 0, ctypes.byref(ctypes.c_void_p())) == -1   # slots < 1
    assert lib.dcg_server_destroy(None) == -1
