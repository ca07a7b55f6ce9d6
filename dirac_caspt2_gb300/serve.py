"""Served CASPT2 request streams: Poisson arrivals into the library's serving loop.

``run_stream`` submits requests to a ``Caspt2Server`` at their arrival times (a submitter
thread sleeps until each one), collects the results as the slots finish them and reports the
latency percentiles (submit to finish, queueing included) beside the solves/s of the stream
(requests / (last finish - first submit)).

    python -m dirac_caspt2_gb300.serve --requests 256 --rate 20 --slots 4 --precision split

generates the stream's systems on the device (``synth_device``; sizes from per-request seeds:
active spinors in {4, 6, 8, 10, 12} half filled, inactive 4-24, secondary 60-400), keeps
their records in HBM, runs the stream and prints one JSON line.  ``--check-alone K`` then
re-runs K of the requests one at a time on an idle server and reports the largest difference
between each result alone and in the mix.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import sys
import threading
import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import api

__all__ = ["poisson_arrivals", "latency_summary", "StreamReport", "run_stream", "max_concurrency",
           "max_result_difference"]


def poisson_arrivals(n: int, rate_hz: float, seed: int = 0) -> np.ndarray:
    """Arrival offsets (s) of n requests of a Poisson process with the given mean rate:
    cumulative sums of exponential gaps, the first request at 0."""
    if n <= 0:
        return np.zeros(0)
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, n)
    gaps[0] = 0.0
    return np.cumsum(gaps)


def latency_summary(lat_s: Sequence[float]) -> Dict[str, float]:
    """p50 / p99 / mean / max of latencies given in seconds, in milliseconds."""
    a = np.asarray(lat_s, dtype=np.float64) * 1e3
    if a.size == 0:
        return {"p50_ms": float("nan"), "p99_ms": float("nan"), "mean_ms": float("nan"), "max_ms": float("nan")}
    return {"p50_ms": float(np.percentile(a, 50)), "p99_ms": float(np.percentile(a, 99)),
            "mean_ms": float(a.mean()), "max_ms": float(a.max())}


@dataclasses.dataclass
class StreamReport:
    requests: int
    failed: int
    solves_per_s: float
    makespan_s: float
    latency: Dict[str, float]
    queue_wait: Dict[str, float]
    service: Dict[str, float]
    max_running: int
    results: Dict[int, api.ServedResult]

    @property
    def failures(self) -> List[Tuple[int, int, str]]:
        """(request id, status, message) of every failed request."""
        return [(r.request_id, r.status, r.error) for r in self.results.values() if r.status != 0]

    def summary(self) -> Dict[str, object]:
        return {"requests": self.requests, "failed": self.failed, "failures": self.failures[:8],
                "solves_per_s": self.solves_per_s,
                "makespan_s": self.makespan_s, **self.latency,
                "queue_wait_p50_ms": self.queue_wait["p50_ms"], "queue_wait_p99_ms": self.queue_wait["p99_ms"],
                "service_p50_ms": self.service["p50_ms"], "service_p99_ms": self.service["p99_ms"],
                "max_running": self.max_running}


def run_stream(server: api.Caspt2Server, requests: Sequence[Tuple[int, object]], arrivals: Sequence[float],
               timeout_s: float = 600.0) -> StreamReport:
    """Submit requests[k] = (request_id, HostBuffers or SystemInput) at arrivals[k] seconds after
    the start and wait for all of them (at most timeout_s)."""
    n = len(requests)
    errors: List[BaseException] = []
    start = time.perf_counter()

    def submitter():
        try:
            for (rid, sysm), t in zip(requests, arrivals):
                delay = start + float(t) - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                server.submit(rid, sysm)
        except BaseException as e:   # surfaced to the caller below
            errors.append(e)

    th = threading.Thread(target=submitter, daemon=True)
    th.start()
    results: Dict[int, api.ServedResult] = {}
    deadline = time.perf_counter() + timeout_s
    while len(results) < n and not errors:
        r = server.poll(50)
        if r is not None:
            results[r.request_id] = r
        if time.perf_counter() > deadline:
            raise TimeoutError(f"served stream: {len(results)} of {n} requests finished in {timeout_s} s")
    th.join()
    if errors:
        raise errors[0]
    rs = list(results.values())
    ok = [r for r in rs if r.status == 0]
    t0 = min(r.t_submit for r in rs)
    t1 = max(r.t_end for r in rs)
    return StreamReport(requests=n, failed=n - len(ok), solves_per_s=len(ok) / (t1 - t0) if t1 > t0 else float("inf"),
                        makespan_s=t1 - t0, latency=latency_summary([r.latency for r in ok]),
                        queue_wait=latency_summary([r.t_start - r.t_submit for r in ok]),
                        service=latency_summary([r.t_end - r.t_start for r in ok]),
                        max_running=max_concurrency([(r.t_start, r.t_end) for r in rs]), results=results)


def max_concurrency(spans: Sequence[Tuple[float, float]]) -> int:
    """Largest number of [start, end) intervals that overlap at one instant."""
    ev = sorted([(a, 1) for a, _ in spans] + [(b, -1) for _, b in spans], key=lambda x: (x[0], x[1]))
    cur = best = 0
    for _, d in ev:
        cur += d
        best = max(best, cur)
    return best


def max_result_difference(a: api.ServedResult, b: api.ServedResult) -> float:
    """Largest absolute difference of the energies of two results of the same request."""
    d = [abs(a.casci_energy - b.casci_energy), abs(a.e0 - b.e0), abs(a.total_energy - b.total_energy)]
    d += [abs(a.e2[k] - b.e2[k]) for k in api.SUBSPACES]
    d += [abs(a.sumc2[k] - b.sumc2[k]) for k in api.SUBSPACES]
    return float(max(d))


def main(argv: Optional[Sequence[str]] = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--requests", type=int, default=256)
    ap.add_argument("--rate", type=float, default=20.0, help="mean arrivals per second")
    ap.add_argument("--slots", default="4", help="slot counts to run the stream with, comma separated")
    ap.add_argument("--precision", default="split", help="fp64, split or both (comma separated)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--hbm-budget-gb", type=float, default=0.0, help="0: 90%% of the free memory after generation")
    ap.add_argument("--max-nsec", type=int, default=400)
    ap.add_argument("--check-alone", type=int, default=0)
    ap.add_argument("--warmup", type=int, default=2, help="requests per slot run before the stream (untimed)")
    a = ap.parse_args(argv)
    import torch
    from . import synth_device as sd
    cfgs = sd.stream_configs(a.requests, a.seed, nsec_range=(60, a.max_nsec))
    t0 = time.perf_counter()
    systems = [sd.make_system_device(c, "cuda") for c in cfgs]
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    gen_s = time.perf_counter() - t0
    bufs = [s.buffers() for s in systems]
    rec_gb = sum(s.record_bytes for s in systems) / 1e9
    arrivals = poisson_arrivals(a.requests, a.rate, a.seed + 1)
    failed = 0
    for prec_name in a.precision.split(","):
        prec = api.DCG_PREC_SPLIT if prec_name == "split" else api.DCG_PREC_FP64
        for slots in (int(x) for x in a.slots.split(",")):
            with api.Caspt2Server(0, prec, slots, int(a.hbm_budget_gb * 1e9)) as srv:
                nw = min(a.warmup * slots, len(bufs))   # warm the slots' workspaces and kernels
                for k in range(nw):
                    srv.submit(2**40 + k, bufs[k])
                for _ in range(nw):
                    while srv.poll(1000) is None:
                        pass
                rep = run_stream(srv, list(enumerate(bufs)), arrivals)
                out = {"stream": "poisson", "rate_hz": a.rate, "slots": slots, "precision": prec_name,
                       "generate_s": round(gen_s, 2), "resident_record_gb": round(rec_gb, 2),
                       "server_device_gb": round(srv.device_bytes() / 1e9, 2), **rep.summary()}
                if a.check_alone > 0:
                    worst = 0.0
                    for k in range(min(a.check_alone, a.requests)):
                        srv.submit(10**6 + k, bufs[k])
                        r = None
                        while r is None:
                            r = srv.poll(1000)
                        worst = max(worst, max_result_difference(r, rep.results[k]))
                    out["alone_vs_mix_max_abs_diff"] = worst
                    out["alone_checked"] = min(a.check_alone, a.requests)
            failed += rep.failed
            print(json.dumps(out), flush=True)
    return 0 if failed == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
