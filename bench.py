"""Benchmark: CASPT2 solves/s on one GB300 (or N independent replicas).

One step = one complete CASCI + CASPT2 solve (integral expansion, CASCI matrix and
eigensolve, Fock build and diagonalisation, CI rotation, densities, 4-index
transformation and the eight subspaces A-H) of the seeded synthetic system
20 inactive / 12 active (6 electrons) / 300 secondary Kramers-paired complex spinors,
CASCI root 1.

  value  : solves/s with the MDCINTNEW records already resident in HBM (device pointers)
  e2e    : solves/s through the public C-ABI call with pinned host buffers; every step
           copies the records and one-electron data host->device and reads the energies back
  cpu_baseline / --impl reference : the CPU restatement of the reference algorithm
           (numpy + the host BLAS, all host cores), the reference's Fortran being unbuildable
           here (no Fortran compiler)

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

CONFIG = "cas_20_12_300"
ROOFLINE_FAMILY = "transform"
PEAKS_FILE = os.path.join(HERE, "MEASURED_PEAKS.json")
FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    try:
        p = json.load(open(PEAKS_FILE))
        return p, "measured"
    except (OSError, ValueError):
        return FALLBACK_PEAKS, "fallback"


def cpu_oracle_solve(S, cfg):
    """One full solve of the CPU restatement (test infrastructure; baseline only)."""
    from oracle import caspt2_oracle as O
    s = O.System(ninact=cfg.ninact, nact=cfg.nact, nsec=cfg.nsec, nelec=cfg.nelec, nmo=S.nmo, nsymrpa=1,
                 multb=S.multb, irpamo=S.irpamo, h=S.h, ecore=S.ecore, rec_idx=S.rec_idx, rec_val=S.rec_val,
                 realonly=cfg.realonly)
    t = time.perf_counter()
    r = O.run(s)
    return time.perf_counter() - t, r


def run_reference(args, cfg_name):
    """Reference arm: the CPU restatement of the reference's FP64 algorithm on the host cores."""
    rank, world, local = _dist()
    if rank != 0:
        return 0
    from dirac_caspt2_gb300 import synth
    cfg = synth.CONFIGS[cfg_name]
    S = synth.make_system(cfg)
    times = []
    for k in range(args.warmup + args.steps):
        dt, r = cpu_oracle_solve(S, cfg)
        if k >= args.warmup:
            times.append(dt)
    mean = sum(times) / len(times)
    cores = os.cpu_count()
    value = 1.0 / mean
    line = {"impl": "reference", "metric": "caspt2_solves_per_s", "value": value, "unit": "solves/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64)",
            "data": "synthetic (seeded Kramers-paired complex spinor system)",
            "config": {"workload": cfg_name, "ninact": cfg.ninact, "nact": cfg.nact, "nsec": cfg.nsec,
                       "nelec": cfg.nelec, "root": 1, "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": f"full CASCI+CASPT2 solve of {cfg_name} by the numpy restatement "
                                       "of the reference (oracle/), host BLAS threads = all cores"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "p50_ms": float(np.percentile(np.array(times) * 1e3, 50)),
            "p99_ms": float(np.percentile(np.array(times) * 1e3, 99)),
            "total_energy": r.total_energy}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, cfg_name):
    import torch
    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="gloo")
    torch.cuda.set_device(local)
    from dirac_caspt2_gb300 import api, build, synth
    build.build()
    cfg = synth.CONFIGS[cfg_name]
    S = synth.make_system(cfg)
    sin = api.SystemInput.from_synth(S)
    prec = api.DCG_PREC_SPLIT if args.precision == "split" else api.DCG_PREC_FP64
    ses = api.Caspt2Session(local, prec)
    stream = torch.cuda.ExternalStream(ses.stream_ptr, device=local)

    # host buffers in page-locked memory (e2e leg) and device-resident copies (value leg)
    hb_host = api.HostBuffers(sin)
    pin = {}
    for nm in ("ijkl", "re", "im"):
        a = getattr(hb_host, nm)
        if a is not None:
            pin[nm] = torch.from_numpy(a).pin_memory()
            setattr(hb_host, nm, pin[nm].numpy())
    hb_host.rebind()
    dev = {nm: t.to(f"cuda:{local}") for nm, t in pin.items()}
    torch.cuda.synchronize()
    hb_dev = api.HostBuffers(sin)
    hb_dev.use_device_records(dev["ijkl"].data_ptr(), dev["re"].data_ptr(),
                              dev["im"].data_ptr() if "im" in dev else 0)
    hb = hb_host

    def one(bufs):
        ses.set_system(sin, bufs)
        ses.casci(1)
        return ses.caspt2(0)

    # warm-up (allocations, module load)
    for _ in range(args.warmup):
        ref = one(hb_dev)
    e_ref = ref[3]

    def timed(bufs, family=None):
        if family:
            ses.time_family(family)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        launches = 0
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()
        clk = ClockSampler(local)
        clk.start()
        energies = []
        t0 = time.perf_counter()
        for k in range(args.steps):
            ev[k][0].record(stream)
            r = one(bufs)
            ev[k][1].record(stream)
            launches += ses.kernel_launches()
            energies.append(r[3])
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        clocks = clk.stop()
        per = [a.elapsed_time(b) for a, b in ev]
        fam = ses.family_stats() if family else None
        if family:
            ses.time_family("none")
        return per, wall, launches, clocks, energies, fam

    per_v, wall_v, launches_v, clocks_v, en_v, fam = timed(hb_dev, ROOFLINE_FAMILY)
    per_e, wall_e, launches_e, clocks_e, en_e, _ = timed(hb_host)
    tot_v = sum(per_v) / 1e3
    tot_e = sum(per_e) / 1e3
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([tot_v, tot_e], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_v, tot_e = float(t[0]), float(t[1])
    value = world * args.steps / tot_v
    e2e = world * args.steps / tot_e
    stage = ses.stage_ms()
    peaks, src = _peaks()
    # roofline of the dominant kernel family
    fam_ms, fam_launch, fam_work = fam
    per_launch_ms = fam_ms / max(1, fam_launch)
    if ROOFLINE_FAMILY in ("hstream", "scatter"):
        achieved = fam_work / (fam_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"]}
    else:
        achieved = fam_work / (fam_ms * 1e-3) / 1e12
        pk = peaks["bf16_tflops_sustained"]
        roof = {"bound": "tensor", "achieved": achieved, "peak": pk, "unit": "TFLOP/s", "frac": achieved / pk}
    roof.update({"traffic": None, "kernel_family": ROOFLINE_FAMILY, "launches_timed": fam_launch,
                 "mean_launch_ms": per_launch_ms, "peak_source": f"{src} ({'sustained' if roof['unit'] == 'TFLOP/s' else 'burst'})"})
    line = {"metric": "caspt2_solves_per_s", "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_v / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128 (f64)" if prec == api.DCG_PREC_FP64 else "c128 (split bf16 -> f64)",
            "data": "synthetic (seeded Kramers-paired complex spinor system; replicas only)",
            "config": {"workload": cfg_name, "ninact": cfg.ninact, "nact": cfg.nact, "nsec": cfg.nsec,
                       "nelec": cfg.nelec, "root": 1, "records": int(len(S.rec_val)),
                       "precision": args.precision, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (1 GB of records, 0.6 GB H class per step)"},
            "p50_ms": float(np.percentile(per_v, 50)), "p99_ms": float(np.percentile(per_v, 99)),
            "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": hb.h2d_bytes,
                    "d2h_bytes_per_step": 8 * (1 + 8 + 8 + 2), "p50_ms": float(np.percentile(per_e, 50)),
                    "p99_ms": float(np.percentile(per_e, 99))},
            "gpu_launches": int(launches_v),
            "clocks": clocks_v, "roofline": roof,
            "stage_ms_last_step": {k: round(v, 3) for k, v in stage.items()},
            "total_energy": e_ref, "energy_spread": float(max(en_v + en_e) - min(en_v + en_e))}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        dt, r = cpu_oracle_solve(S, cfg)
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"one full CASCI+CASPT2 solve of {cfg_name} by the numpy restatement "
                                          "(oracle/), host BLAS threads = all cores",
                                "abs_diff_total_energy": abs(r.total_energy - e_ref)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ses.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default=CONFIG)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "split"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args, args.config)
    return run_ours(args, args.config)


if __name__ == "__main__":
    sys.exit(main())
