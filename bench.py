"""Benchmark: CASPT2 solves/s on one GB300 (or N independent replicas).

One step = one complete CASCI + CASPT2 solve (integral expansion, CASCI matrix and
eigensolve, Fock build and diagonalisation, CI rotation, densities, 4-index
transformation and the eight subspaces A-H) of the seeded synthetic system
20 inactive / 12 active (6 electrons) / 300 secondary Kramers-paired complex spinors,
CASCI root 1.

  value  : solves/s of the split-precision path (transformation on BF16 tensor cores, FP64
           recombination) with the MDCINTNEW records already resident in HBM (device pointers)
  fp64_gpu : the plain FP64 GPU path on the same system, and |dE2| between the two paths
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
REF_BUDGET_S = 150.0   # reference arm: stop adding CPU solves past this much time


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


_FP64_PEAK = {}


def fp64_gemm_peak(local, n=4096, reps=5):
    """Measured FP64 rate of this GPU: a cuBLAS DGEMM of n x n x n through torch, timed with
    CUDA events after two warm-up products (MEASURED_PEAKS.json carries no FP64 figure).
    Measured once per process."""
    if local in _FP64_PEAK:
        return _FP64_PEAK[local]
    import torch
    dev = f"cuda:{local}"
    g = torch.Generator(device=dev).manual_seed(0)
    a = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
    b = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
    for _ in range(2):
        c = a @ b
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        c = a @ b
    e1.record()
    torch.cuda.synchronize()
    del a, b, c
    _FP64_PEAK[local] = 2.0 * n ** 3 * reps / (e0.elapsed_time(e1) * 1e-3) / 1e12
    return _FP64_PEAK[local]


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
    """Reference arm: the CPU restatement of the reference's FP64 algorithm (oracle/) on the
    host cores.  One step is one full solve of the workload.  A CPU solve has no warm-up state,
    so the warm-up steps are not run, and steps stop once REF_BUDGET_S of solves have
    accumulated (at least one); the line states how many ran."""
    rank, world, local = _dist()
    if rank != 0:
        return 0
    from dirac_caspt2_gb300 import synth
    cfg = synth.CONFIGS[cfg_name]
    S = synth.make_system(cfg)
    times = []
    r = None
    for k in range(max(1, args.steps)):
        dt, r = cpu_oracle_solve(S, cfg)
        times.append(dt)
        if sum(times) > REF_BUDGET_S:
            break
    mean = sum(times) / len(times)
    cores = os.cpu_count()
    value = 1.0 / mean
    line = {"impl": "reference", "metric": "caspt2_solves_per_s", "value": value, "unit": "solves/s",
            "n_gpus": args.gpus, "steps": len(times), "steps_requested": args.steps, "warmup": 0,
            "warmup_requested": args.warmup, "ms_per_step": mean * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64)",
            "data": "synthetic (seeded Kramers-paired complex spinor system)",
            "config": {"workload": cfg_name, "ninact": cfg.ninact, "nact": cfg.nact, "nsec": cfg.nsec,
                       "nelec": cfg.nelec, "root": 1, "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": f"{len(times)} full CASCI+CASPT2 solve(s) of {cfg_name} by the numpy "
                                       "restatement of the reference (oracle/); host BLAS threads = all cores; "
                                       "the reference's Fortran needs a Fortran compiler absent here"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "p50_ms": float(np.percentile(np.array(times) * 1e3, 50)),
            "p99_ms": float(np.percentile(np.array(times) * 1e3, 99)),
            "total_energy": r.total_energy}
    print(json.dumps(line), flush=True)
    return 0


def _traffic(family, cfg_name):
    """DRAM bytes per launch of the family, from the ncu capture summarised under profiles/
    (dram__bytes_read.sum + dram__bytes_write.sum, mean over one solve's launches)."""
    import re
    if family != "split_mma":
        return None
    p = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", f"launch_list_{cfg_name}_split.md")
    if not os.path.exists(p):
        return None
    m = re.search(r"^traffic_bytes_per_launch = (\d+)", open(p).read(), re.M)
    return int(m.group(1)) if m else None


def _dominant_traffic(family):
    """DRAM bytes of one launch of the FP64 eigensolver family's kernel, from its ncu summary
    under profiles/ (dram__bytes_read.sum + dram__bytes_write.sum)."""
    import re
    name = {"eig_tri": "tridiag_smem_kernel_n792.md", "eig_back": "backtransform_reg_kernel_n792.md"}.get(family)
    if not name:
        return None
    p = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", name)
    if not os.path.exists(p):
        return None
    m = re.search(r"^traffic_bytes_per_launch = (\d+)", open(p).read(), re.M)
    return int(m.group(1)) if m else None


def run_ours(args, cfg_name):
    import torch
    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="gloo")
    torch.cuda.set_device(local)
    from dirac_caspt2_gb300 import api, build, replicas, synth
    build.build()
    cfg = synth.CONFIGS[cfg_name]
    S = synth.make_system(cfg)
    sin = api.SystemInput.from_synth(S)
    prec = api.DCG_PREC_SPLIT if args.precision == "split" else api.DCG_PREC_FP64
    family = args.roofline_family or ("split_mma" if prec == api.DCG_PREC_SPLIT else "transform")
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

    def one(session, bufs):
        session.set_system(sin, bufs)
        eig, _ = session.casci(1)
        e2, sc2, e0, etot = session.caspt2(0)
        return eig[0], e2, etot

    def timed(session, bufs, steps, fam=None):
        strm = torch.cuda.ExternalStream(session.stream_ptr, device=local)
        if fam:
            session.time_family(fam)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        launches = 0
        replicas.barrier()
        torch.cuda.synchronize()
        clk = ClockSampler(local)
        clk.start()
        results = []
        for k in range(steps):
            ev[k][0].record(strm)
            results.append(one(session, bufs))
            ev[k][1].record(strm)
            launches += session.kernel_launches()
        torch.cuda.synchronize()
        clocks = clk.stop()
        per = [x.elapsed_time(y) for x, y in ev]
        stats = session.family_stats() if fam else None
        if fam:
            session.time_family("none")
        return per, launches, clocks, results, stats

    for _ in range(args.warmup):          # allocations, module load
        one(ses, hb_dev)
    per_v, launches_v, clocks_v, res_v, fam = timed(ses, hb_dev, args.steps, family)
    one(ses, hb_host)                      # untimed: the host-buffer path's record buffers
    per_e, _, clocks_e, res_e, _ = timed(ses, hb_host, args.steps)
    stage = ses.stage_ms()
    tot_v = sum(per_v) / 1e3
    tot_e = sum(per_e) / 1e3

    # end to end through the serving loop: the same host-buffer requests on four slots, so one
    # request's host-to-device copy and set-up overlap the others' solves (each request still
    # copies its records from pinned host memory and reads its energies back)
    def e2e_served(steps, slots=4):
        srv = api.Caspt2Server(local, prec, slots=slots)
        try:
            for k in range(slots):   # slot workspaces
                srv.submit(k, hb_host)
            for _ in range(slots):
                r = srv.poll(600000)
                if r is None or r.status != 0:
                    raise RuntimeError(f"served e2e warm-up failed: {None if r is None else r.error}")
            replicas.barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for k in range(steps):
                srv.submit(100 + k, hb_host)
            got = []
            while len(got) < steps:
                r = srv.poll(600000)
                if r is None:
                    raise RuntimeError("served e2e: no result within 600 s")
                if r.status != 0:
                    raise RuntimeError(f"served e2e request failed: {r.error}")
                got.append(r)
            return time.perf_counter() - t0, got
        finally:
            srv.close()

    # enough requests that the slots stay busy well past the first and the last one
    e2e_steps = max(args.steps, args.e2e_requests)
    tot_s, res_s = e2e_served(e2e_steps, args.e2e_slots)

    # every kernel family timed live on two more steps each, against the roofline that bounds it:
    # the BF16 tensor pipe (measured sustained peak), HBM (measured copy bandwidth) or the FP64
    # pipe (a cuBLAS DGEMM measured here, beside the nominal 152 SMs x 2 FMA per clock x 2.07 GHz:
    # MEASURED_PEAKS.json holds no FP64 figure)
    fp64_nominal = 152 * 4 * 2.070e-3   # TF/s
    fp64_meas = fp64_gemm_peak(local)
    peaks0, src0 = _peaks()
    fam_spec = {   # family: (bound, work unit, what the work counts)
        "split_mma": ("tensor", "flop", "BF16 tensor FLOPs of the 15 slice products"),
        "transform": ("fp64", "flop", "FP64-equivalent FLOPs of the 4-index transformation (complex MAC = 8)"),
        "rdm": ("fp64", "flop", "FP64-equivalent FLOPs of the density GEMMs"),
        "hstream": ("hbm", "byte", "bytes the H-subspace sum must read (the a > b half of the H class)"),
        "scatter": ("hbm", "byte", "record bytes the integral expansion reads"),
        "eig_tri": ("fp64", "flop", "Householder reduction, (16/3) n^3 per matrix (tridiagonal or band form)"),
        "eig_val": ("fp64", "flop", "tridiagonal divide and conquer, (4/3) n^3 per matrix"),
        "eig_back": ("fp64", "flop", "eigenvector back-transformation, 8 n^2 m"),
    }
    fam_live = {}
    for fname, (bound, unit, what) in fam_spec.items():
        if fname == "split_mma" and prec != api.DCG_PREC_SPLIT:
            continue
        _, _, _, _, st = timed(ses, hb_dev, 2, fname)
        f_ms, f_launch, f_work = st
        if not f_launch or f_ms <= 0:
            continue
        ent = {"bound": bound, "ms_per_step": f_ms / 2, "launches_per_step": f_launch / 2, "work": what}
        if unit == "byte":
            ach = f_work / (f_ms * 1e-3) / 1e9
            ent.update({"achieved": ach, "unit": "GB/s", "peak": peaks0["hbm_gbs"],
                        "frac": ach / peaks0["hbm_gbs"], "peak_source": f"{src0} (copy bandwidth)"})
        elif bound == "tensor":
            ach = f_work / (f_ms * 1e-3) / 1e12
            pk = peaks0["bf16_tflops_sustained"]
            ent.update({"achieved": ach, "unit": "TFLOP/s", "peak": pk, "frac": ach / pk,
                        "peak_source": f"{src0} (bf16 sustained)"})
        else:
            ach = f_work / (f_ms * 1e-3) / 1e12
            ent.update({"achieved": ach, "unit": "TFLOP/s", "peak": fp64_meas, "frac": ach / fp64_meas,
                        "peak_source": "measured (cuBLAS DGEMM 4096^3 in this process)",
                        "frac_of_nominal": ach / fp64_nominal})
        fam_live[fname] = ent

    # plain FP64 GPU path on the same system: the comparison the metric names
    fp64 = None
    if prec == api.DCG_PREC_SPLIT and not args.no_fp64_compare:
        s64 = api.Caspt2Session(local, api.DCG_PREC_FP64)
        for _ in range(max(1, min(args.warmup, 2))):
            one(s64, hb_dev)
        n64 = max(3, min(args.steps, 5))
        per_64, _, _, res_64, _ = timed(s64, hb_dev, n64)
        s64.close()
        e_s, e2_s, t_s = res_v[-1]
        e_d, e2_d, t_d = res_64[-1]
        fp64 = {"value": n64 / (sum(per_64) / 1e3), "unit": "solves/s", "ms_per_step": sum(per_64) / n64,
                "p50_ms": float(np.percentile(per_64, 50)), "p99_ms": float(np.percentile(per_64, 99)),
                "max_abs_dE2_subspace": max(abs(e2_s[k] - e2_d[k]) for k in e2_s),
                "abs_dE2_total": abs(sum(e2_s.values()) - sum(e2_d.values())),
                "abs_dE_casci": abs(e_s - e_d), "abs_dE_total": abs(t_s - t_d),
                "dE2_by_subspace": {k: e2_s[k] - e2_d[k] for k in e2_s}}

    # replicas: every rank solves its own copy; the slowest rank bounds the job
    tot_v, tot_e, tot_s = replicas.max_over_ranks([tot_v, tot_e, tot_s])
    value, e2e, e2e_s = world * args.steps / tot_v, world * args.steps / tot_e, world * e2e_steps / tot_s
    peaks, src = _peaks()
    fam_ms, fam_launch, fam_work = fam
    if family in ("hstream", "scatter"):
        achieved = fam_work / (fam_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"]}
    elif family == "split_mma":
        achieved = fam_work / (fam_ms * 1e-3) / 1e12
        pk = peaks["bf16_tflops_sustained"]
        roof = {"bound": "tensor", "achieved": achieved, "peak": pk, "unit": "TFLOP/s", "frac": achieved / pk,
                "work": "BF16 tensor FLOPs of the 15 slice products (15 x 8 M N K per complex M x N x K GEMM)"}
    else:
        achieved = fam_work / (fam_ms * 1e-3) / 1e12
        roof = {"bound": "fp64", "achieved": achieved, "peak": None, "unit": "TFLOP/s", "frac": None,
                "work": "FP64 FLOPs; GB300 has no FP64 tensor rate to compare against"}
    roof.update({"traffic": _traffic(family, cfg_name), "kernel_family": family, "launches_timed": fam_launch,
                 "mean_launch_ms": fam_ms / max(1, fam_launch),
                 "peak_source": f"{src} MEASURED_PEAKS.json ({'sustained' if roof['unit'] == 'TFLOP/s' else 'burst'})"})
    e_casci, e2_last, e_tot = res_v[-1]
    energies = [r[2] for r in res_v + res_e]
    line = {"metric": "caspt2_solves_per_s", "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_v / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": ("c128 (f64)" if prec == api.DCG_PREC_FP64 else
                      "c128: transformation on BF16 tensor cores as 5-slice split products with FP64 "
                      "recombination; eigensolvers, densities and E2 in f64"),
            "data": "synthetic (seeded Kramers-paired complex spinor system; replicas only)",
            "config": {"workload": cfg_name, "ninact": cfg.ninact, "nact": cfg.nact, "nsec": cfg.nsec,
                       "nelec": cfg.nelec, "root": 1, "records": int(len(S.rec_val)),
                       "precision": args.precision, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (1 GB of records, 0.6 GB H class per step)"},
            "p50_ms": float(np.percentile(per_v, 50)), "p99_ms": float(np.percentile(per_v, 99)),
            "e2e": {"value": e2e_s, "unit": "solves/s", "h2d_bytes_per_step": hb_host.h2d_bytes,
                    "d2h_bytes_per_step": 8 * (1 + 8 + 8 + 2),
                    "path": f"dcg_server with {args.e2e_slots} slots (public serving API): each step one request from "
                            "pinned host buffers, host wall clock from the first submit to the last result; "
                            f"up to {args.e2e_slots} requests in flight overlap their copies and latency-bound "
                            "phases. "
                            "single_context below is the same requests one after another on one context "
                            "(dcg_set_system / dcg_casci / dcg_caspt2 from pinned host buffers)",
                    "requests": e2e_steps,
                    "p50_ms": float(np.percentile([(r.t_end - r.t_submit) * 1e3 for r in res_s], 50)),
                    "p99_ms": float(np.percentile([(r.t_end - r.t_submit) * 1e3 for r in res_s], 99)),
                    "max_abs_dE_vs_device_resident": max(abs(r.total_energy - res_v[-1][2]) for r in res_s),
                    "single_context": {"value": e2e, "unit": "solves/s",
                                       "p50_ms": float(np.percentile(per_e, 50)),
                                       "p99_ms": float(np.percentile(per_e, 99)),
                                       "per_step_ms": [round(x, 2) for x in per_e],
                                       "timing": "CUDA events on the context's stream"}},
            "gpu_launches": int(launches_v),
            "clocks": clocks_v, "roofline": roof,
            "stage_ms_last_step": {k: round(v, 3) for k, v in stage.items()},
            "total_energy": e_tot, "energy_spread": float(max(energies) - min(energies))}
    line["families"] = fam_live   # every kernel family against its own roofline
    line["fp64_peak"] = {"measured_tflops": fp64_meas, "nominal_tflops": fp64_nominal,
                         "how": "cuBLAS DGEMM 4096^3 through torch, CUDA events; the FP64 families' frac is "
                                "against it, frac_of_nominal against 152 SMs x 2 FMA/clk x 2.07 GHz"}
    if fam_live:
        dom = max(fam_live, key=lambda k: fam_live[k]["ms_per_step"])
        line["dominant_family"] = {"family": dom, "ms_per_step": fam_live[dom]["ms_per_step"],
                                   "share_of_step": fam_live[dom]["ms_per_step"] / (tot_v / args.steps * 1e3),
                                   "frac": fam_live[dom]["frac"], "bound": fam_live[dom]["bound"]}
        # the dominant kernel's own roofline object (the `roofline` key above stays on the
        # tensor-core family, the kernels the split path adds): its FP64 work per launch over
        # its mean live launch time, against the FP64 peak measured in this process
        fd = fam_live[dom]
        if fd["bound"] == "fp64":
            per_launch_ms = fd["ms_per_step"] / max(fd["launches_per_step"], 1e-9)
            line["roofline_dominant"] = {
                "kernel_family": dom, "bound": "fp64", "unit": "TFLOP/s",
                "achieved": fd["achieved"], "peak": fp64_meas, "frac": fd["achieved"] / fp64_meas,
                "peak_source": "measured (cuBLAS DGEMM 4096^3 in this process; MEASURED_PEAKS.json has no FP64 figure)",
                "work": fd["work"], "launches_per_step": fd["launches_per_step"],
                "mean_launch_ms": per_launch_ms,
                "traffic": _dominant_traffic(dom),
                "traffic_note": "DRAM bytes of one launch on one 792 x 792 matrix (ncu), the A/C metric order"}
    tuned = api.autotune_entries()
    line["autotune"] = {"mode": api.autotune_mode(-1), "keys": len(tuned),
                        "changed_from_heuristic": sum(1 for t in tuned if t["choice"] != 0),
                        "heuristic_ms_sum": round(sum(t["heuristic_ms"] for t in tuned), 3),
                        "tuned_ms_sum": round(sum(t["best_ms"] for t in tuned), 3),
                        "decisions": sorted({t["kind"] for t in tuned})}
    line["cuda_graphs"] = "CASCI Davidson step (device-resident sizes) captured once per eigensolve and replayed"
    if fp64 is not None:
        line["fp64_gpu"] = fp64
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        dt, r = cpu_oracle_solve(S, cfg)
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"one full CASCI+CASPT2 solve of {cfg_name} by the numpy restatement "
                                          "(oracle/), host BLAS threads = all cores",
                                "abs_diff_total_energy": abs(r.total_energy - e_tot),
                                "max_abs_dE2_subspace": max(abs(r.e2[k] - e2_last[k]) for k in r.e2)}
    ses.close()
    del dev, hb_dev
    torch.cuda.empty_cache()
    if args.serve_requests > 0:
        line["serve"] = serve_leg(args, local, world)
    if args.large_config and world == 1:
        line["large_solve"] = large_leg(args, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def large_leg(args, local):
    """The large single solve (40 inactive, 14 active with 8 electrons, 800 secondary spinors;
    650 M records, largest class about 16 GB), generated on the device with its records resident:
    one split-precision solve after a warm-up solve, timed with CUDA events, then one plain FP64
    solve of the same system (after its own warm-up unless args.large_fp64_cold), with the
    largest per-subspace |dE2| between the two paths and the live rates of the kernel families
    the size stresses (tensor-core GEMMs, H streaming, Householder reduction)."""
    import torch
    from dirac_caspt2_gb300 import api, synth, synth_device as sd
    cfg = synth.CONFIGS[args.large_config]
    t0 = time.perf_counter()
    dsys = sd.make_system_device(cfg, f"cuda:{local}")
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    bufs = dsys.buffers()
    sin = dsys.system_input()
    peaks, src = _peaks()
    out = {"workload": args.large_config, "ninact": cfg.ninact, "nact": cfg.nact, "nsec": cfg.nsec,
           "nelec": cfg.nelec, "records": dsys.nrec, "record_gb": round(dsys.record_bytes / 1e9, 2),
           "generate_s": round(gen_s, 1)}
    res = {}
    for name, prec in (("split", api.DCG_PREC_SPLIT), ("fp64", api.DCG_PREC_FP64)):
        with api.Caspt2Session(local, prec) as ses:
            strm = torch.cuda.ExternalStream(ses.stream_ptr, device=local)
            ses.solve(sin, bufs=bufs)                       # warm-up: workspaces, tuner
            fams = {}
            for fam in (("split_mma", "hstream", "eig_tri") if name == "split" else ("hstream",)):
                ses.time_family(fam)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(strm)
                r = ses.solve(sin, bufs=bufs)
                b.record(strm)
                torch.cuda.synchronize()
                f_ms, f_n, f_w = ses.family_stats()
                ses.time_family("none")
                if f_n:
                    if fam == "hstream":
                        ach = f_w / (f_ms * 1e-3) / 1e9
                        fams[fam] = {"ms": f_ms, "achieved": ach, "unit": "GB/s", "frac": ach / peaks["hbm_gbs"]}
                    elif fam == "split_mma":
                        ach = f_w / (f_ms * 1e-3) / 1e12
                        fams[fam] = {"ms": f_ms, "achieved": ach, "unit": "TFLOP/s",
                                     "frac": ach / peaks["bf16_tflops_sustained"]}
                    else:
                        ach = f_w / (f_ms * 1e-3) / 1e12
                        fams[fam] = {"ms": f_ms, "achieved": ach, "unit": "TFLOP/s",
                                     "frac": ach / fp64_gemm_peak(local),
                                     "frac_of_nominal": ach / (152 * 4 * 2.070e-3)}
            ms = a.elapsed_time(b)
            res[name] = r
            out[name] = {"ms_per_solve": ms, "solves_per_s": 1e3 / ms,
                         "stage_ms": {k: round(v, 2) for k, v in r.stage_ms.items()},
                         "total_energy": r.total_energy, "families": fams,
                         "device_gb": round(ses.device_bytes() / 1e9, 1)}
            ses.trim()
        torch.cuda.empty_cache()
    sp, fp = res["split"], res["fp64"]
    out["max_abs_dE2_subspace"] = max(abs(sp.e2[k] - fp.e2[k]) for k in sp.e2)
    out["abs_dE_total"] = abs(sp.total_energy - fp.total_energy)
    out["abs_dE_casci"] = abs(sp.casci_energies[0] - fp.casci_energies[0])
    # CPU-oracle energies of this system, when tests/golden holds them (made once on a host with
    # the memory for it by tests/golden/make_synthetic_fixtures.py --device-generator)
    fx_path = os.path.join(HERE, "tests", "golden", f"synthetic_{args.large_config}.json")
    if os.path.exists(fx_path):
        fx = json.load(open(fx_path))
        if fx["fingerprint"]["nrec"] == out["records"]:
            out["oracle"] = {name: {"max_abs_dE2_subspace": max(abs(r.e2[k] - fx["e2"][k]) for k in "ABCDEFGH"),
                                    "abs_dE_total": abs(r.total_energy - fx["total"]),
                                    "abs_dE_casci": abs(r.casci_energies[0] - fx["casci"])}
                             for name, r in res.items()}
            out["oracle"]["fixture"] = os.path.basename(fx_path)
    out["peak_source"] = src
    del bufs, dsys
    torch.cuda.empty_cache()
    return out


def serve_leg(args, local, world):
    """The served-stream configuration: Poisson arrivals (mean args.serve_rate/s) of
    args.serve_requests independent synthetic systems (per-request seeds; active 4-12 spinors
    half filled, inactive 4-24, secondary 60-400, complex), generated on the device with their
    records resident in HBM, run through the library's serving loop (dcg_server, args.serve_slots
    slots).  Reports solves/s over the stream and the latency percentiles (submit to result),
    and checks that the first requests give the same energies alone as in the mix."""
    import torch
    from dirac_caspt2_gb300 import api, replicas, serve, synth_device as sd
    prec = api.DCG_PREC_SPLIT if args.precision == "split" else api.DCG_PREC_FP64
    cfgs = sd.stream_configs(args.serve_requests, seed=0)
    t0 = time.perf_counter()
    systems = [sd.make_system_device(c, f"cuda:{local}") for c in cfgs]
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    gen_s = time.perf_counter() - t0
    bufs = [s.buffers() for s in systems]
    arrivals = serve.poisson_arrivals(len(bufs), args.serve_rate, seed=1)
    with api.Caspt2Server(local, prec, args.serve_slots) as srv:
        nw = min(2 * args.serve_slots, len(bufs))      # untimed: workspaces and module load
        for k in range(nw):
            srv.submit(2**40 + k, bufs[k])
        for _ in range(nw):
            while srv.poll(1000) is None:
                pass
        replicas.barrier()
        m0 = api.merged_reduction_stats(local)
        rep = serve.run_stream(srv, list(enumerate(bufs)), arrivals)
        m1 = api.merged_reduction_stats(local)
        worst = 0.0
        nchk = min(8, len(bufs))
        for k in range(nchk):
            srv.submit(10**6 + k, bufs[k])
            r = None
            while r is None:
                r = srv.poll(1000)
            worst = max(worst, serve.max_result_difference(r, rep.results[k]))
        dev_gb = srv.device_bytes() / 1e9
    (mk,) = replicas.max_over_ranks([rep.makespan_s])
    out = {"workload": "poisson stream of independent synthetic systems", "requests": rep.requests,
           "rate_hz": args.serve_rate, "slots": args.serve_slots, "precision": args.precision,
           "value": world * (rep.requests - rep.failed) / mk, "unit": "solves/s", "failed": rep.failed, "failures": rep.failures[:8],
           "p50_ms": rep.latency["p50_ms"], "p99_ms": rep.latency["p99_ms"], "mean_ms": rep.latency["mean_ms"],
           "queue_wait_p50_ms": rep.queue_wait["p50_ms"], "service_p50_ms": rep.service["p50_ms"],
           "service_p99_ms": rep.service["p99_ms"], "max_concurrent": rep.max_running, "makespan_s": mk,
           "generate_s": round(gen_s, 2),
           "resident_record_gb": round(sum(s.record_bytes for s in systems) / 1e9, 2),
           "server_workspace_gb": round(dev_gb, 2),
           "alone_vs_mix_max_abs_dE": worst, "alone_checked": nchk,
           "merged_reductions": {"launches": m1["launches"] - m0["launches"],
                                 "joint_launches": m1["joint_launches"] - m0["joint_launches"],
                                 "submissions": m1["submissions"] - m0["submissions"],
                                 "what": "cooperative Householder-reduction launches of the slots during the "
                                         "stream; joint = carrying the reductions of more than one request"},
           "sizes": "nact in {4,6,8,10,12} (nelec = nact/2), ninact 4-24, nsec 60-400 (even), per-request seeds"}
    del bufs, systems
    torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default=CONFIG)
    ap.add_argument("--precision", default="split", choices=["fp64", "split"])
    ap.add_argument("--roofline-family", default=None,
                    help="kernel family timed live for the roofline (default: split_mma, or transform for fp64)")
    ap.add_argument("--no-fp64-compare", action="store_true", help="skip the plain FP64 GPU comparison leg")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=256,
                    help="requests of the served-stream leg (0 skips it)")
    ap.add_argument("--serve-rate", type=float, default=20.0, help="mean Poisson arrival rate of the stream (1/s)")
    ap.add_argument("--serve-slots", type=int, default=4, help="concurrent solves of the serving loop")
    ap.add_argument("--e2e-slots", type=int, default=4, help="server slots of the end-to-end leg")
    ap.add_argument("--e2e-requests", type=int, default=64,
                    help="requests of the end-to-end leg (at least --steps)")
    ap.add_argument("--large-config", default="cas_40_14_800",
                    help="the large single solve reported beside the line ('' to skip)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args, args.config)
    return run_ours(args, args.config)


if __name__ == "__main__":
    sys.exit(main())
