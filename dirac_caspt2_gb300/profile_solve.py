"""Run CASCI/CASPT2 solves of one synthetic workload, for profilers.

A named workload (``--workload cas_20_12_300``) or explicit sizes
(``--ninact 16 --nact 8 --nsec 240 --nelec 4``) is generated with the seeded synthetic
generator, uploaded once, and solved ``--warmup + --solves`` times through the C ABI.
The library marks each stage with an NVTX range (``ints``, ``casci_eig``, ``A`` ... ``H``,
``transformation``) and each transformed integral class with ``tr_<class>``, so a profiler
can select the launches of one stage, e.g.

    ncu --clock-control none --nvtx --nvtx-include "tr_H/" -k regex:zgemm -c 3 ... \\
        python -m dirac_caspt2_gb300.profile_solve --ninact 16 --nact 8 --nsec 240 --nelec 4

Prints the total energy and per-stage device times of the last solve.  With ``--heev N`` it
runs the Hermitian eigensolver alone on a seeded random N x N matrix instead.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

from . import api, synth


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--workload", default=None, choices=sorted(synth.CONFIGS))
    ap.add_argument("--ninact", type=int, default=8)
    ap.add_argument("--nact", type=int, default=6)
    ap.add_argument("--nsec", type=int, default=40)
    ap.add_argument("--nelec", type=int, default=4)
    ap.add_argument("--real", action="store_true")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--warmup", type=int, default=0)
    ap.add_argument("--solves", type=int, default=1)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "split"])
    ap.add_argument("--heev", type=int, default=0,
                    help="instead of a solve: dcg_heev (all eigenpairs) of a seeded random Hermitian matrix "
                         "of this size, --warmup + --solves times")
    ap.add_argument("--zgemm", type=int, nargs=3, default=None, metavar=("M", "N", "K"),
                    help="instead of a solve: dcg_zgemm of seeded random column-major operands, "
                         "--warmup + --solves times, at --gemm-precision")
    ap.add_argument("--gemm-precision", default="split_acc", choices=["fp64", "split", "split_acc"])
    a = ap.parse_args(argv)
    if a.zgemm:
        import numpy as np
        import torch
        M, N, K = a.zgemm
        g = torch.Generator().manual_seed(a.seed)
        dev = lambda r, c: (torch.randn((c, r), dtype=torch.float64, generator=g) +
                            1j * torch.randn((c, r), dtype=torch.float64, generator=g)).cuda()
        A, B = dev(M, K), dev(K, N)           # (cols, rows) storage: column-major M x K and K x N
        C = torch.zeros((N, M), dtype=torch.complex128, device="cuda")
        prec = {"fp64": api.DCG_PREC_FP64, "split": api.DCG_PREC_SPLIT, "split_acc": api.DCG_PREC_SPLIT_ACC}
        ses = api.Caspt2Session(0, api.DCG_PREC_SPLIT)
        t0 = time.time()
        for _ in range(a.warmup + a.solves):
            ses.zgemm(prec[a.gemm_precision], M, N, K, 1, A.data_ptr(), 1, M, 0, B.data_ptr(), K, False,
                      C.data_ptr(), 1, M, 0)
        torch.cuda.synchronize()
        ref = A.T @ B.T
        err = ((C.T - ref).abs().max() / (A.abs().max() * B.abs().max())).item()
        print(json.dumps({"zgemm": [M, N, K], "precision": a.gemm_precision, "calls": a.warmup + a.solves,
                          "wall_s": round(time.time() - t0, 3), "max_rel_error": err}))
        ses.close()
        return 0
    if a.heev > 0:
        import numpy as np
        rng = np.random.default_rng(a.seed)
        m = rng.normal(size=(a.heev, a.heev)) + 1j * rng.normal(size=(a.heev, a.heev))
        m = m + m.conj().T
        ses = api.Caspt2Session(0)
        t0 = time.time()
        for _ in range(a.warmup + a.solves):
            w, _ = ses.heev(m)
        print(json.dumps({"heev": a.heev, "calls": a.warmup + a.solves, "wall_s": round(time.time() - t0, 3),
                          "max_abs_eig_error": float(np.abs(w - np.linalg.eigvalsh(m)).max())}))
        return 0
    if a.workload:
        cfg = synth.CONFIGS[a.workload]
    else:
        cfg = synth.SynthConfig(a.ninact, a.nact, a.nsec, a.nelec, realonly=a.real, seed=a.seed,
                                name=f"cas_{a.ninact}_{a.nact}_{a.nsec}")
    t0 = time.time()
    system = api.SystemInput.from_synth(synth.make_system(cfg))
    t1 = time.time()
    prec = api.DCG_PREC_SPLIT if a.precision == "split" else api.DCG_PREC_FP64
    ses = api.Caspt2Session(0, precision=prec)
    res = None
    warm_launches = 0
    for k in range(a.warmup + a.solves):
        res = ses.solve(system)
        if k < a.warmup:
            warm_launches += res.kernel_launches
    t2 = time.time()
    print(json.dumps({
        "workload": cfg.name, "generate_s": round(t1 - t0, 2), "solve_wall_s": round(t2 - t1, 3),
        "solves": a.warmup + a.solves, "total_energy": res.total_energy,
        "e2": res.e2, "kernel_launches": res.kernel_launches,
        # library launches of the warm-up solves (autotuner trials included): a profiler's
        # launch-skip count to start at the measured solves
        "warmup_kernel_launches": warm_launches,
        "stage_ms": {k: round(v, 3) for k, v in res.stage_ms.items()},
    }))
    return 0


if __name__ == "__main__":
    sys.exit(main())
