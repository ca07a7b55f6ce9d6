"""Oracle energies of the seeded synthetic benchmark systems, for the GPU parity tests at the
benchmark sizes (tests/test_gpu_synthetic_fixtures.py).

For each named configuration of ``dirac_caspt2_gb300.synth.CONFIGS`` given on the command line
(default: cas_8_6_40 and cas_20_12_300) this generates the system from its seed, runs the CPU
oracle (``oracle.caspt2_oracle.run``, RDM mode) and stores in ``synthetic_<name>.json``:
the CASCI energy of root 1, e0, e2X and sumc2,X per subspace, the total energy, and a
fingerprint of the generated system (record count, sums of the record values and of h), so a
test can tell that it regenerated the same system.

With ``--device-generator`` the system is generated on the GPU by
``dirac_caspt2_gb300.synth_device`` (the same records as the host generator, which cannot hold
the 650 M-record 40/14/800 system in reasonable time and memory) and the records are copied to
the host; the oracle then runs with ``lean=True``, releasing each input once it is read.

Usage:  python tests/golden/make_synthetic_fixtures.py [--device-generator] [name ...]
"""
import json
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from dirac_caspt2_gb300 import synth  # noqa: E402
from oracle import caspt2_oracle as O  # noqa: E402


def fingerprint(S) -> dict:
    v = np.asarray(S.rec_val)
    return {"nrec": int(len(v)), "sum_re": float(np.sum(v.real)), "sum_abs": float(np.sum(np.abs(v))),
            "sum_h_re": float(np.sum(S.h.real)), "nmo": int(S.nmo)}


def device_system(cfg):
    """The records of ``cfg`` generated on the GPU, copied to host numpy arrays."""
    import torch
    from dirac_caspt2_gb300 import synth_device
    d = synth_device.make_system_device(cfg, "cuda")
    n = d.nrec
    idx = d.rec_idx.cpu().numpy()
    val = np.empty(n, np.complex128)
    step = 1 << 26
    for a in range(0, n, step):
        b = min(n, a + step)
        val.real[a:b] = d.rec_re[a:b].cpu().numpy()
        val.imag[a:b] = d.rec_im[a:b].cpu().numpy() if d.rec_im is not None else 0.0
    h, ecore, nmo = d.h, d.ecore, d.nmo
    del d
    torch.cuda.empty_cache()
    return types.SimpleNamespace(nmo=nmo, h=h, ecore=ecore, rec_idx=idx, rec_val=val,
                                 multb=np.array([[2, 1], [1, 2]], np.int64), irpamo=np.ones(nmo, np.int64))


def main(names, device_generator=False):
    for name in names:
        cfg = synth.CONFIGS[name]
        t0 = time.time()
        S = device_system(cfg) if device_generator else synth.make_system(cfg)
        fp = fingerprint(S)
        s = O.System(ninact=cfg.ninact, nact=cfg.nact, nsec=cfg.nsec, nelec=cfg.nelec, nmo=S.nmo, nsymrpa=1,
                     multb=S.multb, irpamo=S.irpamo, h=S.h, ecore=S.ecore, rec_idx=S.rec_idx, rec_val=S.rec_val,
                     realonly=cfg.realonly, eshift=cfg.eshift)
        del S
        t1 = time.time()
        print(name, "generated in %.1f s" % (t1 - t0), flush=True)
        r = O.run(s, lean=device_generator)
        t2 = time.time()
        out = {"config": name, "dims": [cfg.ninact, cfg.nact, cfg.nsec, cfg.nelec], "seed": cfg.seed,
               "realonly": cfg.realonly, "fingerprint": fp, "ndet": int(r.ndet),
               "generator": "device" if device_generator else "host",
               "casci": float(r.casci_energies[0]), "e0": float(r.e0),
               "e2": {k: float(v) for k, v in r.e2.items()}, "sumc2": {k: float(v) for k, v in r.sumc2.items()},
               "total": float(r.total_energy), "oracle_mode": "rdm",
               "oracle_seconds": round(t2 - t1, 1), "host_cores": os.cpu_count()}
        with open(os.path.join(HERE, f"synthetic_{name}.json"), "w") as f:
            json.dump(out, f, indent=1)
        print(name, "generated in %.1f s, oracle %.1f s, total %.12f" % (t1 - t0, t2 - t1, r.total_energy))


if __name__ == "__main__":
    args = sys.argv[1:]
    dev = "--device-generator" in args
    args = [a for a in args if a != "--device-generator"]
    main(args or ["cas_8_6_40", "cas_20_12_300"], device_generator=dev)
