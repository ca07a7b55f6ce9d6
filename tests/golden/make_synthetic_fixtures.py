"""Oracle energies of the seeded synthetic benchmark systems, for the GPU parity tests at the
benchmark sizes (tests/test_gpu_synthetic_fixtures.py).

For each named configuration of ``dirac_caspt2_gb300.synth.CONFIGS`` given on the command line
(default: cas_8_6_40 and cas_20_12_300) this generates the system from its seed, runs the CPU
oracle (``oracle.caspt2_oracle.run``, RDM mode) and stores in ``synthetic_<name>.json``:
the CASCI energy of root 1, e0, e2X and sumc2,X per subspace, the total energy, and a
fingerprint of the generated system (record count, sums of the record values and of h), so a
test can tell that it regenerated the same system.

Usage:  python tests/golden/make_synthetic_fixtures.py [name ...]
"""
import json
import os
import sys
import time

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


def main(names):
    for name in names:
        cfg = synth.CONFIGS[name]
        t0 = time.time()
        S = synth.make_system(cfg)
        s = O.System(ninact=cfg.ninact, nact=cfg.nact, nsec=cfg.nsec, nelec=cfg.nelec, nmo=S.nmo, nsymrpa=1,
                     multb=S.multb, irpamo=S.irpamo, h=S.h, ecore=S.ecore, rec_idx=S.rec_idx, rec_val=S.rec_val,
                     realonly=cfg.realonly, eshift=cfg.eshift)
        t1 = time.time()
        r = O.run(s)
        t2 = time.time()
        out = {"config": name, "dims": [cfg.ninact, cfg.nact, cfg.nsec, cfg.nelec], "seed": cfg.seed,
               "realonly": cfg.realonly, "fingerprint": fingerprint(S), "ndet": int(r.ndet),
               "casci": float(r.casci_energies[0]), "e0": float(r.e0),
               "e2": {k: float(v) for k, v in r.e2.items()}, "sumc2": {k: float(v) for k, v in r.sumc2.items()},
               "total": float(r.total_energy), "oracle_mode": "rdm",
               "oracle_seconds": round(t2 - t1, 1), "host_cores": os.cpu_count()}
        with open(os.path.join(HERE, f"synthetic_{name}.json"), "w") as f:
            json.dump(out, f, indent=1)
        print(name, "generated in %.1f s, oracle %.1f s, total %.12f" % (t1 - t0, t2 - t1, r.total_energy))


if __name__ == "__main__":
    main(sys.argv[1:] or ["cas_8_6_40", "cas_20_12_300"])
