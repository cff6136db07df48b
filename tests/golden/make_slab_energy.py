"""FP64 Ewald energy of the 1,002,002-atom half-vacuum slab (systems.cfg_slab_1m:
21.5 x 21.5 x 43 nm, tin-foil boundary), the reference value of the benchmark's
slab line for the energy error per expansion order.  The oracle's Ewald sum
(oracle/ewald64.c, eps 1e-7) takes about 15 minutes on 8 host cores, too long for
a benchmark run, so its value is stored here:

  python tests/golden/make_slab_energy.py   # writes tests/golden/ewald_slab1m.json
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import __graft_entry__ as G  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main():
    systems = G.load_module("systems")
    O.set_threads(os.cpu_count() or 1)
    xyz, q, box = systems.cfg_slab_1m()
    b = np.array([np.float32(box[0]), np.float32(box[1]), np.float32(box[2])], np.float64)
    t0 = time.time()
    _, _, e = O.ewald(xyz.astype(np.float64), q.astype(np.float64), b, eps=1e-7, energy=True)
    out = {"system": "systems.cfg_slab_1m()", "atoms": int(len(q)), "box_nm": b.tolist(), "eps": 1e-7,
           "energy_kj_mol": e, "seconds": round(time.time() - t0, 1),
           "sha256_xyz": __import__("hashlib").sha256(np.ascontiguousarray(xyz).tobytes()).hexdigest()}
    with open(os.path.join(HERE, "ewald_slab1m.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
