"""Generates the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own CompleteBalancedOctree::build and Traverser
(src/gromacs/zeta_fmm/tree.cpp, traverser.cpp, compiled unmodified into
oracle/_ref/libzetaref.so by oracle/ref_build.sh) and records:

* tree_*.npz   -- body order and leaf body counts for seeded inputs, including
                  bodies exactly on cell boundaries and outside the box;
* lists_small.npz -- complete P2P/M2L lists (target, source, offset in periods)
                  for depth 1-2 and images 0, 1, 2, 4;
* lists_hash.json -- counts and SHA-256 of the complete lists for depth 3-4;
* tree_water96k_d4.npz -- the 95,600-atom water/ion box at depth 4 (4,096
                  leaves): coordinates, leaf body counts and the SHA-256 of the
                  body order;
* ref_outputs.npz -- FP64 potentials and forces of the reference's own kernels
                  (kernel.cu p2m ... l2p, run on the host by
                  oracle/ref_kernels_driver.cpp; before the dipole correction) on
                  every 5th atom of seeded water/ion boxes (REF_CASES), with the
                  SHA-256 of the generated coordinates.

Needs the reference checkout (only present where fixtures are generated):
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from oracle import oracle as O  # noqa: E402
import __graft_entry__ as G  # noqa: E402


def list_arrays(lst, cycle):
    t, s, o = lst
    oi = np.rint(np.asarray(o) / cycle).astype(np.int32)
    return np.asarray(t, np.int32), np.asarray(s, np.int32), oi


def digest(t, s, o):
    h = hashlib.sha256()
    for a in (t, s, o):
        h.update(np.ascontiguousarray(a, dtype="<i4").tobytes())
    return h.hexdigest()


# (lattice sites, box edge, ion pairs, order, depth, images); inputs are
# systems.water_ion_box(sites, edge, ions, ions, seed=sites + order)
REF_CASES = [(300, 2.0, 2, 4, 2, 4), (800, 2.0, 4, 5, 1, 4), (1000, 2.2, 4, 8, 2, 4), (1500, 3.0, 6, 10, 3, 0),
             (1500, 3.0, 6, 6, 3, 2)]


def ref_case_inputs(systems, case):
    ns, L, ions, P, D, im = case
    return systems.water_ion_box(ns, L, n_na=ions, n_cl=ions, seed=ns + P)


def tree_case(xyz, cycle, depth):
    R = O.ref_run(xyz.astype(np.float64), cycle, depth, 4)
    leaf = R["depth"] == depth
    return R["order"].astype(np.int32), R["body_num"][leaf].astype(np.int32)


def main():
    obuild.build(ref=True)
    if not O.ref_available():
        raise SystemExit("reference library not built (reference checkout missing)")
    systems = G.load_module("systems")
    out = {}
    # 1. the 9,000-atom water box at depth 3
    xyz, q, box = systems.cfg_small()
    order, cnt = tree_case(xyz, float(box[0]), 3)
    np.savez_compressed(os.path.join(HERE, "tree_water9k_d3.npz"), xyz=xyz, order=order, leaf_count=cnt,
                        box=np.float32(box[0]))
    # 2. boundary and out-of-box bodies (float32 inputs, as GROMACS passes them)
    L = np.float32(3.2)
    rng = np.random.default_rng(11)
    grid = (np.arange(9, dtype=np.float32) * (L / np.float32(8))).astype(np.float32)
    b = np.stack(np.meshgrid(grid, grid, grid, indexing="ij"), -1).reshape(-1, 3)
    extra = rng.uniform(-0.3, 3.5, size=(200, 3)).astype(np.float32)
    xyz2 = np.concatenate([b, extra], 0).astype(np.float32)
    for d in (1, 2, 3):
        order, cnt = tree_case(xyz2, float(L), d)
        np.savez_compressed(os.path.join(HERE, f"tree_edges_d{d}.npz"), xyz=xyz2, order=order, leaf_count=cnt,
                            box=L)
    # 2b. the 95,600-atom box of the benchmark at depth 4 (coordinates stored:
    # the generator's floating-point steps need not round alike on every host)
    xyz, q, box = systems.cfg_96k()
    order, cnt = tree_case(xyz, float(box[0]), 4)
    np.savez_compressed(os.path.join(HERE, "tree_water96k_d4.npz"), xyz=xyz, leaf_count=cnt,
                        order_sha256=np.frombuffer(hashlib.sha256(order.astype("<i4").tobytes()).digest(), np.uint8),
                        box=np.float32(box[0]))
    # 3. complete small lists
    small = {}
    for depth in (1, 2):
        for images in (0, 1, 2, 4):
            R = O.ref_run(np.zeros((0, 3)), 4.5, depth, images)
            for k in ("p2p", "m2l"):
                t, s, o = list_arrays(R[k], 4.5)
                small[f"{k}_d{depth}_i{images}_tgt"] = t
                small[f"{k}_d{depth}_i{images}_src"] = s
                small[f"{k}_d{depth}_i{images}_off"] = o
    np.savez_compressed(os.path.join(HERE, "lists_small.npz"), **small)
    # 4. hashes of large lists
    hashes = {}
    for depth, images in ((3, 0), (3, 1), (3, 4), (4, 4)):
        R = O.ref_run(np.zeros((0, 3)), 9.86, depth, images)
        for k in ("p2p", "m2l"):
            t, s, o = list_arrays(R[k], 9.86)
            hashes[f"{k}_d{depth}_i{images}"] = {"count": int(len(t)), "sha256": digest(t, s, o)}
    with open(os.path.join(HERE, "lists_hash.json"), "w") as f:
        json.dump(hashes, f, indent=1, sort_keys=True)
    out.update(hashes)
    # 5. outputs of the reference's own FP64 kernels
    ref = {}
    for k, case in enumerate(REF_CASES):
        xyz, q, box = ref_case_inputs(systems, case)
        pot, force = O.ref_solve(xyz.astype(np.float64), q.astype(np.float64), float(case[1]), case[3], case[4],
                                 case[5])
        sample = np.arange(0, len(q), 5, dtype=np.int32)
        ref[f"case{k}_params"] = np.array(case, np.float64)
        ref[f"case{k}_xyz_sha256"] = np.frombuffer(hashlib.sha256(xyz.tobytes()).digest(), np.uint8)
        ref[f"case{k}_idx"] = sample
        ref[f"case{k}_pot"] = pot[sample]
        ref[f"case{k}_force"] = force[sample]
    np.savez_compressed(os.path.join(HERE, "ref_outputs.npz"), **ref)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
