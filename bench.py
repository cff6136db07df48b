"""Benchmark of the GB300 FMM Coulomb solver (one JSON line on rank 0).

Workload: the 95,600-atom periodic water+ion box (9.86 nm cube, 31,800 SPC/E
waters + 100 Na+ + 100 Cl-, seeded synthetic input), one FMM step = tree build,
P2M, M2M, FP64 root + lattice, M2L, L2L, L2P, P2P, dipole correction, energy.
metric: atoms*steps/s.

  value  device-resident step: coordinates already in HBM, one CUDA-graph replay
         per step through gbfmm_execute_device, CUDA events on the caller's
         stream, L2 flushed (256 MB write) before every timed step.
  e2e    the reference-facing call gbfmm_execute: host coordinates in (H2D),
         host forces + potentials + energy out (D2H), synchronous.
Multi-GPU (torchrun): independent replicas of the workload per rank ("replicas
only": one system does not shard), value = sum over ranks of atoms / max time.

--impl reference: the reference algorithm's CPU implementation (the oracle's
FP64 restatement of zeta_fmm, OpenMP on all host cores) on a bounded sample.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import __graft_entry__ as G  # noqa: E402

METRIC = "Coulomb FMM atoms·steps/s at 1e-3 rel force err: tuned vs plain GPU FMM, 1×GB300"
UNIT = "atoms*steps/s"
WORKLOAD = "water+ion 95,600 atoms, 9.86 nm cubic periodic box (31,800 SPC/E waters + 100 Na+ + 100 Cl-)"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0}, "fallback"


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    def __init__(self):
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, dev=0):
        rows = [r for r in self.rows if len(r) >= 9 and r[0] == str(dev)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_reference(xyz, q, box, P, depth, steps, warmup, sample_atoms=None):
    """The reference algorithm on the host cores: zeta_fmm restated in FP64 C
    (oracle/zeta64.c), OpenMP over all cores."""
    from oracle import oracle as O
    ncores = os.cpu_count() or 1
    O.set_threads(ncores)
    x = xyz.astype(np.float64)
    qq = q.astype(np.float64)
    if sample_atoms is not None and sample_atoms < len(q):
        x, qq = x[:sample_atoms], qq[:sample_atoms]
    for _ in range(warmup):
        O.zeta_solve(x, qq, float(box[0]), P, depth, 4)
    t0 = time.perf_counter()
    for _ in range(steps):
        O.zeta_solve(x, qq, float(box[0]), P, depth, 4)
    dt = time.perf_counter() - t0
    return len(qq) * steps / dt, ncores, dt / steps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbfmm", choices=["gbfmm", "reference"])
    ap.add_argument("--order", type=int, default=10)
    ap.add_argument("--depth", type=int, default=4)
    ap.add_argument("--cpu-steps", type=int, default=3)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_env()
    systems = G.load_module("systems")
    xyz, q, box = systems.cfg_96k()
    n = len(q)
    config = {"workload": WORKLOAD, "atoms": n, "order": args.order, "depth": args.depth, "images": 4,
              "l2": "flushed (256 MB write) before every timed step", "parallelism": f"replicas{ws}"}

    if args.impl == "reference":
        if rank != 0:
            return
        v, cores, sec = cpu_reference(xyz, q, box, args.order, args.depth, args.steps and min(args.steps, 3), 1)
        line = {"metric": METRIC, "impl": "reference", "value": v, "unit": UNIT, "n_gpus": ws, "steps": min(args.steps, 3),
                "warmup": 1, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": config,
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": f"full {n}-atom system, p={args.order}, depth {args.depth}, "
                                           "zeta_fmm algorithm in FP64 C (oracle/zeta64.c), OpenMP"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    pkg = G.load_package()
    pkg.lib()
    solver = pkg.ZetaFmmSolver(n, q, order=args.order, max_depth=args.depth, images=4)
    x_dev = torch.from_numpy(xyz).to(dev)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2

    def step():
        solver.execute_device(x_dev.data_ptr(), box, stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with Clocks() as clk:
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()
            ev0[i].record(stream)
            step()
            ev1[i].record(stream)
        torch.cuda.synchronize()
    ms = float(sum(a.elapsed_time(b) for a, b in zip(ev0, ev1)))
    if ws > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = n * ws * args.steps / (ms / 1e3)

    # end to end through the host-side reference-facing call
    for _ in range(2):
        solver.execute(xyz, box)
    torch.cuda.synchronize()
    e2e_s = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ta = time.perf_counter()
        solver.execute(xyz, box)
        e2e_s += time.perf_counter() - ta
    e2e = n * ws * args.steps / e2e_s

    # per-stage device times (CUDA events on the solver's stream, kernel-by-kernel launches)
    solver.set_timing(True)
    stage = {}
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        solver.execute(xyz, box)
        for k, v in solver.stage_times().items():
            stage[k] = stage.get(k, 0.0) + v / args.steps
    solver.set_timing(False)

    # accuracy of this configuration against the FP64 Ewald oracle (sampled atoms)
    acc = None
    try:
        from oracle import oracle as O
        solver.execute(xyz, box)
        f = solver.forces()
        tg = np.arange(0, n, 191)
        _, fe, _ = O.ewald(xyz.astype(np.float64), q.astype(np.float64), box[0], eps=1e-9, targets=tg)
        acc = float(np.sqrt(np.sum((f[tg] - fe) ** 2) / np.sum(fe ** 2)))
    except Exception as e:  # the accuracy report must not break the timing line
        acc = f"unavailable: {e}"

    P, D = args.order, args.depth
    pk, src = peaks()
    # dominant stage and its roofline
    dom = max(stage, key=stage.get) if stage else None
    m2l_pairs = sum((1 << (3 * k)) * (107 if k == 1 else 182) for k in range(1, D + 1))
    alg_m2l = 8 * sum((j + 1) * (P - j + 1) ** 2 for j in range(P + 1)) * m2l_pairs
    # P2P pairs: exact count from the tree
    order, lo, ln = solver.tree()
    nd = 1 << D
    cnt = ln.reshape(-1)
    from itertools import product
    ix = np.array([int("".join(str((c >> (3 * (D - 1 - l) + 2)) & 1) for l in range(D)), 2) for c in range(nd ** 3)])
    iy = np.array([int("".join(str((c >> (3 * (D - 1 - l) + 1)) & 1) for l in range(D)), 2) for c in range(nd ** 3)])
    iz = np.array([int("".join(str((c >> (3 * (D - 1 - l))) & 1) for l in range(D)), 2) for c in range(nd ** 3)])
    grid = np.zeros((nd, nd, nd), np.int64)
    grid[ix, iy, iz] = cnt
    near = np.zeros_like(grid)
    for dx, dy, dz in product(range(-3, 4), repeat=3):
        if dx * dx + dy * dy + dz * dz <= 6:
            near += np.roll(grid, (dx, dy, dz), axis=(0, 1, 2))
    p2p_pairs = int(np.sum(grid * near))
    fp32_peak = 152 * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12  # nominal CUDA-core FP32, TFLOP/s
    kern = {}
    if "m2l" in stage:
        a = alg_m2l / (stage["m2l"] * 1e-3) / 1e12
        kern["m2l"] = {"ms": stage["m2l"], "algorithmic_tflop": alg_m2l / 1e12, "achieved_tflops": a,
                       "bound": "fp32-cuda-core", "peak_tflops": fp32_peak, "frac": a / fp32_peak}
    if "p2p" in stage:
        a = 20.0 * p2p_pairs / (stage["p2p"] * 1e-3) / 1e12
        kern["p2p"] = {"ms": stage["p2p"], "pairs": p2p_pairs, "achieved_tflops": a, "bound": "fp32-cuda-core",
                       "peak_tflops": fp32_peak, "frac": a / fp32_peak}
    roof = None
    if dom in kern:
        k = kern[dom]
        roof = {"kernel": dom, "bound": k["bound"], "achieved": k["achieved_tflops"], "peak": k["peak_tflops"],
                "unit": "TFLOP/s", "frac": k["frac"], "traffic": None,
                "peak_source": "nominal 152 SMs x 128 FP32 lanes x 2 x sm_max_mhz (no FP32 entry in "
                               f"MEASURED_PEAKS.json; hbm/bf16 peaks are {src})"}

    launches = solver.step_launches() * args.steps
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "config": config, "path": f"plain FP32 M2L, p={P}, depth {D}",
            "rel_force_err_vs_ewald": acc,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 12 * n,
                    "d2h_bytes_per_step": 12 * n + 4 * n + 8},
            "stage_ms": stage, "kernels": kern, "roofline": roof, "clocks": clk.summary(local),
            "gpu_launches": launches}
    if rank == 0:
        v, cores, sec = cpu_reference(xyz, q, box, P, D, args.cpu_steps, 1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"{args.cpu_steps} steps of the full {n}-atom system, p={P}, depth {D}; "
                                          "zeta_fmm algorithm in FP64 C (oracle/zeta64.c), OpenMP"}
        print(json.dumps(line))
    solver.close()
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
