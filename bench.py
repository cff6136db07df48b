"""Benchmark of the GB300 FMM Coulomb solver (one JSON line on rank 0).

Workload: the 95,600-atom periodic water+ion box (9.86 nm cube, 31,800 SPC/E
waters + 100 Na+ + 100 Cl-, seeded synthetic input).  One step = tree build,
P2M, M2M, FP64 root + lattice, M2L, L2L, L2P, P2P, dipole correction and
energy, from device coordinates to device forces, potentials and energy.
metric: atoms*steps/s at <= 1e-3 relative RMS force error against FP64 Ewald.

  tuned  the mixed-precision path: tensor-core M2L (split bf16) with the
         expansion order, tree depth and precision proposed by the learned
         tuner (gromacs-fmm_gb300/tuner.py) for the 1e-3 tolerance and checked
         against the plain FMM on this configuration; this is 'value'.  Its
         error against FP64 Ewald on sampled atoms is reported, and so is an
         exhaustive sweep over a candidate grid ('sweep').
  plain  the plain FP32 GPU FMM at the same accuracy: the fastest FP32
         (order, depth) of the sweep whose force error against FP64 Ewald meets
         the same 1e-3 ('plain_fp32', the denominator of
         'speedup_tuned_vs_plain'); the FP32 path with the reference parameters
         for this workload (p=10, depth 4) is reported beside it
         ('plain_fp32_order10').
  value  device-resident: one CUDA-graph replay per step through
         gbfmm_execute_device, CUDA events on the caller's stream, L2 flushed
         (256 MB write) before every timed step.
  e2e    the reference-facing call gbfmm_execute: host coordinates in, host
         forces + potentials + energy out, synchronous.  On GB300 the step
         reads and writes that host memory in place over NVLink-C2C; the same
         call with staging copies is reported beside it (value_with_copies).
Multi-GPU (torchrun): independent replicas per rank ("replicas only": a single
system does not shard), value = sum over ranks of atoms / max time.

--impl reference: the reference algorithm's CPU implementation (the oracle's
FP64 restatement of zeta_fmm, OpenMP on all host cores) on the same workload,
at the same order and depth as 'value' and for the same number of steps.
"""
import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time
from itertools import product

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import __graft_entry__ as G  # noqa: E402

METRIC = "Coulomb FMM atoms·steps/s at 1e-3 rel force err: tuned vs plain GPU FMM, 1×GB300"
UNIT = "atoms*steps/s"
WORKLOAD = "water+ion 95,600 atoms, 9.86 nm cubic periodic box (31,800 SPC/E waters + 100 Na+ + 100 Cl-)"
TOL = 1e-3
PLAIN_REF = (0, 10, 4)                  # (precision, order, depth): the reference parameters, FP32
# the configuration the learned tuner chooses for this workload at 1e-3 (checked
# on every run: 'tuner.chosen'); the CPU arms run the same order and depth
HEADLINE = (2, 5, 4)
CANDIDATES = [(p, P, D) for D in (3, 4) for p in (0, 2, 1) for P in (4, 5, 6, 7, 8)]
PREC_NAME = {0: "fp32", 1: "bf16x3", 2: "bf16x1"}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0}, "fallback"


class Clocks:
    """SM clocks and clock-event reasons sampled DURING the timed region.

    NVML through ctypes (libnvidia-ml.so.1, read-only queries), polled every
    millisecond from a thread on the device torch runs on (matched by UUID), plus
    one synchronous sample at each end, so that even a region of a few
    milliseconds is seen.  Falls back to `nvidia-smi -lms 200` where NVML is
    absent."""

    # nvmlClocksEventReasons bits
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, device=0):
        self.device = device
        self.rows = []   # (sm_mhz, max_mhz, reasons mask)
        self.smi_rows = []
        self.proc = None
        self.nv = None
        self.h = None
        self.stop = threading.Event()
        self.t = None

    def _nvml_open(self):
        import ctypes
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            return False
        h = ctypes.c_void_p()
        uuid = None
        try:
            import torch
            u = getattr(torch.cuda.get_device_properties(self.device), "uuid", None)
            uuid = ("GPU-" + str(u)) if u is not None and not str(u).startswith("GPU-") else (str(u) if u else None)
        except Exception:
            uuid = None
        ok = uuid is not None and nv.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(h)) == 0
        if not ok:
            vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
            idx = int(vis.split(",")[self.device]) if vis and vis.split(",")[0].isdigit() else self.device
            if nv.nvmlDeviceGetHandleByIndex_v2(idx, ctypes.byref(h)) != 0:
                return False
        self.nv, self.h = nv, h
        reasons = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self.reasons_fn = reasons or nv.nvmlDeviceGetCurrentClocksThrottleReasons
        return True

    def _sample(self):
        import ctypes
        mhz, mx, mask = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        if (self.nv.nvmlDeviceGetClockInfo(self.h, 1, ctypes.byref(mhz)) == 0 and
                self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(mx)) == 0 and
                self.reasons_fn(self.h, ctypes.byref(mask)) == 0):
            self.rows.append((mhz.value, mx.value, mask.value))

    def _poll(self):
        while not self.stop.is_set():
            self._sample()
            time.sleep(0.001)

    def __enter__(self):
        try:
            if self._nvml_open():
                self._sample()
                self.t = threading.Thread(target=self._poll, daemon=True)
                self.t.start()
                return self
        except Exception:
            self.nv = None
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
            self.smi_rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.nv is not None:
            self.stop.set()
            self.t.join(timeout=2)
            self._sample()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.rows:
            sm = [r[0] for r in self.rows]
            reasons = sorted({name for r in self.rows for bit, name in self.REASONS.items() if r[2] & bit})
            return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(r[1] for r in self.rows)),
                    "reasons": reasons, "samples": len(self.rows), "source": "nvml"}
        rows = [r for r in self.smi_rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "source": "nvidia-smi"}


def ncu_traffic(kernel):
    """DRAM bytes per launch of a kernel from its committed ncu summary
    (profiles/<kernel>_water95600_*.md, line 'traffic_bytes_per_launch: N'), or None."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None, None
    for f in sorted(os.listdir(d)):
        if f.startswith(kernel + "_water95600") and f.endswith(".md"):
            m = re.search(r"traffic_bytes_per_launch:\s*(\d+)", open(os.path.join(d, f)).read())
            if m:
                return int(m.group(1)), "profiles/" + f
    return None, None


def pageable_access(device=0):
    """True where the device reads pageable host memory coherently (the driver's
    CU_DEVICE_ATTRIBUTE_PAGEABLE_MEMORY_ACCESS, a read-only query)."""
    import ctypes
    try:
        cu = ctypes.CDLL("libcuda.so.1")
        if cu.cuInit(0) != 0:
            return False
        d, v = ctypes.c_int(), ctypes.c_int(0)
        if cu.cuDeviceGet(ctypes.byref(d), int(device)) != 0:
            return False
        return cu.cuDeviceGetAttribute(ctypes.byref(v), 88, d) == 0 and v.value != 0
    except OSError:
        return False


def dist_env():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def replica_throughput(atoms_local, steps, ms_local, dist=None, device=None):
    """Whole-job atoms*steps/s of independent replicas: atoms summed over ranks,
    divided by the slowest rank's time (max over ranks)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return atoms_local * steps / (ms_local / 1e3), ms_local
    import torch
    t = torch.tensor([ms_local, float(atoms_local)], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    sm = t.clone()
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return float(sm[1].item()) * steps / (float(mx[0].item()) / 1e3), float(mx[0].item())


def cpu_reference(xyz, q, box, P, depth, steps, warmup):
    """The reference algorithm on the host cores: zeta_fmm restated in FP64 C
    (oracle/zeta64.c), OpenMP over all cores."""
    from oracle import oracle as O
    ncores = os.cpu_count() or 1
    O.set_threads(ncores)
    x = xyz.astype(np.float64)
    qq = q.astype(np.float64)
    for _ in range(warmup):
        O.zeta_solve(x, qq, float(box[0]), P, depth, 4)
    t0 = time.perf_counter()
    for _ in range(steps):
        O.zeta_solve(x, qq, float(box[0]), P, depth, 4)
    dt = time.perf_counter() - t0
    return len(qq) * steps / dt, ncores, dt / steps


def p2p_pair_count(leaf_counts, D):
    nd = 1 << D
    codes = np.arange(nd ** 3)
    ix = np.zeros_like(codes)
    iy = np.zeros_like(codes)
    iz = np.zeros_like(codes)
    for l in range(D):
        ix |= ((codes >> (3 * l + 2)) & 1) << l
        iy |= ((codes >> (3 * l + 1)) & 1) << l
        iz |= ((codes >> (3 * l)) & 1) << l
    grid = np.zeros((nd, nd, nd), np.int64)
    grid[ix, iy, iz] = leaf_counts
    near = np.zeros_like(grid)
    for dx, dy, dz in product(range(-3, 4), repeat=3):
        if dx * dx + dy * dy + dz * dz <= 6:
            near += np.roll(grid, (dx, dy, dz), axis=(0, 1, 2))
    return int(np.sum(grid * near))


def m2l_flops_per_pair(P):
    """The reference's count: 8 * sum_j (j+1)(P-j+1)^2 flops per M2L pair."""
    return 8 * sum((j + 1) * (P - j + 1) ** 2 for j in range(P + 1))


def m2l_pairs(D):
    return sum((1 << (3 * k)) * (107 if k == 1 else 182) for k in range(1, D + 1))


class Runner:
    def __init__(self, pkg, torch, dev, xyz, q, box):
        self.pkg, self.torch, self.dev = pkg, torch, dev
        self.xyz, self.q, self.box = xyz, q, box
        self.n = len(q)
        self.x_dev = torch.from_numpy(xyz).to(dev)
        self.stream = torch.cuda.current_stream(dev)
        self.flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2

    def solver(self, prec, P, D, flags=0):
        return self.pkg.ZetaFmmSolver(self.n, self.q, order=P, max_depth=D, images=4, precision=prec, flags=flags)

    def step(self, s):
        s.execute_device(self.x_dev.data_ptr(), self.box, self.stream.cuda_stream)

    def time_device(self, s, steps, warmup, clocks=None):
        """Total device ms of `steps` steps (L2 flushed before each); the clock
        sampler, when given, runs over the timed steps only."""
        torch = self.torch
        for _ in range(warmup):
            self.step(s)
        torch.cuda.synchronize()
        ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        if clocks is not None:
            clocks.__enter__()
        try:
            for i in range(steps):
                self.flush.zero_()
                ev0[i].record(self.stream)
                self.step(s)
                ev1[i].record(self.stream)
            torch.cuda.synchronize()
        finally:
            if clocks is not None:
                clocks.__exit__(None, None, None)
        return float(sum(a.elapsed_time(b) for a, b in zip(ev0, ev1)))

    def time_e2e(self, s, steps):
        """Host wall time of `steps` calls of the C ABI's gbfmm_execute, as the
        mdrun adapter makes them (host coordinates in; forces, potentials and
        energy on the host when it returns), L2 flushed before each call."""
        for _ in range(2):
            s.execute(self.xyz, self.box)
        x = np.ascontiguousarray(self.xyz, dtype=np.float32)
        m = self.pkg.box_matrix(self.box)
        fn, h = self.pkg.lib().gbfmm_execute, s._h
        xp, mp = self.pkg._fp(x), self.pkg._fp(m)
        tot = 0.0
        for _ in range(steps):
            self.flush.zero_()
            self.torch.cuda.synchronize()
            t0 = time.perf_counter()
            rc = fn(h, xp, mp, 0)
            tot += time.perf_counter() - t0
            if rc != 0:
                raise RuntimeError(f"gbfmm_execute returned {rc}")
        return tot

    def stages(self, s, steps):
        s.set_timing(True)
        acc = {}
        for _ in range(steps):
            self.flush.zero_()
            self.torch.cuda.synchronize()
            s.execute(self.xyz, self.box)
            for k, v in s.stage_times().items():
                acc[k] = acc.get(k, 0.0) + v / steps
        s.set_timing(False)
        return acc


def rel_diff(f, g):
    return float(np.sqrt(np.sum((f - g) ** 2) / np.sum(g ** 2)))


def pot_err(p, g, xyz=None, q=None, tg=None, V=None):
    """Relative RMS potential error modulo a constant, and that constant.  The
    FMM's potentials follow the reference's dipole correction, which subtracts
    the per-atom constant (4 pi / 3V) |M|^2 / (N q_i) (solver.cpp:30-49) where the
    tin-foil Ewald potential subtracts (4 pi / 3V) M . r_i; with the atoms (xyz,
    q), targets tg and volume V given, p is first taken to Ewald's convention.
    What remains differs by a constant: the lattice sum and the Ewald sum (whose
    mean potential is zero) differ in the potential's zero by the box's mean
    inner potential (a term in sum q r^2 / V), which moves no force and, in a
    neutral box, no energy."""
    if xyz is not None:
        x = np.asarray(xyz, np.float64)
        qq = np.asarray(q, np.float64)
        M = (qq[:, None] * x).sum(0)
        c = 138.935457833 * 4.0 * np.pi / (3.0 * V)
        qt = qq[tg]
        own = np.where(qt != 0, np.dot(M, M) / (len(qq) * np.where(qt != 0, qt, 1.0)), 0.0)
        p = p + c * (own - x[tg] @ M)
    k = float(np.mean(p - g))
    return float(np.sqrt(np.sum((p - k - g) ** 2) / np.sum((g - np.mean(g)) ** 2))), k


def large_line(pkg, torch, dev, systems, steps):
    """The inhomogeneous 1,002,002-atom slab: a periodic 21.5 x 21.5 x 43 nm box
    whose lower half is water with 0.15 M NaCl and whose upper half is vacuum
    (aspect_z 2: the tree's root is the 43 nm cube that holds the box twice along
    x and y; depth 6 gives 0.67 nm leaves, 30.6 bodies per water leaf; M2L tiles
    of the vacuum are skipped).  Per expansion order 6, 8, 10, 12: the split-bf16
    tensor-core M2L with FP32 accumulation (BF16X3; BF16X1 beside it), FP64 root
    and lattice; device-resident steps, L2 flushed before each; relative RMS force
    and potential error against the FP64 Ewald sum of the rectangular box (every
    997th atom) and the energy error against the FP64 Ewald energy.  The plain FP32
    FMM at order 10 is reported beside it."""
    from oracle import oracle as O
    xyz, q, box = systems.cfg_slab_1m()
    n = len(q)
    a = float(np.float32(box[0]))
    b3 = np.array([a, a, 2 * a])
    tg = np.arange(0, n, 997)
    O.set_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    pe, fe, _ = O.ewald(xyz.astype(np.float64), q.astype(np.float64), b3, eps=1e-9, targets=tg)
    ewald_s = time.perf_counter() - t0
    # the FP64 Ewald energy of this system (about 15 minutes of host time) is
    # stored with the script that computed it (tests/golden/make_slab_energy.py)
    with open(os.path.join(ROOT, "tests", "golden", "ewald_slab1m.json")) as fh:
        e_ref = json.load(fh)["energy_kj_mol"]
    run = Runner(pkg, torch, dev, xyz, q, [a, a, 2 * a])
    D = 6
    out = {"workload": "water+ion slab, 1,002,002 atoms: periodic 21.5 x 21.5 x 43 nm box, lower half 333,402 SPC/E "
                       "waters + 898 Na+ + 898 Cl- (0.15 M), upper half vacuum", "atoms": n, "depth": D,
           "box_nm": [a, a, 2 * a], "ewald": f"FP64 Ewald (oracle/ewald64.c) of the rectangular box: forces and "
                                           f"potentials on {len(tg)} atoms (every 997th), eps 1e-9, {ewald_s:.1f} s; "
                                           "energy (eps 1e-7) from tests/golden/ewald_slab1m.json", "ewald_energy": e_ref}
    rows = []
    for P in (6, 8, 10, 12):
        for prec in (1, 2):
            s = pkg.ZetaFmmSolver(n, q, order=P, max_depth=D, images=4, precision=prec, aspect_z=2)
            s.execute(xyz, [a, a, 2 * a])
            f, p, e = s.forces(), s.potentials(), s.get_energy()
            ms = run.time_device(s, steps, 3) / steps
            pr, pc = pot_err(p[tg], pe, xyz, q, tg, a * a * 2 * a)
            rows.append({"order": P, "precision": PREC_NAME[prec], "ms_per_step": ms, "value": n / (ms * 1e-3),
                         "rel_force_err_vs_ewald": rel_diff(f[tg], fe), "rel_pot_err_vs_ewald_modulo_constant": pr,
                         "pot_offset_vs_ewald": pc, "energy": e, "rel_energy_err_vs_ewald": abs(e - e_ref) / abs(e_ref)})
            s.close()
    s = pkg.ZetaFmmSolver(n, q, order=10, max_depth=D, images=4, precision=0, aspect_z=2)
    s.execute(xyz, [a, a, 2 * a])
    f, p, e = s.forces(), s.potentials(), s.get_energy()
    ms = run.time_device(s, steps, 3) / steps
    s.close()
    pr, pc = pot_err(p[tg], pe, xyz, q, tg, a * a * 2 * a)
    out["plain_fp32_order10"] = {"ms_per_step": ms, "value": n / (ms * 1e-3), "rel_force_err_vs_ewald":
                                 rel_diff(f[tg], fe), "rel_pot_err_vs_ewald_modulo_constant": pr,
                                 "pot_offset_vs_ewald": pc, "energy": e,
                                 "rel_energy_err_vs_ewald": abs(e - e_ref) / abs(e_ref)}
    out["per_order"] = rows
    ok = [r for r in rows if r["rel_force_err_vs_ewald"] <= TOL]
    if ok:
        best = min(ok, key=lambda r: r["ms_per_step"])
        out["fastest_within_tolerance"] = {"order": best["order"], "precision": best["precision"],
                                           "value": best["value"], "ms_per_step": best["ms_per_step"]}
        out["speedup_vs_plain_order10"] = out["plain_fp32_order10"]["ms_per_step"] / best["ms_per_step"]
    return out


def frames_line(pkg, torch, dev, systems, tuner_mod, n_frames):
    """The 250,002-atom box over a trajectory of kicked frames (sigma 0.01 nm per
    frame).  Per tolerance, the tuner proposes and checks on the first frame and
    the choice serves the following frames; every frame is checked against the
    plain order-10, depth-5 FP32 FMM (the check solve, solved on every frame anyway),
    and a frame whose check misses the tolerance re-runs the checked choice on
    that frame (fallback to the plain FMM if nothing meets it).  On every 25th
    frame both are also held against the FP64 Ewald sum (forces on every 251st
    atom).  Device time per frame: L2 flushed before each."""
    from oracle import oracle as O
    xyz, q, box = systems.cfg_250k()
    n = len(q)
    L = float(box[0])
    frames = list(systems.kicked_frames(xyz, box, n_frames))
    base = pkg.ZetaFmmSolver(n, q, order=10, max_depth=5, images=4)
    fb, tb = [], []
    st = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)

    def dev_time(s, x):
        xd = torch.from_numpy(x).to(dev)
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        s.execute_device(xd.data_ptr(), L, st.cuda_stream)
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1)

    base.execute(frames[0], L)
    for x in frames:
        tb.append(dev_time(base, x))
        fb.append(base.forces().copy())
    base.close()
    O.set_threads(os.cpu_count() or 1)
    tg = np.arange(0, n, 251)
    sampled = list(range(0, n_frames, 25))
    ewald = {}
    for i in sampled:
        _, fe, _ = O.ewald(frames[i].astype(np.float64), q.astype(np.float64), L, eps=1e-9, targets=tg)
        ewald[i] = fe
    out = {"workload": f"water+ion 250,002 atoms, 13.6 nm cube, {n_frames} frames with 0.01 nm Gaussian kicks",
           "baseline": {"order": 10, "depth": 5, "precision": "fp32", "ms_per_frame": float(np.mean(tb)),
                        "rel_force_err_vs_ewald_sampled_frames":
                            [rel_diff(fb[i][tg], ewald[i]) for i in sampled]},
           "ewald": f"FP64 Ewald (oracle/ewald64.c), forces on every 251st atom of frames {sampled}"}
    for tol in (1e-3, 5e-4):
        mlp = tuner_mod.Mlp.load()
        ts = tuner_mod.TunedSolver(q, mlp, tol=tol)
        P, D, prec = ts.propose(frames[0], L)
        choices = [{"frame": 0, "order": P, "depth": D, "precision": PREC_NAME[prec]}]
        diffs, tt, errs = [], [], []
        for i, (x, f0) in enumerate(zip(frames, fb)):
            s = ts.solver
            tt.append(dev_time(s, x))
            d = rel_diff(s.forces(), f0)
            if d > tol:
                # the check of this frame missed: choose again on this frame
                s.close()
                P, D, prec = ts.propose(x, L)
                choices.append({"frame": i, "order": P, "depth": D, "precision": PREC_NAME[prec],
                                "missed_diff": d})
                d = rel_diff(ts.solver.forces(), f0)
            diffs.append(d)
            if i in ewald:
                errs.append(rel_diff(ts.solver.forces()[tg], ewald[i]))
        ts.solver.close()
        mlp.close()
        out[f"tol_{tol:g}"] = {"order": choices[-1]["order"], "depth": choices[-1]["depth"],
                               "precision": choices[-1]["precision"], "choices": choices,
                               "max_rel_force_diff_vs_baseline": max(diffs),
                               "rel_force_err_vs_ewald_sampled_frames": errs,
                               "max_rel_force_err_vs_ewald": max(errs), "ms_per_frame": float(np.mean(tt)),
                               "speedup_vs_baseline": float(np.mean(tb)) / float(np.mean(tt))}
    return out


def batch_spec(tuner_mod, nat):
    """Orders and depths of the 64-system batch: each system's order drawn (seeded)
    from 6..10; its depth the plain depth (16-128 bodies per leaf) or, for a
    seeded third of the systems, one deeper, clamped to 3..5, so that every
    depth of 3..5 occurs."""
    rng = np.random.default_rng(64)
    orders = [int(v) for v in rng.integers(6, 11, size=len(nat))]
    deeper = np.random.default_rng(65).random(len(nat)) < 1.0 / 3.0
    depths = [min(5, max(3, tuner_mod.plain_depth(k) + int(d))) for k, d in zip(nat, deeper)]
    return orders, depths


def batch_line(pkg, torch, dev, systems, steps, warmup):
    """64 independent systems (atom counts log-uniform in [2,000, 200,000], water +
    0.15 M NaCl, one cubic box each), solved in one batched CUDA graph
    (gbfmm_batch_*: each kind of kernel runs for every system in one launch,
    the near fields in one persistent kernel, tiles from gbfmm_batch_autotune),
    device-resident, L2 flushed before every step:
      value  each system's own order drawn (seeded) from 6..10 and its depth in
             3..5 (batch_spec), BF16X3;
      tuned  each system's order and depth proposed by the learned tuner for the
             1e-3 tolerance (each proposal checked against the plain order-10
             FMM), each with its own precision (gbfmm_batch_create_mixed);
             every system's batched forces are checked against its plain FMM
             again.
    Each is compared with the same systems solved one after another (one graph
    per system), and each system's own step time is reported (tuned)."""
    tuner_mod = G.load_module("tuner")
    sy = systems.batch_systems(n_sys=64)
    nat = [len(s[1]) for s in sy]
    off = np.concatenate([[0], np.cumsum(nat)])
    n = int(off[-1])
    X = np.concatenate([s[0] for s in sy]).astype(np.float32)
    Q = np.concatenate([s[1] for s in sy]).astype(np.float32)
    B = np.array([float(s[2][0]) for s in sy], np.float32)
    xd = torch.from_numpy(X).to(dev)
    qd = torch.from_numpy(Q).to(dev)
    st = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)

    def timed(fn, nsteps=steps):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        tot = 0.0
        for _ in range(nsteps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / nsteps

    def run_batch(orders, depths, prec):
        b = pkg.BatchSolver(nat, orders, depths, images=4, precision=prec)
        f, _, _ = b.execute(X, Q, B)  # captures the graph
        ms_default = timed(lambda: b.execute_device(xd.data_ptr(), qd.data_ptr(), B, st.cuda_stream))
        tiles = b.autotune(xd.data_ptr(), qd.data_ptr(), B, reps=2)  # gbfmm_batch_autotune
        b.execute(X, Q, B)  # captures the tuned graph
        ms = timed(lambda: b.execute_device(xd.data_ptr(), qd.data_ptr(), B, st.cuda_stream))
        launches = b.step_launches()
        b.close()
        singles = []
        for i, (xyz, q, box) in enumerate(sy):
            s = pkg.ZetaFmmSolver(len(q), q, order=orders[i], max_depth=depths[i], images=4,
                                  precision=prec[i] if isinstance(prec, list) else prec)
            s.execute(xyz, float(box[0]))
            singles.append(s)

        def seq():
            for i, s in enumerate(singles):
                s.execute_device(xd.data_ptr() + 12 * int(off[i]), float(B[i]), st.cuda_stream)

        ms_seq = timed(seq)
        seq_launches = sum(s.step_launches() for s in singles)
        per = [timed(lambda s=s, i=i: s.execute_device(xd.data_ptr() + 12 * int(off[i]), float(B[i]),
                                                       st.cuda_stream), 3) for i, s in enumerate(singles)]
        for s in singles:
            s.close()
        pn = sorted({PREC_NAME[v] for v in prec}) if isinstance(prec, list) else PREC_NAME[prec]
        return f, {"value": n / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "tile_autotune": tiles,
                   "ms_per_step_default_tiles": ms_default, "precision": pn, "launches_per_step": launches,
                   "sequential_single_solves": {"value": n / (ms_seq * 1e-3), "ms_per_step": ms_seq,
                                                "launches_per_step": seq_launches},
                   "speedup_vs_sequential": ms_seq / ms}, per

    spec_orders, spec_depths = batch_spec(tuner_mod, nat)
    _, spec, spec_per = run_batch(spec_orders, spec_depths, 1)
    spec.update(orders=sorted(set(spec_orders)), depths=sorted(set(spec_depths)),
                per_system_ms={"min": min(spec_per), "median": float(np.median(spec_per)), "max": max(spec_per)})
    # the tuner's proposal per system (statistics and MLP on the device, checked)
    mlp = tuner_mod.Mlp.load()
    props = []
    for xyz, q, box in sy:
        ts = tuner_mod.TunedSolver(q, mlp, tol=TOL)
        props.append(ts.propose(xyz, float(box[0])))
        ts.solver.close()
    mlp.close()
    orders = [p[0] for p in props]
    depths = [p[1] for p in props]
    precs = [p[2] for p in props]
    f, tuned, per = run_batch(orders, depths, precs)
    diffs = []
    for i, (xyz, q, box) in enumerate(sy):
        pl = pkg.ZetaFmmSolver(len(q), q, order=10, max_depth=tuner_mod.plain_depth(len(q)), images=4)
        pl.execute(xyz, float(box[0]))
        diffs.append(rel_diff(f[off[i]:off[i + 1]], pl.forces()))
        pl.close()
    tuned.update(orders=sorted(set(orders)), depths=sorted(set(depths)),
                 max_rel_force_diff_vs_plain=max(diffs), systems_over_tolerance=int(sum(d > TOL for d in diffs)),
                 per_system_ms={"min": min(per), "median": float(np.median(per)), "max": max(per)},
                 per_system=[{"atoms": nat[i], "order": orders[i], "depth": depths[i],
                              "precision": PREC_NAME[precs[i]], "ms": per[i],
                              "rel_force_diff_vs_plain": diffs[i]} for i in range(len(sy))])
    return {"workload": f"64 systems, {n} atoms (log-uniform 2,000-200,000 per system), 0.15 M NaCl, "
                        "order 6-10 and depth 3-5 per system, bf16x3",
            "atoms": n, "value": spec["value"], "unit": UNIT, "ms_per_step": spec["ms_per_step"],
            "spec": spec, "tuned": tuned}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbfmm", choices=["gbfmm", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=5)
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-system batched line")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the 1,002,002-atom line and the 250,002-atom trajectory line")
    ap.add_argument("--frames", type=int, default=200, help="frames of the trajectory line")
    ap.add_argument("--profile", default=None,
                    help="precision,order,depth[,p2p_variant,m2l_split,m2l_stages[,near_after]], or "
                         "batch[,shape,per_sm,m2l_split,m2l_stages,far_lanes,far_prio,near_after]: only run "
                         "--steps device-resident steps of that configuration and tuning, or of the 64-system "
                         "batch (a short, fixed launch sequence for ncu captures); prints no bench line")
    ap.add_argument("--large-only", action="store_true",
                    help="only the 1,002,002-atom slab line (printed alone; no bench line)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_env()
    systems = G.load_module("systems")
    xyz, q, box = systems.cfg_96k()
    n = len(q)
    if args.large_only:
        import torch
        pkg = G.load_package()
        print(json.dumps({"large": large_line(pkg, torch, torch.device("cuda", local), systems, 5)}))
        return
    if args.profile and args.profile.split(",")[0] == "batch":
        # device-resident steps of the 64-system batch of the batch line (orders
        # 6-10, depths 3-5, BF16X3); default tiles and schedule, or
        # batch,shape,per_sm,m2l_split,m2l_stages,far_lanes,far_prio,near_after
        import torch
        pkg = G.load_package()
        tuner_mod = G.load_module("tuner")
        sy = systems.batch_systems(n_sys=64)
        nat = [len(t[1]) for t in sy]
        orders, depths = batch_spec(tuner_mod, nat)
        X = np.concatenate([t[0] for t in sy]).astype(np.float32)
        Q = np.concatenate([t[1] for t in sy]).astype(np.float32)
        B = np.array([float(t[2][0]) for t in sy], np.float32)
        b = pkg.BatchSolver(nat, orders, depths, images=4, precision=1)
        tv = [int(v) for v in args.profile.split(",")[1:]]
        if len(tv) == 7:
            b.set_tuning(*tv[:4])
            b.set_schedule(*tv[4:])
        xd, qd = torch.from_numpy(X).cuda(), torch.from_numpy(Q).cuda()
        st = torch.cuda.current_stream()
        for _ in range(args.steps):
            b.execute_device(xd.data_ptr(), qd.data_ptr(), B, st.cuda_stream)
        torch.cuda.synchronize()
        print(json.dumps({"profile": args.profile, "steps": args.steps, "systems": len(nat), "atoms": int(sum(nat)),
                          "launches_per_step": b.step_launches()}))
        b.close()
        return
    if args.profile:
        # device-resident steps (gbfmm_execute_device, as 'value' is measured)
        import torch
        vals = [int(v) for v in args.profile.split(",")]
        prec, P, D = vals[:3]
        pkg = G.load_package()
        s = pkg.ZetaFmmSolver(n, q, order=P, max_depth=D, images=4, precision=prec)
        if len(vals) >= 6:
            s.set_tuning(*vals[3:6])
        if len(vals) == 7:
            s.set_near_start(vals[6])
        xd = torch.from_numpy(xyz).cuda()
        st = torch.cuda.current_stream()
        for _ in range(args.steps):
            s.execute_device(xd.data_ptr(), box, st.cuda_stream)
        torch.cuda.synchronize()
        print(json.dumps({"profile": args.profile, "steps": args.steps, "energy": s.get_energy(),
                          "launches_per_step": s.step_launches()}))
        s.close()
        return
    config = {"workload": WORKLOAD, "atoms": n, "images": 4, "tolerance": TOL, "order": HEADLINE[1],
              "depth": HEADLINE[2], "l2": "GPU arm: flushed (256 MB write) before every timed step",
              "parallelism": f"replicas{ws}"}

    if args.impl == "reference":
        if rank != 0:
            return
        steps = args.steps
        v, cores, sec = cpu_reference(xyz, q, box, HEADLINE[1], HEADLINE[2], steps, 1)
        line = {"metric": METRIC, "impl": "reference", "value": v, "unit": UNIT, "n_gpus": ws, "steps": steps,
                "warmup": 1, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": config,
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": f"{steps} steps of the full {n}-atom system, p={HEADLINE[1]}, depth "
                                           f"{HEADLINE[2]} (the GPU arm's order and depth); zeta_fmm algorithm in "
                                           "FP64 C (oracle/zeta64.c), OpenMP"},
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
    run = Runner(pkg, torch, dev, xyz, q, box)

    # FP64 Ewald forces on sampled atoms and the total energy: the accuracy reference
    # of every candidate (OpenMP on the host cores)
    from oracle import oracle as O
    O.set_threads(os.cpu_count() or 1)
    tg = np.arange(0, n, 191)
    _, fe, _ = O.ewald(xyz.astype(np.float64), q.astype(np.float64), box[0], eps=1e-9, targets=tg)
    _, _, ee = O.ewald(xyz.astype(np.float64), q.astype(np.float64), box[0], eps=1e-7, energy=True)

    def err_of(s):
        s.execute(xyz, box)
        f = s.forces()
        return float(np.sqrt(np.sum((f[tg] - fe) ** 2) / np.sum(fe ** 2)))

    def energy_err(s):
        return abs(s.get_energy() - ee) / abs(ee)  # after err_of's execute

    # tuned parameters: the learned tuner's proposal for this system (statistics
    # on the device, MLP forward on the device), checked against the plain
    # order-10 FMM on this configuration; the plain FMM is check and fallback
    tuner_mod = G.load_module("tuner")
    mlp = tuner_mod.Mlp.load()
    ts = tuner_mod.TunedSolver(q, mlp, tol=TOL)
    choice = ts.propose(xyz, float(box[0]))
    ts.solver.close()
    best = (choice[2], choice[0], choice[1])
    prop = ts.checks[0]["proposal"]
    tuner_info = {"proposal": None if prop is None else
                  {"order": prop[0], "depth": prop[1], "precision": PREC_NAME[prop[2]],
                   "pred_rel_force_err": prop[3], "pred_ms": prop[4]},
                  "checks": [{"order": c["proposal"][0], "diff_vs_plain": c["diff_vs_plain"],
                              "accepted": c["accepted"]} for c in ts.checks if c["proposal"] is not None],
                  "chosen": {"order": choice[0], "depth": choice[1], "precision": PREC_NAME[choice[2]]}}
    mlp.close()
    # exhaustive sweep over a candidate grid (FP32 included), reported beside the proposal
    tune = []
    for prec, P, D in CANDIDATES:
        s = run.solver(prec, P, D)
        e = err_of(s)
        ee_rel = energy_err(s)
        ms = run.time_device(s, 5, 3) / 5
        tune.append({"precision": PREC_NAME[prec], "order": P, "depth": D, "rel_force_err": e,
                     "rel_energy_err": ee_rel, "ms": ms})
        s.close()
    # the plain FP32 GPU FMM at the same accuracy: the fastest FP32 candidate that
    # meets the tolerance (default tiles in the sweep; autotuned below, as 'tuned')
    ok32 = [t for t in tune if t["precision"] == "fp32" and t["rel_force_err"] <= TOL]
    eq = min(ok32, key=lambda t: t["ms"]) if ok32 else None
    plain_eq = (0, eq["order"], eq["depth"]) if eq else PLAIN_REF

    results = {}
    for name, (prec, P, D) in (("plain_order10", PLAIN_REF), ("plain", plain_eq), ("tuned", best)):
        s = run.solver(prec, P, D)
        tiles = s.autotune(xyz, box, reps=5)  # tile shapes of this configuration (gbfmm_autotune)
        if ws > 1:
            dist.barrier()
        clk = Clocks(local)
        ms = run.time_device(s, args.steps, args.warmup, clocks=clk)
        value, ms = replica_throughput(n, args.steps, ms, dist if ws > 1 else None, dev)
        r = {"prec": prec, "P": P, "D": D, "ms": ms / args.steps, "value": value,
             "err": err_of(s), "clocks": clk.summary(), "launches": s.step_launches()}
        r["eerr"] = energy_err(s)
        r["e2e"] = n * ws * args.steps / run.time_e2e(s, args.steps)
        # the same call with staging copies (GBFMM_FLAG_HOST_COPY), for comparison
        sc = run.solver(prec, P, D, flags=pkg.FLAG_HOST_COPY)
        t = s.tuning()
        sc.set_tuning(t["p2p_variant"], t["m2l_split"], t["m2l_stages"])
        sc.set_near_start(t["near_after"])
        r["e2e_copies"] = n * ws * args.steps / run.time_e2e(sc, args.steps)
        sc.close()
        r["stages"] = run.stages(s, args.steps)
        r["tiles"] = tiles
        _, _, ln = s.tree()
        r["p2p_pairs"] = p2p_pair_count(ln, D)
        results[name] = r
        s.close()

    tuned, plain, plain10 = results["tuned"], results["plain"], results["plain_order10"]
    pk, src = peaks()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = sms * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    P, D = tuned["P"], tuned["D"]
    st = tuned["stages"]
    kern = {}
    alg = m2l_flops_per_pair(P) * m2l_pairs(D)
    if "m2l" in st:
        a = alg / (st["m2l"] * 1e-3) / 1e12
        if tuned["prec"] == 0:
            kern["m2l"] = {"ms": st["m2l"], "bound": "fp32-cuda-core", "achieved": a, "peak": fp32_peak,
                           "unit": "TFLOP/s", "frac": a / fp32_peak}
        else:
            kern["m2l"] = {"ms": st["m2l"], "bound": "tensor", "achieved": a, "peak": pk["bf16_tflops"],
                           "unit": "TFLOP/s", "frac": a / pk["bf16_tflops"],
                           "note": "algorithmic flops (8*sum_j (j+1)(P-j+1)^2 per pair); the split-bf16 MMAs "
                                   "execute more"}
    if "p2p" in st:
        a = 20.0 * tuned["p2p_pairs"] / (st["p2p"] * 1e-3) / 1e12
        # the FMA pipe's own bound: 13 FP32 lane operations per pair (3 differences, 3 for r^2,
        # r^-2, q r^-1, its product with r^-2, the potential sum, 3 gradient FMAs)
        floor_ms = 13.0 * tuned["p2p_pairs"] / (sms * 128 * pk.get("sm_max_mhz", 2070.0) * 1e6) * 1e3
        kern["p2p"] = {"ms": st["p2p"], "bound": "fp32-cuda-core", "achieved": a, "peak": fp32_peak,
                       "unit": "TFLOP/s", "frac": a / fp32_peak, "pairs": tuned["p2p_pairs"],
                       "fma_pipe_floor_ms": floor_ms, "frac_of_fma_pipe_floor": floor_ms / st["p2p"]}
    dom = max((k for k in st if k in kern), key=lambda k: st[k], default=None)
    roof = None
    if dom:
        k = kern[dom]
        tb, tsrc = ncu_traffic("k_" + dom + ("_tc" if dom == "m2l" and tuned["prec"] else ""))
        roof = {"kernel": dom, "bound": k["bound"], "achieved": k["achieved"], "peak": k["peak"], "unit": k["unit"],
                "frac": k["frac"], "traffic": tb, "traffic_source": tsrc,
                "peak_source": (f"bf16 dense, MEASURED_PEAKS.json ({src})" if k["bound"] == "tensor" else
                                f"nominal {sms} SMs x 128 FP32 lanes x 2 x sm_max_mhz (no FP32 entry in "
                                "MEASURED_PEAKS.json)"), "sms": sms}
    line = {"metric": METRIC, "value": tuned["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tuned["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+bf16x3" if tuned["prec"] == 1 else (
                "f32+bf16" if tuned["prec"] == 2 else "f32"), "data": "synthetic",
            "config": dict(config, order=P, depth=D), "m2l_precision": PREC_NAME[tuned["prec"]],
            "rel_force_err_vs_ewald": tuned["err"], "rel_energy_err_vs_ewald": tuned["eerr"],
            "ewald": "FP64 Ewald (oracle/ewald64.c): forces on every 191st atom (eps 1e-9), total energy "
                     "(eps 1e-7)",
            "e2e": {"value": tuned["e2e"], "unit": UNIT, "h2d_bytes_per_step": 12 * n,
                    "d2h_bytes_per_step": 12 * n + 4 * n + 8,
                    "host_io": ("in place: the step reads the host coordinates and writes the host results "
                                "over NVLink-C2C (pageable-memory access), no staging copies")
                    if pageable_access(local) else "staging copies (cudaMemcpyAsync)",
                    "value_with_copies": tuned["e2e_copies"]},
            "plain_fp32": {"value": plain["value"], "ms_per_step": plain["ms"], "order": plain["P"],
                           "depth": plain["D"], "rel_force_err_vs_ewald": plain["err"],
                           "rel_energy_err_vs_ewald": plain["eerr"], "e2e": plain["e2e"],
                           "stage_ms": plain["stages"],
                           "chosen_as": "fastest FP32 (order, depth) of the sweep within the tolerance"
                           if eq else "no FP32 candidate met the tolerance: reference parameters"},
            "plain_fp32_order10": {"value": plain10["value"], "ms_per_step": plain10["ms"], "order": plain10["P"],
                                   "depth": plain10["D"], "rel_force_err_vs_ewald": plain10["err"],
                                   "rel_energy_err_vs_ewald": plain10["eerr"], "e2e": plain10["e2e"],
                                   "stage_ms": plain10["stages"]},
            "speedup_tuned_vs_plain": tuned["value"] / plain["value"],
            "speedup_tuned_vs_plain_order10": tuned["value"] / plain10["value"],
            "headline_matches_tuner": (tuned["prec"], P, D) == HEADLINE,
            "tuner": tuner_info, "tile_autotune": {"tuned": tuned["tiles"], "plain": plain["tiles"]},
            "sweep": tune, "stage_ms": st, "kernels": kern, "roofline": roof, "clocks": tuned["clocks"],
            "gpu_launches": tuned["launches"] * args.steps}
    if rank == 0 and not args.no_batch:
        line["batch"] = batch_line(pkg, torch, dev, systems, max(3, min(args.steps, 10)), 2)
    if rank == 0 and not args.no_extra:
        line["large"] = large_line(pkg, torch, dev, systems, 5)
        line["frames"] = frames_line(pkg, torch, dev, systems, tuner_mod, args.frames)
    if rank == 0:
        v, cores, sec = cpu_reference(xyz, q, box, P, D, args.cpu_steps, 1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"{args.cpu_steps} steps of the full {n}-atom system, p={P}, depth {D} "
                                          "(the order and depth of 'value'); zeta_fmm algorithm in FP64 C "
                                          "(oracle/zeta64.c), OpenMP"}
        print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
