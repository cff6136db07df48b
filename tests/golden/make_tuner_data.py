"""Makes the parameter tuner's training tuples and trains the shipped weights.

Needs a GB300 (the library's kernels time every candidate and train the
network) and the FP64 oracle (the error labels are taken against its converged
Ewald sum):

  python tests/golden/make_tuner_data.py generate --out tests/golden/tuner_tuples.npz
  python tests/golden/make_tuner_data.py train --tuples tests/golden/tuner_tuples.npz \
      --out gromacs-fmm_gb300/tuner_weights.bin

One tuple = the statistics of one seeded system (gbfmm_features) + one candidate
(order 4..10, every depth with 2..200 bodies per stored leaf, BF16X3 and BF16X1
M2L) +
two labels: log10 of the candidate's relative RMS force error against FP64 Ewald
(eps 1e-9) on a stride sample of at most 1000 atoms, and log10 of its step time
in ms (device-resident inputs, CUDA events, L2 flushed before every step, median
of 7 steps).  `train` also reports leave-systems-out validation: the error of
the predictions and the regret of the proposals on systems the network did not
see.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import __graft_entry__ as G  # noqa: E402

PRECS = (1, 2)          # BF16X3, BF16X1
ORDERS = range(4, 11)
SITE_DENSITY = 33.4     # water sites per nm^3 at 1 g/cm^3


def system_specs(n, seed0):
    """Seeded system descriptions: size (1,000 to 330,000 water sites, about 3,000
    to 1,000,000 atoms, log-uniform), density, ion content, box shape (a cube, or
    a slab Lx = Ly, Lz = 2 Lx) and the filled fraction of the box's height (the
    rest is vacuum)."""
    out = []
    for i in range(n):
        rng = np.random.default_rng(seed0 + i)
        n_sites = int(round(10 ** rng.uniform(3.0, 5.52)))
        dens = float(rng.choice([0.7, 1.0, 1.0, 1.35]))
        ion = float(rng.choice([0.0, 0.002, 0.01, 0.03]))
        slab = bool(rng.random() < 0.3)
        fill = float(rng.choice([1.0, 0.5, 0.5])) if slab else float(rng.choice([1.0, 1.0, 1.0, 0.55]))
        out.append(dict(n_sites=n_sites, dens=dens, ion=ion, fill=fill, slab=slab, seed=seed0 + i))
    return out


def make_system(systems, spec):
    """(coords, charges, box [Lx, Ly, Lz])."""
    vol = spec["n_sites"] / (SITE_DENSITY * spec["dens"] * spec["fill"])
    if spec.get("slab"):
        a = (vol / 2.0) ** (1.0 / 3.0)
        box = [a, a, 2 * a]
    else:
        L = vol ** (1.0 / 3.0)
        box = [L, L, L]
    ions = int(spec["n_sites"] * spec["ion"] / 2)
    xyz, q, b = systems.water_ion_box(spec["n_sites"], box, n_na=ions, n_cl=ions, seed=spec["seed"],
                                      fill_z=spec["fill"])
    b32 = [float(np.float32(v)) for v in b]
    b32[2] = 2 * b32[0] if spec.get("slab") else b32[0]
    b32[1] = b32[0]
    return xyz, q, b32


def depths_for(natoms, slab=False):
    stored = (lambda d: 8.0 ** d / 4) if slab else (lambda d: 8.0 ** d)
    return [d for d in range(1, 8) if 2 <= natoms / stored(d) <= 200]


class Timer:
    """Per-step device time of a solver's execute_device (L2 flushed first)."""

    def __init__(self, torch):
        self.torch = torch
        self.flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        self.stream = torch.cuda.Stream()

    def __call__(self, solver, d_coords, box, reps=7):
        torch = self.torch
        ts = []
        with torch.cuda.stream(self.stream):
            for r in range(reps + 2):
                self.flush.fill_(r & 0xff)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(self.stream)
                solver.execute_device(d_coords.data_ptr(), box, self.stream.cuda_stream)
                e1.record(self.stream)
                e1.synchronize()
                if r >= 2:
                    ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))


def generate(args):
    import torch
    pkg = G.load_package()
    pkg.build()
    systems = G.load_module("systems")
    tuner = G.load_module("tuner")
    from oracle import oracle as O
    timer = Timer(torch)
    rows = []
    t_start = time.time()
    O.set_threads(os.cpu_count() or 1)
    for k, spec in enumerate(system_specs(args.systems, args.seed)):
        xyz, q, L = make_system(systems, spec)
        n = len(q)
        stride = max(97, n // 1000)
        tg = np.arange(0, n, stride)
        _, fe, _ = O.ewald(xyz.astype(np.float64), q.astype(np.float64), np.array(L), eps=1e-9, targets=tg)
        xd = torch.from_numpy(np.ascontiguousarray(xyz, np.float32)).cuda()
        qd = torch.from_numpy(np.ascontiguousarray(q, np.float32)).cuda()
        feat = tuner.features(xd.data_ptr(), qd.data_ptr(), n, L, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        aspect = 2 if spec.get("slab") else 1
        for D in depths_for(n, aspect == 2):
            for P in ORDERS:
                for prec in PRECS:
                    s = pkg.ZetaFmmSolver(n, q, order=P, max_depth=D, images=4, precision=prec, aspect_z=aspect)
                    s.execute(xyz, L)
                    f = s.forces()
                    err = float(np.sqrt(np.sum((f[tg] - fe) ** 2) / np.sum(fe ** 2)))
                    ms = timer(s, xd, L)
                    s.close()
                    rows.append(dict(system=k, natoms=n, order=P, depth=D, precision=prec, err=err, ms=ms,
                                     feat=feat.tolist(), spec=spec))
        print(json.dumps({"system": k, "natoms": n, "spec": spec, "tuples": len(rows),
                          "elapsed_s": round(time.time() - t_start, 1)}), flush=True)
    np.savez_compressed(
        args.out,
        system=np.array([r["system"] for r in rows], np.int32),
        natoms=np.array([r["natoms"] for r in rows], np.int32),
        order=np.array([r["order"] for r in rows], np.int32),
        depth=np.array([r["depth"] for r in rows], np.int32),
        precision=np.array([r["precision"] for r in rows], np.int32),
        err=np.array([r["err"] for r in rows]),
        ms=np.array([r["ms"] for r in rows]),
        feat=np.array([r["feat"] for r in rows], np.float32),
        specs=np.array(json.dumps(system_specs(args.systems, args.seed))),
    )


def design(tuner, d):
    x = np.stack([tuner.tuner_input(d["feat"][i], d["order"][i], d["depth"][i], d["precision"][i])
                  for i in range(len(d["order"]))])
    t = np.stack([np.log10(np.maximum(d["err"], 1e-7)), np.log10(d["ms"])], axis=1).astype(np.float32)
    return x, t


def proposal_quality(tuner, m, d, systems_idx, tol, margin):
    """For each system: the proposal's true error and time against the fastest
    candidate that truly meets tol."""
    out = []
    for k in systems_idx:
        sel = np.nonzero(d["system"] == k)[0]
        prop = m.propose(d["feat"][sel[0]], tol, margin)
        ok = sel[d["err"][sel] <= tol]
        best = float(d["ms"][ok].min()) if len(ok) else None
        if prop is None:
            out.append(dict(system=int(k), proposal=None, best_ms=best))
            continue
        P, D, prec = prop[:3]
        hit = sel[(d["order"][sel] == P) & (d["depth"][sel] == D) & (d["precision"][sel] == prec)]
        e, t = float(d["err"][hit[0]]), float(d["ms"][hit[0]])
        out.append(dict(system=int(k), natoms=int(d["natoms"][sel[0]]), proposal=[P, D, prec], err=e, ms=t,
                        best_ms=best, regret=(t / best if best else None), meets_tol=e <= tol))
    return out


def train(args):
    pkg = G.load_package()
    pkg.build()
    tuner = G.load_module("tuner")
    d = dict(np.load(args.tuples))
    x, t = design(tuner, d)
    sysids = np.unique(d["system"])
    # leave-systems-out validation: 4 folds by system
    folds = [sysids[i::4] for i in range(4)]
    val = []
    for f, held in enumerate(folds):
        tr = ~np.isin(d["system"], held)
        m, loss = tuner.fit(x[tr], t[tr], epochs=args.epochs, lr=args.lr, batch=args.batch, seed=args.seed + f)
        y = m.predict(x[~tr])
        mae = np.abs(y - t[~tr]).mean(0)
        q = proposal_quality(tuner, m, d, held, args.tol, args.margin)
        val.append(dict(fold=f, train_loss=loss, mae_log10_err=float(mae[0]), mae_log10_ms=float(mae[1]),
                        proposals=q))
        m.close()
    m, loss = tuner.fit(x, t, epochs=args.epochs, lr=args.lr, batch=args.batch, seed=args.seed)
    m.save(args.out)
    report = dict(tuples=int(len(x)), systems=int(len(sysids)), final_loss=loss, validation=val)
    print(json.dumps(report))
    if args.report:
        with open(args.report, "w") as fh:
            json.dump(report, fh, indent=1)


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    g = sub.add_parser("generate")
    g.add_argument("--out", default=os.path.join(ROOT, "tests", "golden", "tuner_tuples.npz"))
    g.add_argument("--systems", type=int, default=70)
    g.add_argument("--seed", type=int, default=5000)
    tr = sub.add_parser("train")
    tr.add_argument("--tuples", default=os.path.join(ROOT, "tests", "golden", "tuner_tuples.npz"))
    tr.add_argument("--out", default=os.path.join(ROOT, "gromacs-fmm_gb300", "tuner_weights.bin"))
    tr.add_argument("--report", default=None)
    tr.add_argument("--epochs", type=int, default=1500)
    tr.add_argument("--batch", type=int, default=64)
    tr.add_argument("--lr", type=float, default=2e-3)
    tr.add_argument("--seed", type=int, default=0)
    tr.add_argument("--tol", type=float, default=1e-3)
    tr.add_argument("--margin", type=float, default=1.5)
    a = ap.parse_args()
    generate(a) if a.cmd == "generate" else train(a)


if __name__ == "__main__":
    main()
