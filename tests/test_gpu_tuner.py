"""The learned parameter tuner on the GPU: its forward/backward kernels against
the FP64 numpy restatement, training, the weights file, the statistics kernel
against numpy, and the gain of its checked proposals over the plain order-10
FP32 FMM on systems it was not trained on."""
import os

import numpy as np
import pytest

from conftest import G, rel_rms

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
from oracle import mlp64  # noqa: E402


@pytest.fixture(scope="module")
def tuner(pkg):
    return G.load_module("tuner")


def _data(rng, B, I, O):
    x = rng.normal(size=(B, I)).astype(np.float32)
    t = rng.normal(size=(B, O)).astype(np.float32)
    return x, t


def test_forward_and_gradient_match_fp64_oracle(tuner):
    I, H, O, B = 60, 64, 2, 97
    m = tuner.Mlp(I, H, O, seed=3)
    p = m.params()
    x, t = _data(np.random.default_rng(1), B, I, O)
    y = m.forward(x)
    y64 = mlp64.forward(p, x, I, H, O)
    assert np.max(np.abs(y - y64)) <= 1e-5 * max(1.0, np.max(np.abs(y64)))
    loss, g = m.loss_grad(x, t)
    loss64, g64 = mlp64.loss_grad(p, x, t, I, H, O)
    assert abs(loss - loss64) <= 1e-5 * loss64
    assert rel_rms(g, g64) < 1e-5
    # every parameter block, not just the norm
    for lo, hi in [(0, H * I), (H * I + H, H * I + H + H * H), (len(p) - O * H - O, len(p))]:
        assert rel_rms(g[lo:hi], g64[lo:hi]) < 1e-5
    m.close()


def test_training_fits_a_smooth_function(tuner):
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, size=(2048, 6)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2], np.exp(0.5 * x[:, 3]) - x[:, 4] ** 2], 1).astype(np.float32)
    m, loss = tuner.fit(x, t, n_hidden=32, epochs=150, batch=64, lr=3e-3, seed=4)
    y = m.predict(x)
    base = np.mean(np.sum((t - t.mean(0)) ** 2, 1))
    assert np.mean(np.sum((y - t) ** 2, 1)) < 0.02 * base
    # deterministic: the same seed trains the same network
    m2, _ = tuner.fit(x, t, n_hidden=32, epochs=150, batch=64, lr=3e-3, seed=4)
    assert np.array_equal(m.params(), m2.params())
    m.close()
    m2.close()


def test_save_load_and_corruption(tuner, tmp_path, pkg):
    rng = np.random.default_rng(5)
    x, t = _data(rng, 256, 60, 2)
    m, _ = tuner.fit(x, t, epochs=3, seed=1)
    path = str(tmp_path / "w.bin")
    m.save(path)
    m2 = tuner.Mlp.load(path)
    assert np.array_equal(m.params(), m2.params())
    assert np.array_equal(m.predict(x[:10]), m2.predict(x[:10]))
    raw = bytearray(open(path, "rb").read())
    raw[100] ^= 0x10
    bad = str(tmp_path / "bad.bin")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(pkg.FmmError):
        tuner.Mlp.load(bad)
    open(bad, "wb").write(bytes(raw[:len(raw) // 2]))
    with pytest.raises(pkg.FmmError):
        tuner.Mlp.load(bad)
    m.close()
    m2.close()


def _features_numpy(xyz, q, box):
    """Restatement of gbfmm_features' statistics: a cube of edge L, or a slab
    L x L x 2L whose tree root is the cube of edge 2L (only the box's cells)."""
    b = np.broadcast_to(np.asarray(box, np.float64), (3,))
    slab = b[2] != b[0]
    C = b[2]
    sxy = 1 if slab else 0
    x = np.asarray(xyz, np.float32)
    inv = np.float32(64 / np.float64(C))
    hi = np.array([64 >> sxy, 64 >> sxy, 64])
    idx = np.clip(np.floor(x * inv).astype(np.int64), 0, hi - 1)
    N = len(q)
    q64 = q.astype(np.float64)
    V = b[0] * b[1] * b[2]
    f = np.zeros(57)
    f[0] = np.log10(N)
    f[1] = np.log10(N / V)
    f[2] = np.log10(C)
    f[3] = np.sum(q64 ** 2) / N
    f[4] = abs(q64.sum()) / np.sqrt(np.sum(q64 ** 2))
    d = (q64[:, None] * x.astype(np.float64)).sum(0) - q64.sum() * b / 2
    f[5] = np.log10(np.sum(d * d) / (V * np.sum(q64 ** 2)) + 1e-12)
    f[56] = 1.0 if slab else 0.0
    for k in range(2, 7):
        c = idx >> (6 - k)
        nxy = (1 << k) >> sxy
        cell = (c[:, 0] * nxy + c[:, 1]) * (1 << k) + c[:, 2]
        cnt = np.bincount(cell, minlength=nxy * nxy * (1 << k))
        bb = np.zeros(len(cnt), np.int64)
        nz = cnt > 0
        bb[nz] = np.minimum(1 + np.floor(np.log2(cnt[nz])).astype(np.int64), 8)
        f[6 + 9 * (k - 2):6 + 9 * (k - 1)] = np.bincount(bb, minlength=9) / len(cnt)
        f[51 + k - 2] = np.log2(N / nz.sum())
    return f


def test_features_match_numpy(tuner, systems):
    for spec in [(3000, 4.0, 0, 1.0, False), (9000, 5.2, 20, 0.55, False), (6000, 3.6, 10, 0.5, True)]:
        n_sites, L, ions, fill, slab = spec
        box = [L, L, 2 * L] if slab else L
        xyz, q, b = systems.water_ion_box(n_sites, box, n_na=ions, n_cl=ions, seed=11, fill_z=fill)
        xd = torch.from_numpy(xyz).cuda()
        qd = torch.from_numpy(q).cuda()
        bx = [float(np.float32(v)) for v in np.broadcast_to(b, (3,))]
        f = tuner.features(xd.data_ptr(), qd.data_ptr(), len(q), bx, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        ref = _features_numpy(xyz, q, bx)
        assert np.allclose(f[6:51], ref[6:51], atol=1e-7)   # occupancy histograms: exact counts
        assert np.allclose(f[[0, 1, 2, 3, 51, 52, 53, 54, 55, 56]], ref[[0, 1, 2, 3, 51, 52, 53, 54, 55, 56]],
                           rtol=1e-5)
        assert abs(f[4] - ref[4]) <= 1e-4 * max(1.0, ref[4]) + 1e-6
        assert abs(f[5] - ref[5]) <= 1e-3 * max(1.0, abs(ref[5]))


class _Timer:
    def __init__(self):
        self.flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        self.stream = torch.cuda.Stream()

    def __call__(self, solver, xd, L, reps=9):
        ts = []
        with torch.cuda.stream(self.stream):
            for r in range(reps + 2):
                self.flush.fill_(r & 0xff)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(self.stream)
                solver.execute_device(xd.data_ptr(), L, self.stream.cuda_stream)
                e1.record(self.stream)
                e1.synchronize()
                if r >= 2:
                    ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))


# held-out systems: seeds and shapes outside the training specs
HELD_OUT = [(20000, 8.45, 60, 1.0, 901), (32000, 12.0, 0, 0.55, 902), (26000, 8.8, 150, 1.0, 903)]


@pytest.mark.parametrize("n_sites,L,ions,fill,seed", HELD_OUT)
def test_checked_proposal_gain_over_plain(tuner, oracle, systems, pkg, n_sites, L, ions, fill, seed):
    """The proposal (checked against the plain FMM on this configuration) meets
    1e-3 relative RMS force error against FP64 Ewald and runs at least twice as
    fast as the plain order-10 FP32 FMM."""
    tol = 1e-3
    xyz, q, box = systems.water_ion_box(n_sites, L, n_na=ions, n_cl=ions, seed=seed, fill_z=fill)
    L = float(box[0])
    mlp = tuner.Mlp.load()
    ts = tuner.TunedSolver(q, mlp, tol=tol)
    choice = ts.propose(xyz, L)
    assert ts.checks and any(c["accepted"] for c in ts.checks), ts.checks
    assert choice != (tuner.PLAIN_ORDER, tuner.plain_depth(len(q)), pkg.PREC_FP32)
    f = ts.execute(xyz, L)
    tg = np.arange(0, len(q), 53)
    _, fe, _ = oracle.ewald(xyz.astype(np.float64), q.astype(np.float64), L, eps=1e-9, targets=tg)
    assert rel_rms(f[tg], fe) <= tol
    plain = ts._plain()
    plain.execute(xyz, L)
    xd = torch.from_numpy(xyz).cuda()
    timer = _Timer()
    t_tuned = timer(ts.solver, xd, L)
    t_plain = timer(plain, xd, L)
    assert t_plain / t_tuned >= 2.0, (choice, t_tuned, t_plain)
    plain.close()
    ts.solver.close()
    mlp.close()


def test_unreachable_tolerance_falls_back_to_the_plain_fmm(tuner, systems, pkg):
    """No candidate can meet 1e-9 against the plain FMM: gbfmm_tuner_choose keeps
    the plain order-10 FP32 parameters and says so (the fallback of the checked
    choice)."""
    xyz, q, box = systems.water_ion_box(3000, 4.5, seed=77)
    mlp = tuner.Mlp.load()
    ts = tuner.TunedSolver(q, mlp, tol=1e-9)
    choice = ts.propose(xyz, float(box[0]))
    assert choice == (tuner.PLAIN_ORDER, tuner.plain_depth(len(q)), pkg.PREC_FP32)
    assert not any(c["accepted"] for c in ts.checks)
    plain = ts._plain()
    plain.execute(xyz, float(box[0]))
    assert rel_rms(ts.execute(xyz, float(box[0])), plain.forces()) < 1e-6
    plain.close()
    ts.solver.close()
    mlp.close()
