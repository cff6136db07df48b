"""Batched solves: independent systems of uneven sizes, each with its own order
and depth, through one CUDA graph.  With GBFMM_FLAG_DETERMINISTIC each system's
result must equal a separate deterministic single-system solve bit for bit
(same kernels, same summation order); without it the split-entry M2L adds with
atomics, so the comparison is at FP32 rounding level.  Both are checked against
the FP64 oracle."""
import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu


def _systems(systems):
    specs = [(1200, 2.5, 6, 2, 3), (400, 1.7, 8, 2, 1), (3000, 3.3, 5, 3, 6), (150, 1.2, 4, 1, 0),
             (2200, 2.9, 7, 3, 4)]
    out = []
    for k, (nsite, L, P, D, ions) in enumerate(specs):
        xyz, q, box = systems.water_ion_box(nsite, L, n_na=ions, n_cl=ions, seed=100 + k)
        out.append((xyz, q, float(box[0]), P, D))
    return out


@pytest.mark.parametrize("precision,det", [(0, True), (1, True), (0, False)])
def test_batch_matches_single_solves_and_oracle(pkg, oracle, systems, precision, det):
    sy = _systems(systems)
    flags = pkg.FLAG_DETERMINISTIC if det else 0
    b = pkg.BatchSolver([len(s[1]) for s in sy], [s[3] for s in sy], [s[4] for s in sy], images=4,
                        precision=precision, flags=flags)
    X = np.concatenate([s[0] for s in sy])
    Q = np.concatenate([s[1] for s in sy])
    B = np.array([s[2] for s in sy], np.float32)
    for _ in range(2):  # the second call replays the captured graph
        f, p, e = b.execute(X, Q, B)
    off = b.offsets
    tol = 1e-5 if precision == 0 else 1e-4
    for i, (xyz, q, L, P, D) in enumerate(sy):
        s = pkg.ZetaFmmSolver(len(q), q, order=P, max_depth=D, images=4, precision=precision, flags=flags)
        s.execute(xyz, L)
        fi, pi = f[off[i]:off[i + 1]], p[off[i]:off[i + 1]]
        if det:
            assert np.array_equal(fi, s.forces())
            assert np.array_equal(pi, s.potentials())
            assert e[i] == s.get_energy()
        else:
            assert rel_rms(fi, s.forces()) < 2e-6
            assert rel_rms(pi, s.potentials()) < 2e-6
            assert abs(e[i] - s.get_energy()) <= 2e-6 * abs(e[i])
        po, fo, eo = oracle.zeta_solve(xyz.astype(np.float64), q.astype(np.float64), L, P, D, 4)
        assert rel_rms(fi, fo) < tol
        assert abs(e[i] - eo) / abs(eo) < tol
        s.close()
    b.close()


def test_batch_device_path_follows_new_coordinates(pkg, systems):
    torch = pytest.importorskip("torch")
    sy = _systems(systems)[:3]
    b = pkg.BatchSolver([len(s[1]) for s in sy], [s[3] for s in sy], [s[4] for s in sy])
    X = np.concatenate([s[0] for s in sy])
    Q = np.concatenate([s[1] for s in sy])
    B = np.array([s[2] for s in sy], np.float32)
    f1, _, _ = b.execute(X, Q, B)
    X2 = (X * np.float32(1.03)).astype(np.float32)
    B2 = (B * np.float32(1.03)).astype(np.float32)
    xd = torch.from_numpy(X2).cuda()
    qd = torch.from_numpy(Q).cuda()
    st = torch.cuda.current_stream()
    b.execute_device(xd.data_ptr(), qd.data_ptr(), B2, st.cuda_stream)
    st.synchronize()
    f2, _, _ = b.execute(X2, Q, B2)
    s = pkg.ZetaFmmSolver(len(sy[0][1]), sy[0][1], order=sy[0][3], max_depth=sy[0][4])
    s.execute(X2[:len(sy[0][1])], float(B2[0]))
    assert rel_rms(f2[:len(sy[0][1])], s.forces()) < 2e-6
    assert rel_rms(f1, f2) > 1e-3  # the new coordinates were used
    s.close()
    b.close()


def _batch_inputs(pkg, systems, precision, flags=0):
    sy = _systems(systems)
    b = pkg.BatchSolver([len(s[1]) for s in sy], [s[3] for s in sy], [s[4] for s in sy], images=4,
                        precision=precision, flags=flags)
    X = np.concatenate([s[0] for s in sy])
    Q = np.concatenate([s[1] for s in sy])
    B = np.array([s[2] for s in sy], np.float32)
    return b, X, Q, B


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_every_tuning_matches(pkg, systems, precision):
    """Every near-field shape and residency of the batch kernel (a CTA per leaf,
    or resident CTAs walking the queue), and every M2L split and depth, give the
    same forces up to the order of the additions."""
    b, X, Q, B = _batch_inputs(pkg, systems, precision)
    f0, p0, _ = b.execute(X, Q, B)
    for shape in range(5):
        for per_sm in (0, 2, 5):
            b.set_tuning(shape, per_sm, 0, 0)
            f, p, _ = b.execute(X, Q, B)
            assert rel_rms(f, f0) < 1e-5, (shape, per_sm)
            assert rel_rms(p, p0) < 1e-5, (shape, per_sm)
    if precision:
        for split in (1, 2, 4, 8):
            for stages in (1, 2):
                b.set_tuning(0, 4, split, stages)
                f, _, _ = b.execute(X, Q, B)
                assert rel_rms(f, f0) < 1e-5, (split, stages)
    with pytest.raises(pkg.FmmError):
        b.set_tuning(5, 4, 0, 0)
    with pytest.raises(pkg.FmmError):
        b.set_tuning(0, 6, 0, 0)
    b.close()


def test_batch_autotune_keeps_a_valid_tuning(pkg, systems):
    torch = pytest.importorskip("torch")
    b, X, Q, B = _batch_inputs(pkg, systems, 1)
    f0, _, e0 = b.execute(X, Q, B)
    xd = torch.from_numpy(X).cuda()
    qd = torch.from_numpy(Q).cuda()
    t = b.autotune(xd.data_ptr(), qd.data_ptr(), B, reps=2)
    assert t["ms"] > 0 and 0 <= t["p2p_shape"] < 5 and 0 <= t["p2p_per_sm"] <= 5
    assert t["m2l_split"] in (0, 1, 2, 4, 8)
    f1, _, e1 = b.execute(X, Q, B)
    assert rel_rms(f1, f0) < 1e-5
    assert np.allclose(e1, e0, rtol=1e-5, atol=0)
    b.close()


def test_deterministic_batch_keeps_whole_m2l_tiles(pkg, systems):
    b, X, Q, B = _batch_inputs(pkg, systems, 1, flags=pkg.FLAG_DETERMINISTIC)
    with pytest.raises(pkg.FmmError):
        b.set_tuning(0, 4, 2, 0)
    f1, _, _ = b.execute(X, Q, B)
    b.set_tuning(3, 3, 1, 2)
    f2, _, _ = b.execute(X, Q, B)
    f3, _, _ = b.execute(X, Q, B)
    assert np.array_equal(f2, f3)
    assert rel_rms(f2, f1) < 1e-5
    b.close()


def test_batch_mixed_precisions_match_single_solves(pkg, systems):
    """Each system with its own M2L precision (gbfmm_batch_create_mixed): bit for
    bit the deterministic single-system solve at that precision."""
    sy = _systems(systems)
    precs = [0, 1, 2, 1, 0]
    b = pkg.BatchSolver([len(s[1]) for s in sy], [s[3] for s in sy], [s[4] for s in sy], images=4,
                        precision=precs, flags=pkg.FLAG_DETERMINISTIC)
    X = np.concatenate([s[0] for s in sy])
    Q = np.concatenate([s[1] for s in sy])
    B = np.array([s[2] for s in sy], np.float32)
    for _ in range(2):
        f, p, e = b.execute(X, Q, B)
    off = b.offsets
    for i, (xyz, q, L, P, D) in enumerate(sy):
        s = pkg.ZetaFmmSolver(len(q), q, order=P, max_depth=D, images=4, precision=precs[i],
                              flags=pkg.FLAG_DETERMINISTIC)
        s.execute(xyz, L)
        assert np.array_equal(f[off[i]:off[i + 1]], s.forces()), i
        assert e[i] == s.get_energy(), i
        s.close()
    b.close()


def test_batch_launch_count_does_not_grow_with_systems(pkg, systems):
    """The batch step launches each kind of kernel once for all systems (once per
    order or shared-memory size where the kernel depends on them): doubling the
    systems at the same orders and depths keeps the launch count, which stays
    below the sum of the systems' single-solve launches."""
    sy = _systems(systems)
    counts = []
    for rep in (1, 2):
        s2 = sy * rep
        b = pkg.BatchSolver([len(s[1]) for s in s2], [s[3] for s in s2], [s[4] for s in s2], images=4,
                            precision=1, flags=pkg.FLAG_DETERMINISTIC)
        X = np.concatenate([s[0] for s in s2])
        Q = np.concatenate([s[1] for s in s2])
        B = np.array([s[2] for s in s2], np.float32)
        f, _, _ = b.execute(X, Q, B)
        counts.append(b.step_launches())
        if rep == 2:
            n1 = b.offsets[len(sy)]
            assert np.array_equal(f[:n1], f[n1:])  # the same systems twice: the same bits
        b.close()
    singles = 0
    for xyz, q, L, P, D in sy:
        s = pkg.ZetaFmmSolver(len(q), q, order=P, max_depth=D, images=4, precision=1, flags=pkg.FLAG_DETERMINISTIC)
        s.execute(xyz, L)
        singles += s.step_launches()
        s.close()
    assert counts[0] == counts[1], counts
    assert counts[0] < singles, (counts, singles)


def test_batch_schedule_leaves_results_unchanged(pkg, systems):
    """Far-field lanes, their stream priority and the near field's start point
    only move work between streams: under GBFMM_FLAG_DETERMINISTIC every
    schedule gives the same bits."""
    sy = _systems(systems)
    b = pkg.BatchSolver([len(s[1]) for s in sy], [s[3] for s in sy], [s[4] for s in sy], images=4,
                        precision=1, flags=pkg.FLAG_DETERMINISTIC)
    X = np.concatenate([s[0] for s in sy])
    Q = np.concatenate([s[1] for s in sy])
    B = np.array([s[2] for s in sy], np.float32)
    f0, p0, e0 = b.execute(X, Q, B)
    n0 = b.step_launches()
    for sched in [(2, 0, 0), (3, 1, 1), (5, 0, 2), (1, 1, 1)]:
        b.set_schedule(*sched)
        assert b.schedule() == dict(zip(("far_lanes", "far_prio", "near_after"), sched))
        f, p, e = b.execute(X, Q, B)
        assert np.array_equal(f, f0) and np.array_equal(p, p0) and np.array_equal(e, e0), sched
        assert b.step_launches() >= n0
    with pytest.raises(pkg.FmmError):
        b.set_schedule(9, 0, 0)
    with pytest.raises(pkg.FmmError):
        b.set_schedule(1, 0, 3)
    b.close()
