"""The tile-shape autotuner: every P2P warp-step shape and every tensor-core M2L
entry split and pipeline depth gives the same forces (up to the order of the
floating-point additions) and the FP64 oracle's to the path's tolerance; the
autotuner keeps one of them and reports its step time."""
import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu


def _system(systems):
    xyz, q, box = systems.water_ion_box(6000, 5.6, n_na=8, n_cl=8, seed=71)
    return xyz, q, float(box[0])


@pytest.mark.parametrize("precision,tol", [(0, 1e-5), (1, 1e-4), (2, 3e-3)])
def test_every_shape_matches(pkg, oracle, systems, precision, tol):
    xyz, q, L = _system(systems)
    s = pkg.ZetaFmmSolver(len(q), q, order=6, max_depth=3, images=4, precision=precision)
    s.execute(xyz, L)
    f0 = s.forces()
    _, fo, _ = oracle.zeta_solve(xyz.astype(np.float64), q.astype(np.float64), L, 6, 3, 4)
    assert rel_rms(f0, fo) < tol
    ns0 = s.tuning()["m2l_stages"]
    # P2P: 3 warp-step shapes x (one CTA per leaf, or 2..5 persistent CTAs per SM), and
    # two shapes with up to 4 targets per thread
    for pv in range(17):
        s.set_tuning(pv, 1, ns0)
        s.execute(xyz, L)
        assert rel_rms(s.forces(), f0) < 1e-5, pv
    if precision:
        for sp in (1, 2, 4, 8):
            for ns in (1, 2):
                s.set_tuning(0, sp, ns)
                s.execute(xyz, L)
                assert rel_rms(s.forces(), f0) < 1e-5, (sp, ns)
    s.close()


def test_autotune_keeps_a_valid_tuning(pkg, systems):
    xyz, q, L = _system(systems)
    s = pkg.ZetaFmmSolver(len(q), q, order=5, max_depth=3, images=4, precision=2)
    s.execute(xyz, L)
    f0 = s.forces()
    t = s.autotune(xyz, L, reps=3)
    assert t["ms"] > 0 and 0 <= t["p2p_variant"] < 17 and t["m2l_split"] in (1, 2, 4, 8)
    s.execute(xyz, L)
    assert rel_rms(s.forces(), f0) < 1e-5
    s.close()


def test_deterministic_handle_keeps_whole_tiles(pkg, systems):
    xyz, q, L = _system(systems)
    s = pkg.ZetaFmmSolver(len(q), q, order=5, max_depth=3, images=4, precision=1, flags=pkg.FLAG_DETERMINISTIC)
    assert s.tuning()["m2l_split"] == 1
    with pytest.raises(pkg.FmmError):
        s.set_tuning(0, 2, 2)
    s.execute(xyz, L)
    f1 = s.forces()
    s.autotune(xyz, L, reps=2)
    assert s.tuning()["m2l_split"] == 1
    s.execute(xyz, L)
    f2 = s.forces()
    s.set_tuning(s.tuning()["p2p_variant"], 1, s.tuning()["m2l_stages"])
    # the same shapes give bit-identical results on a deterministic handle
    s.execute(xyz, L)
    assert np.array_equal(s.forces(), f2)
    assert rel_rms(f2, f1) < 1e-5
    s.close()


def test_near_field_start_leaves_results_unchanged(pkg, systems):
    """The near field may start after the tree, the P2M or the upper tree: only the
    order of the graph's nodes changes, so a deterministic handle gives the same bits."""
    xyz, q, L = _system(systems)
    s = pkg.ZetaFmmSolver(len(q), q, order=5, max_depth=3, images=4, precision=1, flags=pkg.FLAG_DETERMINISTIC)
    s.execute(xyz, L)
    f0, p0 = s.forces(), s.potentials()
    for after in (1, 2, 0):
        s.set_near_start(after)
        assert s.tuning()["near_after"] == after
        s.execute(xyz, L)
        assert np.array_equal(s.forces(), f0) and np.array_equal(s.potentials(), p0), after
    with pytest.raises(pkg.FmmError):
        s.set_near_start(3)
    s.close()


@pytest.mark.parametrize("order,depth,prec", [(5, 3, 1), (5, 4, 2), (4, 4, 0), (8, 5, 0)])
def test_launch_overlap_leaves_results_unchanged(pkg, systems, order, depth, prec):
    """Programmatic dependent launches only move kernel starts: each kernel still
    waits for the previous one before it touches its data, so a deterministic
    handle gives the same bits with and without them (tensor-core and FP32 M2L,
    the fused and the level-by-level upward pass, the staged and unstaged upper
    tree)."""
    xyz, q, L = _system(systems)
    s = pkg.ZetaFmmSolver(len(q), q, order=order, max_depth=depth, images=4, precision=prec,
                          flags=pkg.FLAG_DETERMINISTIC)
    assert s.launch_overlap()
    s.execute(xyz, L)
    f0, p0, e0 = s.forces(), s.potentials(), s.get_energy()
    for on in (False, True, False):
        s.set_launch_overlap(on)
        assert s.launch_overlap() == on
        for _ in range(2):
            s.execute(xyz, L)
            assert np.array_equal(s.forces(), f0) and np.array_equal(s.potentials(), p0), on
            assert s.get_energy() == e0
    s.close()
