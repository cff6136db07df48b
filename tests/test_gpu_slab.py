"""Slab boxes (Lx = Ly, Lz = 2 Lx; aspect_z = 2): a half-vacuum water slab.

The library solves a slab as the periodic cube of edge Lz that holds it twice
along x and twice along y, storing and computing only the box's own cells.  The
oracle solves that cube literally (oracle.zeta_solve_slab: the four copies,
4N bodies, the reference algorithm in FP64), so the FP32 path must match it to
1e-5 and the split-bf16 tensor-core path to 1e-4; both converge to the FP64
Ewald sum of the rectangular box as the order grows."""
import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu


def _slab(n_sites, a, seed, ions=3):
    import __graft_entry__ as G
    systems = G.load_module("systems")
    xyz, q, box = systems.water_ion_box(n_sites, [a, a, 2 * a], n_na=ions, n_cl=ions, seed=seed, fill_z=0.5)
    return xyz, q, np.float32(a)


def _solve(pkg, xyz, q, a, **kw):
    s = pkg.ZetaFmmSolver(len(q), q, aspect_z=2, **kw)
    s.execute(xyz, [a, a, 2 * a])
    out = s.forces(), s.potentials(), s.get_energy()
    s.close()
    return out


@pytest.mark.parametrize("n_sites,a,P,depth,images,prec,tol", [
    (400, 2.2, 4, 2, 4, 0, 1e-5),
    (400, 2.2, 8, 3, 4, 0, 1e-5),
    (900, 3.0, 6, 3, 2, 0, 1e-5),
    (400, 2.2, 6, 1, 4, 0, 1e-5),   # depth 1: the leaves are the two cubes of the box
    (3000, 4.2, 5, 4, 4, 0, 1e-5),
    (400, 2.2, 6, 2, 4, 1, 1e-4),   # tensor-core M2L, split bf16
    (3000, 4.2, 7, 4, 4, 1, 1e-4),
    (900, 3.0, 10, 3, 4, 1, 1e-4),
])
def test_slab_matches_the_fp64_solver_of_the_periodic_cube(pkg, oracle, n_sites, a, P, depth, images, prec, tol):
    xyz, q, a = _slab(n_sites, a, seed=n_sites + P)
    f, p, e = _solve(pkg, xyz, q, a, order=P, max_depth=depth, images=images, precision=prec)
    po, fo, eo = oracle.zeta_solve_slab(xyz.astype(np.float64), q.astype(np.float64), float(a), P, depth, images)
    assert rel_rms(f, fo) < tol
    assert rel_rms(p, po) < tol
    assert abs(e - eo) / abs(eo) < 1e-5


def test_slab_converges_to_ewald(pkg, oracle):
    xyz, q, a = _slab(1500, 3.4, seed=77)
    box = np.array([a, a, 2 * a], np.float64)
    _, fe, _ = oracle.ewald(xyz.astype(np.float64), q.astype(np.float64), box, eps=1e-10)
    _, _, ee = oracle.ewald(xyz.astype(np.float64), q.astype(np.float64), box, eps=1e-9, energy=True)
    errs = []
    for P in (4, 8, 12):
        f, _, e = _solve(pkg, xyz, q, a, order=P, max_depth=3, images=4)
        errs.append(rel_rms(f, fe))
        assert abs(e - ee) / abs(ee) < 1e-4
    assert errs[1] < 0.2 * errs[0] and errs[2] < 0.3 * errs[1]
    assert errs[2] < 1e-4


def test_slab_box_validation(pkg):
    q = np.zeros(4, np.float32)
    x = np.full((4, 3), 0.5, np.float32)
    s = pkg.ZetaFmmSolver(4, q, order=4, max_depth=2, aspect_z=2)
    with pytest.raises(pkg.FmmError) as e:
        s.execute(x, 2.0)  # cubic box on a slab handle
    assert e.value.status == 2
    s.execute(x, [2.0, 2.0, 4.0])
    s.close()
    c = pkg.ZetaFmmSolver(4, q, order=4, max_depth=2)
    with pytest.raises(pkg.FmmError) as e:
        c.execute(x, [2.0, 2.0, 4.0])  # slab box on a cubic handle
    assert e.value.status == 2
    c.close()


@pytest.mark.parametrize("P,depth,prec", [(5, 4, 2), (8, 3, 0)])
def test_slab_launch_overlap_leaves_results_unchanged(pkg, P, depth, prec):
    """Programmatic dependent launches on a slab (two stored level-1 cells, per-axis
    grids): a deterministic handle gives the same bits with and without them."""
    xyz, q, a = _slab(3000, 4.2, seed=61)
    s = pkg.ZetaFmmSolver(len(q), q, aspect_z=2, order=P, max_depth=depth, images=4, precision=prec,
                          flags=pkg.FLAG_DETERMINISTIC)
    box = [a, a, 2 * a]
    s.execute(xyz, box)
    f0, p0, e0 = s.forces(), s.potentials(), s.get_energy()
    s.set_launch_overlap(False)
    s.execute(xyz, box)
    assert np.array_equal(s.forces(), f0) and np.array_equal(s.potentials(), p0) and s.get_energy() == e0
    s.close()
