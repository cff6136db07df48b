"""The Coulomb virial (gbfmm_get_virial) against the FP64 Ewald virial.

Xi = -1/2 sum over pairs (periodic images included) of r_ij (x) F_ij, the
quantity mdrun's ForceWithVirial takes from a force provider.  The library
computes it from the step's own tree, expansions and fields (the image-shift
term of every interaction that crosses the box, the far lattice and the
tin-foil term); the oracle's Ewald sum gives it analytically (real-space pair
sum and the reciprocal-space strain derivative, checked on the host against
finite differences of the energy).  Homogeneity gives a second, exact check:
the Coulomb energy scales as 1/length, so trace(Xi) = -E/2 for the FMM's own
energy E."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n_sites,L,P,depth,prec,tol", [
    (1500, 3.0, 8, 3, 0, 2e-3),
    (3000, 4.5, 10, 3, 0, 1e-3),
    (1500, 3.0, 6, 2, 1, 5e-3),
    (800, 2.2, 8, 1, 0, 5e-3),   # depth 1: 1.1 nm leaves, the coarsest tree (3.2e-3 measured)
])
def test_virial_matches_ewald_cube(pkg, oracle, systems, n_sites, L, P, depth, prec, tol):
    xyz, q, box = systems.water_ion_box(n_sites, L, n_na=4, n_cl=4, seed=n_sites + P)
    s = pkg.ZetaFmmSolver(len(q), q, order=P, max_depth=depth, images=4, precision=prec)
    s.execute(xyz, box)
    v, e = s.virial(), s.get_energy()
    s.close()
    b = np.full(3, float(np.float32(box[0])))
    ee, ve = oracle.ewald_virial(xyz.astype(np.float64), q.astype(np.float64), b, eps=1e-10)
    assert _rel(v, ve) < tol, (v, ve)
    assert abs(np.trace(v) + 0.5 * e) < 1e-4 * abs(e)
    assert np.allclose(v, v.T, atol=1e-3 * np.abs(v).max())


def test_virial_matches_ewald_slab(pkg, oracle, systems):
    a = 2.6
    xyz, q, _ = systems.water_ion_box(600, [a, a, 2 * a], n_na=3, n_cl=3, seed=71, fill_z=0.5)
    a32 = float(np.float32(a))
    s = pkg.ZetaFmmSolver(len(q), q, order=8, max_depth=3, images=4, aspect_z=2)
    s.execute(xyz, [a32, a32, 2 * a32])
    v, e = s.virial(), s.get_energy()
    s.close()
    ee, ve = oracle.ewald_virial(xyz.astype(np.float64), q.astype(np.float64), np.array([a32, a32, 2 * a32]),
                                 eps=1e-10)
    assert _rel(v, ve) < 2e-3, (v, ve)
    assert abs(np.trace(v) + 0.5 * e) < 1e-4 * abs(e)


def test_virial_needs_a_step(pkg):
    s = pkg.ZetaFmmSolver(4, np.zeros(4, np.float32), order=4, max_depth=1)
    with pytest.raises(pkg.FmmError) as e:
        s.virial()
    assert e.value.status == 7
    s.close()
