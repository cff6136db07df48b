"""Tensor-core (tcgen05) M2L: split-bf16 products with FP32 accumulation.

BF16X3 keeps ~16 bits of every operand (hi*hi + hi*lo + lo*hi); its force and
potential error against the FP64 oracle is bounded at 1e-4 relative RMS here.
BF16X1 (hi*hi) is bounded at 1e-3, the benchmark metric's own tolerance.  Both must agree with the plain FP32 path
on the near field exactly, so they are also compared against it."""
import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_sites,L,P,depth,images", [
    (1000, 2.2, 4, 2, 4),
    (3000, 4.5, 8, 3, 4),
    (1500, 3.0, 6, 3, 0),
    (1500, 3.0, 10, 3, 4),
    (800, 2.0, 5, 1, 4),
    (8000, 6.2, 7, 4, 2),
    (1000, 2.2, 2, 2, 4),     # the lowest orders
    (1000, 2.2, 3, 2, 4),
    (7000, 4.3, 4, 5, 4),     # depth 5
])
def test_tc_bf16x3_parity(pkg, oracle, systems, n_sites, L, P, depth, images):
    xyz, q, box = systems.water_ion_box(n_sites, L, n_na=4, n_cl=4, seed=n_sites * 3 + P)
    s = pkg.ZetaFmmSolver(len(q), q, order=P, max_depth=depth, images=images, precision=pkg.PREC_BF16X3)
    s.execute(xyz, box)
    f, p, e = s.forces(), s.potentials(), s.get_energy()
    po, fo, eo = oracle.zeta_solve(xyz.astype(np.float64), q.astype(np.float64), float(box[0]), P, depth, images)
    assert rel_rms(f, fo) < 1e-4
    assert rel_rms(p, po) < 1e-4
    assert abs(e - eo) / abs(eo) < 1e-5
    s.close()


def test_tc_bf16x1_parity(pkg, oracle, systems):
    xyz, q, box = systems.water_ion_box(3000, 4.5, n_na=5, n_cl=5, seed=21)
    s = pkg.ZetaFmmSolver(len(q), q, order=8, max_depth=3, images=4, precision=pkg.PREC_BF16X1)
    s.execute(xyz, box)
    f = s.forces()
    _, fo, _ = oracle.zeta_solve(xyz.astype(np.float64), q.astype(np.float64), float(box[0]), 8, 3, 4)
    assert rel_rms(f, fo) < 1e-3
    s.close()


def test_tc_matches_fp32_path_and_is_deterministic(pkg, systems):
    xyz, q, box = systems.water_ion_box(4000, 3.4, n_na=3, n_cl=3, seed=22)
    a = pkg.ZetaFmmSolver(len(q), q, order=6, max_depth=3, images=4)
    b = pkg.ZetaFmmSolver(len(q), q, order=6, max_depth=3, images=4, precision=pkg.PREC_BF16X3,
                          flags=pkg.FLAG_DETERMINISTIC)
    a.execute(xyz, box)
    b.execute(xyz, box)
    fb1 = b.forces()
    assert rel_rms(fb1, a.forces()) < 1e-4
    b.execute(xyz, box)
    assert np.array_equal(fb1, b.forces())
    a.close()
    b.close()


def test_tc_rejects_high_order(pkg):
    with pytest.raises(pkg.FmmError) as e:
        pkg.ZetaFmmSolver(10, np.zeros(10, np.float32), order=13, max_depth=1, precision=pkg.PREC_BF16X3)
    assert e.value.status == 6


@pytest.mark.parametrize("P,prec,tol,tol_pot", [(11, 1, 1e-4, 1e-4), (12, 1, 1e-4, 1e-4), (12, 2, 1e-3, 5e-3)])
def test_tc_orders_11_and_12(pkg, oracle, systems, P, prec, tol, tol_pot):
    """Three K atoms per multipole row (up to 169 coefficients); one pipeline
    stage of the split-precision form, two of the single product (whose
    potentials keep about 8 bits of the far field: 3.6e-3 measured here)."""
    xyz, q, box = systems.water_ion_box(1500, 3.0, n_na=4, n_cl=4, seed=50 + P)
    s = pkg.ZetaFmmSolver(len(q), q, order=P, max_depth=3, images=4, precision=prec)
    s.execute(xyz, box)
    f, p, e = s.forces(), s.potentials(), s.get_energy()
    s.close()
    po, fo, eo = oracle.zeta_solve(xyz.astype(np.float64), q.astype(np.float64), float(box[0]), P, 3, 4)
    assert rel_rms(f, fo) < tol
    assert rel_rms(p, po) < tol_pot
    assert abs(e - eo) / abs(eo) < (1e-4 if prec == 2 else 1e-5)  # one product: 3.2e-5 measured
