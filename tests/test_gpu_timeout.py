"""The bounded device waits: a wait that runs out reports GBFMM_ERR_TIMEOUT to
the caller, and the context stays usable.

Every spin on an mbarrier in the library's kernels (the tensor-core M2L's
copy/MMA pipeline, the upper-tree kernel's staged copies) polls at most a given
number of times, then records an error bit that the host turns into
GBFMM_ERR_TIMEOUT.  The probe runs that same wait in a one-warp kernel on a
barrier that nothing completes, with no copies or MMAs in flight, so the wait
runs out without any fault; then a normal solve must still succeed."""
import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu


def test_a_bounded_wait_that_runs_out_reports_timeout(pkg):
    with pytest.raises(pkg.FmmError) as e:
        pkg.debug_bounded_wait(1 << 12)
    assert e.value.status == 8  # GBFMM_ERR_TIMEOUT
    assert "gave up" in str(e.value)


def test_the_context_stays_usable_after_a_timeout(pkg, oracle, systems):
    with pytest.raises(pkg.FmmError):
        pkg.debug_bounded_wait(1 << 10)
    xyz, q, box = systems.water_ion_box(300, 2.2, n_na=2, n_cl=2, seed=41)
    s = pkg.ZetaFmmSolver(len(q), q, order=6, max_depth=2, images=4, precision=pkg.PREC_BF16X3)
    s.execute(xyz, box)
    f = s.forces()
    s.close()
    _, fo, _ = oracle.zeta_solve(xyz.astype(np.float64), q.astype(np.float64), float(box[0]), 6, 2, 4)
    assert rel_rms(f, fo) < 1e-4
