"""GPU parity: the sm_103a FP32 path against the FP64 oracle and against the
outputs of the reference's own FP64 kernels (relative RMS force and potential
error <= 1e-5, relative energy error <= 1e-6), and the tree against fixtures made
by the reference's own tree.cpp (bit-exact)."""
import numpy as np
import pytest

from conftest import golden, rel_rms

pytestmark = pytest.mark.gpu

TOL_F = 1e-5   # relative RMS force / potential error of the FP32 path vs the FP64 oracle
TOL_E = 1e-6   # relative energy error


def _solve(pkg, xyz, q, box, **kw):
    s = pkg.ZetaFmmSolver(len(q), q, **kw)
    s.execute(xyz, box)
    return s.forces(), s.potentials(), s.get_energy(), s


@pytest.mark.parametrize("n_sites,L,ions,P,depth,images", [
    (300, 2.0, 2, 4, 2, 4),
    (1000, 2.2, 4, 8, 2, 4),
    (3000, 4.5, 0, 8, 3, 4),
    (1500, 3.0, 6, 10, 3, 0),
    (1500, 3.0, 6, 6, 3, 1),
    (1500, 3.0, 6, 6, 3, 2),
    (3000, 4.5, 10, 12, 3, 4),
    (800, 2.0, 4, 5, 1, 4),
    (800, 2.0, 4, 16, 2, 4),    # the highest order
    (800, 2.0, 4, 2, 2, 4),     # the lowest order
    (1500, 3.0, 6, 6, 3, 6),
    (1500, 3.0, 6, 6, 3, 8),    # the most lattice images
    (7000, 4.3, 6, 4, 5, 4),    # depth 5: 32,768 leaves, fewer than one body per leaf
])
def test_parity_vs_oracle(pkg, oracle, systems, n_sites, L, ions, P, depth, images):
    xyz, q, box = systems.water_ion_box(n_sites, L, n_na=ions, n_cl=ions, seed=n_sites + P)
    f, p, e, s = _solve(pkg, xyz, q, box, order=P, max_depth=depth, images=images)
    po, fo, eo = oracle.zeta_solve(xyz.astype(np.float64), q.astype(np.float64), float(box[0]), P, depth, images)
    assert rel_rms(f, fo) < TOL_F
    assert rel_rms(p, po) < TOL_F
    assert abs(e - eo) / abs(eo) < TOL_E
    s.close()


def test_parity_vs_reference_kernel_outputs(pkg, oracle, systems):
    """The FP32 path against the outputs of the reference's own FP64 kernels
    (kernel.cu, committed fixture): the dipole correction, which the reference
    applies on the host after its kernels, is taken off the GPU results with the
    oracle's correction term."""
    g = golden("ref_outputs.npz")
    k = 0
    while f"case{k}_params" in g:
        ns, L, ions, P, D, im = g[f"case{k}_params"]
        xyz, q, box = systems.water_ion_box(int(ns), float(L), n_na=int(ions), n_cl=int(ions), seed=int(ns) + int(P))
        f, p, e, s = _solve(pkg, xyz, q, box, order=int(P), max_depth=int(D), images=int(im))
        s.close()
        x64, q64 = xyz.astype(np.float64), q.astype(np.float64)
        p1, f1, _ = oracle.zeta_solve(x64, q64, float(L), int(P), int(D), int(im))
        p0, f0, _ = oracle.zeta_solve(x64, q64, float(L), int(P), int(D), int(im), stages=3)
        idx = g[f"case{k}_idx"]
        assert rel_rms(f[idx] - (f1 - f0)[idx], g[f"case{k}_force"]) < TOL_F
        assert rel_rms(p[idx] - (p1 - p0)[idx], g[f"case{k}_pot"]) < TOL_F
        k += 1
    assert k == 5


def test_parity_water_96k(pkg, oracle, systems):
    """The 95,600-atom 9.86 nm box at p=10, depth 4, at full size."""
    xyz, q, box = systems.cfg_96k()
    f, p, e, s = _solve(pkg, xyz, q, box, order=10, max_depth=4, images=4)
    po, fo, eo = oracle.zeta_solve(xyz.astype(np.float64), q.astype(np.float64), float(box[0]), 10, 4, 4)
    assert rel_rms(f, fo) < TOL_F
    assert rel_rms(p, po) < TOL_F
    assert abs(e - eo) / abs(eo) < TOL_E
    # against the converged Ewald sum on a sample of atoms (FMM truncation error)
    tg = np.arange(0, len(q), 97)
    _, fe, _ = oracle.ewald(xyz.astype(np.float64), q.astype(np.float64), box[0], eps=1e-9, targets=tg)
    assert rel_rms(f[tg], fe) < 2e-4
    s.close()


@pytest.mark.parametrize("name,depth", [("tree_water9k_d3.npz", 3), ("tree_edges_d1.npz", 1),
                                        ("tree_edges_d2.npz", 2), ("tree_edges_d3.npz", 3)])
def test_tree_bit_exact_vs_reference(pkg, name, depth):
    g = golden(name)
    xyz = g["xyz"]
    q = np.where(np.arange(len(xyz)) % 2 == 0, 1.0, -1.0).astype(np.float32)
    s = pkg.ZetaFmmSolver(len(q), q, order=4, max_depth=depth, images=4)
    s.execute(xyz, float(g["box"]))
    order, lo, ln = s.tree()
    assert np.array_equal(order, g["order"])
    assert np.array_equal(ln, g["leaf_count"])
    assert np.array_equal(lo, np.concatenate([[0], np.cumsum(ln)[:-1]]))
    s.close()


def test_tree_bit_exact_vs_reference_96k_depth4(pkg):
    """The benchmark's 95,600-atom box at depth 4: the GPU tree's body order
    (SHA-256) and leaf counts equal the reference tree.cpp's."""
    import hashlib
    g = golden("tree_water96k_d4.npz")
    xyz = g["xyz"]
    q = np.where(np.arange(len(xyz)) % 2 == 0, 1.0, -1.0).astype(np.float32)
    s = pkg.ZetaFmmSolver(len(q), q, order=5, max_depth=4, images=4, precision=pkg.PREC_BF16X1)
    s.execute(xyz, float(g["box"]))
    order, lo, ln = s.tree()
    assert hashlib.sha256(np.ascontiguousarray(order, dtype="<i4").tobytes()).digest() == g["order_sha256"].tobytes()
    assert np.array_equal(ln, g["leaf_count"])
    assert np.array_equal(lo, np.concatenate([[0], np.cumsum(ln)[:-1]]))
    s.close()


def test_crowded_leaves(pkg, oracle, systems):
    """Ragged occupancy: most bodies in a few leaves (> 256 per leaf, > 2048 near
    sources), many empty leaves."""
    rng = np.random.default_rng(4)
    L = 4.0
    a = rng.uniform(0.05, 0.45, (1400, 3))
    b = rng.uniform(0, L, (200, 3))
    xyz = np.concatenate([a, b]).astype(np.float32)
    q = np.where(np.arange(len(xyz)) % 2 == 0, 0.5, -0.5).astype(np.float32)
    f, p, e, s = _solve(pkg, xyz, q, L, order=6, max_depth=3, images=4)
    po, fo, eo = oracle.zeta_solve(xyz.astype(np.float64), q.astype(np.float64), L, 6, 3, 4)
    assert rel_rms(f, fo) < TOL_F
    assert rel_rms(p, po) < TOL_F
    s.close()


@pytest.mark.parametrize("depth,images", [(3, 4), (1, 4), (2, 0)])
def test_faces_outside_box_and_coincident_bodies(pkg, oracle, systems, depth, images):
    """Bodies exactly on leaf faces, outside the box, coincident with another body
    (r = 0: skipped), and two bodies that coincide only through the periodic
    shift (exact in float and double: a 4 nm box).  Every r = 0 pair must be
    skipped, as kernel.cu:480-490 does, wherever the two bodies are staged."""
    xyz, q, box = systems.water_ion_box(2100, 4.0, n_na=5, n_cl=5, seed=21)
    L = 4.0
    h = L / 2 ** depth
    rng = np.random.default_rng(3)
    x = xyz.copy()
    idx = rng.choice(len(q), 200, replace=False)
    for k, i in enumerate(idx[:60]):           # on leaf faces, the box faces included
        x[i, k % 3] = np.float32(h * rng.integers(0, 2 ** depth + 1))
    for k, i in enumerate(idx[60:100]):        # just outside the box
        x[i, k % 3] = np.float32(-0.0625 if k % 2 else L + 0.0625)
    for k in range(10):                        # coincident pairs
        x[idx[100 + k]] = x[idx[110 + k]]
    for k in range(6):                         # coincident through the periodic shift
        a, b = idx[120 + 2 * k], idx[121 + 2 * k]
        d = k % 3
        x[b] = x[a]
        x[a, d] = np.float32(-0.125)
        x[b, d] = np.float32(L - 0.125)
    f, p, e, s = _solve(pkg, x, q, L, order=6, max_depth=depth, images=images)
    assert np.isfinite(f).all() and np.isfinite(p).all()
    po, fo, eo = oracle.zeta_solve(x.astype(np.float64), q.astype(np.float64), L, 6, depth, images)
    assert rel_rms(f, fo) < TOL_F
    assert rel_rms(p, po) < TOL_F
    s.close()


def test_device_execute_matches_host_execute(pkg, systems):
    torch = pytest.importorskip("torch")
    xyz, q, box = systems.water_ion_box(1200, 2.5, seed=12)
    s = pkg.ZetaFmmSolver(len(q), q, order=6, max_depth=2, images=4, flags=pkg.FLAG_DETERMINISTIC)
    s.execute(xyz, box)
    f_host = s.forces()
    x = torch.from_numpy(xyz).cuda()
    st = torch.cuda.Stream()
    s.execute_device(x.data_ptr(), box, st.cuda_stream)
    st.synchronize()
    f_dev = s.forces()
    assert np.array_equal(f_host, f_dev)
    fp, pp, ep = s.device_outputs()
    assert fp and pp and ep
    s.close()


class _CudaView:
    """Zero-copy view of a device buffer of float32 (no stream synchronisation)."""

    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": "<f4", "data": (int(ptr), False), "version": 2}


def test_device_execute_is_ordered_on_the_callers_stream(pkg, systems):
    """Work enqueued on the caller's stream after gbfmm_execute_device sees the
    step's results without any other synchronisation, on the legacy default
    stream (handle 0) as on a created stream."""
    torch = pytest.importorskip("torch")
    xyz, q, box = systems.water_ion_box(3000, 3.0, seed=21)
    xyz2 = np.mod(xyz + np.float32(0.37), np.float32(box[0])).astype(np.float32)
    s = pkg.ZetaFmmSolver(len(q), q, order=6, max_depth=3, images=4, flags=pkg.FLAG_DETERMINISTIC)
    s.execute(xyz2, box)
    f_ref = s.forces().copy()
    x2 = torch.from_numpy(xyz2).cuda()
    torch.cuda.synchronize()
    for stream in (torch.cuda.default_stream(), torch.cuda.Stream()):
        s.execute(xyz, box)  # the output buffers now hold another configuration
        with torch.cuda.stream(stream):
            s.execute_device(x2.data_ptr(), box, stream.cuda_stream)
            fp, _, _ = s.device_outputs()
            f_dev = torch.as_tensor(_CudaView(fp, (len(q), 3)), device="cuda").clone()
        stream.synchronize()
        assert np.array_equal(f_dev.cpu().numpy(), f_ref)
    s.close()


def test_host_call_in_place_matches_copies(pkg, systems):
    """gbfmm_execute reads the host coordinates and writes the host results in
    place where the device reaches pageable memory (GB300 over NVLink-C2C), and
    copies through device buffers with GBFMM_FLAG_HOST_COPY: the results are
    the same bit for bit, on repeated calls."""
    xyz, q, box = systems.water_ion_box(3000, 3.0, n_na=4, n_cl=4, seed=31)
    out = []
    for flags in (pkg.FLAG_DETERMINISTIC, pkg.FLAG_DETERMINISTIC | pkg.FLAG_HOST_COPY):
        s = pkg.ZetaFmmSolver(len(q), q, order=6, max_depth=3, images=4, flags=flags)
        res = []
        for k in range(2):
            s.execute(xyz if k else xyz * np.float32(1.01), box)
            res.append((s.forces(), s.potentials(), s.get_energy()))
        out.append(res[1])
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


def test_deterministic_flag_is_bitwise_repeatable(pkg, systems):
    xyz, q, box = systems.water_ion_box(2000, 2.8, seed=13)
    s = pkg.ZetaFmmSolver(len(q), q, order=8, max_depth=3, images=4, flags=pkg.FLAG_DETERMINISTIC)
    s.execute(xyz, box)
    f1, p1, e1 = s.forces(), s.potentials(), s.get_energy()
    s.execute(xyz, box)
    f2, p2, e2 = s.forces(), s.potentials(), s.get_energy()
    assert np.array_equal(f1, f2) and np.array_equal(p1, p2)
    assert abs(e1 - e2) <= 1e-12 * abs(e1)
    s.close()


def test_graph_replay_follows_new_box_and_coords(pkg, oracle, systems):
    xyz, q, box = systems.water_ion_box(900, 2.1, seed=14)
    s = pkg.ZetaFmmSolver(len(q), q, order=6, max_depth=2, images=4)
    s.execute(xyz, box)
    xyz2 = (xyz * np.float32(1.05)).astype(np.float32)
    L2 = float(np.float32(box[0] * 1.05))
    s.execute(xyz2, L2)
    f = s.forces()
    _, fo, _ = oracle.zeta_solve(xyz2.astype(np.float64), q.astype(np.float64), L2, 6, 2, 4)
    assert rel_rms(f, fo) < TOL_F
    s.close()


def test_back_to_back_steps_each_see_their_own_box(pkg, systems):
    """Device steps queued without a host synchronisation between them, the box
    and coordinates alternating: the tree kernel of each step reads that step's
    constants (written by the host into pinned memory that the next call rewrites
    once the previous step's tree kernel has read it), so every step gives the
    bits of a separate solve of its own configuration."""
    torch = pytest.importorskip("torch")
    xyz, q, box = systems.water_ion_box(3000, 3.0, seed=23)
    L1 = float(box[0])
    xyz2 = (xyz * np.float32(1.05)).astype(np.float32)
    L2 = float(np.float32(L1 * 1.05))
    cfgs = [(xyz, L1), (xyz2, L2)]
    ref = []
    for x, L in cfgs:
        r = pkg.ZetaFmmSolver(len(q), q, order=5, max_depth=3, images=4, precision=1, flags=pkg.FLAG_DETERMINISTIC)
        r.execute(x, L)
        ref.append(r.forces())
        r.close()
    s = pkg.ZetaFmmSolver(len(q), q, order=5, max_depth=3, images=4, precision=1, flags=pkg.FLAG_DETERMINISTIC)
    xd = [torch.from_numpy(x).cuda() for x, _ in cfgs]
    torch.cuda.synchronize()
    st = torch.cuda.Stream()
    outs = []
    with torch.cuda.stream(st):
        for k in range(6):
            s.execute_device(xd[k % 2].data_ptr(), cfgs[k % 2][1], st.cuda_stream)
            fp, _, _ = s.device_outputs()
            outs.append(torch.as_tensor(_CudaView(fp, (len(q), 3)), device="cuda").clone())
    st.synchronize()
    for k, f in enumerate(outs):
        assert np.array_equal(f.cpu().numpy(), ref[k % 2]), k
    s.close()


def test_nonfinite_input_reports_error_and_recovers(pkg, systems):
    xyz, q, box = systems.water_ion_box(300, 2.0, seed=15)
    s = pkg.ZetaFmmSolver(len(q), q, order=4, max_depth=2, images=4)
    bad = xyz.copy()
    bad[7, 1] = np.nan
    with pytest.raises(pkg.FmmError) as e:
        s.execute(bad, box)
    assert e.value.status == 3
    s.execute(xyz, box)
    assert np.isfinite(s.forces()).all()
    s.close()


def test_box_validation(pkg, systems):
    xyz, q, box = systems.water_ion_box(100, 1.5, seed=16)
    s = pkg.ZetaFmmSolver(len(q), q, order=4, max_depth=1, images=4)
    for bad in ([1.5, 1.5, 1.6], [0.0, 0.0, 0.0], [np.inf, 1.5, 1.5]):
        with pytest.raises(pkg.FmmError) as e:
            s.execute(xyz, bad)
        assert e.value.status == 2
    with pytest.raises(pkg.FmmError) as e:
        pkg.ZetaFmmSolver(len(q), q, order=4, max_depth=1).forces()
    assert e.value.status == 7
    s.close()


def test_add_force_and_compare_forces(pkg, oracle, systems):
    xyz, q, box = systems.water_ion_box(500, 1.8, seed=17)
    s = pkg.ZetaFmmSolver(len(q), q, order=6, max_depth=2, images=4)
    s.execute(xyz, box)
    acc = np.ones((len(q), 3), np.float32)
    s.add_force(acc)
    assert np.allclose(acc - 1.0, s.forces(), rtol=0, atol=1e-3)
    _, fo, _ = oracle.zeta_solve(xyz.astype(np.float64), q.astype(np.float64), float(box[0]), 6, 2, 4)
    l2f = s.compare_forces(fo.astype(np.float32), verbose=False)
    assert l2f < TOL_F
    s.close()


def test_empty_and_zero_charge_systems(pkg):
    s = pkg.ZetaFmmSolver(0, np.zeros(0, np.float32), order=4, max_depth=1, images=4)
    s.execute(np.zeros((0, 3), np.float32), 2.0)
    assert s.get_energy() == 0.0
    s.close()
    xyz = np.random.default_rng(0).uniform(0, 2, (50, 3)).astype(np.float32)
    s = pkg.ZetaFmmSolver(50, np.zeros(50, np.float32), order=4, max_depth=1, images=4)
    s.execute(xyz, 2.0)
    assert np.all(s.forces() == 0) and np.all(s.potentials() == 0) and s.get_energy() == 0.0
    s.close()
