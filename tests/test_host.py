"""Host-side logic of the library (no GPU compute): ABI exports, operator tables,
stencil-driven interaction lists, argument validation, input generator."""
import hashlib
import json
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "gbfmm.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbfmm_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol(pkg):
    L = pkg.lib()
    names = _declared_functions()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings(pkg):
    L = pkg.lib()
    for code in range(10):
        assert L.gbfmm_status_string(code).decode() == pkg.STATUS[code]


def _pk(n, m):
    return n * (n + 1) // 2 + m


def _r2c(x, P):
    z = np.zeros((P + 1) * (P + 2) // 2, complex)
    for n in range(P + 1):
        z[_pk(n, 0)] = x[n * n]
        for m in range(1, n + 1):
            z[_pk(n, m)] = x[n * n + 2 * m - 1] + 1j * x[n * n + 2 * m]
    return z


def _c2r(z, P):
    x = np.zeros((P + 1) ** 2)
    for n in range(P + 1):
        x[n * n] = z[_pk(n, 0)].real
        for m in range(1, n + 1):
            x[n * n + 2 * m - 1] = z[_pk(n, m)].real
            x[n * n + 2 * m] = z[_pk(n, m)].imag
    return x


@pytest.mark.parametrize("P", [3, 8, 12])
def test_harmonics_match_oracle(pkg, oracle, P):
    rng = np.random.default_rng(P)
    for _ in range(4):
        d = rng.normal(size=3)
        for kind, okind in ((0, 0), (1, 2)):
            a = pkg.debug_harmonics(P, kind, d)
            b = oracle.harmonics(okind, P, d)
            bb = np.array([b[n * n + n + m] for n in range(P + 1) for m in range(n + 1)])
            assert np.max(np.abs(a - bb) / np.maximum(np.abs(bb), 1e-300)) < 1e-10


@pytest.mark.parametrize("P", [4, 10])
def test_operator_matrices_match_oracle_loops(pkg, oracle, P):
    """The real matrices the kernels apply equal the reference-form loops of the
    oracle (kernel.cu:310-454, 550-606) in scaled units."""
    R = (P + 1) ** 2
    deg = np.array([int(np.floor(np.sqrt(r))) for r in range(R)])
    rng = np.random.default_rng(1)
    x = rng.normal(size=R)
    for c in range(0, 724, 53):
        A, cv = pkg.debug_operator(P, 2, c)
        kind, v = int(cv[0]), cv[1:]
        d = v if kind == 0 else v / 2
        xin = x * 2.0 ** deg if kind == 1 else x
        y = _c2r(oracle.apply_op(2, P, d, _r2c(xin, P)), P)
        assert np.max(np.abs(A @ x - y)) <= 1e-12 * np.max(np.abs(y))
    for o in range(8):
        s = np.array([1 if (o >> b) & 1 else -1 for b in (2, 1, 0)], float)
        A, _ = pkg.debug_operator(P, 0, o)
        y = _c2r(oracle.apply_op(0, P, -s / 2, _r2c(x, P)), P) * 2.0 ** (-deg)
        assert np.max(np.abs(A @ x - y)) <= 1e-13 * np.max(np.abs(y))
        A, _ = pkg.debug_operator(P, 1, o)
        y = _c2r(oracle.apply_op(1, P, s / 2, _r2c(x * 2.0 ** (-(deg + 1)), P)), P)
        assert np.max(np.abs(A @ x - y)) <= 1e-13 * np.max(np.abs(y))


def test_lattice_operator_matches_image_loops(pkg, oracle):
    """The fused FP64 lattice operator equals the reference's image M2M
    (kernel.cu:356-406) followed by the 3 x 26 x 27 root M2L entries
    (traverser.cpp:162-214), applied one by one in the oracle."""
    P, images = 5, 4
    R = (P + 1) ** 2
    rng = np.random.default_rng(5)
    x = rng.normal(size=R)
    A, _ = pkg.debug_operator(P, 3, 0, images=images)
    M = _r2c(x, P)
    Lacc = np.zeros_like(M)
    src = M
    c3 = 1.0
    for m in range(images - 1):
        for pz in (-1, 0, 1):
            for py in (-1, 0, 1):
                for px in (-1, 0, 1):
                    if px == py == pz == 0:
                        continue
                    for cz in (-1, 0, 1):
                        for cy in (-1, 0, 1):
                            for cx in (-1, 0, 1):
                                off = np.array([px * 3 + cx, py * 3 + cy, pz * 3 + cz]) * c3
                                Lacc = Lacc + oracle.apply_op(2, P, -off, src)
        if m < images - 2:
            nxt = np.zeros_like(src)
            for pz in (-1, 0, 1):
                for py in (-1, 0, 1):
                    for px in (-1, 0, 1):
                        nxt = nxt + oracle.apply_op(0, P, -np.array([px, py, pz]) * c3, src)
            src = nxt
        c3 *= 3
    y = _c2r(Lacc, P)
    assert np.max(np.abs(A @ x - y)) <= 1e-11 * np.max(np.abs(y))


@pytest.mark.parametrize("depth", [1, 2])
@pytest.mark.parametrize("images", [0, 1, 2, 4])
def test_lists_bit_exact_vs_reference_small(pkg, depth, images):
    g = golden("lists_small.npz")
    for k in ("p2p", "m2l"):
        t, s, o = pkg.lists(depth, images, k)
        assert np.array_equal(t, g[f"{k}_d{depth}_i{images}_tgt"])
        assert np.array_equal(s, g[f"{k}_d{depth}_i{images}_src"])
        assert np.array_equal(o, g[f"{k}_d{depth}_i{images}_off"])


def test_lists_bit_exact_vs_reference_hash(pkg):
    with open(os.path.join(GOLDEN, "lists_hash.json")) as f:
        ref = json.load(f)
    for key, v in ref.items():
        kind, d, i = key.split("_")
        t, s, o = pkg.lists(int(d[1:]), int(i[1:]), kind)
        assert len(t) == v["count"], key
        h = hashlib.sha256()
        for a in (t, s, o):
            h.update(np.ascontiguousarray(a, dtype="<i4").tobytes())
        assert h.hexdigest() == v["sha256"], key


@pytest.mark.parametrize("kw,status", [({"order": 1}, 1), ({"order": 17}, 1), ({"max_depth": 0}, 1),
                                       ({"max_depth": 8}, 1), ({"images": -1}, 1), ({"theta": 0.5}, 6),
                                       ({"rega": 0.1}, 6), ({"precision": 7}, 1), ({"m2l_split": 99}, 1),
                                       ({"aspect_z": 3}, 1), ({"aspect_z": 2, "images": 0}, 6),
                                       ({"precision": 1, "order": 13}, 6)])
def test_invalid_parameters_rejected_before_device_use(pkg, kw, status):
    import ctypes
    p = pkg.default_params(**kw)
    h = ctypes.c_void_p()
    rc = pkg.lib().gbfmm_create(ctypes.byref(p), 10, ctypes.byref(h))
    assert rc == status
    assert not h.value
    assert len(pkg.lib().gbfmm_last_error()) > 0


def test_create_without_device_fails_loudly(pkg):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(pkg.FmmError) as e:
        pkg.ZetaFmmSolver(10, np.zeros(10, np.float32), order=4, max_depth=1)
    assert e.value.status == 4


def test_systems_generator(systems):
    xyz, q, box = systems.cfg_small()
    assert xyz.shape == (9000, 3) and xyz.dtype == np.float32
    assert abs(float(q.astype(np.float64).sum())) < 1e-3
    assert (xyz >= 0).all() and (xyz < box[0]).all()
    # rigid geometry (before wrapping; check molecules away from the faces)
    w = xyz.reshape(-1, 3, 3).astype(np.float64)
    inner = np.all((w[:, 0] > 0.2) & (w[:, 0] < box[0] - 0.2), axis=1)
    d1 = np.linalg.norm(w[inner, 1] - w[inner, 0], axis=1)
    d2 = np.linalg.norm(w[inner, 2] - w[inner, 0], axis=1)
    assert np.allclose(d1, 0.1, atol=1e-5) and np.allclose(d2, 0.1, atol=1e-5)
    ang = np.degrees(np.arccos(np.sum((w[inner, 1] - w[inner, 0]) * (w[inner, 2] - w[inner, 0]), 1) / (d1 * d2)))
    assert np.allclose(ang, 109.47, atol=1e-2)
    x2, q2, _ = systems.cfg_small()
    assert np.array_equal(xyz, x2) and np.array_equal(q, q2)
    xb, qb, bb = systems.cfg_96k()
    assert len(qb) == 95600 and np.sum(qb == 1.0) == 100 and np.sum(qb == -1.0) == 100
    assert abs(float(qb.astype(np.float64).sum())) < 1e-2


def test_batch_arguments_rejected_before_device_use(pkg):
    import ctypes
    lib = pkg.lib()
    ip = ctypes.POINTER(ctypes.c_int)
    b = ctypes.c_void_p()
    off = np.array([0, 10, 5], np.int32)  # decreasing
    o = np.array([4, 4], np.int32)
    d = np.array([1, 1], np.int32)
    assert lib.gbfmm_batch_create(2, off.ctypes.data_as(ip), o.ctypes.data_as(ip), d.ctypes.data_as(ip), 4, 0, 0,
                                  ctypes.byref(b)) == 1
    assert not b.value
    off = np.array([1, 10, 20], np.int32)  # must start at 0
    assert lib.gbfmm_batch_create(2, off.ctypes.data_as(ip), o.ctypes.data_as(ip), d.ctypes.data_as(ip), 4, 0, 0,
                                  ctypes.byref(b)) == 1
    assert lib.gbfmm_batch_create_mixed(2, off.ctypes.data_as(ip), o.ctypes.data_as(ip), d.ctypes.data_as(ip),
                                        None, 4, 0, ctypes.byref(b)) == 1
    assert lib.gbfmm_batch_set_tuning(None, 0, 4, 0, 0) == 1
    assert lib.gbfmm_batch_get_tuning(None, None, None, None, None) == 1
    assert lib.gbfmm_batch_autotune(None, None, None, None, 3, None) == 1


def test_schedule_entry_points_reject_a_null_handle(pkg):
    """The single-solve scheduling entry points check their arguments before any
    device use: a NULL handle or output pointer is GBFMM_ERR_ARG."""
    import ctypes
    lib = pkg.lib()
    v = ctypes.c_int()
    for fn, args in (("gbfmm_set_launch_overlap", (None, 1)), ("gbfmm_get_launch_overlap", (None, ctypes.byref(v))),
                     ("gbfmm_set_near_start", (None, 1)), ("gbfmm_get_near_start", (None, ctypes.byref(v))),
                     ("gbfmm_set_tuning", (None, 0, 1, 2)), ("gbfmm_step_launches", (None, ctypes.byref(v))),
                     ("gbfmm_autotune", (None, None, None, 3, None)),
                     ("gbfmm_batch_set_schedule", (None, 1, 0, 0)),
                     ("gbfmm_batch_step_launches", (None, ctypes.byref(v)))):
        assert getattr(lib, fn)(*args) == 1, fn


def test_bench_pair_count_matches_the_reference_lists(oracle, systems):
    """bench.py's P2P pair count (the unit of its roofline) equals the sum over
    the reference-ordered P2P list of |target leaf| x |source leaf|."""
    import bench
    xyz, q, box = systems.water_ion_box(3000, 4.5, n_na=5, n_cl=5, seed=9)
    L, D = float(box[0]), 3
    tree = oracle.zeta_tree(xyz.astype(np.float64), L, D)
    leaves = np.nonzero(tree["depth"] == D)[0]
    counts = tree["body_num"][leaves]  # BFS order = Morton order of the leaves
    t, s, _ = oracle.zeta_lists(D, 4, L)["p2p"]
    want = int(np.sum(tree["body_num"][t].astype(np.int64) * tree["body_num"][s]))
    assert bench.p2p_pair_count(counts, D) == want


@pytest.mark.parametrize("depth", [2, 3, 4])
def test_bench_m2l_pair_count_matches_the_reference_lists(oracle, depth):
    """bench.py's M2L pair count (levels 1..depth; the root row is the lattice
    operator's) equals the reference-ordered M2L list's entries with targets below
    the root."""
    import bench
    t, _, _ = oracle.zeta_lists(depth, 4, 1.0)["m2l"]
    below_root = int(np.sum(t >= 1))  # BFS index 0 is the root
    assert bench.m2l_pairs(depth) == below_root
