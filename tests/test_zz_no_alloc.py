"""The tree build that allocates nothing (gbfmm_tree_build_noalloc).

It exists for callers that cannot allocate device memory when they call in,
such as an MD engine whose memory pool reserved the GPU at start-up.  Its
scratch is one static device array, shared by every call.  The test checks,
through the C ABI, that two calls in a row reproduce the body order and leaf
offsets of the allocating entry point exactly (integer outputs: tolerance 0),
and that sizes beyond the static limits are rejected."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fn(pkg):
    f = pkg.lib().gbfmm_tree_build_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _reference_tree(pkg, xyz, q, box, depth):
    s = pkg.ZetaFmmSolver(len(q), q, order=4, max_depth=depth, images=4)
    s.execute(xyz, box)
    order, lo, ln = s.tree()
    s.close()
    return order, np.concatenate([lo, [len(q)]]).astype(np.int32)


def test_noalloc_tree_matches_allocating_entry_point(pkg, systems):
    torch = pytest.importorskip("torch")
    f = _fn(pkg)
    stream = torch.cuda.current_stream()
    cases = [systems.water_ion_box(3000, 4.5, n_na=5, n_cl=5, seed=31) + (3,),
             systems.water_ion_box(700, 2.4, seed=32) + (2,)]
    for xyz, q, box, depth in cases:
        ref_order, ref_off = _reference_tree(pkg, xyz, q, box, depth)
        x = torch.from_numpy(xyz).cuda()
        qq = torch.from_numpy(q).cuda()
        order = torch.empty(len(q), dtype=torch.int32, device="cuda")
        off = torch.empty(8 ** depth + 1, dtype=torch.int32, device="cuda")
        bm = pkg.box_matrix(box)
        for _ in range(2):  # two calls in a row share (and reuse) the static scratch
            order.fill_(-1)
            off.fill_(-1)
            rc = f(x.data_ptr(), qq.data_ptr(), len(q), bm.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), depth,
                   order.data_ptr(), off.data_ptr(), stream.cuda_stream)
            assert rc == 0
            torch.cuda.synchronize()
            assert np.array_equal(order.cpu().numpy(), ref_order)
            assert np.array_equal(off.cpu().numpy(), ref_off)


def _call(pkg, f, xyz, q, box, depth, stream, calls=2):
    """Calls the entry point `calls` times in a row on the same inputs and returns
    each call's (order, leaf offsets)."""
    import torch
    x = torch.from_numpy(np.ascontiguousarray(xyz, np.float32)).cuda()
    qq = torch.from_numpy(np.ascontiguousarray(q, np.float32)).cuda()
    order = torch.empty(max(len(q), 1), dtype=torch.int32, device="cuda")
    off = torch.empty(8 ** depth + 1, dtype=torch.int32, device="cuda")
    bm = pkg.box_matrix(box)
    out = []
    for _ in range(calls):
        order.fill_(-1)
        off.fill_(-1)
        rc = f(x.data_ptr(), qq.data_ptr(), len(q), bm.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), depth,
               order.data_ptr(), off.data_ptr(), stream.cuda_stream)
        assert rc == 0
        torch.cuda.synchronize()
        out.append((order.cpu().numpy()[:len(q)], off.cpu().numpy()))
    return out


@pytest.mark.parametrize("name,depth", [("tree_edges_d1.npz", 1), ("tree_edges_d2.npz", 2),
                                        ("tree_edges_d3.npz", 3)])
def test_noalloc_tree_on_the_reference_edge_fixtures(pkg, name, depth):
    """Bodies exactly on cell boundaries and outside the box: body order and
    leaf counts equal the reference's own tree build (fixtures made by its
    tree.cpp), on two calls in a row."""
    torch = pytest.importorskip("torch")
    from conftest import golden
    g = golden(name)
    q = np.where(np.arange(len(g["xyz"])) % 2 == 0, 1.0, -1.0).astype(np.float32)
    for order, off in _call(pkg, _fn(pkg), g["xyz"], q, float(g["box"]), depth, torch.cuda.current_stream()):
        assert np.array_equal(order, g["order"])
        assert np.array_equal(np.diff(off), g["leaf_count"])
        assert off[0] == 0


def test_noalloc_tree_at_its_stated_limits(pkg, systems):
    """65,536 bodies at depth 4, the largest call the static scratch takes: equal
    to the allocating entry point, on two calls in a row."""
    torch = pytest.importorskip("torch")
    xyz, q, box = systems.water_ion_box(21846, 6.0, seed=33)
    xyz, q = xyz[:65536], q[:65536]
    assert len(q) == 65536
    ref_order, ref_off = _reference_tree(pkg, xyz, q, box, 4)
    for order, off in _call(pkg, _fn(pkg), xyz, q, box, 4, torch.cuda.current_stream()):
        assert np.array_equal(order, ref_order)
        assert np.array_equal(off, ref_off)


def test_noalloc_tree_rejects_sizes_beyond_its_limits(pkg):
    torch = pytest.importorskip("torch")
    f = _fn(pkg)
    bm = pkg.box_matrix(3.0)
    bp = bm.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    dummy = torch.zeros(16, device="cuda")
    assert f(dummy.data_ptr(), dummy.data_ptr(), 65537, bp, 3, dummy.data_ptr(), dummy.data_ptr(), None) == 1
    assert f(dummy.data_ptr(), dummy.data_ptr(), 4, bp, 5, dummy.data_ptr(), dummy.data_ptr(), None) == 1
    assert f(dummy.data_ptr(), dummy.data_ptr(), 4, pkg.box_matrix([3.0, 3.0, 3.5]).ctypes.data_as(
        ctypes.POINTER(ctypes.c_float)), 3, dummy.data_ptr(), dummy.data_ptr(), None) == 2
