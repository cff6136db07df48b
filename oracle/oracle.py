"""ctypes wrapper of the oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg import this
module; the product library never does.  It exposes:

* ``zeta_solve`` -- FP64 restatement of the zeta_fmm solver (zeta64.c),
* ``zeta_tree`` / ``zeta_lists`` -- restated tree build and traversal,
* ``ewald`` / ``direct`` -- FP64 Ewald and direct lattice sums (ewald64.c),
* ``ref_run`` -- the reference's own tree/traverser (oracle/_ref), when built.
"""
import ctypes
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libzetaref.so")

_lib = None
_ref = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        L.z64_solve.restype = ctypes.c_int
        L.z64_solve.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp]
        L.z64_tree.restype = ctypes.c_int
        L.z64_tree.argtypes = [ctypes.c_int, _dp, ctypes.c_double, _dp, ctypes.c_int, _ip, _ip, _ip, _ip,
                               _dp, ctypes.c_int]
        L.z64_lists.restype = ctypes.c_int
        L.z64_lists.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, _lp, _lp]
        L.z64_lists_fetch.restype = None
        L.z64_lists_fetch.argtypes = [ctypes.c_int, _ip, _ip, _dp]
        L.z64_harmonics.restype = None
        L.z64_harmonics.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp]
        L.z64_apply.restype = None
        L.z64_apply.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
        L.z64_set_threads.restype = None
        L.z64_set_threads.argtypes = [ctypes.c_int]
        L.ew64_solve.restype = ctypes.c_int
        L.ew64_solve.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                 _ip, _dp, _dp, ctypes.c_int, _dp]
        L.ew64_virial.restype = ctypes.c_int
        L.ew64_virial.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, _dp, _dp]
        L.direct64_solve.restype = ctypes.c_int
        L.direct64_solve.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_int, _dp, _dp]
        _lib = L
    return _lib


def set_threads(n):
    lib().z64_set_threads(int(n))


def zeta_solve(xyz, q, cycle, P, depth, images=4, theta=0.4, stages=7):
    """Reference-algorithm FMM in FP64. xyz (n,3) float64 (already float32-rounded
    by the caller when mimicking GROMACS RVec input), q (n,). Returns pot, force, energy."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    n = len(q)
    pot = np.zeros(n)
    force = np.zeros((n, 3))
    e = np.zeros(1)
    rc = lib().z64_solve(n, _d(xyz), _d(q), float(cycle), int(P), int(depth), int(images), float(theta),
                         int(stages), _d(pot), _d(force), _d(e))
    if rc != 0:
        raise ValueError("z64_solve rejected its arguments")
    return pot, force, float(e[0])


def zeta_solve_slab(xyz, q, a, P, depth, images=4, theta=0.4):
    """The same FP64 solver for a periodic slab box a x a x 2a: the slab is the
    periodic cube of edge 2a that holds it twice along x and twice along y (the
    same periodic charge density, so the same tin-foil Ewald limit), solved here
    literally on the four copies (4N bodies, cycle 2a, depth counted from that
    cube).  Returns the first copy's potentials and forces, and the box's energy."""
    xyz = np.asarray(xyz, dtype=np.float64)
    q = np.asarray(q, dtype=np.float64)
    n = len(q)
    shifts = np.array([[0.0, 0.0, 0.0], [a, 0.0, 0.0], [0.0, a, 0.0], [a, a, 0.0]])
    x4 = np.concatenate([xyz + s for s in shifts])
    q4 = np.concatenate([q] * 4)
    pot, force, e = zeta_solve(x4, q4, 2.0 * a, P, depth, images, theta)
    return pot[:n], force[:n], e / 4.0


def zeta_tree(xyz, cycle, depth):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    n = len(xyz)
    maxc = (8 ** (depth + 1) - 1) // 7
    order = np.zeros(max(n, 1), np.int32)
    cd = np.zeros(maxc, np.int32)
    bo = np.zeros(maxc, np.int32)
    bn = np.zeros(maxc, np.int32)
    cc = np.zeros((maxc, 3))
    center = np.full(3, cycle / 2.0)
    nc = lib().z64_tree(n, _d(xyz), cycle / 2.0, _d(center), int(depth), _i(order), _i(cd), _i(bo), _i(bn),
                        _d(cc), maxc)
    return dict(order=order[:n], depth=cd[:nc], body_off=bo[:nc], body_num=bn[:nc], center=cc[:nc])


def zeta_lists(depth, images, cycle=1.0, theta=0.4):
    np2p = ctypes.c_long()
    nm2l = ctypes.c_long()
    nimg = lib().z64_lists(int(depth), int(images), float(cycle), float(theta), ctypes.byref(np2p),
                           ctypes.byref(nm2l))
    out = {"n_image_cells": nimg}
    for which, name, cnt in ((0, "p2p", np2p.value), (1, "m2l", nm2l.value)):
        t = np.zeros(max(cnt, 1), np.int32)
        s = np.zeros(max(cnt, 1), np.int32)
        o = np.zeros((max(cnt, 1), 3))
        lib().z64_lists_fetch(which, _i(t), _i(s), _d(o))
        out[name] = (t[:cnt], s[:cnt], o[:cnt])
    return out


def harmonics(kind, P, d):
    d = np.ascontiguousarray(d, dtype=np.float64)
    out = np.zeros(2 * (P + 1) ** 2)
    lib().z64_harmonics(int(kind), int(P), _d(d), _d(out))
    return out[0::2] + 1j * out[1::2]


def apply_op(kind, P, d, vec):
    """kind 0: M2M, 1: L2L, 2: M2L; vec packed complex of length (P+1)(P+2)/2."""
    d = np.ascontiguousarray(d, dtype=np.float64)
    v = np.ascontiguousarray(np.stack([np.real(vec), np.imag(vec)], -1).reshape(-1), dtype=np.float64)
    out = np.zeros_like(v)
    lib().z64_apply(int(kind), int(P), _d(d), _d(v), _d(out))
    return out[0::2] + 1j * out[1::2]


def ewald(xyz, q, box, eps=1e-10, targets=None, rc=0.0, energy=False):
    """Converged FP64 Ewald (tin-foil). Returns (pot[targets], force[targets], energy|None)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    box = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    n = len(q)
    if energy:
        tg = np.arange(n, dtype=np.int32)
    else:
        tg = np.ascontiguousarray(np.arange(n) if targets is None else targets, dtype=np.int32)
    nt = len(tg)
    pot = np.zeros(nt)
    force = np.zeros((nt, 3))
    e = np.zeros(1)
    lib().ew64_solve(n, _d(xyz), _d(q), _d(box), float(eps), float(rc), nt, _i(tg), _d(pot), _d(force),
                     1 if energy else 0, _d(e))
    return pot, force, (float(e[0]) if energy else None)


def ewald_virial(xyz, q, box, eps=1e-9):
    """FP64 Ewald energy and virial tensor Xi = -1/2 sum_pairs r_ij (x) F_ij
    (kJ/mol, 3 x 3), tin-foil boundary."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    box = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    e = np.zeros(1)
    vir = np.zeros(9)
    lib().ew64_virial(len(q), _d(xyz), _d(q), _d(box), float(eps), _d(e), _d(vir))
    return float(e[0]), vir.reshape(3, 3)


def direct(xyz, q, L, nmax):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    n = len(q)
    pot = np.zeros(n)
    force = np.zeros((n, 3))
    lib().direct64_solve(n, _d(xyz), _d(q), float(L), int(nmax), _d(pot), _d(force))
    return pot, force


# ------------------------------------------------------------------ reference itself

RTFMM_LIB = os.path.join(HERE, "_ref", "librtfmmref.so")
_rt = None


def rtfmm_available():
    """The reference's own CPU FMM (src/gromacs/rtfmm, built by rtfmm_build.sh on
    an x86-64 host where the reference checkout exists)."""
    return os.path.exists(RTFMM_LIB)


def rtfmm_solve(xyz, q, cycle, P=10, depth=3, images=4):
    """The reference's own CPU FMM (kernel-independent, P surface points per
    edge, OpenMP) on a cubic periodic box: potentials and forces in GROMACS
    units, as rtFmmSolver::execute leaves them."""
    global _rt
    if _rt is None:
        L = ctypes.CDLL(RTFMM_LIB)
        L.rtfmm_ref_solve.restype = ctypes.c_int
        L.rtfmm_ref_solve.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, _dp, _dp]
        _rt = L
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    n = len(q)
    pot = np.zeros(n)
    force = np.zeros((n, 3))
    rc = _rt.rtfmm_ref_solve(n, _d(xyz), _d(q), float(cycle), int(P), int(depth), int(images), _d(pot), _d(force))
    if rc != 0:
        raise ValueError("rtfmm_ref_solve rejected its arguments")
    return pot, force


def ref_available():
    return os.path.exists(REF_LIB)


def ref_lib():
    global _ref
    if _ref is None:
        R = ctypes.CDLL(REF_LIB)
        R.zref_run.restype = ctypes.c_int
        R.zref_run.argtypes = [ctypes.c_int, _dp, ctypes.c_double, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               ctypes.c_double]
        R.zref_cells.restype = None
        R.zref_cells.argtypes = [_ip, _dp, _dp, _ip, _ip, _ip, _ip]
        R.zref_order.restype = None
        R.zref_order.argtypes = [_ip]
        R.zref_nlist.restype = ctypes.c_long
        R.zref_nlist.argtypes = [ctypes.c_int]
        R.zref_list.restype = None
        R.zref_list.argtypes = [ctypes.c_int, _ip, _ip, _dp]
        R.zref_solve.restype = ctypes.c_int
        R.zref_solve.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 _dp, _dp]
        _ref = R
    return _ref


def ref_run(xyz, cycle, depth, images, theta=0.4):
    """Run the reference's own CompleteBalancedOctree + Traverser."""
    R = ref_lib()
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(xyz)
    center = np.full(3, cycle / 2.0)
    nc = R.zref_run(n, _d(xyz), cycle / 2.0, _d(center), int(depth), int(images), float(cycle), float(theta))
    depth_a = np.zeros(nc, np.int32)
    r = np.zeros(nc)
    c = np.zeros((nc, 3))
    co = np.zeros(nc, np.int32)
    cn = np.zeros(nc, np.int32)
    bo = np.zeros(nc, np.int32)
    bn = np.zeros(nc, np.int32)
    R.zref_cells(_i(depth_a), _d(r), _d(c), _i(co), _i(cn), _i(bo), _i(bn))
    order = np.zeros(max(n, 1), np.int32)
    R.zref_order(_i(order))
    out = dict(depth=depth_a, r=r, center=c, child_off=co, child_num=cn, body_off=bo, body_num=bn,
               order=order[:n])
    for which, name in ((0, "p2p"), (1, "m2l")):
        cnt = R.zref_nlist(which)
        t = np.zeros(max(cnt, 1), np.int32)
        s = np.zeros(max(cnt, 1), np.int32)
        o = np.zeros((max(cnt, 1), 3))
        R.zref_list(which, _i(t), _i(s), _d(o))
        out[name] = (t[:cnt], s[:cnt], o[:cnt])
    return out


def ref_solve(xyz, q, cycle, P, depth, images=4):
    """The reference's own FP64 kernels (kernel.cu p2m ... l2p, run on the host by
    oracle/ref_kernels_driver.cpp) on its own tree and lists.  Returns potentials
    (kJ/mol/e) and forces (kJ/mol/nm) in input order, before the dipole correction:
    the quantities of zeta_solve(..., stages=3)."""
    R = ref_lib()
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    q = np.ascontiguousarray(q, dtype=np.float64)
    n = len(q)
    pot = np.zeros(n)
    force = np.zeros((n, 3))
    rc = R.zref_solve(n, _d(xyz), _d(q), float(cycle), int(P), int(depth), int(images), _d(pot), _d(force))
    if rc != 0:
        raise ValueError("zref_solve rejected its arguments")
    return pot, force

