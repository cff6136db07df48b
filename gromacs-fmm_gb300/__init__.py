"""GB300-native FMM Coulomb solver: host-side mirror of the reference plugin API.

``ZetaFmmSolver`` mirrors ``coulomb_solver::BaseSolver`` as implemented by the
fork's GPU FMM (src/gromacs/coulomb_solvers/basesolver.h:43-90,
src/gromacs/zeta_fmm/zeta_fmm_solver.cpp): ``set_parameter`` takes the charges,
``execute(coords, box)`` computes, ``add_force`` accumulates forces,
``get_energy`` returns the Coulomb energy and ``compare_forces`` prints and
returns the relative L2 force error.  All compute goes through the C ABI of
lib/libgbfmm.so (include/gbfmm.h); there is no CPU path: if the library or a
CUDA device is missing the calls raise.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libgbfmm.so")

PREC_FP32 = 0
PREC_BF16X3 = 1
PREC_BF16X1 = 2
FLAG_NO_GRAPH = 1
FLAG_DETERMINISTIC = 2
FLAG_HOST_COPY = 4

STATUS = {0: "ok", 1: "invalid argument", 2: "invalid box", 3: "non-finite coordinate or charge", 4: "CUDA error",
          5: "out of memory", 6: "unsupported", 7: "call out of order", 8: "device wait timed out",
          9: "system not neutral"}


class FmmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Params(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("max_depth", ctypes.c_int), ("images", ctypes.c_int),
                ("theta", ctypes.c_double), ("rega", ctypes.c_double), ("precision", ctypes.c_int),
                ("m2l_tile", ctypes.c_int), ("m2l_split", ctypes.c_int), ("flags", ctypes.c_int),
                ("aspect_z", ctypes.c_int)]


_lib = None


def build(force=False):
    import importlib
    return importlib.import_module(__name__ + ".build").build(force=force)


def lib():
    """Loads the in-tree library (raises if it is missing: no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FmmError(4, f"{LIB_PATH} not built; run build()")
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        ip = ctypes.POINTER(ctypes.c_int)
        fp = ctypes.POINTER(ctypes.c_float)
        dp = ctypes.POINTER(ctypes.c_double)
        sig = {
            "gbfmm_params_default": (None, [ctypes.POINTER(Params)]),
            "gbfmm_status_string": (ctypes.c_char_p, [ctypes.c_int]),
            "gbfmm_last_error": (ctypes.c_char_p, []),
            "gbfmm_version": (ctypes.c_char_p, []),
            "gbfmm_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.c_int, ctypes.POINTER(vp)]),
            "gbfmm_destroy": (ctypes.c_int, [vp]),
            "gbfmm_set_charges": (ctypes.c_int, [vp, ctypes.c_int, fp]),
            "gbfmm_execute": (ctypes.c_int, [vp, fp, fp, ctypes.c_int]),
            "gbfmm_execute_device": (ctypes.c_int, [vp, vp, fp, vp]),
            "gbfmm_device_outputs": (ctypes.c_int, [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]),
            "gbfmm_add_forces": (ctypes.c_int, [vp, fp]),
            "gbfmm_get_forces": (ctypes.c_int, [vp, fp]),
            "gbfmm_get_potentials": (ctypes.c_int, [vp, fp]),
            "gbfmm_get_energy": (ctypes.c_int, [vp, dp]),
            "gbfmm_compare_forces": (ctypes.c_int, [vp, fp, dp]),
            "gbfmm_set_timing": (ctypes.c_int, [vp, ctypes.c_int]),
            "gbfmm_stage_times": (ctypes.c_int, [vp, fp, ctypes.c_int, ip]),
            "gbfmm_autotune": (ctypes.c_int, [vp, fp, fp, ctypes.c_int, fp]),
            "gbfmm_get_tuning": (ctypes.c_int, [vp, ip, ip, ip]),
            "gbfmm_set_tuning": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
            "gbfmm_stage_name": (ctypes.c_char_p, [ctypes.c_int]),
            "gbfmm_step_launches": (ctypes.c_int, [vp, ip]),
            "gbfmm_get_tree": (ctypes.c_int, [vp, ip, ip, ip]),
            "gbfmm_get_lists": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_long), ip, ip, ip]),
            "gbfmm_lists": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_long), ip,
                                           ip, ip]),
            "gbfmm_debug_operator": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, ip, dp]),
            "gbfmm_debug_harmonics": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, dp, dp]),
            "gbfmm_debug_bounded_wait": (ctypes.c_int, [ctypes.c_uint, vp]),
            "gbfmm_batch_status": (ctypes.c_int, [vp]),
            "gbfmm_set_near_start": (ctypes.c_int, [vp, ctypes.c_int]),
            "gbfmm_get_near_start": (ctypes.c_int, [vp, ip]),
            "gbfmm_set_launch_overlap": (ctypes.c_int, [vp, ctypes.c_int]),
            "gbfmm_get_launch_overlap": (ctypes.c_int, [vp, ip]),
            "gbfmm_batch_step_launches": (ctypes.c_int, [vp, ip]),
            "gbfmm_batch_set_schedule": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
            "gbfmm_batch_get_schedule": (ctypes.c_int, [vp, ip, ip, ip]),
            "gbfmm_get_virial": (ctypes.c_int, [vp, dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise FmmError(rc, lib().gbfmm_last_error().decode())


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def default_params(**kw):
    p = Params()
    lib().gbfmm_params_default(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def box_matrix(box):
    """Cubic/rectangular edge(s) -> row-major float[9] GROMACS matrix."""
    b = np.asarray(box, dtype=np.float64)
    if b.size == 9:
        return _f32(b.reshape(9))
    b = np.broadcast_to(b, (3,))
    m = np.zeros(9, np.float32)
    m[0], m[4], m[8] = b
    return m


class ZetaFmmSolver:
    """Mirror of zeta_fmm::ZetaFmmSolver over the GB300 library.

    Parameters default to the reference's constants (P=10, max_depth=3,
    images=4, zeta_fmm_solver.cpp:10-13)."""

    def __init__(self, natoms, charges=None, order=10, max_depth=3, images=4, precision=PREC_FP32, flags=0,
                 m2l_split=0, aspect_z=1):
        self.natoms = int(natoms)
        self.params = default_params(order=order, max_depth=max_depth, images=images, precision=precision,
                                     flags=flags, m2l_split=m2l_split, aspect_z=aspect_z)
        h = ctypes.c_void_p()
        _check(lib().gbfmm_create(ctypes.byref(self.params), self.natoms, ctypes.byref(h)))
        self._h = h
        if charges is not None:
            self.set_parameter(charges)

    def close(self):
        if getattr(self, "_h", None):
            lib().gbfmm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- BaseSolver API
    def set_parameter(self, charges):
        q = _f32(charges)
        if q.shape != (self.natoms,):
            raise FmmError(1, f"expected {self.natoms} charges, got {q.shape}")
        self._q = q
        _check(lib().gbfmm_set_charges(self._h, self.natoms, _fp(q)))

    def execute(self, coords, box, verbose=0, dummy=0):
        x = _f32(coords).reshape(-1)
        if x.size != 3 * self.natoms:
            raise FmmError(1, f"expected {3 * self.natoms} coordinates, got {x.size}")
        m = box_matrix(box)
        _check(lib().gbfmm_execute(self._h, _fp(x), _fp(m), int(verbose)))

    def add_force(self, forces):
        f = np.asarray(forces)
        if f.dtype != np.float32 or not f.flags.c_contiguous or f.size != 3 * self.natoms:
            raise FmmError(1, "forces must be a C-contiguous float32 array of natoms x 3")
        _check(lib().gbfmm_add_forces(self._h, _fp(f)))

    def get_energy(self):
        e = ctypes.c_double()
        _check(lib().gbfmm_get_energy(self._h, ctypes.byref(e)))
        return e.value

    def compare_forces(self, fs, verbose=True):
        g = _f32(fs).reshape(-1)
        out = ctypes.c_double()
        _check(lib().gbfmm_compare_forces(self._h, _fp(g), ctypes.byref(out)))
        if verbose:
            print("L2f = %.8f" % out.value)
        return out.value

    # -- extensions
    def forces(self):
        f = np.zeros((self.natoms, 3), np.float32)
        _check(lib().gbfmm_get_forces(self._h, _fp(f)))
        return f

    def virial(self):
        """Coulomb virial of the last execute, -1/2 sum_pairs r_ij (x) F_ij (kJ/mol, 3 x 3)."""
        v = np.zeros(9)
        _check(lib().gbfmm_get_virial(self._h, v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return v.reshape(3, 3)

    def potentials(self):
        p = np.zeros(self.natoms, np.float32)
        _check(lib().gbfmm_get_potentials(self._h, _fp(p)))
        return p

    def execute_device(self, coords_ptr, box, stream_ptr=0):
        m = box_matrix(box)
        _check(lib().gbfmm_execute_device(self._h, ctypes.c_void_p(int(coords_ptr)), _fp(m),
                                          ctypes.c_void_p(int(stream_ptr))))

    def device_outputs(self):
        f, p, e = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        _check(lib().gbfmm_device_outputs(self._h, ctypes.byref(f), ctypes.byref(p), ctypes.byref(e)))
        return f.value, p.value, e.value

    def set_timing(self, on=True):
        _check(lib().gbfmm_set_timing(self._h, 1 if on else 0))

    def step_launches(self):
        n = ctypes.c_int()
        _check(lib().gbfmm_step_launches(self._h, ctypes.byref(n)))
        return n.value

    def autotune(self, coords, box, reps=5):
        """Times the P2P and tensor-core M2L tile shapes on this configuration and
        keeps the fastest (gbfmm_autotune); returns the tuning and its step time."""
        L = lib()
        x = _f32(coords).reshape(-1)
        m = box_matrix(box)
        ms = ctypes.c_float()
        _check(L.gbfmm_autotune(self._h, _fp(x), _fp(m), int(reps), ctypes.byref(ms)))
        t = self.tuning()
        t["ms"] = ms.value
        return t

    def tuning(self):
        a, b, c, d = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().gbfmm_get_tuning(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        _check(lib().gbfmm_get_near_start(self._h, ctypes.byref(d)))
        return {"p2p_variant": a.value, "m2l_split": b.value, "m2l_stages": c.value, "near_after": d.value}

    def set_near_start(self, after):
        _check(lib().gbfmm_set_near_start(self._h, int(after)))

    def launch_overlap(self):
        e = ctypes.c_int()
        _check(lib().gbfmm_get_launch_overlap(self._h, ctypes.byref(e)))
        return bool(e.value)

    def set_launch_overlap(self, enable):
        """Programmatic dependent launches between the step's consecutive kernels
        (gbfmm_set_launch_overlap); on by default."""
        _check(lib().gbfmm_set_launch_overlap(self._h, 1 if enable else 0))

    def set_tuning(self, p2p_variant=0, m2l_split=1, m2l_stages=2):
        _check(lib().gbfmm_set_tuning(self._h, int(p2p_variant), int(m2l_split), int(m2l_stages)))

    def stage_times(self):
        ms = np.zeros(16, np.float32)
        n = ctypes.c_int()
        _check(lib().gbfmm_stage_times(self._h, _fp(ms), 16, ctypes.byref(n)))
        return {lib().gbfmm_stage_name(i).decode(): float(ms[i]) for i in range(n.value)}

    def tree(self):
        # stored leaves: all 8^depth of a cube, the box's quarter of the root cube of a slab
        nleaf = 8 ** self.params.max_depth // (4 if self.params.aspect_z == 2 else 1)
        order = np.zeros(max(self.natoms, 1), np.int32)
        lo = np.zeros(nleaf, np.int32)
        ln = np.zeros(nleaf, np.int32)
        ip = ctypes.POINTER(ctypes.c_int)
        _check(lib().gbfmm_get_tree(self._h, order.ctypes.data_as(ip), lo.ctypes.data_as(ip), ln.ctypes.data_as(ip)))
        return order[:self.natoms], lo, ln

    def lists(self, which):
        """which 'p2p' or 'm2l': (target, source, offset[n,3] in periods), reference order."""
        w = 0 if which == "p2p" else 1
        cnt = ctypes.c_long()
        _check(lib().gbfmm_get_lists(self._h, w, ctypes.byref(cnt), None, None, None))
        n = cnt.value
        t = np.zeros(max(n, 1), np.int32)
        s = np.zeros(max(n, 1), np.int32)
        o = np.zeros((max(n, 1), 3), np.int32)
        ip = ctypes.POINTER(ctypes.c_int)
        _check(lib().gbfmm_get_lists(self._h, w, ctypes.byref(cnt), t.ctypes.data_as(ip), s.ctypes.data_as(ip),
                                     o.ctypes.data_as(ip)))
        return t[:n], s[:n], o[:n]


class BatchSolver:
    """Many independent cubic systems solved together through one CUDA graph
    (gbfmm_batch_*).  systems: list of (coords (n,3), charges (n,), box edge);
    orders/depths: one per system; precision: one for every system, or a list
    with each system's own (gbfmm_batch_create_mixed)."""

    def __init__(self, natoms_list, orders, depths, images=4, precision=PREC_FP32, flags=0):
        L = lib()
        vp = ctypes.c_void_p
        ip = ctypes.POINTER(ctypes.c_int)
        fp = ctypes.POINTER(ctypes.c_float)
        dp = ctypes.POINTER(ctypes.c_double)
        L.gbfmm_batch_create.restype = ctypes.c_int
        L.gbfmm_batch_create.argtypes = [ctypes.c_int, ip, ip, ip, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(vp)]
        L.gbfmm_batch_create_mixed.restype = ctypes.c_int
        L.gbfmm_batch_create_mixed.argtypes = [ctypes.c_int, ip, ip, ip, ip, ctypes.c_int, ctypes.c_int,
                                               ctypes.POINTER(vp)]
        L.gbfmm_batch_execute.restype = ctypes.c_int
        L.gbfmm_batch_execute.argtypes = [vp, fp, fp, fp, fp, fp, dp]
        L.gbfmm_batch_execute_device.restype = ctypes.c_int
        L.gbfmm_batch_execute_device.argtypes = [vp, vp, vp, fp, vp]
        L.gbfmm_batch_device_outputs.restype = ctypes.c_int
        L.gbfmm_batch_device_outputs.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]
        L.gbfmm_batch_destroy.restype = ctypes.c_int
        L.gbfmm_batch_destroy.argtypes = [vp]
        L.gbfmm_batch_autotune.restype = ctypes.c_int
        L.gbfmm_batch_autotune.argtypes = [vp, vp, vp, fp, ctypes.c_int, fp]
        L.gbfmm_batch_get_tuning.restype = ctypes.c_int
        L.gbfmm_batch_get_tuning.argtypes = [vp, ip, ip, ip, ip]
        L.gbfmm_batch_set_tuning.restype = ctypes.c_int
        L.gbfmm_batch_set_tuning.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        self.n_sys = len(natoms_list)
        self.offsets = np.concatenate([[0], np.cumsum(natoms_list)]).astype(np.int32)
        o = np.ascontiguousarray(orders, dtype=np.int32)
        d = np.ascontiguousarray(depths, dtype=np.int32)
        h = ctypes.c_void_p()
        if np.ndim(precision) == 0:
            _check(L.gbfmm_batch_create(self.n_sys, self.offsets.ctypes.data_as(ip), o.ctypes.data_as(ip),
                                        d.ctypes.data_as(ip), images, int(precision), flags, ctypes.byref(h)))
        else:  # each system's own precision
            pr = np.ascontiguousarray(precision, dtype=np.int32)
            _check(L.gbfmm_batch_create_mixed(self.n_sys, self.offsets.ctypes.data_as(ip), o.ctypes.data_as(ip),
                                              d.ctypes.data_as(ip), pr.ctypes.data_as(ip), images, flags,
                                              ctypes.byref(h)))
        self._b = h

    def close(self):
        if getattr(self, "_b", None):
            lib().gbfmm_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def execute(self, coords, charges, box_edges):
        """Host arrays (packed in system order); returns forces, potentials, energies."""
        x = _f32(coords).reshape(-1)
        q = _f32(charges)
        b = _f32(box_edges)
        n = int(self.offsets[-1])
        f = np.zeros((n, 3), np.float32)
        p = np.zeros(n, np.float32)
        e = np.zeros(self.n_sys)
        _check(lib().gbfmm_batch_execute(self._b, _fp(x), _fp(q), _fp(b), _fp(f), _fp(p),
                                         e.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return f, p, e

    def execute_device(self, coords_ptr, charges_ptr, box_edges, stream_ptr=0):
        b = _f32(box_edges)
        _check(lib().gbfmm_batch_execute_device(self._b, ctypes.c_void_p(int(coords_ptr)),
                                                ctypes.c_void_p(int(charges_ptr)), _fp(b),
                                                ctypes.c_void_p(int(stream_ptr))))

    def status(self):
        """Waits for the last step; raises FmmError if a system reported an error."""
        _check(lib().gbfmm_batch_status(self._b))

    def schedule(self):
        v = [ctypes.c_int() for _ in range(3)]
        _check(lib().gbfmm_batch_get_schedule(self._b, *[ctypes.byref(x) for x in v]))
        return {"far_lanes": v[0].value, "far_prio": v[1].value, "near_after": v[2].value}

    def set_schedule(self, far_lanes=1, far_prio=0, near_after=0):
        _check(lib().gbfmm_batch_set_schedule(self._b, int(far_lanes), int(far_prio), int(near_after)))

    def step_launches(self):
        """Kernels one batch step launches (counted when its graph is captured)."""
        n = ctypes.c_int()
        _check(lib().gbfmm_batch_step_launches(self._b, ctypes.byref(n)))
        return n.value

    def tuning(self):
        v = [ctypes.c_int() for _ in range(4)]
        _check(lib().gbfmm_batch_get_tuning(self._b, *[ctypes.byref(x) for x in v]))
        return {"p2p_shape": v[0].value, "p2p_per_sm": v[1].value, "m2l_split": v[2].value,
                "m2l_stages": v[3].value}

    def set_tuning(self, p2p_shape=0, p2p_per_sm=4, m2l_split=0, m2l_stages=0):
        _check(lib().gbfmm_batch_set_tuning(self._b, int(p2p_shape), int(p2p_per_sm), int(m2l_split),
                                            int(m2l_stages)))

    def autotune(self, coords_ptr, charges_ptr, box_edges, reps=3):
        """Device inputs (as execute_device); keeps the fastest batch tuning and
        returns it with its step time."""
        b = _f32(box_edges)
        ms = ctypes.c_float()
        _check(lib().gbfmm_batch_autotune(self._b, ctypes.c_void_p(int(coords_ptr)), ctypes.c_void_p(int(charges_ptr)),
                                          _fp(b), int(reps), ctypes.byref(ms)))
        return dict(self.tuning(), **self.schedule(), ms=ms.value)


def lists(max_depth, images, which):
    """Reference-ordered interaction lists without a handle (host only)."""
    w = 0 if which == "p2p" else 1
    cnt = ctypes.c_long()
    _check(lib().gbfmm_lists(max_depth, images, w, ctypes.byref(cnt), None, None, None))
    n = cnt.value
    t = np.zeros(max(n, 1), np.int32)
    s = np.zeros(max(n, 1), np.int32)
    o = np.zeros((max(n, 1), 3), np.int32)
    ip = ctypes.POINTER(ctypes.c_int)
    _check(lib().gbfmm_lists(max_depth, images, w, ctypes.byref(cnt), t.ctypes.data_as(ip), s.ctypes.data_as(ip),
                             o.ctypes.data_as(ip)))
    return t[:n], s[:n], o[:n]


def debug_operator(order, kind, index, images=4):
    R = (order + 1) ** 2
    mat = np.zeros((R, R))
    dim = ctypes.c_int()
    cv = np.zeros(4)
    dp = ctypes.POINTER(ctypes.c_double)
    _check(lib().gbfmm_debug_operator(order, images, kind, index, mat.ctypes.data_as(dp), ctypes.byref(dim),
                                      cv.ctypes.data_as(dp)))
    return mat, cv


def debug_bounded_wait(polls, stream_ptr=0):
    """The library's bounded mbarrier wait on a barrier nothing completes
    (gbfmm_debug_bounded_wait): raises FmmError(GBFMM_ERR_TIMEOUT) when it gives up."""
    _check(lib().gbfmm_debug_bounded_wait(int(polls), ctypes.c_void_p(int(stream_ptr))))


def debug_harmonics(order, kind, d):
    n = (order + 1) * (order + 2) // 2
    out = np.zeros(2 * n)
    d = np.ascontiguousarray(d, dtype=np.float64)
    dp = ctypes.POINTER(ctypes.c_double)
    _check(lib().gbfmm_debug_harmonics(order, kind, d.ctypes.data_as(dp), out.ctypes.data_as(dp)))
    return out[0::2] + 1j * out[1::2]
