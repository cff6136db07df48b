"""Learned choice of (order, depth, precision) for a force-error tolerance.

Host side of the tuner in include/gbfmm.h: per-step statistics computed on the
GPU (gbfmm_features), a 3-layer MLP whose forward, backward and Adam kernels
are the library's own (gbfmm_mlp_*), and the proposal (gbfmm_tuner_propose).

`TunedSolver` checks every proposal through the library's gbfmm_tuner_choose:
it solves the system once with the proposal and once with the plain
fixed-parameter FMM (order 10, the check solve) and keeps the proposal only if their
forces agree within the tolerance (retrying one and two orders higher);
otherwise it falls back to the plain FMM.  Nothing here uses an FP64
reference: training tuples come from tests/golden/make_tuner_data.py.
"""
import ctypes
import importlib
import os

import numpy as np

_pkg = importlib.import_module(__name__.rsplit(".", 1)[0])
lib, _check, FmmError = _pkg.lib, _pkg._check, _pkg.FmmError

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "tuner_weights.bin")
NFEAT = 57
N_IN = NFEAT + 4
PLAIN_ORDER = 10
MAX_CHECKS = 8  # GBFMM_TUNER_MAX_CHECKS

class TunerChoice(ctypes.Structure):
    """gbfmm_tuner_choice of include/gbfmm.h."""
    _fields_ = [("order", ctypes.c_int), ("depth", ctypes.c_int), ("precision", ctypes.c_int),
                ("fallback", ctypes.c_int), ("diff_vs_plain", ctypes.c_double),
                ("proposed_order", ctypes.c_int), ("proposed_depth", ctypes.c_int),
                ("proposed_precision", ctypes.c_int), ("pred_rel_force_err", ctypes.c_float),
                ("pred_ms", ctypes.c_float), ("nchecks", ctypes.c_int), ("check_order", ctypes.c_int * MAX_CHECKS),
                ("check_diff", ctypes.c_double * MAX_CHECKS)]


_fp = ctypes.POINTER(ctypes.c_float)
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p


def _sig():
    L = lib()
    if getattr(L, "_tuner_sig", False):
        return L
    sig = {
        "gbfmm_features": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _fp, _fp, _vp]),
        "gbfmm_mlp_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong,
                                            ctypes.POINTER(_vp)]),
        "gbfmm_mlp_destroy": (ctypes.c_int, [_vp]),
        "gbfmm_mlp_num_params": (ctypes.c_int, [_vp, _ip]),
        "gbfmm_mlp_get_params": (ctypes.c_int, [_vp, _fp]),
        "gbfmm_mlp_set_params": (ctypes.c_int, [_vp, _fp]),
        "gbfmm_mlp_set_normalization": (ctypes.c_int, [_vp, _fp, _fp, _fp, _fp]),
        "gbfmm_mlp_forward": (ctypes.c_int, [_vp, _fp, ctypes.c_int, _fp]),
        "gbfmm_mlp_loss_grad": (ctypes.c_int, [_vp, _fp, _fp, ctypes.c_int, _dp, _fp]),
        "gbfmm_mlp_train": (ctypes.c_int, [_vp, _fp, _fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                           ctypes.c_ulonglong, _dp]),
        "gbfmm_mlp_predict": (ctypes.c_int, [_vp, _fp, ctypes.c_int, _fp]),
        "gbfmm_mlp_save": (ctypes.c_int, [_vp, ctypes.c_char_p]),
        "gbfmm_mlp_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_vp)]),
        "gbfmm_tuner_input": (ctypes.c_int, [_fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _fp]),
        "gbfmm_tuner_propose": (ctypes.c_int, [_vp, _fp, ctypes.c_double, ctypes.c_double, _ip, _ip, _ip, _fp, _fp]),
        "gbfmm_tuner_choose": (ctypes.c_int, [_vp, ctypes.c_int, _fp, _fp, _fp, ctypes.c_int, ctypes.c_double,
                                              ctypes.c_double, ctypes.POINTER(TunerChoice)]),
        "gbfmm_plain_depth": (ctypes.c_int, [ctypes.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    L._tuner_sig = True
    return L


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def features(d_coords, d_charges, natoms, box, stream=0):
    """Statistics of a system whose coordinates/charges are on the device."""
    out = np.zeros(NFEAT, np.float32)
    m = _pkg.box_matrix(box)
    _check(_sig().gbfmm_features(_vp(int(d_coords)), _vp(int(d_charges)), int(natoms), m.ctypes.data_as(_fp),
                                 out.ctypes.data_as(_fp), _vp(int(stream))))
    return out


def tuner_input(feat, order, depth, precision):
    row = np.zeros(N_IN, np.float32)
    f = _f(feat)
    _check(_sig().gbfmm_tuner_input(f.ctypes.data_as(_fp), int(order), int(depth), int(precision),
                                    row.ctypes.data_as(_fp)))
    return row


class Mlp:
    """The tuner network (n_in -> n_hidden -> n_hidden -> n_out, tanh)."""

    def __init__(self, n_in=N_IN, n_hidden=64, n_out=2, seed=0, _handle=None):
        L = _sig()
        if _handle is None:
            h = _vp()
            _check(L.gbfmm_mlp_create(n_in, n_hidden, n_out, seed, ctypes.byref(h)))
            _handle = h
        self._h = _handle
        self.n_in, self.n_hidden, self.n_out = n_in, n_hidden, n_out

    @classmethod
    def load(cls, path=WEIGHTS):
        h = _vp()
        _check(_sig().gbfmm_mlp_load(path.encode(), ctypes.byref(h)))
        # the network's shape from the file header: "GBFMMMLP", version, I, H, O (int32)
        with open(path, "rb") as fh:
            hdr = fh.read(24)
        _, n_in, n_hidden, n_out = np.frombuffer(hdr[8:24], "<i4")
        return cls(n_in=int(n_in), n_hidden=int(n_hidden), n_out=int(n_out), _handle=h)

    def close(self):
        if getattr(self, "_h", None):
            _sig().gbfmm_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_params(self):
        n = ctypes.c_int()
        _check(_sig().gbfmm_mlp_num_params(self._h, ctypes.byref(n)))
        return n.value

    def params(self):
        p = np.zeros(self.num_params(), np.float32)
        _check(_sig().gbfmm_mlp_get_params(self._h, p.ctypes.data_as(_fp)))
        return p

    def set_params(self, p):
        p = _f(p)
        _check(_sig().gbfmm_mlp_set_params(self._h, p.ctypes.data_as(_fp)))

    def set_normalization(self, xm, xs, ym, ys):
        a = [_f(v) for v in (xm, xs, ym, ys)]
        _check(_sig().gbfmm_mlp_set_normalization(self._h, *[v.ctypes.data_as(_fp) for v in a]))

    def forward(self, x):
        x = _f(x).reshape(-1, self.n_in)
        y = np.zeros((len(x), self.n_out), np.float32)
        _check(_sig().gbfmm_mlp_forward(self._h, x.ctypes.data_as(_fp), len(x), y.ctypes.data_as(_fp)))
        return y

    def loss_grad(self, x, t):
        x = _f(x).reshape(-1, self.n_in)
        t = _f(t).reshape(-1, self.n_out)
        loss = ctypes.c_double()
        g = np.zeros(self.num_params(), np.float32)
        _check(_sig().gbfmm_mlp_loss_grad(self._h, x.ctypes.data_as(_fp), t.ctypes.data_as(_fp), len(x),
                                          ctypes.byref(loss), g.ctypes.data_as(_fp)))
        return loss.value, g

    def train(self, x, t, epochs=200, batch=128, lr=2e-3, seed=1):
        x = _f(x).reshape(-1, self.n_in)
        t = _f(t).reshape(-1, self.n_out)
        loss = ctypes.c_double()
        _check(_sig().gbfmm_mlp_train(self._h, x.ctypes.data_as(_fp), t.ctypes.data_as(_fp), len(x), epochs, batch,
                                      lr, seed, ctypes.byref(loss)))
        return loss.value

    def predict(self, x):
        x = _f(x).reshape(-1, self.n_in)
        y = np.zeros((len(x), self.n_out), np.float32)
        _check(_sig().gbfmm_mlp_predict(self._h, x.ctypes.data_as(_fp), len(x), y.ctypes.data_as(_fp)))
        return y

    def save(self, path=WEIGHTS):
        _check(_sig().gbfmm_mlp_save(self._h, path.encode()))

    def propose(self, feat, tol, margin=1.5):
        """(order, depth, precision, predicted error, predicted ms) or None."""
        f = _f(feat)
        o, d, p = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        pe, pm = ctypes.c_float(), ctypes.c_float()
        rc = _sig().gbfmm_tuner_propose(self._h, f.ctypes.data_as(_fp), float(tol), float(margin), ctypes.byref(o),
                                        ctypes.byref(d), ctypes.byref(p), ctypes.byref(pe), ctypes.byref(pm))
        if rc == 6:
            return None
        _check(rc)
        return o.value, d.value, p.value, pe.value, pm.value


def fit(x, t, n_hidden=64, epochs=400, batch=128, lr=2e-3, seed=0):
    """Normalises the tuples and trains a fresh network on the GPU."""
    x = _f(x)
    t = _f(t)
    m = Mlp(x.shape[1], n_hidden, t.shape[1], seed=seed)
    xm, xs = x.mean(0), x.std(0)
    xs[xs < 1e-6] = 1.0
    ym, ys = t.mean(0), t.std(0)
    ys[ys < 1e-6] = 1.0
    m.set_normalization(xm, xs, ym, ys)
    loss = m.train(x, t, epochs=epochs, batch=batch, lr=lr, seed=seed + 1)
    return m, loss


def plain_depth(natoms):
    """Depth of the plain FMM: about 16-128 bodies per leaf, as the reference's
    fixed depth gives for its systems (gbfmm_plain_depth)."""
    return int(_sig().gbfmm_plain_depth(int(natoms)))


class TunedSolver:
    """Solves a system with the MLP-proposed parameters, checked against the
    plain fixed-parameter FMM (check and fallback) whenever a proposal is made."""

    def __init__(self, charges, mlp, tol=1e-3, margin=1.5, images=4):
        self.q = _f(charges)
        self.n = len(self.q)
        self.mlp, self.tol, self.margin, self.images = mlp, tol, margin, images
        self.solver = None
        self.choice = None
        self.checks = []

    def _plain(self, box=None):
        slab = box is not None and np.size(box) == 3 and float(np.ravel(box)[2]) != float(np.ravel(box)[0])
        return _pkg.ZetaFmmSolver(self.n, self.q, order=PLAIN_ORDER, max_depth=plain_depth(4 * self.n if slab else self.n),
                                  images=self.images, aspect_z=2 if slab else 1)

    def propose(self, coords, box):
        """Computes statistics, proposes, and checks the proposal against the
        plain FMM on this configuration (gbfmm_tuner_choose).  Returns the
        accepted choice; self.solver holds a solver of that choice with this
        configuration's results."""
        x = _f(coords).reshape(-1)
        m = _pkg.box_matrix(box)
        c = TunerChoice()
        _check(_sig().gbfmm_tuner_choose(self.mlp._h, self.n, self.q.ctypes.data_as(_fp), x.ctypes.data_as(_fp),
                                         m.ctypes.data_as(_fp), self.images, float(self.tol), float(self.margin),
                                         ctypes.byref(c)))
        if c.proposed_order == 0:
            self.checks.append({"proposal": None, "accepted": False})
        else:
            prop = (c.proposed_order, c.proposed_depth, c.proposed_precision, c.pred_rel_force_err, c.pred_ms)
            for k in range(c.nchecks):
                self.checks.append({"proposal": prop if k == 0 else (c.check_order[k], prop[1], prop[2]),
                                    "diff_vs_plain": c.check_diff[k],
                                    "accepted": not c.fallback and c.check_order[k] == c.order})
        self.choice = (c.order, c.depth, c.precision)
        self.solver = _pkg.ZetaFmmSolver(self.n, self.q, order=c.order, max_depth=c.depth, images=self.images,
                                         precision=c.precision, aspect_z=2 if m[8] != m[0] else 1)
        self.solver.execute(coords, box)
        return self.choice

    def execute(self, coords, box):
        if self.solver is None:
            self.propose(coords, box)
        self.solver.execute(coords, box)
        return self.solver.forces()
