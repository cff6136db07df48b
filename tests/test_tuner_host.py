"""Tuner host side without a GPU: the FP64 MLP restatement against finite
differences, the candidate encoding of the C ABI, the shipped weights file
(format and FNV-1a checksum) and the committed training tuples."""
import ctypes
import os
import struct

import numpy as np
import pytest

from conftest import GOLDEN, G
from oracle import mlp64

WEIGHTS = os.path.join(G.PKG_DIR, "tuner_weights.bin")
TUPLES = os.path.join(GOLDEN, "tuner_tuples.npz")


def test_mlp64_gradient_matches_finite_differences():
    I, H, O, B = 7, 5, 2, 6
    rng = np.random.default_rng(0)
    npar = H * I + H + H * H + H + O * H + O
    p = rng.normal(0, 0.5, npar)
    x = rng.normal(size=(B, I))
    t = rng.normal(size=(B, O))
    _, g = mlp64.loss_grad(p, x, t, I, H, O)
    h = 1e-6
    for k in range(npar):
        e = np.zeros(npar)
        e[k] = h
        fd = (mlp64.loss_grad(p + e, x, t, I, H, O)[0] - mlp64.loss_grad(p - e, x, t, I, H, O)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-7 * max(1.0, abs(fd))
    # the forward pass is the loss's prediction
    y = mlp64.forward(p, x, I, H, O)
    assert np.isclose(np.sum((y - t) ** 2) / B, mlp64.loss_grad(p, x, t, I, H, O)[0])


def test_candidate_encoding(pkg):
    tuner = G.load_module("tuner")
    feat = np.arange(tuner.NFEAT, dtype=np.float32) * 0.01
    feat[0] = np.log10(95600)
    feat[56] = 0.0  # a cube
    for prec, bits in [(0, 1.0), (1, 16 / 24), (2, 8 / 24)]:
        r = tuner.tuner_input(feat, 7, 4, prec)
        assert np.array_equal(r[:tuner.NFEAT], feat)
        assert np.isclose(r[tuner.NFEAT], 0.7)
        assert np.isclose(r[tuner.NFEAT + 1], 4 / 6)
        assert np.isclose(r[tuner.NFEAT + 2], bits)
        assert np.isclose(r[tuner.NFEAT + 3], np.log2(95600 / 8 ** 4) / 5, rtol=1e-5)
    # a slab (statistic 56 = 1) stores a quarter of the root cube's leaves
    feat[56] = 1.0
    r = tuner.tuner_input(feat, 7, 4, 1)
    assert np.isclose(r[tuner.NFEAT + 3], np.log2(95600 / (8 ** 4 / 4)) / 5, rtol=1e-5)
    with pytest.raises(pkg.FmmError):
        tuner.tuner_input(feat, 7, 4, 3)


def _fnv1a(data, h=1469598103934665603):
    for c in data:
        h ^= c
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def test_weights_file_format_and_checksum():
    raw = open(WEIGHTS, "rb").read()
    assert raw[:8] == b"GBFMMMLP"
    ver, I, H, O = struct.unpack("<4i", raw[8:24])
    assert (ver, I, O) == (1, 61, 2) and 8 <= H <= 256
    npar = H * I + H + H * H + H + O * H + O
    body = raw[24:24 + 4 * (npar + 2 * I + 2 * O)]
    assert len(raw) == 24 + len(body) + 8
    (h_file,) = struct.unpack("<Q", raw[-8:])
    assert _fnv1a(raw[8:24] + body) == h_file
    p = np.frombuffer(body, np.float32)
    assert np.all(np.isfinite(p))
    xs = p[npar + I:npar + 2 * I]
    assert np.all(xs > 0)


def test_training_tuples():
    d = np.load(TUPLES)
    n = len(d["order"])
    assert n >= 2000
    assert d["natoms"].max() >= 500000  # sizes up to about a million atoms
    assert np.all(np.isfinite(d["err"])) and np.all(d["err"] > 0)
    assert np.all(np.isfinite(d["ms"])) and np.all(d["ms"] > 0)
    assert d["feat"].shape == (n, 57)
    slab = d["feat"][:, 56] > 0.5
    assert slab.any() and (~slab).any()  # both box shapes
    # within one system, depth and precision: the error falls with the order
    falls = total = 0
    for k in np.unique(d["system"]):
        for D in np.unique(d["depth"][d["system"] == k]):
            for prec in (1, 2):
                sel = (d["system"] == k) & (d["depth"] == D) & (d["precision"] == prec)
                e = d["err"][sel][np.argsort(d["order"][sel])]
                falls += int(e[-1] < e[0])
                total += 1
    assert falls == total


def test_plain_depth_rule(pkg):
    """gbfmm_plain_depth: the deepest level with at least 16 bodies per leaf
    (depths 1-7), the reference-like fixed depth the checked choice falls back to."""
    lib = pkg.lib()
    lib.gbfmm_plain_depth.restype = ctypes.c_int
    lib.gbfmm_plain_depth.argtypes = [ctypes.c_int]
    for n in (10, 300, 1023, 1024, 9000, 95600, 250002, 1002002, 2 ** 31 - 1):
        d = lib.gbfmm_plain_depth(n)
        want = 1
        while n / 8.0 ** (want + 1) >= 16 and want < 7:
            want += 1
        assert d == want, n
        if 1 < d < 7:
            assert 16 <= n / 8.0 ** d < 128, n


def test_tuner_choose_rejects_bad_arguments_before_device_use(pkg):
    tuner = G.load_module("tuner")
    f = tuner._sig().gbfmm_tuner_choose
    q = np.ones(4, np.float32)
    x = np.zeros(12, np.float32)
    box = np.eye(3, dtype=np.float32).reshape(-1) * 2
    fp = ctypes.POINTER(ctypes.c_float)
    out = tuner.TunerChoice()
    args = [q.ctypes.data_as(fp), x.ctypes.data_as(fp), box.ctypes.data_as(fp)]
    assert f(None, 4, *args, 4, 1e-3, 1.5, ctypes.byref(out)) == 1   # no network
    assert f(None, 0, *args, 4, 1e-3, 1.5, ctypes.byref(out)) == 1   # no atoms
    assert f(None, 4, *args, 4, 1e-3, 1.5, None) == 1                # no output
