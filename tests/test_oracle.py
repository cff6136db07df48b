"""The oracle pinned against the reference: tree and lists against fixtures made
by the reference's own tree.cpp/traverser.cpp, potentials and forces against the
outputs of the reference's own FP64 kernels (kernel.cu, run on the host), and the
operators against physics (FP64 Ewald and direct lattice sums)."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden, rel_rms


def _digest(t, s, o):
    h = hashlib.sha256()
    for a in (t, s, o):
        h.update(np.ascontiguousarray(a, dtype="<i4").tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name,depth", [("tree_water9k_d3.npz", 3), ("tree_edges_d1.npz", 1),
                                        ("tree_edges_d2.npz", 2), ("tree_edges_d3.npz", 3)])
def test_oracle_tree_matches_reference(oracle, name, depth):
    g = golden(name)
    T = oracle.zeta_tree(g["xyz"].astype(np.float64), float(g["box"]), depth)
    assert np.array_equal(T["order"], g["order"])
    leaf = T["depth"] == depth
    assert np.array_equal(T["body_num"][leaf], g["leaf_count"])


def test_oracle_tree_matches_reference_96k_depth4(oracle):
    """The 95,600-atom box of the benchmark at depth 4 (4,096 leaves): leaf counts
    and the SHA-256 of the body order of the reference's tree.cpp."""
    g = golden("tree_water96k_d4.npz")
    T = oracle.zeta_tree(g["xyz"].astype(np.float64), float(g["box"]), 4)
    order = np.ascontiguousarray(T["order"], dtype="<i4")
    assert hashlib.sha256(order.tobytes()).digest() == g["order_sha256"].tobytes()
    leaf = T["depth"] == 4
    assert np.array_equal(T["body_num"][leaf], g["leaf_count"])


@pytest.mark.parametrize("depth", [1, 2])
@pytest.mark.parametrize("images", [0, 1, 2, 4])
def test_oracle_lists_match_reference(oracle, depth, images):
    g = golden("lists_small.npz")
    L = oracle.zeta_lists(depth, images, cycle=4.5)
    for k in ("p2p", "m2l"):
        t, s, o = L[k]
        assert np.array_equal(t, g[f"{k}_d{depth}_i{images}_tgt"])
        assert np.array_equal(s, g[f"{k}_d{depth}_i{images}_src"])
        assert np.array_equal(np.rint(o / 4.5).astype(np.int32), g[f"{k}_d{depth}_i{images}_off"])


def test_oracle_lists_hash_matches_reference(oracle):
    with open(os.path.join(GOLDEN, "lists_hash.json")) as f:
        ref = json.load(f)
    for key, v in ref.items():
        kind, d, i = key.split("_")
        L = oracle.zeta_lists(int(d[1:]), int(i[1:]), cycle=9.86)
        t, s, o = L[kind]
        assert len(t) == v["count"], key
        assert _digest(t, s, np.rint(o / 9.86).astype(np.int32)) == v["sha256"], key


def test_ewald_matches_direct_lattice_sum(oracle):
    rng = np.random.default_rng(3)
    L = 2.0
    x = rng.uniform(0, L, (8, 3))
    q = np.array([1.0, -1.0] * 4)
    _, fd = oracle.direct(x, q, L, 24)
    _, fe, _ = oracle.ewald(x, q, L, eps=1e-12)
    # the shell sum converges slowly; forces agree to ~1e-6
    assert rel_rms(fd, fe) < 5e-6


def test_ewald_accuracy_parameter_is_consistent(oracle, systems):
    xyz, q, box = systems.water_ion_box(500, 1.75, seed=3)
    x = xyz.astype(np.float64)
    tg = np.arange(0, len(q), 5)
    _, f1, _ = oracle.ewald(x, q, box[0], eps=1e-8, targets=tg)
    _, f2, _ = oracle.ewald(x, q, box[0], eps=1e-12, targets=tg)
    assert rel_rms(f1, f2) < 1e-7


def test_zeta_oracle_converges_to_ewald(oracle, systems):
    xyz, q, box = systems.water_ion_box(1000, 2.2, n_na=4, n_cl=4, seed=9)
    x = xyz.astype(np.float64)
    q = q.astype(np.float64)
    _, fe, ee = oracle.ewald(x, q, box[0], eps=1e-11, energy=True)
    errs = []
    for P in (4, 6, 8, 10):
        _, f, e = oracle.zeta_solve(x, q, float(box[0]), P, 2, 4)
        errs.append(rel_rms(f, fe))
    assert all(errs[i + 1] < errs[i] for i in range(len(errs) - 1)), errs
    assert errs[-1] < 2e-4
    _, _, e10 = oracle.zeta_solve(x, q, float(box[0]), 12, 2, 4)
    assert abs(e10 - ee) / abs(ee) < 1e-5


def test_zeta_oracle_near_and_far_split(oracle, systems):
    """Stage masks: near (P2P) + far (multipole) + dipole add up to the full solve."""
    xyz, q, box = systems.water_ion_box(300, 1.6, seed=2)
    x = xyz.astype(np.float64)
    q = q.astype(np.float64)
    p_all, f_all, _ = oracle.zeta_solve(x, q, float(box[0]), 6, 2, 4, stages=7)
    p1, f1, _ = oracle.zeta_solve(x, q, float(box[0]), 6, 2, 4, stages=1)
    p2, f2, _ = oracle.zeta_solve(x, q, float(box[0]), 6, 2, 4, stages=2)
    p4, f4, _ = oracle.zeta_solve(x, q, float(box[0]), 6, 2, 4, stages=4)
    assert np.allclose(f1 + f2 + f4, f_all, rtol=1e-12, atol=1e-9)


def ref_cases():
    g = golden("ref_outputs.npz")
    k = 0
    while f"case{k}_params" in g:
        yield k, g
        k += 1


def ref_case_inputs(systems, g, k):
    ns, L, ions, P, D, im = g[f"case{k}_params"]
    xyz, q, box = systems.water_ion_box(int(ns), float(L), n_na=int(ions), n_cl=int(ions), seed=int(ns) + int(P))
    assert hashlib.sha256(xyz.tobytes()).digest() == g[f"case{k}_xyz_sha256"].tobytes(), "input generator drifted"
    return xyz, q, float(L), int(P), int(D), int(im)


def test_oracle_equals_reference_kernels(oracle, systems):
    """FP64 potentials and forces of the oracle's restatement equal those of the
    reference's own kernels (before the dipole correction) to rounding."""
    n_cases = 0
    for k, g in ref_cases():
        xyz, q, L, P, D, im = ref_case_inputs(systems, g, k)
        pot, force, _ = oracle.zeta_solve(xyz.astype(np.float64), q.astype(np.float64), L, P, D, im, stages=3)
        idx = g[f"case{k}_idx"]
        assert rel_rms(pot[idx], g[f"case{k}_pot"]) < 1e-12
        assert rel_rms(force[idx], g[f"case{k}_force"]) < 1e-12
        n_cases += 1
    assert n_cases == 5


def test_reference_kernels_reproduce_their_fixture(oracle, systems):
    """Where the reference is built, its kernels reproduce the committed fixture."""
    if not oracle.ref_available():
        pytest.skip("reference library not built")
    for k, g in ref_cases():
        xyz, q, L, P, D, im = ref_case_inputs(systems, g, k)
        pot, force = oracle.ref_solve(xyz.astype(np.float64), q.astype(np.float64), L, P, D, im)
        idx = g[f"case{k}_idx"]
        assert np.array_equal(pot[idx], g[f"case{k}_pot"])
        assert np.array_equal(force[idx], g[f"case{k}_force"])
        break



def test_oracle_slab_converges_to_rectangular_ewald(oracle, systems):
    """A half-vacuum slab a x a x 2a: the four-copy periodic cube of edge 2a has
    the slab's periodic charge density, so the solver on it converges with the
    order to the FP64 Ewald sum of the rectangular box."""
    a = 2.6
    xyz, q, _ = systems.water_ion_box(500, [a, a, 2 * a], n_na=2, n_cl=2, seed=91, fill_z=0.5)
    x64, q64 = xyz.astype(np.float64), q.astype(np.float64)
    a32 = float(np.float32(a))
    _, fe, _ = oracle.ewald(x64, q64, np.array([a32, a32, 2 * a32]), eps=1e-10)
    _, _, ee = oracle.ewald(x64, q64, np.array([a32, a32, 2 * a32]), eps=1e-9, energy=True)
    errs = []
    for P in (4, 8):
        _, fo, eo = oracle.zeta_solve_slab(x64, q64, a32, P, 2, 4)
        errs.append(rel_rms(fo, fe))
        assert abs(eo - ee) / abs(ee) < 1e-4
    assert errs[1] < 0.2 * errs[0] and errs[1] < 5e-4


def test_reference_cpu_fmm_converges_to_ewald(oracle, systems):
    """The reference's own CPU FMM (src/gromacs/rtfmm, built unmodified by
    oracle/rtfmm_build.sh with the FFTW-subset and BLAS shims) on the 9,000-atom
    box: its forces agree with the FP64 Ewald sum (P = 10 surface points, depth
    3, images 4), and with this FP64 restatement of the GPU solver's algorithm.
    It builds only on an x86-64 host with the reference checkout."""
    if not oracle.rtfmm_available():
        pytest.skip("reference CPU FMM not built on this host")
    xyz, q, box = systems.cfg_small()
    L = float(box[0])
    x64, q64 = xyz.astype(np.float64), q.astype(np.float64)
    p, f = oracle.rtfmm_solve(x64, q64, L, 10, 3, 4)
    tg = np.arange(0, len(q), 7)
    _, fe, _ = oracle.ewald(x64, q64, L, eps=1e-10, targets=tg)
    assert rel_rms(f[tg], fe) < 1e-5
    _, fo, _ = oracle.zeta_solve(x64, q64, L, 10, 3, 4)
    assert rel_rms(fo, f) < 1e-4
