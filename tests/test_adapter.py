"""The GROMACS-side drop-in (gromacs-fmm_gb300/adapter/gbfmm_solver.h): a
coulomb_solver::BaseSolver subclass over the C ABI.  It is compiled against
stand-ins of the few GROMACS types it uses (tests/adapter/gromacs/) and driven
by tests/adapter/mdrun_steps.cpp the way mdrun drives a solver: construct, then
per step set_parameter, execute, add_force into the step's force buffer and
get_energy."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_rms

DRIVER = os.path.join(ROOT, "tests", "adapter", "mdrun_steps.cpp")
FLAGS = ["-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
         "-I", os.path.join(ROOT, "gromacs-fmm_gb300", "adapter"), "-I", os.path.join(ROOT, "tests", "adapter")]


def _gxx():
    g = shutil.which("g++")
    if not g:
        pytest.skip("no g++")
    return g


def test_adapter_compiles_against_the_base_solver_interface():
    subprocess.run([_gxx(), "-fsyntax-only", *FLAGS, DRIVER], check=True)


def _run_driver(pkg, tmp_path, xyz, q, L, args):
    lib_dir = os.path.dirname(pkg.LIB_PATH)
    exe = str(tmp_path / "mdrun_steps")
    subprocess.run([_gxx(), *FLAGS, DRIVER, "-L", lib_dir, "-lgbfmm", f"-Wl,-rpath,{lib_dir}", "-o", exe],
                   check=True)
    rng = np.random.default_rng(5)
    steps = [xyz, np.mod(xyz + rng.normal(0, 0.01, xyz.shape), L).astype(np.float32)]
    n = len(q)
    with open(tmp_path / "in.bin", "wb") as f:
        np.array([n, len(steps)], np.int32).tofile(f)
        np.array([L, 0, 0, 0, L, 0, 0, 0, L], np.float32).tofile(f)
        q.astype(np.float32).tofile(f)
        for x in steps:
            x.astype(np.float32).tofile(f)
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), *[str(a) for a in args]],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "L2f = 0.00000000" in r.stdout
    raw = (tmp_path / "out.bin").read_bytes()
    rec = 12 * n + 8 + 72
    assert len(raw) == rec * len(steps)
    out = []
    for k, x in enumerate(steps):
        f = np.frombuffer(raw[k * rec:k * rec + 12 * n], np.float32).reshape(n, 3) - 1.0  # added to ones
        e = np.frombuffer(raw[k * rec + 12 * n:k * rec + 12 * n + 8], np.float64)[0]
        v = np.frombuffer(raw[k * rec + 12 * n + 8:(k + 1) * rec], np.float64).reshape(3, 3)
        out.append((x, f, e, v))
    return out, r.stdout


@pytest.mark.gpu
def test_adapter_steps_match_the_oracle(pkg, oracle, systems, tmp_path):
    xyz, q, box = systems.water_ion_box(1500, 3.0, n_na=4, n_cl=4, seed=41)
    L = float(box[0])
    P, D, images = 8, 2, 4
    steps, _ = _run_driver(pkg, tmp_path, xyz, q, L, [P, D, images])
    for x, f, e, v in steps:
        po, fo, eo = oracle.zeta_solve(x.astype(np.float64), q.astype(np.float64), L, P, D, images)
        assert rel_rms(f, fo) < 1e-5
        assert abs(e - eo) / abs(eo) < 1e-6
        # the virial the adapter adds to ForceWithVirial, against the FP64 Ewald virial
        _, ve = oracle.ewald_virial(x.astype(np.float64), q.astype(np.float64), np.full(3, L), eps=1e-10)
        assert np.linalg.norm(v - ve) / np.linalg.norm(ve) < 5e-3


@pytest.mark.gpu
def test_adapter_with_the_learned_tuner(pkg, oracle, systems, tmp_path):
    """Given a force tolerance instead of fixed parameters, the adapter takes the
    tuner's checked choice (gbfmm_tuner_choose) at the first step; both steps stay
    within the tolerance of the plain order-10 FMM."""
    tuner = pytest.importorskip("gromacs_fmm_gb300.tuner")
    xyz, q, box = systems.water_ion_box(16000, 8.0, n_na=12, n_cl=12, seed=43)
    L = float(box[0])
    tol = 1e-3
    steps, out = _run_driver(pkg, tmp_path, xyz, q, L, [0, 0, 4, tol, tuner.WEIGHTS])
    line = [ln for ln in out.splitlines() if ln.startswith("choice ")][0]
    order, depth, prec, fallback = (int(v) for v in line.split()[1:])
    assert 4 <= order <= 10 and 1 <= depth <= 7 and prec in (0, 1, 2)
    D0 = tuner.plain_depth(len(q))
    for x, f, e, _ in steps:
        _, fo, eo = oracle.zeta_solve(x.astype(np.float64), q.astype(np.float64), L, 10, D0, 4)
        assert rel_rms(f, fo) < tol
        assert abs(e - eo) / abs(eo) < tol
