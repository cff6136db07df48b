"""Build recipe for the oracle's C restatement (TEST INFRASTRUCTURE ONLY).

Compiles oracle/zeta64.c and oracle/ewald64.c into oracle/lib/liboracle.so with
OpenMP.  Portable C: no architecture flags, so the same recipe builds on x86_64
and aarch64.  ``build(ref=True)`` additionally runs oracle/ref_build.sh, which
compiles the reference's own tree/traverser sources when the reference checkout
is present (it is absent on GPU machines; the recipe then does nothing), and
oracle/rtfmm_build.sh, which builds the reference's own CPU FMM there (x86-64).
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "lib", "liboracle.so")
SRCS = [os.path.join(HERE, "zeta64.c"), os.path.join(HERE, "ewald64.c")]


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    with open(out, "rb") as f:
        hdr = f.read(20)
    if want is not None and (len(hdr) < 20 or int.from_bytes(hdr[18:20], "little") != want):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(ref=False, force=False):
    os.makedirs(os.path.join(HERE, "lib"), exist_ok=True)
    deps = SRCS + [os.path.join(HERE, "zeta64.h")]
    if force or _stale(LIB, deps):
        cmd = ["gcc", "-O2", "-std=c11", "-D_DEFAULT_SOURCE", "-fPIC", "-shared", "-fopenmp",
               "-o", LIB] + SRCS + ["-lm"]
        subprocess.run(cmd, check=True)
    if ref:
        subprocess.run(["bash", os.path.join(HERE, "ref_build.sh")], check=True)
        rt = os.path.join(HERE, "_ref", "librtfmmref.so")
        deps = [os.path.join(HERE, f) for f in ("rtfmm_build.sh", "rtfmm_driver.cpp", "rtfmm_fftw.cpp",
                                                 "rtfmm_lapack.cpp")]
        if force or not os.path.exists(rt) or any(os.path.getmtime(d) > os.path.getmtime(rt) for d in deps):
            subprocess.run(["bash", os.path.join(HERE, "rtfmm_build.sh")], check=True)
    return LIB


if __name__ == "__main__":
    build(ref=True, force=True)
    print(LIB)
