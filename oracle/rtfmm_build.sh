#!/usr/bin/env bash
# Builds oracle/_ref/librtfmmref.so: the reference's own CPU FMM (the
# kernel-independent FMM of src/gromacs/rtfmm), compiled from its unmodified
# sources where the reference checkout is present, with
#   - oracle/rtfmm_shim/fftw3.h + oracle/rtfmm_fftw.cpp for the FFTW calls,
#   - oracle/rtfmm_shim/cblas.h and the OpenBLAS that scipy bundles for BLAS and
#     dgesvd_,
#   - the tree depth literal of fmm.cpp:21 replaced by a call (fmm.cpp is piped
#     through sed to the compiler: no copy of the source is written),
#   - oracle/rtfmm_driver.cpp.
# The sources use AVX intrinsics: x86-64 hosts only.  Outputs stay out of git.
set -euo pipefail
REF=${GB_FMM_REFERENCE:-/root/reference}
SRC="$REF/src/gromacs/rtfmm"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$SRC/fmm.cpp" ]; then
    echo "reference sources not found at $SRC; skipping oracle/_ref/librtfmmref.so" >&2
    exit 0
fi
if [ "$(uname -m)" != "x86_64" ]; then
    echo "the reference CPU FMM uses x86 AVX intrinsics; skipping on $(uname -m)" >&2
    exit 0
fi
BLASDIR=$(python3 -c "import os, scipy; d = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), 'scipy.libs'); print(d)")
BLAS=$(ls "$BLASDIR"/libscipy_openblas-*.so | head -1)
CUDA_INC=${CUDA_HOME:-/usr/local/cuda}/include
OUT="$HERE/_ref"
mkdir -p "$OUT/rtfmm_obj"
FLAGS=(-std=c++17 -O3 -fopenmp -mavx2 -mfma -fPIC -w -DNDEBUG -I"$HERE/rtfmm_shim" -I"$CUDA_INC" -I"$SRC")
objs=()
for f in argument body tree traverser kernel mathfunc surface; do
    g++ "${FLAGS[@]}" -c "$SRC/$f.cpp" -o "$OUT/rtfmm_obj/$f.o" &
    objs+=("$OUT/rtfmm_obj/$f.o")
done
sed 's/args\.r, 3, Tree::TreeType::uniform/args.r, rtfmm_depth(), Tree::TreeType::uniform/' "$SRC/fmm.cpp" |
    g++ "${FLAGS[@]}" -x c++ -include "$HERE/rtfmm_shim/depth.h" -c - -o "$OUT/rtfmm_obj/fmm.o" &
objs+=("$OUT/rtfmm_obj/fmm.o")
g++ "${FLAGS[@]}" -c "$HERE/rtfmm_fftw.cpp" -o "$OUT/rtfmm_obj/fftw.o" &
objs+=("$OUT/rtfmm_obj/fftw.o")
g++ "${FLAGS[@]}" -c "$HERE/rtfmm_driver.cpp" -o "$OUT/rtfmm_obj/driver.o" &
objs+=("$OUT/rtfmm_obj/driver.o")
g++ "${FLAGS[@]}" -c "$HERE/rtfmm_lapack.cpp" -o "$OUT/rtfmm_obj/lapack.o" &
objs+=("$OUT/rtfmm_obj/lapack.o")
wait
g++ -shared -fopenmp -o "$OUT/librtfmmref.so" "${objs[@]}" "$BLAS" -Wl,-rpath,"$BLASDIR"
echo "built $OUT/librtfmmref.so"
