#!/usr/bin/env bash
# Builds oracle/_ref/libzetaref.so from the reference's own, unmodified zeta_fmm
# sources: tree.cpp and traverser.cpp, and the FP64 kernels of kernel.cu (the part
# before GPUKernel::GPUKernel(), piped to the compiler as host code through
# oracle/ref_cuda_shim.h, so that no copy of the source is written), plus
# oracle/ref_driver.cpp and oracle/ref_kernels_driver.cpp.  Runs only where the
# reference checkout is present; the outputs stay out of git (oracle/_ref/).
set -euo pipefail
REF=${GB_FMM_REFERENCE:-/root/reference}
SRC="$REF/src/gromacs/zeta_fmm"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$SRC/tree.cpp" ]; then
    echo "reference sources not found at $SRC; skipping oracle/_ref" >&2
    exit 0
fi
CUDA_INC=${CUDA_HOME:-/usr/local/cuda}/include
mkdir -p "$HERE/_ref"
FLAGS=(-std=c++17 -O2 -fPIC -w -I"$CUDA_INC" -I"$SRC")
last=$(grep -n "zeta_fmm::GPUKernel::GPUKernel()" "$SRC/kernel.cu" | cut -d: -f1)
sed -n "1,$((last - 1))p" "$SRC/kernel.cu" |
    g++ "${FLAGS[@]}" -x c++ -include "$HERE/ref_cuda_shim.h" -c - -o "$HERE/_ref/ref_kernels.o"
g++ "${FLAGS[@]}" -shared \
    "$SRC/tree.cpp" "$SRC/traverser.cpp" "$HERE/ref_driver.cpp" "$HERE/ref_kernels_driver.cpp" \
    "$HERE/_ref/ref_kernels.o" -o "$HERE/_ref/libzetaref.so"
echo "built $HERE/_ref/libzetaref.so"
