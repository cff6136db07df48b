#!/usr/bin/env bash
# Builds oracle/_ref/libzetaref.so from the reference's own, unmodified zeta_fmm
# tree and traverser sources plus oracle/ref_driver.cpp.  Runs only where the
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
g++ -std=c++17 -O2 -fPIC -shared -w -I"$CUDA_INC" -I"$SRC" \
    "$SRC/tree.cpp" "$SRC/traverser.cpp" "$HERE/ref_driver.cpp" \
    -o "$HERE/_ref/libzetaref.so"
echo "built $HERE/_ref/libzetaref.so"
