#!/bin/bash
# Builds the reference's BRMerge path unmodified from its own sources into
# oracle/_ref/libbrm_ref.so (git-ignored).  Needs the reference tree; the
# default location is /root/reference (override with BRM_REFERENCE_DIR).
# Only spgemm.h (header-only kernels), src/Timings.cpp and src/CSR.cpp (the
# MatrixMarket reader) are compiled; two
# small shims in oracle/ref_shim replace TBB malloc and the x86 TSC timer.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${BRM_REFERENCE_DIR:-/root/reference}/BRMerge-SpGEMM"
if [ ! -f "$REF/inc/spgemm.h" ]; then
  echo "reference sources not found at $REF; skipping" >&2
  exit 3
fi
mkdir -p "$HERE/_ref"
g++ -O2 -fopenmp -std=c++17 -DTBB -ffp-contract=off -fPIC -shared \
    -include "$HERE/ref_shim/prelude.h" -I "$HERE/ref_shim" -I "$REF/inc" \
    "$HERE/ref_wrap.cpp" "$REF/src/Timings.cpp" "$REF/src/CSR.cpp" -o "$HERE/_ref/libbrm_ref.so.tmp"
mv "$HERE/_ref/libbrm_ref.so.tmp" "$HERE/_ref/libbrm_ref.so"
echo "built $HERE/_ref/libbrm_ref.so"
