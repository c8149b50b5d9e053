#!/bin/bash
# Builds oracle/_ref/libref_host.so from the reference's own sources, in place
# (read-only) -- TEST INFRASTRUCTURE ONLY.  Skips quietly when the reference
# tree is absent (e.g. on a machine that only runs the GPU tests).
set -e
REF=${GBSP_REFERENCE_DIR:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/sparse_fft_bluestein.cu" ]; then
    echo "reference sources not found at $REF; oracle/_ref not built" >&2
    exit 0
fi
mkdir -p "$OUT"
NVCC=${NVCC:-nvcc}
"$NVCC" -std=c++17 -O2 -shared -Xcompiler -fPIC --expt-relaxed-constexpr -w \
    -gencode arch=compute_103a,code=sm_103a \
    -I"$REF/include" -I"$REF/src" \
    "$HERE/ref_shim.cu" -o "$OUT/libref_host.so.tmp" -lcufft -lcublas
mv "$OUT/libref_host.so.tmp" "$OUT/libref_host.so"
echo "built $OUT/libref_host.so" >&2
