#!/bin/bash
# Builds, from the reference's own sources in place (read-only) -- TEST
# INFRASTRUCTURE ONLY:
#   oracle/_ref/libref_host.so     the reference's host functions (this
#                                  machine's CPU architecture), via ref_shim.cu
#   oracle/_ref/ref_kernels.fatbin the reference's GPU kernels for sm_103a
#                                  (device code only, so it runs on a GPU host
#                                  of any CPU architecture; launched by
#                                  oracle/ref_gpu_driver.cpp)
#   oracle/_ref/REFERENCE_DIR      where the sources were read from
# The reference tree is taken from GBSP_REFERENCE_DIR, else the path this
# recipe was written for; without it nothing is built.
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
COMMON=(-std=c++17 -O3 --expt-relaxed-constexpr -w -gencode arch=compute_103a,code=sm_103a
        -I"$REF/include" -I"$REF/src")
"$NVCC" "${COMMON[@]}" -shared -Xcompiler -fPIC \
    "$HERE/ref_shim.cu" -o "$OUT/libref_host.so.tmp" -lcufft -lcublas
mv "$OUT/libref_host.so.tmp" "$OUT/libref_host.so"
"$NVCC" "${COMMON[@]}" -fatbin "$HERE/ref_shim.cu" -o "$OUT/ref_kernels.fatbin.tmp"
mv "$OUT/ref_kernels.fatbin.tmp" "$OUT/ref_kernels.fatbin"
echo "$REF" > "$OUT/REFERENCE_DIR"
echo "built $OUT/libref_host.so and $OUT/ref_kernels.fatbin" >&2
