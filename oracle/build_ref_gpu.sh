#!/usr/bin/env bash
# Compiles the reference's standard-filter GPU source, read in place under the
# reference checkout, into a device-only cubin for sm_103a -- test
# infrastructure only, never part of the product.  The tests load it through
# the CUDA driver API and run the reference's own kernels, with the host-side
# steps of each reference entry point restated in oracle/ref_gpu.py.
#   REF   reference checkout (default: the checkout this recipe was written for)
# Output:
#   _ref/ref_sqf_gpu.cubin
# The source is compiled unmodified.  ref_gpu_shim/ supplies what CUDA 13
# lacks: the toolkit's CUB in place of the vendored CUB 1.7.4 (pre.cuh), and a
# parse-only stand-in for the un-vendored moderngpu header.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${REF:-/root/reference}"
OUT="$HERE/_ref"
SRC="$REF/standardQuotientFilter/GPU_version/quotientFilter.cu"
if [ ! -f "$SRC" ]; then
  echo "build_ref_gpu: reference sources not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT"
# The reference includes "../../moderngpu/src/moderngpu/kernel_merge.hxx"
# relative to its own folder, where the file is absent; the preprocessor then
# tries the -I folders with the same relative path, so an -I folder two levels
# below the shim root resolves it to ref_gpu_shim/moderngpu/...
INC="$OUT/shim_inc/a/b"
mkdir -p "$INC" "$OUT/shim_inc/moderngpu/src/moderngpu"
cp "$HERE/ref_gpu_shim/moderngpu/src/moderngpu/kernel_merge.hxx" \
   "$OUT/shim_inc/moderngpu/src/moderngpu/kernel_merge.hxx"
NVCC="${NVCC:-nvcc}"
$NVCC -gencode arch=compute_103a,code=sm_103a -cubin -O3 -w \
  -I "$INC" -include "$HERE/ref_gpu_shim/pre.cuh" \
  -o "$OUT/ref_sqf_gpu.cubin.tmp" "$SRC"
mv "$OUT/ref_sqf_gpu.cubin.tmp" "$OUT/ref_sqf_gpu.cubin"
rm -rf "$OUT/shim_inc"
echo "build_ref_gpu: ok -> $OUT/ref_sqf_gpu.cubin"
