#!/usr/bin/env bash
# Compiles the reference's CPU code from its own sources (read in place under
# the reference checkout) into oracle/_ref/ -- test infrastructure only; never
# part of the product.  Nothing here runs the reference's build system.
#   REF   reference checkout (default: the checkout this recipe was written for)
# Outputs:
#   _ref/libref_sqf_fnv.so   SQF CPU_version as shipped (FNV hash)
#   _ref/libref_sqf_ap.so    SQF CPU_version with fnv_hash made weak and
#                            resolved to the reference's Normal_APHash
#   _ref/libref_rsqf.so      RSQF CPU_version + mt19937ar
#   _ref/libref_rsqf8.so     the same with RBITS 8
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${REF:-/root/reference}"
OUT="$HERE/_ref"
SQF="$REF/standardQuotientFilter/CPU_version"
RSQF="$REF/rankSelectQuotientFilter/CPU_version"
if [ ! -f "$SQF/quotientFilter.cpp" ]; then
  echo "build_ref: reference sources not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS="-O2 -fPIC -w"
$CXX $FLAGS -c "$SQF/quotientFilter.cpp" -o "$OUT/sqf_cpu.o"
$CXX $FLAGS -I"$SQF" -c "$HERE/ref_shim_sqf.cpp" -o "$OUT/ref_shim_sqf.o"
$CXX -shared -o "$OUT/libref_sqf_fnv.so" "$OUT/sqf_cpu.o" "$OUT/ref_shim_sqf.o"
# GPU-hash variant: fnv_hash weak in a copy of the object; the strong
# forwarder in ref_shim_aphash.cpp wins at link time.  -fPIC keeps the
# calls to fnv_hash as relocations against the symbol.
objcopy --weaken-symbol=_Z8fnv_hashjj "$OUT/sqf_cpu.o" "$OUT/sqf_cpu_weak.o"
$CXX $FLAGS -c "$RSQF/RSQF.cpp" -o "$OUT/rsqf_cpu.o"
$CXX $FLAGS -c "$HERE/ref_shim_aphash.cpp" -o "$OUT/ref_shim_aphash.o"
$CXX -shared -o "$OUT/libref_sqf_ap.so" "$OUT/sqf_cpu_weak.o" "$OUT/ref_shim_sqf.o" \
     "$OUT/ref_shim_aphash.o" "$OUT/rsqf_cpu.o"
$CXX $FLAGS -c "$REF/mt19937ar.cpp" -o "$OUT/mt.o"
$CXX $FLAGS -I"$RSQF" -I"$REF" -c "$HERE/ref_shim_rsqf.cpp" -o "$OUT/ref_shim_rsqf.o"
$CXX -shared -o "$OUT/libref_rsqf.so" "$OUT/rsqf_cpu.o" "$OUT/mt.o" "$OUT/ref_shim_rsqf.o"
# the same RSQF with 8-bit remainders: RSQF.h's declarations pre-included
# with RBITS 8 (ref_rsqf8_pre.h), sources unmodified
$CXX $FLAGS -include "$HERE/ref_rsqf8_pre.h" -c "$RSQF/RSQF.cpp" -o "$OUT/rsqf8_cpu.o"
$CXX $FLAGS -include "$HERE/ref_rsqf8_pre.h" -I"$RSQF" -I"$REF" -c "$HERE/ref_shim_rsqf.cpp" -o "$OUT/ref_shim_rsqf8.o"
$CXX -shared -o "$OUT/libref_rsqf8.so" "$OUT/rsqf8_cpu.o" "$OUT/mt.o" "$OUT/ref_shim_rsqf8.o"
rm -f "$OUT"/*.o
echo "build_ref: ok -> $OUT"
