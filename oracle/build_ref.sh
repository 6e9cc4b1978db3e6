#!/usr/bin/env bash
# Builds the REFERENCE library's own algorithm sources (read in place from the reference tree)
# against the stand-in headers in oracle/shim/, plus oracle/ref_capi.cpp, into
# oracle/_ref/libref.so. Test infrastructure: the reference build pins the oracle restatement
# and generates tests/golden/. It needs the reference tree, so it only runs where that exists.
#
#   REF_ROOT   reference checkout (default /root/reference)
#   REF_FLAGS  extra flags; the parity build uses -ffp-contract=off so that host GCC never fuses
#              a*b+c (aarch64 GCC would otherwise contract; x86-64 without -march does not).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_ROOT="${REF_ROOT:-/root/reference}"
LIB="$REF_ROOT/lidar_processing_lib"
if [ ! -d "$LIB/src" ]; then
  echo "build_ref: reference tree not found at $REF_ROOT; skipping" >&2
  exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS="-std=c++17 -O3 -fPIC -ffp-contract=off -w ${REF_FLAGS:-}"
INC="-I$HERE/shim -I$LIB/include -I$LIB/include/lidar_processing_lib -I$HERE/../include"
pids=()
for src in segmenter noise_remover clusterer polygonizer; do
  $CXX $FLAGS $INC -c "$LIB/src/$src.cpp" -o "$OUT/$src.o" & pids+=($!)
done
$CXX $FLAGS $INC -c "$HERE/ref_capi.cpp" -o "$OUT/ref_capi.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
$CXX -shared -o "$OUT/libref.so" "$OUT"/segmenter.o "$OUT"/noise_remover.o "$OUT"/clusterer.o \
  "$OUT"/polygonizer.o "$OUT"/ref_capi.o -lm
echo "build_ref: $OUT/libref.so"
