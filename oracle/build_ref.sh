#!/usr/bin/env bash
# Builds the REFERENCE library's own algorithm sources (read in place from the reference tree)
# against the stand-in headers in oracle/shim/, plus oracle/ref_capi.cpp, into
# oracle/_ref/libref.so. Test infrastructure: the reference build pins the oracle restatement
# and generates tests/golden/. It needs the reference tree, so it only runs where that exists.
# Dataloader::addRingInfo (src/dataloader/src/dataloader.cpp:68-137) sits inside a ROS node; that
# one function is extracted into oracle/_ref/add_ring_info.cpp (a build output, never committed)
# between ring_ref_prelude.h and ring_ref_capi.inc, and compiled into the same library.
#
#   REF_ROOT   reference checkout (default /root/reference; absent tree: nothing is built)
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
DL="$REF_ROOT/src/dataloader/src/dataloader.cpp"
{
  echo "#include \"$HERE/ring_ref_prelude.h\""
  echo "namespace dataloading {"
  awk '/^void Dataloader::addRingInfo\(/{f=1} f{print} f&&/^}/{exit}' "$DL"
  echo "} // namespace dataloading"
  echo "#include \"$HERE/ring_ref_capi.inc\""
} > "$OUT/add_ring_info.cpp"
grep -q "addRingInfo" "$OUT/add_ring_info.cpp" || { echo "build_ref: addRingInfo not found in $DL" >&2; exit 1; }
$CXX $FLAGS $INC -c "$OUT/add_ring_info.cpp" -o "$OUT/add_ring_info.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
$CXX -shared -o "$OUT/libref.so" "$OUT"/segmenter.o "$OUT"/noise_remover.o "$OUT"/clusterer.o \
  "$OUT"/polygonizer.o "$OUT"/ref_capi.o "$OUT"/add_ring_info.o -lm
echo "build_ref: $OUT/libref.so"
