#!/usr/bin/env bash
# Compiles the reference's own accel sources, in place under the reference
# tree, into a CPU oracle binary oracle/_ref/ref_accel.  Test infrastructure
# only: nothing in the product links or runs it.
#
# The reference library cannot be built as shipped (boost, TBB, FreeImage,
# yaml-cpp and Embree are absent), so:
#   * oracle/refharness/shim/pch.h replaces the boost-based precompiled header;
#   * each source is preprocessed and its `#pragma region` lines are dropped,
#     because GCC 13 rejects them inside the default-member-initialiser lambdas
#     that LM_IMPL_F creates;
#   * oracle/refharness/ref_runtime.cpp stands in for the component factory and
#     logger exports of liblightmetrica.
# x86-64 only: the reference forces SSE intrinsics (math.h:69, accel_qbvh.cpp:34).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/src/liblightmetrica" ]; then
  echo "reference tree not found at $REF; nothing to build" >&2
  exit 0
fi
case "$(uname -m)" in
  x86_64) ;;
  *) echo "reference sources need SSE4.2 (x86-64); skipping on $(uname -m)" >&2; exit 0 ;;
esac
mkdir -p "$OUT"
CXX="${CXX:-g++}"
DEFS="-DLM_EXPORTS -DLM_USE_SINGLE_PRECISION -DNDEBUG"
INC="-I$HERE/refharness/shim -I$REF/include"
FLAGS="-std=c++14 -O3 -msse4.2 -ffp-contract=off -w"

SRCS=(
  "$REF/src/liblightmetrica/accel/accel_naive.cpp"
  "$REF/src/liblightmetrica/accel/accel_bvh_sahbin.cpp"
  "$REF/src/liblightmetrica/accel/accel_qbvh.cpp"
  "$HERE/refharness/ref_runtime.cpp"
  "$HERE/refharness/ref_accel_cli.cpp"
)
OBJS=()
pids=()
for src in "${SRCS[@]}"; do
  base="$(basename "$src" .cpp)"
  (
    $CXX $FLAGS $DEFS $INC -E "$src" -o "$OUT/$base.ii"
    sed -i -E '/^[[:space:]]*#[[:space:]]*pragma[[:space:]]+(end)?region/d' "$OUT/$base.ii"
    $CXX $FLAGS -c -x c++ "$OUT/$base.ii" -o "$OUT/$base.o"
    rm -f "$OUT/$base.ii"
  ) &
  pids+=($!)
  OBJS+=("$OUT/$base.o")
done
for p in "${pids[@]}"; do wait "$p"; done
$CXX -O3 -o "$OUT/ref_accel" "${OBJS[@]}" -lpthread
rm -f "${OBJS[@]}"
echo "built $OUT/ref_accel"
