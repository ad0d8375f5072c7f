#!/usr/bin/env bash
# Compiles the reference's own accel and renderer sources, in place under the
# reference tree, into CPU oracle binaries in oracle/_ref/:
#   ref_accel     accel::naive / bvh_sahbin / qbvh driver (single precision)
#   ref_render    renderer::pt, bdpt, ptmis, ptdirect, ltdirect and vcm with bsdf::diffuse, bsdf::null, bsdf::flesnel,
#                 bsdf::cook_torrance, light::area, light::env,
#                 sensor::pinhole, Random (dSFMT) and accel::qbvh (single)
#   ref_render64  the same in double precision (LM_USE_DOUBLE_PRECISION,
#                 cmake/LMBuildOptions.cmake:32-43) with accel::bvh_sahbin
#   ref_isect / ref_isect64  IntersectionUtils::CreateTriangleIntersection
#                 (single / double precision)
#   ref_plugin    the reference-side accel plugin (plugin/accel_cuda.cpp)
#                 driven through the reference's component interfaces
#   ref_render_plugins  the render harness with the renderer plugins
#                 (plugin/renderer_*_cuda.cpp) registered beside the
#                 reference's renderers
#   (both link oracle/refharness/lmgpu_cpu_fake.cpp, a CPU stand-in for the
#   C ABI of include/lmgpu.h, since this machine has no GPU)
# Test infrastructure only: nothing in the product links or runs them.
#
# The reference library cannot be built as shipped (boost, TBB, FreeImage,
# yaml-cpp and Embree are absent), so:
#   * oracle/refharness/shim/pch.h replaces the boost-based precompiled header;
#   * each source is preprocessed and its `#pragma region` lines are dropped,
#     because GCC 13 rejects them inside the default-member-initialiser lambdas
#     that LM_IMPL_F creates;
#   * oracle/refharness/*.cpp stand in for the component factory, logger,
#     property tree, assets, film, scheduler and scene of liblightmetrica.
# x86-64 only: the reference forces SSE intrinsics (math.h:69, accel_qbvh.cpp:34).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   default: $LM_REFERENCE_ROOT, else a `reference` directory beside the repository
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${LM_REFERENCE_ROOT:-$HERE/../../reference}}"
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
CC="${CC:-gcc}"
REPO_ROOT="$(cd "$HERE/.." && pwd)"
PLUGIN="$REPO_ROOT/lightmetrica-v2_gb300/plugin"
INC="-I$HERE/refharness/shim -I$REF/include -I$REF/external-src/dSFMT-src-2.2.3 -I$REPO_ROOT/include -I$PLUGIN"
FLAGS="-std=c++14 -O3 -msse4.2 -ffp-contract=off -w"
L="$REF/src/liblightmetrica"

ACCEL_SRCS=("$L/accel/accel_naive.cpp" "$L/accel/accel_bvh_sahbin.cpp" "$L/accel/accel_bvh_sah.cpp" "$L/accel/accel_qbvh.cpp" "$HERE/refharness/ref_runtime.cpp")
RENDER_SRCS=("$L/renderer/renderer_pt.cpp" "$L/renderer/renderer_bdpt.cpp" "$L/renderer/renderer_ptmis.cpp" "$L/renderer/renderer_ptdirect.cpp" "$L/renderer/renderer_ltdirect.cpp" "$L/renderer/renderer_vcm.cpp" "$L/renderer/subpathsampler.cpp" "$L/asset/bsdf/bsdf_diffuse.cpp" "$L/asset/bsdf/bsdf_null.cpp"
             "$L/asset/bsdf/bsdf_flesnel.cpp" "$L/asset/bsdf/bsdf_cooktorrance.cpp"
             "$L/asset/light/light_area.cpp" "$L/asset/light/light_env.cpp" "$L/asset/sensor/sensor_pinhole.cpp"
             "$L/random.cpp" "$HERE/refharness/ref_render_cli.cpp")

# compile_set <tag> <defs> <sources...>: objects into $OUT/<tag>_*.o
compile_set() {
  local tag="$1" defs="$2"; shift 2
  local pids=()
  for src in "$@"; do
    local base; base="$(basename "$src" .cpp)"
    (
      $CXX $FLAGS $defs $INC -E "$src" -o "$OUT/${tag}_$base.ii"
      sed -i -E '/^[[:space:]]*#[[:space:]]*pragma[[:space:]]+(end)?region/d' "$OUT/${tag}_$base.ii"
      $CXX $FLAGS -c -x c++ "$OUT/${tag}_$base.ii" -o "$OUT/${tag}_$base.o"
      rm -f "$OUT/${tag}_$base.ii"
    ) &
    pids+=($!)
  done
  for p in "${pids[@]}"; do wait "$p"; done
}

S="-DLM_EXPORTS -DLM_USE_SINGLE_PRECISION -DNDEBUG"
D="-DLM_EXPORTS -DLM_USE_DOUBLE_PRECISION -DNDEBUG"
ISECT="$HERE/refharness/ref_isect_cli.cpp"
PLUGIN_SRCS=("$PLUGIN/accel_cuda.cpp" "$PLUGIN/renderer_pt_cuda.cpp" "$PLUGIN/renderer_ptmis_cuda.cpp"
             "$PLUGIN/renderer_ptdirect_cuda.cpp" "$PLUGIN/renderer_ltdirect_cuda.cpp" "$PLUGIN/renderer_bdpt_cuda.cpp"
             "$PLUGIN/renderer_vcm_cuda.cpp" "$PLUGIN/renderer_pt_guided_cuda.cpp")
compile_set f "$S" "${ACCEL_SRCS[@]}" "${RENDER_SRCS[@]}" "$HERE/refharness/ref_accel_cli.cpp" "$ISECT" \
  "${PLUGIN_SRCS[@]}" "$HERE/refharness/ref_plugin_cli.cpp"
# the C-ABI stand-in and the oracle it runs on (plain C/C++, no reference headers)
ORACLE_C=("$HERE/lmoracle_accel.c" "$HERE/lmoracle_pt.c" "$HERE/lmoracle_bdpt.c" "$HERE/lmoracle_surface.c")
for c in "${ORACLE_C[@]}"; do
  $CC -O2 -std=c11 -ffp-contract=off -fno-fast-math -w -c "$c" -o "$OUT/o_$(basename "$c" .c).o" &
done
$CXX -std=c++14 -O2 -ffp-contract=off -w -I"$REPO_ROOT/include" -c "$HERE/refharness/lmgpu_cpu_fake.cpp" -o "$OUT/fake_lmgpu.o" &
wait
compile_set d "$D" "${ACCEL_SRCS[@]}" "${RENDER_SRCS[@]}" "$ISECT"
$CC -O3 -msse2 -DDSFMT_MEXP=19937 -DNDEBUG -w -c "$REF/external-src/dSFMT-src-2.2.3/dSFMT.c" -o "$OUT/dsfmt.o"

obj() { local tag="$1"; shift; for s in "$@"; do echo "$OUT/${tag}_$(basename "$s" .cpp).o"; done; }
$CXX -O3 -o "$OUT/ref_accel" $(obj f "${ACCEL_SRCS[@]}" "$HERE/refharness/ref_accel_cli.cpp") -lpthread
$CXX -O3 -o "$OUT/ref_render" $(obj f "${ACCEL_SRCS[@]}" "${RENDER_SRCS[@]}") "$OUT/dsfmt.o" -lpthread
$CXX -O3 -o "$OUT/ref_render64" $(obj d "${ACCEL_SRCS[@]}" "${RENDER_SRCS[@]}") "$OUT/dsfmt.o" -lpthread
$CXX -O3 -o "$OUT/ref_isect" $(obj f "$HERE/refharness/ref_runtime.cpp" "$ISECT") -lpthread
$CXX -O3 -o "$OUT/ref_isect64" $(obj d "$HERE/refharness/ref_runtime.cpp" "$ISECT") -lpthread
FAKE=("$OUT/fake_lmgpu.o" "$OUT"/o_*.o)
$CXX -O3 -o "$OUT/ref_plugin" $(obj f "$HERE/refharness/ref_runtime.cpp" "$PLUGIN/accel_cuda.cpp" "$HERE/refharness/ref_plugin_cli.cpp") \
  "${FAKE[@]}" -lpthread -lm
$CXX -O3 -o "$OUT/ref_render_plugins" $(obj f "${ACCEL_SRCS[@]}" "${RENDER_SRCS[@]}" "${PLUGIN_SRCS[@]}") "$OUT/dsfmt.o" \
  "${FAKE[@]}" -lpthread -lm
rm -f "$OUT"/*.o
echo "built $OUT/ref_accel $OUT/ref_render $OUT/ref_render64 $OUT/ref_isect $OUT/ref_isect64 $OUT/ref_plugin $OUT/ref_render_plugins"
