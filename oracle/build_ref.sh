#!/usr/bin/env bash
# Builds the unmodified reference sources (RealCausticsEngine, "Real Caustics/src")
# plus oracle/ref_harness.cpp into oracle/_ref/libref_oracle.so.
#
# Test infrastructure only: the library is the checker that pins the oracle
# restatement and generates tests/golden fixtures; nothing in the product links it.
#
# Shims (no source edits):
#   -D'__declspec(x)='           MSVC export keyword
#   BVH\BVH_mesh.h, BVH\BVH_world.h   forwarding headers named with a literal
#                                backslash, for the includes at src/main.cpp:20,
#                                src/mesh.h:5, src/Debug_scene.cpp:10-11
#   -include powf_shim.h         libstdc++ has no std::powf (src/MLT_Sampler.cpp:34,36)
#   -Dmain=ref_main              the reference exports its render entry as `main`
#                                (src/DLL.h:14); renamed so the harness can call it
# Floating point: -O2 -ffp-contract=off, SSE2 only (the x86-64 baseline ISA), so
# every float operation rounds exactly as written in the source.
set -euo pipefail
REF_ROOT="${REF_ROOT:-/root/reference}"
SRC="$REF_ROOT/Real Caustics/src"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$SRC" ]; then
  echo "reference sources not found at $SRC; oracle/_ref not built" >&2
  exit 3
fi
mkdir -p "$OUT/obj" "$OUT/shim"
printf '#include "%s/BVH/BVH_mesh.h"\n' "$SRC" > "$OUT/shim/BVH\\BVH_mesh.h"
printf '#include "%s/BVH/BVH_world.h"\n' "$SRC" > "$OUT/shim/BVH\\BVH_world.h"
printf '#pragma once\n#include <cmath>\nnamespace std { using ::powf; }\n' > "$OUT/shim/powf_shim.h"
CXXFLAGS=(-std=c++17 -O2 -fPIC -ffp-contract=off -w "-D__declspec(x)=" -Dmain=ref_main
          -I"$OUT/shim" -I"$SRC" -include "$OUT/shim/powf_shim.h")
SOURCES=(aabb.cpp BXDF.cpp BVH/BVH_mesh.cpp BVH/BVH_world.cpp Debug_scene.cpp Lights.cpp
         Light_list.cpp materials.cpp matrix.cpp mesh.cpp main.cpp KD_Tree.cpp MLT_Sampler.cpp
         Scene.cpp Transform.cpp Triangle.cpp vec3.cpp Vertex_Merging.cpp)
pids=()
for s in "${SOURCES[@]}"; do
  o="$OUT/obj/$(echo "$s" | tr '/' '_').o"
  g++ "${CXXFLAGS[@]}" -c "$SRC/$s" -o "$o" &
  pids+=($!)
done
g++ "${CXXFLAGS[@]}" -c "$HERE/ref_harness.cpp" -o "$OUT/obj/ref_harness.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/libref_oracle.so" "$OUT"/obj/*.o
echo "built $OUT/libref_oracle.so"
