#!/usr/bin/env bash
# Builds oracle/_ref/libsph_ref.so: the reference SPH core compiled UNMODIFIED from its
# own sources where they lie, plus oracle/ref_harness.cpp (extern "C" marshalling) and
# the project-written GLM stand-in oracle/glm_shim/.
#
# TEST INFRASTRUCTURE ONLY (the oracle).  The reference's CMake is bypassed on purpose:
# it requires OpenGL (CMakeLists.txt:15) and its -mavx2 flag breaks the build
# (kernels.h:107-108, spatial_hash.cpp:115-116).  Two workarounds are needed and nothing
# else: -include memory (kernels.h:100 uses std::unique_ptr without <memory>) and the GLM
# stand-in.
#
#   libsph_ref.so           canonical oracle: IEEE float, no FMA contraction, no fast-math
#   libsph_ref_fastmath.so  the reference's own -ffast-math flag (CMakeLists.txt:148),
#                           kept for the sensitivity check only
#
# Usage: oracle/build_ref.sh [REFERENCE_DIR]   (default /root/reference)
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ref="${1:-${SPH_REFERENCE_DIR:-/root/reference}}"
src="$ref/src"
if [ ! -f "$src/sph_engine.cpp" ]; then
    echo "build_ref: reference sources not found under $src" >&2
    exit 2
fi
out="$here/_ref"
mkdir -p "$out"
tus=("$src/particle.cpp" "$src/kernels.cpp" "$src/spatial_hash.cpp" "$src/sph_engine.cpp"
     "$here/ref_harness.cpp")
common=(-std=gnu++17 -O2 -fopenmp -DUSE_OPENMP -fPIC -shared -w -include memory
        -I"$here/glm_shim" -I"$src")
g++ "${common[@]}" -ffp-contract=off "${tus[@]}" -o "$out/libsph_ref.so" &
p1=$!
g++ "${common[@]}" -ffast-math "${tus[@]}" -o "$out/libsph_ref_fastmath.so" &
p2=$!
wait $p1
wait $p2
echo "build_ref: built $out/libsph_ref.so $out/libsph_ref_fastmath.so"
