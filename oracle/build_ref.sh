#!/usr/bin/env bash
# Builds oracle/_ref/libref_kernels.so: the reference's own OpenCL kernels
# (kernels/grid.cl, wcsph.cl, normals.cl, pcisph.cl, boundary.cl, bilateral.cl,
# curvatureflow.cl and their headers)
# compiled for the CPU through oracle/ref_shim/clshim.hpp, its host scene samplers
# (BoxVolume::particles, FishTank::surface_sampling, Cube::surface_sampling, through
# oracle/ref_shim/ref_scene.cpp), and its mesh code
# (mesh/modelmesh.cpp, mesh/icospheremesh.cpp, external/voxelizer/voxelizer.h).  Used only to pin the oracle
# and to generate tests/golden/ fixtures, in a container where the reference is mounted.
#
# The one source transformation rewrites OpenCL vector literals "(int4)(" / "(float4)("
# into function calls, on copies written under oracle/_ref/src (never committed).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#        oracle/build_ref.sh --root      (prints the reference root it would use)
# The root is the argument, else $FLUIDS_REFERENCE_ROOT, else the container's mount point.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
if [ "${1:-}" = "--root" ]; then
    echo "${FLUIDS_REFERENCE_ROOT:-/root/reference}"
    exit 0
fi
ref="${1:-${FLUIDS_REFERENCE_ROOT:-/root/reference}}"
out="$here/_ref"
have_ref=0
if [ -d "$ref/kernels" ]; then
    have_ref=1
elif [ ! -f "$out/src/grid.cl" ]; then
    echo "build_ref: no reference kernels under $ref; skipped" >&2
    exit 0
fi
mkdir -p "$out/src" "$out/obj"
if [ "$have_ref" = 1 ]; then
    for f in "$ref"/kernels/*.cl "$ref"/kernels/*.h; do
        sed -E 's/\((int4|float4)\)[[:space:]]*\(/make_\1(/g' "$f" > "$out/src/$(basename "$f")"
    done
    # the host scene samplers: each function's text, from its signature line to its closing
    # brace, unchanged (the rest of those files is OpenGL / Qt / Bullet code)
    extract() {   # file, signature prefix, output
        awk -v sig="$2" 'index($0, sig) == 1 {on = 1} on {print} on && /^}/ {exit}' "$1" > "$3"
        [ -s "$3" ] || { echo "build_ref: $2 not found in $1" >&2; exit 1; }
    }
    extract "$ref/fluid/simulation/boxvolume.cpp" "vector<cl_float4> BoxVolume::particles(" "$out/src/boxvolume_particles.inc"
    extract "$ref/scene/fishtank.cpp" "vector<btVector3> FishTank::surface_sampling(" "$out/src/fishtank_surface_sampling.inc"
    extract "$ref/scene/cube.cpp" "vector<btVector3> Cube::surface_sampling(" "$out/src/cube_surface_sampling.inc"
fi
# (without the reference mounted, e.g. on the GPU machine, the kernel copies made here
# under oracle/_ref/src, which travel with the working tree, are compiled again)
CXX="${CXX:-g++}"
flags=(-O2 -std=c++17 -fPIC -ffp-contract=off -pthread -Wall -Wno-sign-compare -Wno-unused -Wno-narrowing -I "$here/ref_shim" -I "$out/src")
pids=()
for u in clshim_runtime ref_grid ref_wcsph ref_normals ref_pcisph ref_boundary ref_render ref_scene; do
    "$CXX" "${flags[@]}" -c "$here/ref_shim/$u.cpp" -o "$out/obj/$u.o" &
    pids+=($!)
done
# the mesh code (mesh/modelmesh.cpp with the vendored tinyobj, mesh/icospheremesh.cpp and
# the vendored voxelizer) compiles from its own sources under the reference root
rm -f "$out"/obj/ref_modelmesh.o "$out"/obj/ref_icospheremesh.o "$out"/obj/ref_mesh.o
if [ "$have_ref" = 1 ]; then
    mflags=(-O2 -std=c++17 -fPIC -ffp-contract=off -pthread -w -I "$here/ref_shim" -I "$ref")
    "$CXX" "${mflags[@]}" -c "$ref/mesh/modelmesh.cpp" -o "$out/obj/ref_modelmesh.o" &
    pids+=($!)
    "$CXX" "${mflags[@]}" -c "$ref/mesh/icospheremesh.cpp" -o "$out/obj/ref_icospheremesh.o" &
    pids+=($!)
    "$CXX" "${mflags[@]}" -c "$here/ref_shim/ref_mesh.cpp" -o "$out/obj/ref_mesh.o" &
    pids+=($!)
fi
# the same kernel files built without USE_MULLER_KERNELS (the Monaghan kernels of
# kernels/monaghan_kernels.h, compiled out in the reference): entry points *_monaghan
for u in ref_wcsph ref_normals ref_pcisph ref_boundary; do
    "$CXX" "${flags[@]}" -DCLSHIM_MONAGHAN -c "$here/ref_shim/$u.cpp" -o "$out/obj/${u}_monaghan.o" &
    pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" -shared -pthread -o "$out/libref_kernels.so" "$out"/obj/*.o
echo "build_ref: built $out/libref_kernels.so"
