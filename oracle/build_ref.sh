#!/usr/bin/env bash
# Build recipe for oracle/_ref/libpcisph_ref.so: the reference's own OpenCL
# kernels (PCISPH/data/kernels/sort_utils.cl, pcisph.cl and the grid_utils.cl /
# Simulation_Params.h they include) compiled as C++ on the host, plus the
# host-side driver in oracle/ref_shim/ref_driver.cpp.
#
# TEST INFRASTRUCTURE ONLY: the output generates golden vectors and pins the
# oracle restatement. It reads the reference sources where they lie and writes
# only into oracle/_ref/. The one textual change -- OpenCL cast literals
# "(float3)(a,b,c)" / "(uint2)(a,b)" become constructor calls -- happens in a
# pipe on the way into g++; no edited copy of any reference file is written.
# Without it, pcisph.cl:167 would parse as a comma expression and lose gravity.
#
# usage: oracle/build_ref.sh <reference_root>   (the checkout holding PCISPH/data/kernels)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
if [[ $# -ne 1 ]]; then
    echo "usage: $0 <reference_root>" >&2
    exit 2
fi
REF_ROOT="$1"
SRC="$REF_ROOT/PCISPH"
OUT="$HERE/_ref"
if [[ ! -f "$SRC/data/kernels/pcisph.cl" ]]; then
    echo "build_ref.sh: reference kernels not found under $SRC" >&2
    exit 2
fi
mkdir -p "$OUT"
rewrite() { sed -E 's/\((float3|uint2)\)[[:space:]]*\(/\1(/g' "$1"; }
{
    echo "#line 1 \"PCISPH/data/kernels/sort_utils.cl\""
    rewrite "$SRC/data/kernels/sort_utils.cl"
    echo ""
    echo "#line 1 \"PCISPH/data/kernels/pcisph.cl\""
    rewrite "$SRC/data/kernels/pcisph.cl"
    echo ""
    # Fluid::update_deduced_attributes up to (not including) its "// buffers" part,
    # i.e. the parameter derivation and the delta computation (Fluid.cpp:377-443).
    echo "#line 1 \"oracle/ref_shim/deduced_prefix.hpp\""
    cat "$HERE/ref_shim/deduced_prefix.hpp"
    echo "#line 377 \"PCISPH/src/sim/Fluid.cpp\""
    sed -n '/void Fluid::update_deduced_attributes()/,/\/\/ buffers/p' "$SRC/src/sim/Fluid.cpp" | sed '$d'
    echo "} }  // end of update_deduced_attributes, namespace sim"
    echo "#line 1 \"oracle/ref_shim/ref_driver.cpp\""
    cat "$HERE/ref_shim/ref_driver.cpp"
} | g++ -x c++ -std=c++17 -O2 -fwrapv -ffp-contract=off -fopenmp -fPIC -shared \
        -DOPENCL_COMPILING -include "$HERE/ref_shim/cl_shim.h" -I "$SRC" -I "$SRC/src" \
        -o "$OUT/libpcisph_ref.so.tmp" -
mv "$OUT/libpcisph_ref.so.tmp" "$OUT/libpcisph_ref.so"
echo "built $OUT/libpcisph_ref.so"

# The reference's scene loader: scenes.cpp from "namespace scene {" up to (not including) load_xraw, which
# needs OpenGL; utils::read_file comes from ref_shim/scene_shim.cpp.
{
    echo "#line 1 \"oracle/ref_shim/scene_shim.cpp\""
    cat "$HERE/ref_shim/scene_shim.cpp"
    echo "#line 11 \"PCISPH/src/scenes.cpp\""
    sed -n '/^namespace scene {/,/void load_xraw(const std::string& path/p' "$SRC/src/scenes.cpp" | sed '$d'
    echo "}  // namespace scene"
    echo "#line 1 \"oracle/ref_shim/scene_entry.cpp\""
    cat "$HERE/ref_shim/scene_entry.cpp"
} | g++ -x c++ -std=c++17 -O2 -ffp-contract=off -w -fPIC -shared -o "$OUT/libpcisph_ref_scene.so.tmp" -
mv "$OUT/libpcisph_ref_scene.so.tmp" "$OUT/libpcisph_ref_scene.so"
echo "built $OUT/libpcisph_ref_scene.so"
