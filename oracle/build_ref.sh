#!/usr/bin/env bash
# Builds the reference engine from its own sources into oracle/_ref/ (test
# infrastructure only).  Only the four engine sources are compiled; the CLI
# (src/main.cpp, src/args.cpp) needs Boost, which is absent, and is not built.
# Flags follow the reference's CMakeLists.txt (-std=c++11 -O3, OpenMP) plus
# -ffp-contract=off so that an aarch64 host rounds like the x86 build.
#
# The reference checkout is $REF_ROOT (its engine sources $REF_SRC, default
# $REF_ROOT/src).  This recipe is the one place that names the checkout's
# default location; `build_ref.sh --root` prints the checkout it would use.
#
# usage: oracle/build_ref.sh [--root | REFERENCE_SRC_DIR]
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
root="${REF_ROOT:-/root/reference}"
if [ "${1:-}" = "--root" ]; then
    echo "$root"
    exit 0
fi
src="${1:-${REF_SRC:-$root/src}}"
out="$here/_ref"
if [ ! -f "$src/boid_simulation_grid.cpp" ]; then
    echo "build_ref.sh: reference sources not found at $src" >&2
    exit 3
fi
mkdir -p "$out"
flags="-std=c++11 -O3 -fopenmp -ffp-contract=off -fPIC -shared -w"
g++ $flags -DREF_GRID -I"$src" "$here/ref_driver.cpp" \
    "$src/boid_simulation_grid.cpp" "$src/boid.cpp" "$src/vector3D.cpp" \
    -o "$out/libref_grid.so" &
g++ $flags -I"$src" "$here/ref_driver.cpp" \
    "$src/boid_simulation.cpp" "$src/boid.cpp" "$src/vector3D.cpp" \
    -o "$out/libref_allpairs.so" &
wait %1 && wait %2
echo "built $out/libref_grid.so $out/libref_allpairs.so"
