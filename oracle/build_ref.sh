#!/usr/bin/env bash
# Builds oracle/_ref/libref{2d,3d}.so: the reference's own CPU solver headers
# (Local_code/level-set_MPI_{2D,3D}/include), unmodified, behind the
# extern "C" drivers in this folder and the single-rank MPI stub; and
# oracle/_ref/libref_sample.so: the sample surface's sources
# (sample/field.cpp, sample/weno5_rk3.cpp, sample/first_order_upwind.cpp)
# compiled in place behind ref_sample_driver.cpp.
# Test infrastructure only.  Nothing is copied out of the reference tree: the
# headers and sources are read in place, and only the shared libraries are
# written (into oracle/_ref/, which git ignores).
#
# -ffp-contract=off keeps the arithmetic free of fused multiply-adds on every
# host (gcc contracts by default on aarch64), so the results are the plain
# IEEE double operations the reference source spells out.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
# the reference tree: first argument, else $LSGB_REFERENCE_ROOT (no default)
ref_root="${1:-${LSGB_REFERENCE_ROOT:-}}"
out="$here/_ref"
if [ -z "$ref_root" ]; then
    echo "usage: build_ref.sh <reference root>  (or set LSGB_REFERENCE_ROOT)" >&2
    exit 2
fi
if [ ! -d "$ref_root/Local_code/level-set_MPI_3D/include" ]; then
    echo "build_ref.sh: reference tree not found at $ref_root" >&2
    exit 2
fi
mkdir -p "$out"
CXX="${CXX:-g++}"
FLAGS="-O2 -std=c++14 -fPIC -shared -ffp-contract=off -fno-fast-math -w"
"$CXX" $FLAGS -I"$here/mpi_stub" -I"$ref_root/Local_code/level-set_MPI_3D/include" \
    "$here/ref_driver3d.cpp" -o "$out/libref3d.so" &
"$CXX" $FLAGS -I"$here/mpi_stub" -I"$ref_root/Local_code/level-set_MPI_2D/include" \
    "$here/ref_driver2d.cpp" -o "$out/libref2d.so" &
"$CXX" $FLAGS -fopenmp -std=c++17 -I"$ref_root/sample" "$here/ref_sample_driver.cpp" \
    "$ref_root/sample/field.cpp" "$ref_root/sample/weno5_rk3.cpp" "$ref_root/sample/first_order_upwind.cpp" \
    -o "$out/libref_sample.so" &
wait %1 && wait %2 && wait %3
echo "built $out/libref3d.so $out/libref2d.so $out/libref_sample.so"
