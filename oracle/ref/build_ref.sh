#!/usr/bin/env bash
# ORACLE / TEST INFRASTRUCTURE — builds the reference Veritas sources, unmodified and in
# place, into oracle/_ref/veritas_ref.  Only the path's own translation units are
# compiled (the reference's CMake build is not used):
#   BoundaryCondition.cpp Level.cpp Rectangle.cpp SolverManager.cpp EMSolver.cpp
#   Mesh.cpp Settings.cpp
# plus this directory's harness.cpp (problem hooks + driver, replacing veritas.cpp) and
# mkl_shim.cpp (the four MKL routines, see shim/mkl.h).  USINGMKL/MKL_ILP64 select the
# reference's default configuration (CMakeLists.txt:9,26).  -ffp-contract=off keeps
# IEEE double arithmetic identical on x86-64 and aarch64.
# Usage: build_ref.sh [reference_dir]   (default: $VERITAS_REFERENCE_DIR)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${VERITAS_REFERENCE_DIR:-}}"
if [ -z "$REF" ]; then
  echo "no reference tree given (argument or VERITAS_REFERENCE_DIR)" >&2
  exit 3
fi
OUT="$HERE/../_ref"
if [ ! -f "$REF/Rectangle.cpp" ]; then
  echo "reference sources not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT/gen" "$OUT/obj"
sed 's/@GIT_SHA1@/reference/' "$REF/gitsha1.hpp.in" > "$OUT/gen/gitsha1.hpp"
CXX="${CXX:-g++}"
FLAGS=(-O3 -std=c++14 -fopenmp -ffp-contract=off -DUSINGMKL -DMKL_ILP64 -w
       -I"$HERE/shim" -I"$OUT/gen" -I"$REF")
pids=()
for src in BoundaryCondition Level Rectangle SolverManager EMSolver Mesh Settings; do
  "$CXX" "${FLAGS[@]}" -c "$REF/$src.cpp" -o "$OUT/obj/$src.o" & pids+=($!)
done
"$CXX" "${FLAGS[@]}" -c "$HERE/harness.cpp" -o "$OUT/obj/harness.o" & pids+=($!)
"$CXX" "${FLAGS[@]}" -c "$HERE/mkl_shim.cpp" -o "$OUT/obj/mkl_shim.o" & pids+=($!)
# the same driver over a user problem written against the C hooks (tests/hooks)
HOOKS="$HERE/../../tests/hooks"
mkdir -p "$OUT/hobj"
"$CXX" "${FLAGS[@]}" -DVX_HOOKS_PROBLEM -I"$HOOKS" -c "$HERE/harness.cpp" -o "$OUT/hobj/harness_hooks.o" & pids+=($!)
"${CC:-gcc}" -O2 -ffp-contract=off -c "$HOOKS/sin2_problem.c" -o "$OUT/hobj/sin2_problem.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" -fopenmp "$OUT"/obj/*.o -o "$OUT/veritas_ref"
REFOBJ=()
for src in BoundaryCondition Level Rectangle SolverManager EMSolver Mesh Settings mkl_shim; do
  REFOBJ+=("$OUT/obj/$src.o")
done
"$CXX" -fopenmp "${REFOBJ[@]}" "$OUT/hobj/harness_hooks.o" "$OUT/hobj/sin2_problem.o" -lm -o "$OUT/veritas_ref_hooks"
echo "built $OUT/veritas_ref $OUT/veritas_ref_hooks"
