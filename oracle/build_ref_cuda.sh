#!/usr/bin/env bash
# Recipe (measurement infrastructure only): builds the reference gpuPfem2 library and the
# Cylinder2D timing driver oracle/refcuda/cylinder_driver.cu into one executable,
# $OUT/ref_cylinder, for sm_103a.
#
#   oracle/build_ref_cuda.sh stage   copies the reference's src/ and
#                                    cases/Cylinder2D/main.cu into baseline/_ref/gpuPfem2
#                                    (needs the reference tree; git-ignored, travels with
#                                    the working copy to a machine without it)
#   oracle/build_ref_cuda.sh         compiles from that staged copy
#
# The reference's CMake build (CMakeLists.txt, cmake/functions.cmake) compiles the same
# sources with separable compilation and links cuBLAS and cuSPARSE; its architecture list
# 61;70;75 is not accepted by CUDA 13, so the sources are compiled here for sm_103a with
# the build type's -O2.  Nothing is written outside baseline/_ref.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/.." && pwd)
STAGE=$ROOT/baseline/_ref/gpuPfem2
OUT=${OUT:-$ROOT/baseline/_ref/bin}
if [ "${1:-}" = "stage" ]; then
  REF=${PF2_REFERENCE_DIR:-/root/reference}
  [ -d "$REF/src" ] || { echo "reference tree not found at $REF" >&2; exit 1; }
  mkdir -p "$STAGE/cases/Cylinder2D"
  cp -r "$REF/src" "$STAGE/"
  cp "$REF/cases/Cylinder2D/main.cu" "$STAGE/cases/Cylinder2D/main.cu"
  echo "staged $STAGE"
  exit 0
fi
[ -d "$STAGE/src" ] || { echo "no staged reference sources at $STAGE (run: $0 stage)" >&2; exit 1; }
NVCC=${NVCC:-nvcc}
FLAGS="-gencode arch=compute_103a,code=sm_103a -rdc=true -std=c++17 -O2 -I$STAGE/src -Xcompiler -fopenmp -w"
SRCS="data_export.cu data_export_3d.cu Dirichlet_bcs.cu mesh_2d.cu mesh_3d.cu common/cuda_helper.cu
      common/cuda_math.cu common/utilities.cpp integration/quadrature_formula_1d.cu
      integration/quadrature_formula_2d.cu integration/quadrature_formula_3d.cu
      linear_algebra/linear_solver.cu linear_algebra/preconditioners.cu linear_algebra/sparse_matrix.cu
      particles/particle_2d.cu particles/particle_handler_2d.cu"
mkdir -p "$OUT/obj"
pids=""
objs=""
for s in $SRCS; do
  o=$OUT/obj/$(echo "$s" | tr '/' '_').o
  objs="$objs $o"
  if [[ "$s" == *.cpp ]]; then
    $NVCC $FLAGS -x cu -c "$STAGE/src/$s" -o "$o" &
  else
    $NVCC $FLAGS -c "$STAGE/src/$s" -o "$o" &
  fi
  pids="$pids $!"
done
$NVCC $FLAGS -I"$STAGE/cases/Cylinder2D" -c "$HERE/refcuda/cylinder_driver.cu" -o "$OUT/obj/cylinder_driver.o" &
pids="$pids $!"
for p in $pids; do wait "$p"; done
$NVCC -gencode arch=compute_103a,code=sm_103a -rdc=true -o "$OUT/ref_cylinder" $objs "$OUT/obj/cylinder_driver.o" \
  -lcublas -lcusparse -lgomp
echo "built $OUT/ref_cylinder"
