#!/usr/bin/env bash
# Recipe: compiles the reference's host-side setup code (DAT reader, CSR pattern,
# neighbour lists, particle-handler constructor, quadrature tables) from its sources
# where they lie, into oracle/_ref/ref_host_dump, linked against the host-memory
# runtime stand-in oracle/refhost/stub_cudart.c.  Test infrastructure only; outputs go
# to oracle/_ref/ and nothing else.  Needs the reference tree and nvcc; x86-64 or
# aarch64 host.
set -euo pipefail
REF=${REF:-/root/reference/src}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
[ -d "$REF" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
mkdir -p "$OUT/obj"
NVCC=${NVCC:-nvcc}
FLAGS="-arch=sm_103a -rdc=true -std=c++17 -O2 -I$REF -Xcompiler -fopenmp -w"
SRCS="mesh_2d.cu linear_algebra/sparse_matrix.cu particles/particle_2d.cu particles/particle_handler_2d.cu
      integration/quadrature_formula_1d.cu integration/quadrature_formula_2d.cu"
OBJS=""
for s in $SRCS; do
  o=$OUT/obj/$(basename "$s" .cu).o
  $NVCC $FLAGS -c "$REF/$s" -o "$o"
  OBJS="$OBJS $o"
done
$NVCC $FLAGS -c "$HERE/refhost/dump_ref_host.cu" -o "$OUT/obj/dump_ref_host.o"
$NVCC -arch=sm_103a -dlink $OBJS "$OUT/obj/dump_ref_host.o" -o "$OUT/obj/dlink.o"
gcc -O2 -c "$HERE/refhost/stub_cudart.c" -o "$OUT/obj/stub_cudart.o"
g++ -o "$OUT/ref_host_dump" $OBJS "$OUT/obj/dump_ref_host.o" "$OUT/obj/dlink.o" "$OUT/obj/stub_cudart.o" -fopenmp
echo "built $OUT/ref_host_dump"
