#!/usr/bin/env bash
# Recipe (test infrastructure only; outputs go to oracle/_ref/ and nothing else):
#  1. the reference's host-side setup code (DAT reader, CSR pattern, neighbour lists,
#     particle-handler constructor, quadrature tables), compiled from its sources where
#     they lie into oracle/_ref/ref_host_dump, linked against the host-memory runtime
#     stand-in oracle/refhost/stub_cudart.c;
#     and the 3D host setup (DAT reader, CSR pattern, quadrature) into ref_host_dump3d;
#     and the VTU writers (data_export.cu) into ref_vtu_dump;
#  2. the reference's GPU kernels, compiled from the same sources into linked sm_103a
#     cubins (device code only) with the mangled name of every kernel:
#     ref_flow.cubin (mesh, particles, Dirichlet BCs, Cylinder2D kernels) and
#     ref_poisson.cubin (Poisson2D kernel), plus ref_kernels.names;
#  3. ref_poisson3d.cubin (Mesh3D and Poisson3D kernels) with ref_kernels3d.names.
# Needs the reference tree and nvcc (x86-64 or aarch64 host).
set -euo pipefail
REF=${REF:-${PF2_REFERENCE_DIR:-/root/reference}/src}
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
# the VTU writers (data_export.cu) on the same stand-in
$NVCC $FLAGS -c "$REF/data_export.cu" -o "$OUT/obj/data_export.o"
$NVCC $FLAGS -c "$HERE/refhost/dump_ref_vtu.cu" -o "$OUT/obj/dump_ref_vtu.o"
$NVCC -arch=sm_103a -dlink $OBJS "$OUT/obj/data_export.o" "$OUT/obj/dump_ref_vtu.o" -o "$OUT/obj/dlink_vtu.o"
g++ -o "$OUT/ref_vtu_dump" $OBJS "$OUT/obj/data_export.o" "$OUT/obj/dump_ref_vtu.o" "$OUT/obj/dlink_vtu.o" \
  "$OUT/obj/stub_cudart.o" -fopenmp
echo "built $OUT/ref_vtu_dump"
# the 3D host setup: DAT reader, CSR pattern, quadrature table (neighbour lists are built
# by GPU kernels there and left out)
OBJS3=""
for s in mesh_3d.cu linear_algebra/sparse_matrix.cu integration/quadrature_formula_3d.cu mesh_2d.cu; do
  o=$OUT/obj/h3_$(basename "$s" .cu).o
  $NVCC $FLAGS -c "$REF/$s" -o "$o"
  OBJS3="$OBJS3 $o"
done
$NVCC $FLAGS -c "$HERE/refhost/dump_ref_host3d.cu" -o "$OUT/obj/dump_ref_host3d.o"
$NVCC -arch=sm_103a -dlink $OBJS3 "$OUT/obj/dump_ref_host3d.o" -o "$OUT/obj/dlink3.o"
g++ -o "$OUT/ref_host_dump3d" $OBJS3 "$OUT/obj/dump_ref_host3d.o" "$OUT/obj/dlink3.o" "$OUT/obj/stub_cudart.o" -fopenmp
echo "built $OUT/ref_host_dump3d"

# ---- 2. device code of the reference kernels
CFLAGS="-arch=sm_103a -rdc=true -std=c++17 -I$REF -w"
CASES=$(cd "$REF/.." && pwd)/cases
flow=""
for s in mesh_2d.cu particles/particle_2d.cu particles/particle_handler_2d.cu Dirichlet_bcs.cu; do
  c=$OUT/obj/$(basename "$s" .cu).cubin
  $NVCC $CFLAGS -cubin "$REF/$s" -o "$c"
  flow="$flow $c"
done
$NVCC $CFLAGS -cubin "$CASES/Cylinder2D/main.cu" -o "$OUT/obj/cylinder_main.cubin"
nvlink -arch=sm_103a $flow "$OUT/obj/cylinder_main.cubin" -o "$OUT/ref_flow.cubin"
# Poisson2D/main.cu uses quadrature_formula_1d.cuh without including it
$NVCC $CFLAGS -include integration/quadrature_formula_1d.cuh -cubin "$CASES/Poisson2D/main.cu" -o "$OUT/obj/poisson_main.cubin"
nvlink -arch=sm_103a "$OUT/obj/poisson_main.cubin" -o "$OUT/ref_poisson.cubin"
# kernel names: the host objects of the same translation units carry the same symbols
$NVCC $FLAGS -c "$CASES/Cylinder2D/main.cu" -o "$OUT/obj/cylinder_main.o"
$NVCC $FLAGS -include integration/quadrature_formula_1d.cuh -c "$CASES/Poisson2D/main.cu" -o "$OUT/obj/poisson_main.o"
$NVCC $FLAGS -c "$REF/Dirichlet_bcs.cu" -o "$OUT/obj/Dirichlet_bcs.o"
for o in mesh_2d particle_handler_2d Dirichlet_bcs cylinder_main poisson_main; do
  nm "$OUT/obj/$o.o" | awk -v src=$o '$2 == "T" && $3 ~ /^_Z[0-9]+k[A-Z]/ && $3 !~ /device_stub/ {
      name = $3; sub(/^_Z[0-9]+/, "", name); len = substr($3, 3) + 0; print src, substr(name, 1, len), $3 }'
done > "$OUT/ref_kernels.names"
echo "built $OUT/ref_flow.cubin $OUT/ref_poisson.cubin ($(wc -l < "$OUT/ref_kernels.names") kernels)"

# ---- 3. device code of the 3D kernels (mesh_3d.cu, cases/Poisson3D/main.cu)
$NVCC $CFLAGS -cubin "$REF/mesh_3d.cu" -o "$OUT/obj/mesh_3d.cubin"
$NVCC $CFLAGS -cubin "$CASES/Poisson3D/main.cu" -o "$OUT/obj/poisson3d_main.cubin"
nvlink -arch=sm_103a "$OUT/obj/mesh_3d.cubin" "$OUT/obj/poisson3d_main.cubin" -o "$OUT/ref_poisson3d.cubin"
$NVCC $FLAGS -c "$CASES/Poisson3D/main.cu" -o "$OUT/obj/poisson3d_main.o"
for o in h3_mesh_3d poisson3d_main; do
  nm "$OUT/obj/$o.o" | awk -v src=$o '$2 == "T" && $3 ~ /^_Z[0-9]+k[A-Z]/ && $3 !~ /device_stub/ {
      name = $3; sub(/^_Z[0-9]+/, "", name); len = substr($3, 3) + 0; print src, substr(name, 1, len), $3 }'
done > "$OUT/ref_kernels3d.names"
echo "built $OUT/ref_poisson3d.cubin ($(wc -l < "$OUT/ref_kernels3d.names") kernels)"
