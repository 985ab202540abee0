// dump_ref_host3d.cu - runs the reference's 3D host-side setup on a mesh and dumps its
// results as raw little-endian arrays (TEST INFRASTRUCTURE ONLY; see stub_cudart.c).
//
// usage: ref_host_dump3d <mesh.dat> <out_prefix>
// writes <out_prefix>.{xyz.f64,tet.i32,rowptr.i32,col.i32,quad.f64}: the vertices and
// tetrahedra of Mesh3D::loadMeshFromFile (neighbour lists off: the reference builds them
// with GPU kernels), the pattern of SparseMatrixCSR(const Mesh3D&), and the rule of
// createCellQuadratureFormula(1) as (x, y, z, w, weight) per point.
#include <cstdio>
#include <string>
#include <vector>

#include "integration/quadrature_formula_3d.cuh"
#include "linear_algebra/sparse_matrix.cuh"
#include "mesh_3d.cuh"

template <class T>
static void dump(const std::string& path, const T* p, size_t n) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) { perror(path.c_str()); exit(1); }
    fwrite(p, sizeof(T), n, f);
    fclose(f);
}

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s mesh.dat out_prefix\n", argv[0]); return 1; }
    const std::string out = argv[2];
    Mesh3D mesh;
    if (!mesh.loadMeshFromFile(argv[1], false)) return 1;
    const auto& hv = mesh.getHostVertices();
    const auto& hc = mesh.getHostCells();
    dump(out + ".xyz.f64", reinterpret_cast<const double*>(hv.data()), 3 * hv.size());
    dump(out + ".tet.i32", reinterpret_cast<const unsigned*>(hc.data()), 4 * hc.size());
    SparseMatrixCSR A(mesh);
    dump(out + ".rowptr.i32", A.getRowOffset(), A.getRows() + 1);
    dump(out + ".col.i32", A.getColIndices(), A.getTotalElements());
    std::vector<double> q;
    for (const auto& gp : createCellQuadratureFormula(1)) {
        q.push_back(gp.coordinates.x); q.push_back(gp.coordinates.y); q.push_back(gp.coordinates.z);
        q.push_back(gp.coordinates.w); q.push_back(gp.weight);
    }
    dump(out + ".quad.f64", q.data(), q.size());
    printf("%s: %zu vertices, %zu tetrahedra, nnz %d\n", argv[1], hv.size(), hc.size(), A.getTotalElements());
    return 0;
}
