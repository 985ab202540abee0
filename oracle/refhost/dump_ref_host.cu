// dump_ref_host.cu - runs the reference's host-side setup on a mesh and dumps its
// results as raw little-endian arrays (TEST INFRASTRUCTURE ONLY; see stub_cudart.c).
//
// usage: ref_host_dump <mesh.dat> <out_prefix>
// writes <out_prefix>.{xy.f64,tri.i32,nboff.i32,nbidx.i32,rowptr.i32,col.i32} and, once,
// <out_prefix>.centers<L>.f64 for L = 1..4 and <out_prefix>.quad.f64.
#include <cstdio>
#include <string>
#include <vector>

#include "integration/quadrature_formula_1d.cuh"
#include "integration/quadrature_formula_2d.cuh"
#include "linear_algebra/sparse_matrix.cuh"
#include "mesh_2d.cuh"
#include "particles/particle_handler_2d.cuh"

extern __constant__ Point3 subcellCenters[CONSTANTS::MAX_PARTICLES_PER_CELL];

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
    Mesh2D mesh;
    if (!mesh.loadMeshFromFile(argv[1])) return 1;
    const auto& hv = mesh.getHostVertices();
    const auto& hc = mesh.getHostCells();
    dump(out + ".xy.f64", reinterpret_cast<const double*>(hv.data()), 2 * hv.size());
    dump(out + ".tri.i32", reinterpret_cast<const unsigned*>(hc.data()), 3 * hc.size());
    const int nc = mesh.getCells().size;  // device count (the host list can hold one more)
    dump(out + ".nboff.i32", mesh.getCellNeighborsOffsets().data, nc + 1);
    dump(out + ".nbidx.i32", mesh.getCellNeighborIndices().data, mesh.getCellNeighborIndices().size);
    SparseMatrixCSR A(mesh);
    dump(out + ".rowptr.i32", A.getRowOffset(), A.getRows() + 1);
    dump(out + ".col.i32", A.getColIndices(), A.getTotalElements());
    for (int L = 1; L <= 4; ++L) {
        ParticleHandler2D ph(&mesh, L);
        Point3 c[CONSTANTS::MAX_PARTICLES_PER_CELL];
        cudaMemcpyFromSymbol(c, subcellCenters, sizeof(c), 0, cudaMemcpyDeviceToHost);
        dump(out + ".centers" + std::to_string(L) + ".f64", reinterpret_cast<const double*>(c), 3 * L * L);
    }
    std::vector<double> q;
    for (const auto& gp : createFaceQuadratureFormula(1)) {
        q.push_back(gp.coordinates.x); q.push_back(gp.coordinates.y); q.push_back(gp.coordinates.z); q.push_back(gp.weight);
    }
    for (const auto& gp : createEdgeQuadratureFormula(1)) { q.push_back(gp.coordinate); q.push_back(gp.weight); }
    dump(out + ".quad.f64", q.data(), q.size());
    printf("%s: %zu vertices, %d cells (host list %zu), %d neighbour entries, nnz %d\n", argv[1], hv.size(), nc,
           hc.size(), mesh.getCellNeighborIndices().size, A.getTotalElements());
    return 0;
}
