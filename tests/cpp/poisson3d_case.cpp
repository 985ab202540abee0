// poisson3d_case.cpp - the reference's Poisson3D driver flow (cases/Poisson3D/main.cu:86-176)
// written against include/gpupfem2/gpupfem2.hpp: load a DAT mesh of tetrahedra, the
// case's Dirichlet values on the six faces of the box, assemble (lambda 0.5, Gaussian
// source), apply BCs, Jacobi-PCG to 1e-8 with 1000 iterations at most, export VTU.
// Prints the iterations and the solution range.
#include <cmath>
#include <cstdio>
#include <vector>

#include "gpupfem2/gpupfem2.hpp"

using namespace gpupfem2;

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s mesh.dat out.vtu\n", argv[0]); return 2; }
    Mesh3D mesh;
    if (!mesh.loadMeshFromFile(argv[1])) return 1;
    const int n = mesh.numVertices();
    DirichletBCs bcs;
    std::vector<DirichletNode> hostBcs;
    for (unsigned i = 0; i < (unsigned)n; ++i) {
        const double3 p = mesh.getHostVertices()[i];
        if (std::fabs(p.x - (-1.0)) < 2e-6) hostBcs.push_back({ i, -1.0 });
        else if (std::fabs(p.x - 1.0) < 2e-6) hostBcs.push_back({ i, 1.0 });
        else if (std::fabs(p.y) < 2e-6) hostBcs.push_back({ i, 0.0 });
        else if (std::fabs(p.y - 1.0) < 2e-6) hostBcs.push_back({ i, 2.0 });
        else if (std::fabs(p.z - (-0.25)) < 2e-6) hostBcs.push_back({ i, 3.0 });
        else if (std::fabs(p.z - 0.25) < 2e-6) hostBcs.push_back({ i, -2.0 });
    }
    bcs.setupDirichletBCs(hostBcs);
    SparseMatrixCSR matrix(mesh);
    deviceVector<double> rhs, solution;
    rhs.allocate(n);
    rhs.clearValues();
    solution.allocate(n);
    solution.clearValues();
    check(pf2_assemble_poisson_3d(mesh.handle(), matrix.handle(), rhs.data, PF2_RHS3D_GAUSSIAN, 0.5, nullptr,
                                  nullptr),
          "pf2_assemble_poisson_3d");
    bcs.applyBCs(matrix, rhs);
    LinearAlgebra LA;
    PreconditionerJacobi precond(n, &LA);
    SolverCG cg(1e-8, 1000, &LA, &precond);
    cg.init(matrix);
    const bool ok = cg.solve(matrix, solution, rhs);
    DataExport3D dataExport(mesh);
    dataExport.addScalarDataVector(solution, "solution");
    dataExport.exportToVTK(argv[2]);
    const std::vector<double> x = solution.toHost();
    double lo = 1e300, hi = -1e300;
    for (double v : x) {
        lo = std::fmin(lo, v);
        hi = std::fmax(hi, v);
    }
    printf("cg_converged=%d cg_iterations=%d min=%.9g max=%.9g\n", ok, cg.lastInfo().iterations, lo, hi);
    return ok ? 0 : 3;
}
