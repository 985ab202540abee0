// poisson_case.cpp - the reference's Poisson2D driver flow (cases/Poisson2D/main.cu:87-183)
// written against include/gpupfem2/gpupfem2.hpp: load a DAT mesh, Dirichlet nodes,
// assemble, apply BCs, Jacobi-PCG then GMRES.  Prints iterations and the max error
// against sin(pi x) sin(pi y) (the mesh is the unit square, f = 2 pi^2 sin sin, u = 0).
#include <cmath>
#include <cstdio>
#include <vector>

#include "gpupfem2/gpupfem2.hpp"

using namespace gpupfem2;

int main(int argc, char** argv) {
    if (argc < 2) { fprintf(stderr, "usage: %s mesh.dat\n", argv[0]); return 2; }
    Mesh2D mesh;
    if (!mesh.loadMeshFromFile(argv[1])) return 1;
    const int n = mesh.numVertices();
    DirichletBCs bcs;
    std::vector<DirichletNode> hostBcs;
    for (unsigned i = 0; i < (unsigned)n; ++i) {
        const double2 p = mesh.getHostVertices()[i];
        if (std::fabs(p.x) < 2e-6 || std::fabs(p.x - 1.0) < 2e-6 || std::fabs(p.y) < 2e-6 || std::fabs(p.y - 1.0) < 2e-6)
            hostBcs.push_back({ i, 0.0 });
    }
    bcs.setupDirichletBCs(hostBcs);
    SparseMatrixCSR matrix(mesh);
    deviceVector<double> rhs, solution;
    rhs.allocate(n);
    solution.allocate(n);
    solution.clearValues();
    check(pf2_assemble_poisson(mesh.handle(), matrix.handle(), rhs.data, PF2_RHS_SINSIN, 1.0, nullptr, nullptr),
          "pf2_assemble_poisson");
    bcs.applyBCs(matrix, rhs);
    LinearAlgebra LA;
    PreconditionerJacobi precond(n, &LA);
    SolverCG cg(1e-10, 2000, &LA, &precond);
    cg.init(matrix);
    const bool ok = cg.solve(matrix, solution, rhs);
    const int cgIt = cg.lastInfo().iterations;
    SolverGMRES gmres(1e-10, 1000, &LA, &precond);
    gmres.init(matrix);
    const bool ok2 = gmres.solve(matrix, solution, rhs);
    const std::vector<double> x = solution.toHost();
    double err = 0.0;
    for (int i = 0; i < n; ++i) {
        const double2 p = mesh.getHostVertices()[i];
        err = std::fmax(err, std::fabs(x[i] - std::sin(M_PI * p.x) * std::sin(M_PI * p.y)));
    }
    printf("cg_converged=%d cg_iterations=%d gmres_converged=%d gmres_iterations=%d max_error=%.6e\n", ok, cgIt, ok2,
           gmres.lastInfo().iterations, err);
    return (ok && ok2) ? 0 : 3;
}
