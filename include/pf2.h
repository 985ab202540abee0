/*
 * pf2.h - C ABI of the GB300-native PFEM-2 time-step engine.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and returns a
 * pf2_status; none allocates or frees user memory.  Objects (mesh, CSR matrix,
 * Dirichlet set, solver, particle set, flow engine) own their device memory; device
 * pointers handed out by the *_view functions stay valid until the object is destroyed
 * (particle arrays until the next call that changes the particle count).  `stream` is
 * a cudaStream_t (NULL = the legacy default stream); work is enqueued on it and the
 * call returns without waiting unless its comment says "synchronises".
 *
 * Each declaration names the reference interface it replaces (andreyypopov/gpuPfem2,
 * paths relative to its source tree).  The reference reports failures by exit()
 * (src/common/cuda_helper.cuh:32-94) or by a bool plus printf; here they come back as a
 * status, and pf2_last_error() holds the message of the calling thread's last failure.
 */
#ifndef PF2_H
#define PF2_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PF2_ABI_VERSION 1

typedef enum pf2_status {
    PF2_OK = 0,
    PF2_NOT_CONVERGED = 1, /* solver hit maxit (reference: solve() returns false) */
    PF2_BAD_INPUT = 2,     /* invalid argument, mesh or size                      */
    PF2_OVERFLOW = 3,      /* a fixed-capacity buffer (particles) would overflow  */
    PF2_CUDA_ERROR = 4,    /* a CUDA runtime call failed                          */
    PF2_TIMEOUT = 5,       /* a bounded device-side wait gave up                  */
    PF2_IO_ERROR = 6       /* file could not be read                              */
} pf2_status;

typedef struct pf2_mesh pf2_mesh;
typedef struct pf2_csr pf2_csr;
typedef struct pf2_bc pf2_bc;
typedef struct pf2_solver pf2_solver;
typedef struct pf2_particles pf2_particles;
typedef struct pf2_flow pf2_flow;

/* Message of the calling thread's last failed call ("" if none). */
const char* pf2_last_error(void);
const char* pf2_status_string(pf2_status s);
int pf2_abi_version(void);
/* Number of kernels the engine has launched in this process (diagnostics; no
 * reference counterpart). */
unsigned long long pf2_kernel_launches(void);

/* ------------------------------------------------------------------ Mesh2D
 * Replaces Mesh2D (src/mesh_2d.cuh:11-69). */

/* Mesh2D::loadMeshFromFile(filename, fillNeighborLists, scale), src/mesh_2d.cu:36-96:
 * SALOME DAT, triangles (type 203) kept, other entities skipped, 1-based ids.
 * Builds cell areas and inverse Jacobians (mesh_2d.cu:10-34, :98-105), the
 * vertex-sharing neighbour lists (mesh_2d.cu:107-139) when fill_neighbors != 0, and the
 * node incidence and CSR pattern the assembly uses.  Synchronises. */
pf2_status pf2_mesh_load_dat(const char* path, int fill_neighbors, double scale, void* stream, pf2_mesh** out);

/* The same mesh from host arrays: xy[2*nv] (x,y pairs), tri[3*nc] (0-based). Synchronises. */
pf2_status pf2_mesh_create(int nv, const double* xy, int nc, const int* tri, int fill_neighbors,
                           void* stream, pf2_mesh** out);
pf2_status pf2_mesh_destroy(pf2_mesh* mesh);
pf2_status pf2_mesh_sizes(const pf2_mesh* mesh, int* nv, int* nc, int* n_neighbor_entries);

/* Device arrays of the mesh (Mesh2D::getVertices/getCells/getCellArea/getInvJacobi/
 * getCellNeighborsOffsets/getCellNeighborIndices/getEdgeBoundaryIDs, mesh_2d.cuh:18-44).
 * xy: double2[nv]; tri: int[3*nc]; area: double[nc]; inv_jacobi: double[4*nc] row-major;
 * neighbor_offsets: int[nc+1]; neighbor_indices: int[n]; edge_ids: int[3*nc]. */
typedef struct pf2_mesh_view {
    int nv, nc, n_neighbor_entries;
    const double* xy;
    const int* tri;
    const double* area;
    const double* inv_jacobi;
    const int* neighbor_offsets;
    const int* neighbor_indices;
    const int* edge_boundary_ids;
} pf2_mesh_view;
pf2_status pf2_mesh_view_get(const pf2_mesh* mesh, pf2_mesh_view* out);

enum { PF2_MESH_XY = 0, PF2_MESH_TRI = 1, PF2_MESH_AREA = 2, PF2_MESH_INV_JACOBI = 3,
       PF2_MESH_NEIGHBOR_OFFSETS = 4, PF2_MESH_NEIGHBOR_INDICES = 5, PF2_MESH_EDGE_IDS = 6 };
/* Copies one mesh array to host memory (sizes as in pf2_mesh_view). Synchronises. */
pf2_status pf2_mesh_download(const pf2_mesh* mesh, int field, void* host_dst);

/* kSetEdgeBoundaryIDs of the channel drivers (cases/Cylinder2D/main.cu:35-70): edge i of
 * a cell (vertex i -> vertex (i+1)%3) gets 0 inlet x=0, 1 outlet x=lx, 2 walls y=0 or
 * y=ly, 3 cylinder (|midpoint - c| - r| < 0.001 when has_cylinder), else -1. */
pf2_status pf2_mesh_set_channel_boundary_ids(pf2_mesh* mesh, double lx, double ly, int has_cylinder,
                                             double cx, double cy, double r, void* stream);
/* Edge boundary ids from host memory, int[3*nc]. */
pf2_status pf2_mesh_set_edge_boundary_ids(pf2_mesh* mesh, const int* ids_host);

/* --------------------------------------------------------- SparseMatrixCSR
 * Replaces SparseMatrixCSR (src/linear_algebra/sparse_matrix.cuh:9-58). */

/* SparseMatrixCSR(const Mesh2D&), sparse_matrix.cu:8-54: rows = nodes, columns =
 * {i} U edge neighbours, ascending, int32 offsets/indices, double values (zeroed).  All
 * matrices of one mesh share the mesh's pattern arrays. */
pf2_status pf2_csr_create(const pf2_mesh* mesh, pf2_csr** out);
pf2_status pf2_csr_destroy(pf2_csr* A);
/* getRows(), getTotalElements() */
pf2_status pf2_csr_sizes(const pf2_csr* A, int* rows, int* nnz);
/* getRowOffset(), getColIndices(), getMatrixValues(): device pointers */
pf2_status pf2_csr_view(const pf2_csr* A, const int** row_offsets, const int** col_indices, double** values);
/* clearValues(), sparse_matrix.cuh:50-52 */
pf2_status pf2_csr_clear_values(pf2_csr* A, void* stream);
/* Copies pattern and/or values to host (NULL skips). Synchronises. */
pf2_status pf2_csr_download(const pf2_csr* A, int* row_offsets, int* col_indices, double* values);
pf2_status pf2_csr_upload_values(pf2_csr* A, const double* values_host);

/* ------------------------------------------------------------ DirichletBCs
 * Replaces DirichletBCs (src/Dirichlet_bcs.cuh:14-29).  pf2_dirichlet_node has the
 * layout of the reference's DirichletNode {unsigned nodeIdx; double bcValue}. */
typedef struct pf2_dirichlet_node {
    unsigned int node;
    double value;
} pf2_dirichlet_node;

/* setupDirichletBCs + setupNodeMap (Dirichlet_bcs.cu:53-71). */
pf2_status pf2_bc_create(int n_nodes, int n_bc, const pf2_dirichlet_node* nodes_host, pf2_bc** out);
pf2_status pf2_bc_destroy(pf2_bc* bc);
pf2_status pf2_bc_size(const pf2_bc* bc, int* n_bc);
/* Replaces the boundary values (device double[n_bc]). */
pf2_status pf2_bc_set_values(pf2_bc* bc, const double* values_dev, void* stream);
/* Copies the current boundary values to device memory double[n_bc]. */
pf2_status pf2_bc_get_values(const pf2_bc* bc, double* values_dev, void* stream);
/* DirichletBCs::applyBCs(matrix, rhs), Dirichlet_bcs.cu:73-86: boundary rows -> e_i with
 * rhs g; other rows lose their boundary columns (rhs_r -= a_rd g_d), unless the row's
 * first off-diagonal value, read before elimination, is below 2e-6 in magnitude. */
pf2_status pf2_bc_apply(const pf2_bc* bc, pf2_csr* A, double* rhs_dev, void* stream);

/* ------------------------------------------------------ Assembly (integrators)
 * The reference's assembly entry points live in its case drivers; each function below
 * assembles matrix values and rhs (overwriting them: clearValues + assemble), and with
 * a non-NULL bc applies the Dirichlet rule of pf2_bc_apply in the same pass. */

enum { PF2_RHS_GAUSSIAN = 0, /* exp(-(x^2+10y^2)), cases/Poisson2D/main.cu:24-26 */
       PF2_RHS_SINSIN = 1 /* 2 pi^2 sin(pi x) sin(pi y) */ };

/* PoissonIntegrator::assembleSystem, cases/Poisson2D/main.cu:28-85 (lambda = 0.5 in the
 * shipped case): A_ij = lambda int grad N_i . grad N_j, b_i = int f N_i, 3-point rule. */
pf2_status pf2_assemble_poisson(const pf2_mesh* mesh, pf2_csr* A, double* rhs_dev, int rhs_kind, double lambda,
                                const pf2_bc* bc, void* stream);

/* ------------------------------------------------------- Mesh3D / Poisson3D
 * Replaces Mesh3D (src/mesh_3d.cuh:11-70), SparseMatrixCSR(const Mesh3D&)
 * (sparse_matrix.cu:56-97), the Poisson3D integrator (cases/Poisson3D/main.cu:26-85)
 * and DataExport3D (src/data_export_3d.cuh:9-23): linear tetrahedra. */
typedef struct pf2_mesh3d pf2_mesh3d;
/* Mesh3D::loadMeshFromFile(path, fillNeighborLists, scale), mesh_3d.cu:84-147: DAT file
 * with "nv ne", nv lines "id x y z", then entities "id type v..." of which type 304
 * (tetrahedron, 1-based vertex ids) are kept; 102 and 203 entities are skipped. */
pf2_status pf2_mesh3d_load_dat(const char* path, int fill_neighbors, double scale, void* stream, pf2_mesh3d** out);
/* From host arrays: xyz double[3*nv], tet int[4*nc] (0-based).  Builds the cell volumes
 * and inverse Jacobians (kCalculateCellVolume / kCalculateInvJacobi, mesh_3d.cu:12-35:
 * J has rows v0 - v3, v1 - v3, v2 - v3), the face-sharing neighbour lists of
 * fillCellNeighborIndices (mesh_3d.cu:37-82,198-227: cells sharing 3 vertices,
 * ascending) when fill_neighbors != 0, and the CSR pattern of the node graph. */
pf2_status pf2_mesh3d_create(int nv, const double* xyz, int nc, const int* tet, int fill_neighbors, void* stream,
                             pf2_mesh3d** out);
pf2_status pf2_mesh3d_destroy(pf2_mesh3d* mesh);
pf2_status pf2_mesh3d_sizes(const pf2_mesh3d* mesh, int* nv, int* nc, int* n_neighbor_entries);
/* Device arrays of the mesh (Mesh3D getters, mesh_3d.cuh:18-52).  xyz4 holds (x, y, z, 0)
 * per vertex (a 32-byte stride, not the reference's 24-byte Point3); inv_jacobi holds 9
 * doubles per cell, row-major (the reference's GenericMatrix3x3 adds a vtable slot). */
typedef struct pf2_mesh3d_view {
    int nv, nc, n_neighbor_entries;
    const double* xyz4;
    const int* tet;
    const double* volume;
    const double* inv_jacobi;
    const int* neighbor_offsets;
    const int* neighbor_indices;
} pf2_mesh3d_view;
pf2_status pf2_mesh3d_view_get(const pf2_mesh3d* mesh, pf2_mesh3d_view* out);
enum { PF2_MESH3D_XYZ = 0,              /* double[3*nv] */
       PF2_MESH3D_TET = 1,              /* int[4*nc] */
       PF2_MESH3D_VOLUME = 2,           /* double[nc] */
       PF2_MESH3D_INV_JACOBI = 3,       /* double[9*nc], row-major */
       PF2_MESH3D_NEIGHBOR_OFFSETS = 4, /* int[nc+1] */
       PF2_MESH3D_NEIGHBOR_INDICES = 5  /* int[n_neighbor_entries] */ };
/* Copies one mesh array to host memory. Synchronises. */
pf2_status pf2_mesh3d_download(const pf2_mesh3d* mesh, int field, void* host_dst);
/* SparseMatrixCSR(const Mesh3D&): rows = nodes, columns = {i} U nodes sharing a
 * tetrahedron with i, ascending; values zeroed.  Usable with every solver and with
 * pf2_bc_apply. */
pf2_status pf2_csr_create_3d(const pf2_mesh3d* mesh, pf2_csr** out);

enum { PF2_RHS3D_GAUSSIAN = 0, /* exp(-(x^2+10y^2+z^2)), cases/Poisson3D/main.cu:22-24 */
       PF2_RHS3D_SINSINSIN = 1 /* 3 pi^2 sin(pi x) sin(pi y) sin(pi z) */ };
/* PoissonIntegrator::assembleSystem of cases/Poisson3D/main.cu:26-85: A_ij = lambda
 * int grad N_i . grad N_j, b_i = int f N_i with the 6-point rule of
 * createCellQuadratureFormula(1) (quadrature_formula_3d.cu); overwrites A's values and
 * rhs; applies bc (pf2_bc_apply) when non-NULL. */
pf2_status pf2_assemble_poisson_3d(const pf2_mesh3d* mesh, pf2_csr* A, double* rhs_dev, int rhs_kind, double lambda,
                                   const pf2_bc* bc, void* stream);
/* DataExport3D::exportToVTK (data_export_3d.cu:15-93): ASCII VTU, tetrahedra as VTK type
 * 10, one Float32 point array per field (device double[nv]). */
pf2_status pf2_export_vtu_3d(const pf2_mesh3d* mesh, const char* path, int nfields, const char* const* names,
                             const double* const* fields_dev, void* stream);

/* SimulationParameters, src/parameters.cuh:6-51 (the fields the step uses). */
typedef struct pf2_params {
    double rho, mu, dt, tolerance;
    int max_iterations;
    int scheme;            /* 0 = Scheme A, 1 = Scheme B (pressure increment) */
    int substeps;          /* particleAdvectionSubsteps */
    int level;             /* cellDivisionLevel: level^2 particles per cell, 1..4 */
    int n_outer;           /* outer iterations of the step (2 in Cylinder2D, 1 in PoiseuilleFlow2D) */
    int pressure_precond;  /* PF2_PRECOND_* for the pressure solve */
    int calculate_loads, body_boundary_id;
    double thickness, mean_velocity;
    double body_cx, body_cy; /* body centre for the load normals (0.2, 0.2 in Cylinder2D/main.cu:344) */
    int pressure_precision;  /* PF2_PRECISION_* for the pressure solve */
    int pressure_x0;         /* PF2_X0_* for the pressure solve: GIVEN starts from the previous
                                pressure p (the reference); LEARNED from the energy-norm Galerkin
                                start over the network's increment and the last 8 increments */
    int gmres_restart;       /* Krylov dimension of the prediction GMRES, 0 = no restart */
    int pressure_criterion;  /* PF2_CRITERION_* of the pressure solve */
    int learn_steps;         /* PF2_X0_LEARNED: train the network on the first learn_steps steps */
    float learn_rate;        /* AdamW learning rate of that training */
    int pressure_ordering;   /* PF2_ORDERING_* of an ILU(0)/IC(0) pressure preconditioner */
    int gmres_orthogonalization; /* PF2_GS_* of the prediction GMRES */
    int cg_variant;          /* PF2_CG_* of the pressure and correction CG solves */
    int prediction_solver;   /* PF2_SOLVER_GMRES (the reference's) or PF2_SOLVER_BICGSTAB */
    double pressure_tolerance;   /* tolerance of the pressure solve; 0 = tolerance (the reference
                                    has one tolerance for every solve) */
    int pressure_max_iterations; /* iteration limit of the pressure solve; 0 = max_iterations */
} pf2_params;
/* SimulationParameters::setDefaultParameters(), parameters.cuh:30-50 */
pf2_status pf2_params_default(pf2_params* p);

/* kIntegrateVelocityPrediction (cases/Cylinder2D/main.cu:72-167): rho M + mu dt K_visc
 * with the outlet edge term on boundary id 1; rhs from u_old, u and (Scheme B) p_old.
 * ux/uy: current velocity, ux_old/uy_old: projected velocity, p_old may be NULL. */
pf2_status pf2_assemble_velocity_prediction(const pf2_mesh* mesh, const pf2_params* p,
                                            const double* ux, const double* uy,
                                            const double* ux_old, const double* uy_old, const double* p_old,
                                            pf2_csr* Ax, pf2_csr* Ay, double* rhs_x, double* rhs_y,
                                            const pf2_bc* bc_x, const pf2_bc* bc_y, void* stream);
/* kIntegratePressureEquation (:169-211). */
pf2_status pf2_assemble_pressure(const pf2_mesh* mesh, const pf2_params* p, const double* pred_x,
                                 const double* pred_y, const double* p_old, pf2_csr* A, double* rhs,
                                 const pf2_bc* bc, void* stream);
/* kIntegrateVelocityCorrection (:213-259). */
pf2_status pf2_assemble_velocity_correction(const pf2_mesh* mesh, const pf2_params* p, const double* pred_x,
                                            const double* pred_y, const double* pressure, const double* p_old,
                                            pf2_csr* Ax, pf2_csr* Ay, double* rhs_x, double* rhs_y,
                                            const pf2_bc* bc_x, const pf2_bc* bc_y, void* stream);
/* VelocityDirichletBCs::setDirichletValues (:467-479, kernels :261-297): writes into
 * `target` the values of `source` plus dt/rho * area-weighted pressure gradient
 * (component 0/1) at each boundary node.  source and target share the node list. */
pf2_status pf2_prediction_bc_values(const pf2_mesh* mesh, const pf2_params* p, const pf2_bc* source,
                                    pf2_bc* target, const double* pressure, const double* p_old, int component,
                                    void* stream);
/* boundaryLoadsCalculator::calculateLoads (:414-428, kernels :299-376): drag and lift
 * coefficients on the edges with body_boundary_id; cxcy_host[2]. The body centre is
 * (cx, cy).  Synchronises. */
pf2_status pf2_body_loads(const pf2_mesh* mesh, const pf2_params* p, double cx, double cy, const double* ux,
                          const double* uy, const double* pressure, double* cxcy_host, void* stream);

/* ---------------------------------------------------------------- Solvers
 * Replaces LinearSolver/SolverCG/SolverGMRES (src/linear_algebra/linear_solver.cuh:15-137)
 * and Preconditioner{Jacobi,ILU,IC} (src/linear_algebra/preconditioners.cuh:9-106). */
enum { PF2_SOLVER_CG = 0, PF2_SOLVER_GMRES = 1,
       PF2_SOLVER_BICGSTAB = 2 /* no reference counterpart: right-preconditioned BiCGStab,
                                  Jacobi or no preconditioner, FP64 */ };
enum { PF2_PRECOND_NONE = -1, PF2_PRECOND_JACOBI = 0, PF2_PRECOND_ILU = 1, PF2_PRECOND_IC = 2 };
enum { PF2_CRITERION_ABS = 0,   /* CG: r^T z < tol^2; GMRES: |beta_k| < tol (the reference's) */
       PF2_CRITERION_REL = 1 }; /* ||b - A x|| <= tol ||b|| */
enum { PF2_PRECISION_FP64 = 0,    /* the reference's FP64 PCG */
       PF2_PRECISION_MIXED = 1 };  /* CG iteration in FP32 (FP64 sums across threads) with reliable
                                      updates: x += d, r = b - A x and the test in FP64 whenever
                                      the iterated residual drops to 0.3 of the last true
                                      residual; CG only */
enum { PF2_X0_GIVEN = 0, PF2_X0_LEARNED = 1 };
enum { PF2_ORDERING_NATURAL = 0,    /* ILU(0)/IC(0) on A as numbered (the reference's)     */
       PF2_ORDERING_MULTICOLOR = 1 }; /* on P A P^T, P a greedy colouring whose thin tail of
                                        high colours is moved down by Kempe-chain swaps (4
                                        colours on the cylinder meshes): a different
                                        preconditioner, parallel triangular solves */
enum { PF2_GS_MODIFIED = 0,           /* GMRES Gram-Schmidt as the reference (linear_solver.cu:480-487) */
       PF2_GS_CLASSICAL_TWICE = 1 };  /* classical Gram-Schmidt with one reorthogonalisation */
enum { PF2_CG_STANDARD = 0,           /* PCG as the reference (linear_solver.cu:301-376): two
                                         grid-wide reductions per iteration */
       PF2_CG_ONE_REDUCTION = 1,      /* Chronopoulos-Gear PCG: the same iterates in exact
                                         arithmetic with r.z, (A z).z and r.r in one reduction;
                                         FP64 with Jacobi/none, or ILU(0)/IC(0) on few-level
                                         orderings (else the standard iteration runs) */
       PF2_CG_PIPELINED = 2 };        /* pipelined PCG (Ghysels-Vanroose 2014): the same
                                         iterates in exact arithmetic with one grid-wide step
                                         per iteration; FP64 ILU(0)/IC(0) on few-level
                                         orderings (else the standard iteration runs) */

typedef struct pf2_solver_options {
    int kind;          /* PF2_SOLVER_* */
    int precond;       /* PF2_PRECOND_* */
    double tolerance;
    int max_iterations;
    int criterion;     /* PF2_CRITERION_* */
    int precision;     /* PF2_PRECISION_* (CG only; MIXED always stops on ||b - A x|| <= tol ||b||) */
    int restart;       /* GMRES Krylov dimension; 0 = max_iterations (no restart, as the reference) */
    int ordering;      /* PF2_ORDERING_* of ILU(0)/IC(0) */
    int orthogonalization; /* GMRES: PF2_GS_MODIFIED (the reference's, one reduction per basis
                              vector) or PF2_GS_CLASSICAL_TWICE (two batched reductions) */
    int cg_variant;        /* CG: PF2_CG_* */
} pf2_solver_options;

/* The multicolour order of PF2_ORDERING_MULTICOLOR for a symmetric CSR pattern (host
 * arrays; no GPU work): perm[r] = row of A at position r of P A P^T; starts receives
 * *nstarts (<= n + 1) sweep-group starts ending with n (NULL: sizes only); kempe != 0
 * moves greedy colouring's tail of high colours down by Kempe-chain swaps (the solver's
 * choice), 0 keeps greedy's colours. */
pf2_status pf2_multicolour_order(int n, const int* rowptr, const int* col, int kempe, int* perm, int* ncolours,
                                 int* nstarts, int* starts);

/* The row partition of the partitioned CG solve (host arrays; no GPU work): part[i] in
 * [0, parts) for each row of a symmetric CSR pattern, by recursive bisection of its graph
 * in breadth-first order from a pseudo-peripheral node; part sizes differ by at most one
 * row per bisection level.  The solver cuts a CG system into one part per SM (at least
 * 512 rows each) and keeps each part's vectors in that block's shared memory; no
 * reference counterpart (the reference's CG runs on cuSPARSE / cuBLAS). */
pf2_status pf2_graph_parts(int n, const int* rowptr, const int* col, int parts, int* part);

typedef struct pf2_solve_info {
    int iterations;      /* total inner iterations */
    int converged;
    double residual;     /* sqrt(r^T z) (CG, ABS), |beta| (GMRES), or ||r||/||b|| (REL) */
    int outer_iterations; /* refinement sweeps (mixed precision) */
    int status;          /* pf2_status of the device-side run */
} pf2_solve_info;

/* SolverCG/SolverGMRES(tol, maxIt, LA, precond) + init(A): allocates the work vectors
 * for A's size (and the factor storage of ILU/IC). */
pf2_status pf2_solver_create(const pf2_csr* A, const pf2_solver_options* opt, pf2_solver** out);
pf2_status pf2_solver_destroy(pf2_solver* s);
/* solve(A, x, b) -> bool: x (device, in/out: initial guess in, solution out), b device.
 * Preconditioner::initialize(A) runs inside, as in the reference (ILU/IC factorise A).
 * Returns PF2_NOT_CONVERGED when maxit is reached.  info may be NULL; when non-NULL the
 * call synchronises to fill it. */
pf2_status pf2_solver_solve(pf2_solver* s, const pf2_csr* A, double* x, const double* b, pf2_solve_info* info,
                            void* stream);
/* Preconditioner::applyPreconditioner(dest, src) with the factors of the last solve or
 * pf2_solver_setup(). */
pf2_status pf2_solver_setup(pf2_solver* s, const pf2_csr* A, void* stream);
pf2_status pf2_precond_apply(pf2_solver* s, double* dst, const double* src, void* stream);

/* y = A x (device vectors); the cusparseSpMV call of LinearAlgebra::sparseMV
 * (src/linear_algebra/linear_algebra.h:56-80). */
pf2_status pf2_spmv(const pf2_csr* A, const double* x, double* y, void* stream);

/* ------------------------------------------------------------------ Output
 * DataExport::exportToVTK (src/data_export.cu:17-122): the mesh and `nfields` node
 * fields (device arrays of mesh nodes, named by `names`) as an ASCII VTU file in the
 * reference's layout (Float32 points and data, triangles as VTK type 5).  Synchronises. */
pf2_status pf2_export_vtu(const pf2_mesh* mesh, const char* path, int nfields, const char* const* names,
                          const double* const* fields, void* stream);
/* DataExport::exportParticlesToVTK (src/data_export.cu:124-171): particle positions as
 * VTK vertices with their velocity.  Synchronises. */
pf2_status pf2_export_particles_vtu(const pf2_particles* ph, const char* path);

/* Jacobi-preconditioned CG that allocates no memory (no reference counterpart): the same
 * kernel and arithmetic as a PF2_SOLVER_CG / PF2_PRECOND_JACOBI solver from
 * pf2_solver_create + pf2_solver_solve, with its work vectors in a fixed file-scope device
 * array of the library sized for PF2_STATIC_MAX_ROWS rows (about 5.3 MB).  For callers
 * that must not allocate device memory per solve: a loop of many small solves where a
 * cudaMalloc/cudaFree pair per solve would dominate (and cudaFree synchronises the
 * device, stalling work on other streams), or a program whose remaining device memory is
 * held by its own pool so that a new allocation would fail.
 * - A with more than PF2_STATIC_MAX_ROWS rows is rejected with PF2_BAD_INPUT.
 * - The barrier, error and timeout words are zeroed by this call (cudaMemsetAsync on
 *   `stream`) before the launch; nothing else needs to start at zero.  x is the initial
 *   guess in, the solution out, as in pf2_solver_solve.
 * - The storage is one per device: two calls whose work overlaps on one device (other
 *   streams, other host threads) race on it and give undefined results; order them.
 * - The first call on a device looks up the array's address (cudaGetSymbolAddress) and
 *   caches it; make that first call before any stream capture.  The cached address
 *   belongs to the device's current primary context: after cudaDeviceReset on that
 *   device it is stale, so do not call this function again in that process.
 * - The solve record in the array is cleared before each launch, so a device-side
 *   timeout reports no iterations rather than the previous call's.
 * info may be NULL (no synchronisation); otherwise the call synchronises `stream` and
 * fills it, returning PF2_NOT_CONVERGED when max_iterations is reached. */
enum { PF2_STATIC_MAX_ROWS = 131072 };
pf2_status pf2_pcg_jacobi_static(const pf2_csr* A, double* x, const double* b, double tolerance, int max_iterations,
                                 int criterion, pf2_solve_info* info, void* stream);

/* ------------------------------------------------------ ParticleHandler2D
 * Replaces ParticleHandler2D (src/particles/particle_handler_2d.cuh:9-54).  Velocity
 * fields are two device arrays (the reference passes a device array of two device
 * pointers, deviceVector<double*>). */

/* ParticleHandler2D(mesh, cellDivisionLevel): level clamped to [1,4]; capacity =
 * capacity_factor * level^2 * nc particles (>= 1.1, the reference's resize margin). */
pf2_status pf2_particles_create(const pf2_mesh* mesh, int level, double capacity_factor, pf2_particles** out);
pf2_status pf2_particles_destroy(pf2_particles* ph);
/* seedParticles(), particle_handler_2d.cu:304-320: level^2 particles per cell at the
 * sub-triangle centroids, zero velocity, ordered by cell. */
pf2_status pf2_particles_seed(pf2_particles* ph, void* stream);
/* initParticleVelocity(u), :322-326 */
pf2_status pf2_particles_init_velocity(pf2_particles* ph, const double* ux, const double* uy, void* stream);
/* advectParticles(u, dt, substeps), :328-342: advection, cell location (own cell, then
 * vertex-sharing neighbours in ascending order), deletion of particles not found, then
 * the sub-cell population check and reseed.  Particles end up ordered by cell. */
pf2_status pf2_particles_advect(pf2_particles* ph, const double* ux, const double* uy, double dt, int substeps,
                                void* stream);
/* correctParticleVelocity(u, u_old), :344-348 */
pf2_status pf2_particles_correct(pf2_particles* ph, const double* ux, const double* uy, const double* ux_old,
                                 const double* uy_old, void* stream);
/* projectVelocityOntoGrid(u), :350-361: u_node = sum L_i v_p / sum L_i. */
pf2_status pf2_particles_project(pf2_particles* ph, double* ux, double* uy, void* stream);
/* getParticleCount(). Synchronises. */
pf2_status pf2_particles_count(const pf2_particles* ph, int* count);
/* getParticles(): copies the particle state to host arrays (NULL skips a field); l2 is
 * the third barycentric coordinate; cell is the containing cell. Synchronises. */
pf2_status pf2_particles_download(const pf2_particles* ph, double* x, double* y, double* l0, double* l1,
                                  double* l2, double* u, double* v, int* cell);
/* Replaces the particle state from host arrays (l2 taken as 1 - l0 - l1 unless it
 * differs, in which case the particle keeps it until it is next located).  Particles
 * are reordered by cell.  Synchronises. */
pf2_status pf2_particles_upload(pf2_particles* ph, int n, const double* x, const double* y, const double* l0,
                                const double* l1, const double* l2, const double* u, const double* v,
                                const int* cell);

/* ---------------------------------------------------- Checkpoint / restart
 * No reference counterpart (its drivers always start from the seed).  A checkpoint is a
 * binary file: magic "PF2CKPT", format version, object kind, then tagged sections, each
 * with its length.  Loading checks every section against the receiving object (mesh
 * size, level, capacity, parameter count) and fails with PF2_BAD_INPUT naming the first
 * section that differs (PF2_OVERFLOW: more particles than the capacity; PF2_IO_ERROR:
 * the file cannot be opened).  A load that fails part-way leaves the object's state
 * unspecified.  All synchronise.
 * Particles: count, x, y, l0, l1, u, v, the cell words (with the sub-cell marks) and the
 * cell segments of the last sort, so that a restored handler continues exactly. */
/* Grows the particle buffers to hold `capacity` particles, keeping the particles (the
 * reference reallocates its particle vector when reseeding outgrows it).  The flow
 * engine does this by itself before a step when the last step left them three
 * quarters full. Synchronises. */
pf2_status pf2_particles_reserve(pf2_particles* ph, long long capacity);
pf2_status pf2_particles_save(const pf2_particles* ph, const char* path);
pf2_status pf2_particles_load(pf2_particles* ph, const char* path);

/* ------------------------------------------------------------- Flow engine
 * One PFEM-2 time step of the channel drivers (cases/Cylinder2D/main.cu:793-880): the
 * state (particles, velocity, prediction, pressure, matrices, solvers) lives on the
 * device; pf2_flow_step enqueues the whole step without host round trips. */
pf2_status pf2_flow_create(const pf2_mesh* mesh, const pf2_params* p,
                           int n_bc_x, const pf2_dirichlet_node* bc_x,
                           int n_bc_y, const pf2_dirichlet_node* bc_y,
                           int n_bc_p, const pf2_dirichlet_node* bc_p, double particle_capacity_factor,
                           pf2_flow** out);
pf2_status pf2_flow_destroy(pf2_flow* f);
/* seedParticles + initParticleVelocity of the zero initial field. */
pf2_status pf2_flow_seed(pf2_flow* f, void* stream);
pf2_status pf2_flow_step(pf2_flow* f, void* stream);
/* From the second step on, pf2_flow_step replays the step as a CUDA graph captured on
 * the engine's own stream (on by default; 0 launches every kernel each step). */
pf2_status pf2_flow_set_graphs(pf2_flow* f, int enable);
enum { PF2_FIELD_UX = 0, PF2_FIELD_UY = 1, PF2_FIELD_UX_OLD = 2, PF2_FIELD_UY_OLD = 3, PF2_FIELD_PRED_X = 4,
       PF2_FIELD_PRED_Y = 5, PF2_FIELD_P = 6, PF2_FIELD_P_OLD = 7 };
pf2_status pf2_flow_field(pf2_flow* f, int which, double** device_ptr);
/* Host copies of a node field (double[nv]). Synchronise. */
pf2_status pf2_flow_download_field(pf2_flow* f, int which, double* host_dst);
pf2_status pf2_flow_upload_field(pf2_flow* f, int which, const double* host_src);
pf2_status pf2_flow_particles(pf2_flow* f, pf2_particles** ph);
/* The flow's own systems (0 prediction x, 1 prediction y, 2 pressure, 3 correction x,
 * 4 correction y) as assembled by the last step: matrix handle (owned by the flow) and
 * device rhs pointer. */
pf2_status pf2_flow_system(pf2_flow* f, int which, pf2_csr** A, double** rhs);
/* New values for a Dirichlet set of the flow (0 velocity x, 1 velocity y, 2 pressure),
 * device double[n_bc] in the order the set was created with (a time-dependent inflow). */
pf2_status pf2_flow_set_boundary_values(pf2_flow* f, int which, const double* values_dev, void* stream);
/* Checkpoint of the flow between steps: step count, the eight node fields, the values of
 * the three Dirichlet sets, the particles and (PF2_X0_LEARNED) the learned guess's
 * history, network parameters and AdamW moments.  Load into an engine created with the
 * same mesh, parameters and Dirichlet node sets; from there the steps repeat the
 * uninterrupted run bit for bit. */
pf2_status pf2_flow_save(pf2_flow* f, const char* path, void* stream);
pf2_status pf2_flow_load(pf2_flow* f, const char* path, void* stream);

typedef struct pf2_step_info {
    int particles;
    int it_prediction[2][8];
    int it_pressure[8];
    int it_correction[2][8];
    int converged;       /* all solves converged */
    int status;          /* first device-side error (pf2_status) */
    double cx, cy;       /* loads, when calculate_loads */
    int guess_used;      /* PF2_X0_LEARNED: 1 if the network's increment got a nonzero coefficient */
    double guess_residual[2]; /* ||b - A p|| of the previous pressure and ||b - A x0|| of the start */
    double pressure_residual[8]; /* ||r|| / ||b|| at the end of each pressure solve (the CG's
                                    iterated residual; the true residual for PF2_PRECISION_MIXED) */
} pf2_step_info;
/* Statistics of the last completed step. Synchronises. */
pf2_status pf2_flow_step_info(pf2_flow* f, pf2_step_info* info);

/* Per-phase device time of the steps (the reference prints per-phase ms with its
 * GpuTimer and NVTX scopes, src/common/gpu_timer.cuh, Cylinder2D/main.cu:795-879).
 * pf2_flow_enable_timing records CUDA events around each phase of the next max_steps
 * steps (0 disables); pf2_flow_phase_times sums them per phase (ms) over the recorded
 * steps and synchronises. */
enum { PF2_PHASE_PARTICLES = 0, PF2_PHASE_PROJECTION = 1, PF2_PHASE_PREDICTION_ASSEMBLY = 2,
       PF2_PHASE_PREDICTION_SOLVE = 3, PF2_PHASE_PRESSURE_ASSEMBLY = 4, PF2_PHASE_PRESSURE_SOLVE = 5,
       PF2_PHASE_CORRECTION_ASSEMBLY = 6, PF2_PHASE_CORRECTION_SOLVE = 7, PF2_PHASE_PARTICLE_CORRECTION = 8,
       PF2_PHASES = 9 };
pf2_status pf2_flow_enable_timing(pf2_flow* f, int max_steps);
pf2_status pf2_flow_phase_times(pf2_flow* f, double* ms_per_phase, int* steps);

/* ------------------------------------------------- Learned initial guess
 * No reference counterpart.  A message-passing network over the mesh graph (nodes;
 * edges = off-diagonal CSR entries): 5 input features per node, 64 hidden units, 3
 * layers (h0 = relu(W0 f + c0); h += relu(Wl [h ; mean of neighbours' h] + cl);
 * y = w4 . h + c4), FP32 master parameters, BF16 tensor-core MLPs with FP32
 * accumulation, training by AdamW (beta 0.9/0.999, eps 1e-8, weight decay 0.01) on the
 * device.  Parameter order: W0[64x5], c0, (Wl[64x128], cl) x 3, w4[64], c4. */
typedef struct pf2_mpnn pf2_mpnn;
pf2_status pf2_mpnn_create(const pf2_mesh* mesh, unsigned long long seed, pf2_mpnn** out);
pf2_status pf2_mpnn_destroy(pf2_mpnn* net);
int pf2_mpnn_param_count(void);
/* Host copies of the parameters / of the last gradient (NULL skips). Synchronise. */
pf2_status pf2_mpnn_set_params(pf2_mpnn* net, const float* params_host);
pf2_status pf2_mpnn_get_params(const pf2_mpnn* net, float* params_host, float* grad_host);
/* y = network(features); feat: device float[nv*5] node-major, y: device float[nv]. */
pf2_status pf2_mpnn_forward(pf2_mpnn* net, const float* feat, float* y, void* stream);
/* One training step on L = mean (y - target)^2: forward, backward (gradient kept for
 * pf2_mpnn_get_params) and, if apply != 0, an AdamW update with rate lr.  loss_host may
 * be NULL; when not, the call synchronises to fill it. */
pf2_status pf2_mpnn_train_step(pf2_mpnn* net, const float* feat, const float* target, float lr, int apply,
                               double* loss_host, void* stream);
/* The network's trained state (parameters, AdamW moments and step count) to or from a
 * checkpoint file. */
pf2_status pf2_mpnn_save(const pf2_mpnn* net, const char* path);
pf2_status pf2_mpnn_load(pf2_mpnn* net, const char* path);

#ifdef __cplusplus
}
#endif
#endif /* PF2_H */
