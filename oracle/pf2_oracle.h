/*
 * pf2_oracle.h - CPU oracle for the PFEM-2 time-step path (TEST INFRASTRUCTURE ONLY).
 *
 * A single-thread FP64 C restatement of the reference gpuPfem2 algorithms on the
 * PFEM-2 step path.  Only the test suite, the smoke check and the CPU-baseline leg of
 * the benchmark load it, always as the checker; the product never links it.
 *
 * Conventions: 0-based node and cell indices, int32 CSR (row offsets + sorted column
 * indices), SoA particle arrays, all floating point in double.  Every function names
 * the reference file:line it restates.  Compiled with -ffp-contract=off: where the
 * reference's GPU code is contracted into fused multiply-adds by nvcc, the oracle calls
 * fma() explicitly at the same place (marked "FMA as nvcc contracts"), so results on
 * x86-64 and aarch64 hosts are identical.
 */
#ifndef PF2_ORACLE_H
#define PF2_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- constants (src/common/constants.h:4-17) ---- */
#define OR_DOUBLE_MIN 2e-6
#define OR_MAX_LEVEL 4

/* ---- quadrature (src/integration/quadrature_formula_2d.cu:17-24, _1d.cu:15-18) ---- */
int or_face_quadrature(int index, double* coords3, double* weights); /* returns #points */
int or_edge_quadrature(int index, double* coords, double* weights);

/* ---- mesh (src/mesh_2d.cu) ---- */
void or_mesh_geometry(int nc, const double* xy, const int* tri, double* area, double* invJ);
int or_node_cells(int nv, int nc, const int* tri, int* offsets, int* cells); /* CSR node->cells, ascending */
int or_neighbors(int nv, int nc, const int* tri, int* offsets, int* idx);   /* idx may be NULL: count only */
int or_csr_structure(int nv, int nc, const int* tri, int* rowptr, int* col); /* col may be NULL */
void or_edge_boundary_ids(int nc, const double* xy, const int* tri, double lx, double ly,
                          int has_cylinder, double cx, double cy, double r, int* ids3);

/* ---- CSR helpers ---- */
int or_find_in_row(const int* rowptr, const int* col, int row, int target);
void or_spmv(int n, const int* rowptr, const int* col, const double* val, const double* x, double* y);

/* ---- assembly ---- */
enum { OR_RHS_GAUSSIAN = 0, OR_RHS_SINSIN = 1 };
void or_assemble_poisson(int nc, const double* xy, const int* tri, const double* area, const double* invJ,
                         int rhs_kind, double lambda, const int* rowptr, const int* col, double* val, double* rhs);

/* ---- Dirichlet BCs (src/Dirichlet_bcs.cu) ---- */
void or_apply_bcs(int n, const int* rowptr, const int* col, double* val, double* rhs,
                  int nbc, const int* bc_node, const double* bc_val);

/* ---- solvers (src/linear_algebra/linear_solver.cu, preconditioners.cu) ---- */
enum { OR_PRECOND_NONE = -1, OR_PRECOND_JACOBI = 0, OR_PRECOND_ILU = 1, OR_PRECOND_IC = 2 };
typedef struct {
    int iterations;
    int converged;
    double residual; /* sqrt(r^T z) for CG, |beta_k| for GMRES */
} or_solve_info;
void or_ilu0(int n, const int* rowptr, const int* col, double* lu);   /* in place on a copy of A */
void or_ic0(int n, const int* rowptr, const int* col, double* l);     /* lower part holds L */
void or_precond_apply(int kind, int n, const int* rowptr, const int* col, const double* fact,
                      const double* invdiag, const double* src, double* dst, double* tmp);
int or_pcg(int n, const int* rowptr, const int* col, const double* val, double* x, const double* b,
           double tol, int maxit, int precond, or_solve_info* info);
int or_gmres(int n, const int* rowptr, const int* col, const double* val, double* x, const double* b,
             double tol, int maxit, int precond, or_solve_info* info);

/* ---- solver options of the engine beyond the reference (pf2_oracle_solvers.c) ---- */
/* Greedy colouring in row order with Kempe-chain trimming of the tail (kempe != 0);
 * perm[r] = row at position r of P A P^T, starts (may be NULL) gets the colour starts
 * and n.  Returns the number of colours. */
int or_multicolour_order(int n, const int* rowptr, const int* col, int kempe, int* perm, int* starts);
/* CG with ordering 0 (natural) / 1 (multicolour, ILU/IC only) and criterion 0 (r^T z <
 * tol^2, the reference's) / 1 (||r|| <= tol ||b||); rel_residual may be NULL. */
int or_cg(int n, const int* rowptr, const int* col, const double* val, double* x, const double* b, double tol,
          int maxit, int precond, int ordering, int criterion, or_solve_info* info, double* rel_residual);
/* Right-preconditioned BiCGStab, Jacobi or none; criterion 0: ||M^{-1} r|| < tol. */
int or_bicgstab(int n, const int* rowptr, const int* col, const double* val, double* x, const double* b,
                double tol, int maxit, int precond, int criterion, or_solve_info* info);
/* GMRES as or_gmres with classical Gram-Schmidt applied twice (DGKS test, 0.7). */
int or_gmres_cgs2(int n, const int* rowptr, const int* col, const double* val, double* x, const double* b,
                  double tol, int maxit, int precond, or_solve_info* info);

/* ---- particles (src/particles/particle_handler_2d.cu) ---- */
int or_subcell_centers(int level, double* centers3);
int or_determine_subcell(int level, double step, const double* l3);
int or_seed(int nc, const double* xy, const int* tri, int level, const double* centers3,
            double* px, double* py, double* l0, double* l1, double* l2, double* pu, double* pv, int* cell);
void or_correct_velocity(int np, const int* tri, const int* cell, const double* l0, const double* l1,
                         const double* l2, const double* ux, const double* uy,
                         const double* ux_old, const double* uy_old, double* pu, double* pv);
void or_project(int np, const int* tri, const int* cell, const double* l0, const double* l1, const double* l2,
                const double* pu, const double* pv, int nv, double* ux, double* uy);
/* Advection with cell location over `substeps` substeps, then the population check and
 * reseed; the output is ordered by cell (stable), reseeded particles at the end of each
 * cell in sub-cell order.  Returns the new particle count, or -1 if cap is too small. */
int or_advect(int np, int cap, double* px, double* py, double* l0, double* l1, double* l2,
              double* pu, double* pv, int* cell,
              int nv, const double* xy, int nc, const int* tri, const double* invJ,
              const int* nb_off, const int* nb_idx, const double* ux, const double* uy,
              double dt, int substeps, int level, const double* centers3, int* n_deleted, int* n_added);
int or_locate(double x, double y, int cell, const double* xy, const int* tri, const double* invJ,
              const int* nb_off, const int* nb_idx, double* l3);

/* ---- flow (cases/Cylinder2D/main.cu) ---- */
typedef struct {
    double rho, mu, dt, tol;
    int maxit, scheme, substeps, level, n_outer, pressure_precond;
    int calc_loads, body_id;
    double thickness, mean_velocity;
    double lx, ly;
    int has_cylinder;
    double cx, cy, radius;
    /* solver choices of the engine (0 everywhere: the reference's) */
    int pressure_ordering;   /* 0 natural, 1 multicolour (ILU/IC) */
    int prediction_solver;   /* 0 or 1: GMRES, 2: BiCGStab (Jacobi) */
    int gmres_orth;          /* 0 modified Gram-Schmidt, 1 classical twice */
    int pressure_criterion;  /* 0 r^T z < tol^2, 1 ||r|| <= tol ||b|| */
    double pressure_tol;     /* 0: tol */
    int pressure_maxit;      /* 0: maxit */
} or_params;

typedef struct {
    int particles;
    int deleted, added;
    int it_pred[2][8], it_pres[8], it_corr[2][8];
    int conv_ok;
    double cx, cy;
    double res_pres[8]; /* ||r|| / ||b|| of each pressure solve's recursive residual at its end */
} or_step_info;

typedef struct or_flow or_flow;
or_flow* or_flow_create(int nv, const double* xy, int nc, const int* tri, const or_params* p,
                        int nbu, const int* bu_node, const double* bu_val,
                        int nbv, const int* bv_node, const double* bv_val,
                        int nbp, const int* bp_node, const double* bp_val, int particle_cap);
void or_flow_destroy(or_flow* f);
int or_flow_step(or_flow* f, or_step_info* info);
int or_flow_particle_count(const or_flow* f);
/* Changes the solver choices of the following steps (the or_params fields of the same
 * names); the state is kept. */
void or_flow_set_solvers(or_flow* f, int pressure_precond, int pressure_ordering, int prediction_solver,
                         int gmres_orth, int pressure_criterion);
/* field ids: 0 ux,1 uy,2 ux_old,3 uy_old,4 pred_x,5 pred_y,6 p,7 p_old */
void or_flow_get_field(const or_flow* f, int which, double* out);
void or_flow_set_field(or_flow* f, int which, const double* in);
void or_flow_get_particles(const or_flow* f, double* px, double* py, double* l0, double* l1, double* l2,
                           double* pu, double* pv, int* cell);
void or_flow_set_particles(or_flow* f, int np, const double* px, const double* py, const double* l0,
                           const double* l1, const double* l2, const double* pu, const double* pv, const int* cell);
int or_flow_csr_nnz(const or_flow* f);
/* matrix ids: 0 pred_x, 1 pred_y, 2 pressure, 3 corr_x, 4 corr_y; rhs ids the same */
void or_flow_get_matrix(const or_flow* f, int which, double* val, double* rhs);

/* The individual flow stages, on explicit arrays (used by the parity tests). */
void or_assemble_prediction(int nc, const double* xy, const int* tri, const double* area, const double* invJ,
                            const int* edge_ids, const or_params* p, const double* ux, const double* uy,
                            const double* ux_old, const double* uy_old, const double* p_old,
                            const int* rowptr, const int* col, double* val_x, double* val_y,
                            double* rhs_x, double* rhs_y);
void or_assemble_pressure(int nc, const int* tri, const double* area, const double* invJ, const or_params* p,
                          const double* predx, const double* predy, const double* p_old,
                          const int* rowptr, const int* col, double* val, double* rhs);
void or_assemble_correction(int nc, const int* tri, const double* area, const double* invJ, const or_params* p,
                            const double* predx, const double* predy, const double* pres, const double* p_old,
                            const int* rowptr, const int* col, double* val_x, double* val_y,
                            double* rhs_x, double* rhs_y);
void or_prediction_bc(int nc, const int* tri, const double* area, const double* invJ, const or_params* p,
                      const double* pres, const double* p_old, int nbc, const int* bc_node,
                      const double* bc_val, const int* node_to_bc, int component, double* out_val);
int or_body_loads(int nc, const double* xy, const int* tri, const double* invJ, const int* edge_ids,
                  const or_params* p, const double* ux, const double* uy, const double* pres, double* cxcy);

/* ---- learned initial guess: message-passing network (no reference counterpart) ----
 * Graph: mesh nodes, edges = off-diagonal CSR entries (symmetric), d_i = #neighbours.
 * features f_i (5): x, y, b, p^n, p^{n-1}, each already scaled by the caller.
 *   h0 = relu(W0 f + c0)                       W0: 64x5   (row-major, [out][in])
 *   l = 1..3: m_i = mean_{j in N(i)} h_j
 *             h  = h + relu(Wl [h ; m] + cl)   Wl: 64x128
 *   y_i = w4 . h_i + c4                        w4: 64
 * Parameter vector order: W0, c0, (W1, c1), (W2, c2), (W3, c3), w4, c4.
 * Loss L = (1/N) sum_i (y_i - t_i)^2.  or_mpnn_forward returns L (t may be NULL: y only);
 * or_mpnn_backward writes dL/dtheta. */
#define OR_MPNN_H 64
#define OR_MPNN_IN 5
#define OR_MPNN_LAYERS 3
int or_mpnn_param_count(void);
double or_mpnn_forward(int n, const int* rowptr, const int* col, const double* feat, const double* theta,
                       double* y, const double* t);
double or_mpnn_backward(int n, const int* rowptr, const int* col, const double* feat, const double* theta,
                        const double* t, double* grad);
void or_adamw(int np, double* theta, const double* grad, double* m, double* v, int step, double lr, double b1,
              double b2, double eps, double wd);

/* ---- 3D (pf2_oracle3d.c) ---- */
void or_mesh3d_geometry(int nc, const double* xyz, const int* tet, double* volume, double* invJ);
int or_mesh3d_neighbors(int nc, const int* tet, int* offsets, int* idx);   /* idx may be NULL */
int or_csr_structure_3d(int nv, int nc, const int* tet, int* rowptr, int* col); /* col may be NULL */
int or_cell_quadrature_3d(double* coords4, double* weights);
void or_assemble_poisson_3d(int nc, const double* xyz, const int* tet, const double* volume, const double* invJ,
                            int rhs_kind, double lambda, const int* rowptr, const int* col, double* val,
                            double* rhs);

#ifdef __cplusplus
}
#endif
#endif
