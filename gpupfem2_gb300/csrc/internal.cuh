// internal.cuh - entry points shared between the translation units of the engine.
#pragma once

#include "common.cuh"

namespace pf2 {

struct FlowCoef {
    double rho, mu, dt;
};

pf2_status launch_prediction(const pf2_mesh* m, const FlowCoef& P, bool matrix, const double* ux, const double* uy,
                             const double* uxo, const double* uyo, const double* pold, double* valx, double* valy,
                             double* rhsx, double* rhsy, const pf2_bc* bcx, const pf2_bc* bcy, cudaStream_t st);
pf2_status launch_pressure(const pf2_mesh* m, const FlowCoef& P, bool matrix, const double* px, const double* py,
                           const double* pold, double* val, double* rhs, const pf2_bc* bc, cudaStream_t st);
pf2_status launch_correction(const pf2_mesh* m, const FlowCoef& P, bool matrix, const double* px, const double* py,
                             const double* pres, const double* pold, double* valx, double* valy, double* rhsx,
                             double* rhsy, const pf2_bc* bcx, const pf2_bc* bcy, cudaStream_t st);
pf2_status launch_prediction_bc(const pf2_mesh* m, const FlowCoef& P, const pf2_bc* src, pf2_bc* dst,
                                const double* pres, const double* pold, int comp, cudaStream_t st);
pf2_status launch_body_loads(const pf2_mesh* m, const FlowCoef& P, int body_id, double thickness, double umean,
                             double cx, double cy, const double* ux, const double* uy, const double* pres,
                             double* out_dev, cudaStream_t st);

pf2_status particles_advect(pf2_particles* H, const double* ux, const double* uy, double dt, int substeps,
                            cudaStream_t st);
pf2_status particles_project(pf2_particles* H, double* ux, double* uy, double* uxo, double* uyo, cudaStream_t st);
pf2_status particles_correct(pf2_particles* H, const double* ux, const double* uy, const double* uxo,
                             const double* uyo, cudaStream_t st);
pf2_status particles_seed(pf2_particles* H, cudaStream_t st);
pf2_status particles_status(pf2_particles* H, cudaStream_t st);
const int* particles_count_ptr(const pf2_particles* H);
// which of the two particle buffers holds the state (the cell sort alternates them)
int particles_parity(const pf2_particles* H);
void particles_set_parity(pf2_particles* H, int parity);

// Device-side record of one solve: copies of the solver's result and error word.
struct SolveRecord {
    int iterations;
    int converged;
    double residual;
    int status;
    int err;
};
// refactor = false reuses the preconditioner of the previous solve (same matrix values)
pf2_status solver_solve_async(pf2_solver* s, const pf2_csr* A, double* x, const double* b, SolveRecord* rec,
                              cudaStream_t st, bool refactor = true);

// Learned initial guess of the pressure solve (guess.cu).
struct Guess;
pf2_status guess_create(const pf2_mesh* m, Guess** out);
void guess_destroy(Guess* g);
// Before the first pressure solve of a step: features from (x, y, b, p, p_prev), the
// network's increment, and x <- the energy-norm Galerkin start over the network's
// increment and the stored increments.  ||b - A p|| and ||b - A x0|| go to res_out[2].
pf2_status guess_apply(Guess* g, const pf2_csr* A, const double* b, double* x, const double* p_prev,
                       double* res_out, int* used_out, cudaStream_t st);
// After the step: the step's increment p_new - p joins the history (with A times it), then
// one AdamW step (lr > 0) on the target (p_new - p) of the features of guess_apply.
pf2_status guess_train(Guess* g, const pf2_csr* A, const double* p_new, float lr, cudaStream_t st);

}  // namespace pf2
