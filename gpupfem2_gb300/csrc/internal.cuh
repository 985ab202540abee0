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
// Drag and lift coefficients into out_dev[0..1]; out_dev holds kBodyLoadsDoubles doubles
// (the blocks' partial sums and a ticket after the two results), zeroed before first use.
constexpr int kLoadBlocks = 1024;
constexpr int kBodyLoadsDoubles = 2 + 4 * kLoadBlocks + 1;
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
long long particles_capacity(const pf2_particles* H);
// grows the particle buffers to cap (no-op when already as large), keeping the particles
pf2_status particles_reserve(pf2_particles* H, long long cap, cudaStream_t st);

// Device-side record of one solve: copies of the solver's result and error word.
struct SolveRecord {
    int iterations;
    int converged;
    double residual;
    int status;
    int err;
    double relres;  // ||r|| / ||b|| at the end of the solve (CG and BiCGStab)
};
// refactor = false reuses the preconditioner of the previous solve (same matrix values)
pf2_status solver_solve_async(pf2_solver* s, const pf2_csr* A, double* x, const double* b, SolveRecord* rec,
                              cudaStream_t st, bool refactor = true);

// A checkpoint file (checkpoint.cu): a header (magic, format version, kind of object) and
// tagged sections (8-byte tag, 8-byte length, payload) written and read in one order.
// Reading checks each tag and length against what the reader expects, so a file of
// another object, mesh or size is rejected with the section that differs.
enum CkptKind : uint32_t { CKPT_PARTICLES = 1, CKPT_FLOW = 2, CKPT_MPNN = 3 };
class CkptFile {
public:
    CkptFile() = default;
    CkptFile(const CkptFile&) = delete;
    CkptFile& operator=(const CkptFile&) = delete;
    ~CkptFile();
    pf2_status open_write(const char* path, CkptKind kind);
    pf2_status open_read(const char* path, CkptKind kind);
    // writing: flush and report any write error; reading: the file must end here
    pf2_status close();
    bool writing() const { return wr_; }
    // host bytes: written, or read into p after the tag and length check
    pf2_status host(const char* tag, void* p, size_t bytes);
    // device bytes, staged through host memory (the stream is synchronised)
    pf2_status device(const char* tag, void* d, size_t bytes, cudaStream_t st);

private:
    pf2_status header(const char* tag, size_t bytes);
    FILE* f_ = nullptr;
    bool wr_ = false;
    std::string path_;
    std::vector<unsigned char> stage_;
};

// The particle state (count, the SoA arrays of the current buffer, the cell words and
// the cell segments) to or from a checkpoint.
pf2_status particles_checkpoint(pf2_particles* H, CkptFile& io, cudaStream_t st);

// The network's trained state (parameters, AdamW moments and step) to or from a checkpoint.
pf2_status mpnn_checkpoint(pf2_mpnn* net, CkptFile& io, cudaStream_t st);

// Learned initial guess of the pressure solve (guess.cu).
struct Guess;
// the guess's state across steps (previous pressure, increment history, network
// parameters and AdamW moments) to or from a checkpoint
pf2_status guess_checkpoint(Guess* g, CkptFile& io, cudaStream_t st);
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
