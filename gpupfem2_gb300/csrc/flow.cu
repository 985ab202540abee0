// flow.cu - one PFEM-2 time step on the device (cases/Cylinder2D/main.cu:793-880).
//
// pf2_flow owns the whole state of the channel drivers: particles, node fields,
// five CSR systems sharing the mesh pattern, the Dirichlet sets and three solvers.
// pf2_flow_step enqueues the step on one stream with no host round trip; iteration
// counts, the device status words and the loads are copied to pinned host memory at
// the end of the step and read by pf2_flow_step_info.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.cuh"

using namespace pf2;

namespace {
constexpr int kMaxOuter = 8;
constexpr int kRecords = 5 * kMaxOuter;  // pred x/y, pressure, corr x/y per outer iteration
}  // namespace

struct pf2_flow {
    const pf2_mesh* mesh = nullptr;
    pf2_params P{};
    pf2_particles* ph = nullptr;
    DevBuf<double> f[8];
    pf2_csr* A[5] = { nullptr, nullptr, nullptr, nullptr, nullptr };
    DevBuf<double> b[5];
    pf2_bc* bc[3] = { nullptr, nullptr, nullptr };
    pf2_bc* pbc[2] = { nullptr, nullptr };
    pf2_solver* gmres = nullptr;
    pf2_solver* cg_p = nullptr;
    pf2_solver* cg_c = nullptr;
    Guess* guess = nullptr;
    long long steps_done = 0;
    // the five matrices (and the pressure factors) do not change between steps: after
    // the first step only the right-hand sides are assembled
    bool assembled = false;
    // CUDA graphs of the step body, one per particle-buffer parity (the cell sort
    // alternates two buffers); captured on the engine's own stream
    bool use_graph = true;
    cudaStream_t cs = nullptr;
    cudaGraphExec_t gexec[2] = { nullptr, nullptr };
    int glr[2] = { -1, -1 };
    DevBuf<double> guess_res;
    DevBuf<int> guess_used;
    PinnedBuf<double> h_guess_res;
    PinnedBuf<int> h_guess_used;
    DevBuf<SolveRecord> rec;
    DevBuf<double> loads;
    PinnedBuf<SolveRecord> h_rec;
    PinnedBuf<double> h_loads;
    PinnedBuf<int> h_np;
    cudaEvent_t done = nullptr;
    bool stepped = false;
    // phase timing: events of up to tmax steps, each with (1 + events per step)
    std::vector<cudaEvent_t> tev;
    std::vector<int> tphase;  // phase closed by each event of a step
    int tmax = 0, tsteps = 0, tper = 0, tcur = 0;

    void mark(cudaStream_t st, int phase) {
        if (tmax == 0 || tsteps >= tmax) return;
        const int k = tsteps * tper + tcur;
        if (tcur < tper) {
            cudaEventRecord(tev[k], st);
            if (tsteps == 0) tphase[tcur] = phase;
            ++tcur;
        }
    }

    ~pf2_flow() {
        for (auto g : gexec)
            if (g) cudaGraphExecDestroy(g);
        if (cs) cudaStreamDestroy(cs);
        for (auto e : tev) cudaEventDestroy(e);
        if (done) cudaEventDestroy(done);
        for (auto* a : A) pf2_csr_destroy(a);
        for (auto* x : bc) pf2_bc_destroy(x);
        for (auto* x : pbc) pf2_bc_destroy(x);
        pf2_solver_destroy(gmres);
        pf2_solver_destroy(cg_p);
        pf2_solver_destroy(cg_c);
        guess_destroy(guess);
        pf2_particles_destroy(ph);
    }
};

extern "C" {

pf2_status pf2_flow_create(const pf2_mesh* mesh, const pf2_params* p, int nbx, const pf2_dirichlet_node* bx, int nby,
                           const pf2_dirichlet_node* by, int nbp, const pf2_dirichlet_node* bp, double cap_factor,
                           pf2_flow** out) {
    PF2_REQUIRE(mesh && p && out, PF2_BAD_INPUT, "null argument");
    *out = nullptr;
    PF2_REQUIRE(p->n_outer >= 1 && p->n_outer <= kMaxOuter, PF2_BAD_INPUT, "n_outer must be in 1..%d", kMaxOuter);
    PF2_REQUIRE(p->substeps >= 1, PF2_BAD_INPUT, "substeps must be >= 1");
    PF2_REQUIRE(p->dt > 0 && p->rho > 0, PF2_BAD_INPUT, "dt and rho must be positive");
    PF2_REQUIRE(p->scheme == 0 || p->scheme == 1, PF2_BAD_INPUT, "scheme must be 0 (A) or 1 (B)");
    PF2_REQUIRE(p->prediction_solver == PF2_SOLVER_GMRES || p->prediction_solver == PF2_SOLVER_BICGSTAB,
                PF2_BAD_INPUT, "prediction_solver must be PF2_SOLVER_GMRES or PF2_SOLVER_BICGSTAB");
    pf2_flow* F = new pf2_flow();
    F->mesh = mesh;
    F->P = *p;
    auto fail = [&](pf2_status s) { delete F; return s; };
    const int nv = mesh->nv;
    pf2_status s;
    for (auto& a : F->f) {
        if ((s = a.alloc(nv))) return fail(s);
        if (cudaMemset(a.p, 0, sizeof(double) * nv) != cudaSuccess) return fail(PF2_CUDA_ERROR);
    }
    for (int k = 0; k < 5; ++k) {
        if ((s = pf2_csr_create(mesh, &F->A[k]))) return fail(s);
        if ((s = F->b[k].alloc(nv))) return fail(s);
        if (cudaMemset(F->b[k].p, 0, sizeof(double) * nv) != cudaSuccess) return fail(PF2_CUDA_ERROR);
    }
    if ((s = pf2_bc_create(nv, nbx, bx, &F->bc[0])) || (s = pf2_bc_create(nv, nby, by, &F->bc[1])) ||
        (s = pf2_bc_create(nv, nbp, bp, &F->bc[2])) || (s = pf2_bc_create(nv, nbx, bx, &F->pbc[0])) ||
        (s = pf2_bc_create(nv, nby, by, &F->pbc[1])))
        return fail(s);
    if ((s = pf2_particles_create(mesh, p->level, cap_factor, &F->ph))) return fail(s);
    // Cylinder2D/main.cu:768-774: GMRES(Jacobi) for the prediction, CG for the rest
    pf2_solver_options o{};
    o.tolerance = p->tolerance;
    o.max_iterations = p->max_iterations;
    o.criterion = PF2_CRITERION_ABS;
    o.precision = PF2_PRECISION_FP64;
    o.kind = p->prediction_solver == PF2_SOLVER_BICGSTAB ? PF2_SOLVER_BICGSTAB : PF2_SOLVER_GMRES;
    o.precond = PF2_PRECOND_JACOBI;
    o.restart = p->gmres_restart;
    o.orthogonalization = p->gmres_orthogonalization;
    if ((s = pf2_solver_create(F->A[0], &o, &F->gmres))) return fail(s);
    o.kind = PF2_SOLVER_CG;
    o.restart = 0;
    o.orthogonalization = PF2_GS_MODIFIED;
    o.cg_variant = p->cg_variant;
    o.precond = p->pressure_precond;
    o.precision = p->pressure_precision;
    o.criterion = p->pressure_criterion;
    if (p->pressure_tolerance > 0) o.tolerance = p->pressure_tolerance;
    if (p->pressure_max_iterations > 0) o.max_iterations = p->pressure_max_iterations;
    o.ordering = p->pressure_ordering;
    if ((s = pf2_solver_create(F->A[2], &o, &F->cg_p))) return fail(s);
    o.tolerance = p->tolerance;
    o.max_iterations = p->max_iterations;
    o.precision = PF2_PRECISION_FP64;
    o.criterion = PF2_CRITERION_ABS;
    o.ordering = PF2_ORDERING_NATURAL;
    o.precond = PF2_PRECOND_JACOBI;
    if ((s = pf2_solver_create(F->A[3], &o, &F->cg_c))) return fail(s);
    if ((s = F->rec.alloc(kRecords)) || (s = F->h_rec.alloc(kRecords)) ||
        (s = F->loads.alloc(kBodyLoadsDoubles)) || (s = F->h_loads.alloc(2)) || (s = F->h_np.alloc(2)))
        return fail(s);
    if (cudaMemset(F->rec.p, 0, sizeof(SolveRecord) * kRecords) != cudaSuccess ||
        cudaMemset(F->loads.p, 0, sizeof(double) * kBodyLoadsDoubles) != cudaSuccess)
        return fail(PF2_CUDA_ERROR);
    if (cudaEventCreateWithFlags(&F->done, cudaEventDisableTiming) != cudaSuccess) return fail(PF2_CUDA_ERROR);
    if ((s = F->guess_res.alloc(2)) || (s = F->guess_used.alloc(1)) || (s = F->h_guess_res.alloc(2)) ||
        (s = F->h_guess_used.alloc(1)))
        return fail(s);
    if (cudaMemset(F->guess_res.p, 0, 2 * sizeof(double)) != cudaSuccess ||
        cudaMemset(F->guess_used.p, 0, sizeof(int)) != cudaSuccess)
        return fail(PF2_CUDA_ERROR);
    if (p->pressure_x0 == PF2_X0_LEARNED && (s = guess_create(mesh, &F->guess))) return fail(s);
    if (cudaStreamCreateWithFlags(&F->cs, cudaStreamNonBlocking) != cudaSuccess) return fail(PF2_CUDA_ERROR);
    *out = F;
    return PF2_OK;
}

pf2_status pf2_flow_destroy(pf2_flow* f) {
    delete f;
    return PF2_OK;
}

pf2_status pf2_flow_seed(pf2_flow* F, void* stream) {
    PF2_REQUIRE(F, PF2_BAD_INPUT, "null flow");
    cudaStream_t st = as_stream(stream);
    PF2_TRY(particles_seed(F->ph, st));
    return particles_correct(F->ph, F->f[0].p, F->f[1].p, nullptr, nullptr, st);
}

}  // extern "C"

// The work of one step, enqueued on st (also what a graph capture records).
static pf2_status step_body(pf2_flow* F, cudaStream_t st) {
    const pf2_params& P = F->P;
    const FlowCoef K{ P.rho, P.mu, P.dt };
    double *ux = F->f[0].p, *uy = F->f[1].p, *uxo = F->f[2].p, *uyo = F->f[3].p;
    double *px = F->f[4].p, *py = F->f[5].p, *pr = F->f[6].p, *po = F->f[7].p;
    const double* pold = (P.scheme == 1) ? po : nullptr;
    F->tcur = 0;
    F->mark(st, -1);
    // particle phase (:797-803); the projection also writes u_old (:805-806)
    PF2_TRY(particles_advect(F->ph, ux, uy, P.dt, P.substeps, st));
    F->mark(st, PF2_PHASE_PARTICLES);
    PF2_TRY(particles_project(F->ph, ux, uy, uxo, uyo, st));
    if (P.scheme == 1) PF2_CUDA(cudaMemcpyAsync(po, pr, sizeof(double) * F->mesh->nv, cudaMemcpyDeviceToDevice, st));
    F->mark(st, PF2_PHASE_PROJECTION);
    SolveRecord* R = F->rec.p;
    for (int it = 0; it < P.n_outer; ++it) {
        // velocity prediction (:812-828): boundary values from the pressure gradient,
        // assembly with the Dirichlet rule, GMRES per component
        for (int k = 0; k < 2; ++k) PF2_TRY(launch_prediction_bc(F->mesh, K, F->bc[k], F->pbc[k], pr, pold, k, st));
        const bool mat = !F->assembled && it == 0;
        PF2_TRY(launch_prediction(F->mesh, K, mat, ux, uy, uxo, uyo, pold, F->A[0]->val.p, F->A[1]->val.p, F->b[0].p,
                                  F->b[1].p, F->pbc[0], F->pbc[1], st));
        F->mark(st, PF2_PHASE_PREDICTION_ASSEMBLY);
        PF2_TRY(solver_solve_async(F->gmres, F->A[0], px, F->b[0].p, &R[5 * it + 0], st, mat));
        PF2_TRY(solver_solve_async(F->gmres, F->A[1], py, F->b[1].p, &R[5 * it + 1], st, true));
        F->mark(st, PF2_PHASE_PREDICTION_SOLVE);
        // pressure (:831-842)
        PF2_TRY(launch_pressure(F->mesh, K, mat, px, py, pold, F->A[2]->val.p, F->b[2].p, F->bc[2], st));
        F->mark(st, PF2_PHASE_PRESSURE_ASSEMBLY);
        if (F->guess && it == 0)
            PF2_TRY(guess_apply(F->guess, F->A[2], F->b[2].p, pr, nullptr, F->guess_res.p, F->guess_used.p, st));
        PF2_TRY(solver_solve_async(F->cg_p, F->A[2], pr, F->b[2].p, &R[5 * it + 2], st, mat));
        F->mark(st, PF2_PHASE_PRESSURE_SOLVE);
        // velocity correction (:845-860)
        PF2_TRY(launch_correction(F->mesh, K, mat, px, py, pr, pold, F->A[3]->val.p, F->A[4]->val.p, F->b[3].p,
                                  F->b[4].p, F->bc[0], F->bc[1], st));
        F->mark(st, PF2_PHASE_CORRECTION_ASSEMBLY);
        PF2_TRY(solver_solve_async(F->cg_c, F->A[3], ux, F->b[3].p, &R[5 * it + 3], st, true));
        PF2_TRY(solver_solve_async(F->cg_c, F->A[4], uy, F->b[4].p, &R[5 * it + 4], st, true));
        F->mark(st, PF2_PHASE_CORRECTION_SOLVE);
    }
    // particle velocity correction (:863-865) and loads (:874-876)
    PF2_TRY(particles_correct(F->ph, ux, uy, uxo, uyo, st));
    if (P.calculate_loads)
        PF2_TRY(launch_body_loads(F->mesh, K, P.body_boundary_id, P.thickness, P.mean_velocity, P.body_cx, P.body_cy,
                                  ux, uy, pr, F->loads.p, st));
    F->mark(st, PF2_PHASE_PARTICLE_CORRECTION);
    if (F->guess)
        PF2_TRY(guess_train(F->guess, F->A[2], pr, F->steps_done < P.learn_steps ? P.learn_rate : 0.0f, st));
    ++F->steps_done;
    F->assembled = true;
    if (F->tmax && F->tsteps < F->tmax) ++F->tsteps;
    PF2_CUDA(cudaMemcpyAsync(F->h_rec.p, F->rec.p, sizeof(SolveRecord) * kRecords, cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaMemcpyAsync(F->h_loads.p, F->loads.p, sizeof(double) * 2, cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaMemcpyAsync(F->h_np.p, particles_count_ptr(F->ph), sizeof(int), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaMemcpyAsync(F->h_guess_res.p, F->guess_res.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaMemcpyAsync(F->h_guess_used.p, F->guess_used.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    return PF2_OK;
}

extern "C" {

pf2_status pf2_flow_step(pf2_flow* F, void* stream) {
    PF2_REQUIRE(F, PF2_BAD_INPUT, "null flow");
    cudaStream_t st = as_stream(stream);
    // reseeding only adds particles: once the last step left the buffers three quarters
    // full, grow them by half (the step graphs hold the old buffers: recapture)
    if (F->stepped) {
        PF2_CUDA(cudaEventSynchronize(F->done));
        const long long np = F->h_np.p[0], cap = particles_capacity(F->ph);
        if (np > cap - cap / 4) {
            PF2_TRY(particles_reserve(F->ph, std::max(cap + cap / 2, 2 * np), st));
            for (auto& gx : F->gexec)
                if (gx) {
                    cudaGraphExecDestroy(gx);
                    gx = nullptr;
                }
        }
    }
    const bool learning = F->guess && F->steps_done < F->P.learn_steps;
    // graphs replay identical work: from the second step on (matrices assembled), and
    // not while phase timing records events
    if (F->use_graph && F->assembled && F->tmax == 0) {
        const int par = particles_parity(F->ph);
        const long long steps0 = F->steps_done;
        if (!F->gexec[par] || F->glr[par] != (int)learning) {
            if (F->gexec[par]) cudaGraphExecDestroy(F->gexec[par]);
            F->gexec[par] = nullptr;
            PF2_CUDA(cudaStreamBeginCapture(F->cs, cudaStreamCaptureModeThreadLocal));
            const pf2_status sb = step_body(F, F->cs);
            cudaGraph_t graph = nullptr;
            const cudaError_t ec = cudaStreamEndCapture(F->cs, &graph);
            cudaGetLastError();
            F->steps_done = steps0;  // the capture did not run the step
            particles_set_parity(F->ph, par);
            cudaGraphExec_t ex = nullptr;
            if (sb == PF2_OK && ec == cudaSuccess && graph &&
                cudaGraphInstantiate(&ex, graph, 0) == cudaSuccess) {
                F->gexec[par] = ex;
                F->glr[par] = (int)learning;
            } else {
                cudaGetLastError();
                F->use_graph = false;  // capture refused: launch eagerly from now on
            }
            if (graph) cudaGraphDestroy(graph);
        }
        if (F->gexec[par]) {
            PF2_CUDA(cudaGraphLaunch(F->gexec[par], st));
            particles_set_parity(F->ph, 1 - par);
            ++F->steps_done;
            PF2_CUDA(cudaEventRecord(F->done, st));
            F->stepped = true;
            return PF2_OK;
        }
    }
    PF2_TRY(step_body(F, st));
    PF2_CUDA(cudaEventRecord(F->done, st));
    F->stepped = true;
    return PF2_OK;
}

pf2_status pf2_flow_set_graphs(pf2_flow* F, int enable) {
    PF2_REQUIRE(F, PF2_BAD_INPUT, "null flow");
    F->use_graph = enable != 0;
    return PF2_OK;
}

pf2_status pf2_flow_enable_timing(pf2_flow* F, int max_steps) {
    PF2_REQUIRE(F && max_steps >= 0, PF2_BAD_INPUT, "bad argument");
    PF2_CUDA(cudaDeviceSynchronize());
    for (auto e : F->tev) cudaEventDestroy(e);
    F->tev.clear();
    F->tmax = max_steps;
    F->tsteps = 0;
    F->tper = 3 + 6 * F->P.n_outer + 1;
    F->tphase.assign(F->tper, -1);
    F->tev.resize((size_t)max_steps * F->tper);
    for (auto& e : F->tev) PF2_CUDA(cudaEventCreate(&e));
    return PF2_OK;
}

pf2_status pf2_flow_phase_times(pf2_flow* F, double* ms, int* steps) {
    PF2_REQUIRE(F && ms, PF2_BAD_INPUT, "null argument");
    for (int k = 0; k < PF2_PHASES; ++k) ms[k] = 0.0;
    if (steps) *steps = F->tsteps;
    if (!F->tsteps) return PF2_OK;
    PF2_CUDA(cudaDeviceSynchronize());
    for (int s = 0; s < F->tsteps; ++s)
        for (int k = 1; k < F->tper; ++k) {
            float t = 0.0f;
            PF2_CUDA(cudaEventElapsedTime(&t, F->tev[(size_t)s * F->tper + k - 1], F->tev[(size_t)s * F->tper + k]));
            const int ph = F->tphase[k];
            if (ph >= 0) ms[ph] += t;
        }
    return PF2_OK;
}

pf2_status pf2_flow_field(pf2_flow* F, int which, double** ptr) {
    PF2_REQUIRE(F && ptr && which >= 0 && which < 8, PF2_BAD_INPUT, "bad field request");
    *ptr = F->f[which].p;
    return PF2_OK;
}

pf2_status pf2_flow_download_field(pf2_flow* F, int which, double* dst) {
    PF2_REQUIRE(F && dst && which >= 0 && which < 8, PF2_BAD_INPUT, "bad field request");
    PF2_CUDA(cudaDeviceSynchronize());
    PF2_CUDA(cudaMemcpy(dst, F->f[which].p, sizeof(double) * F->mesh->nv, cudaMemcpyDeviceToHost));
    return PF2_OK;
}

pf2_status pf2_flow_upload_field(pf2_flow* F, int which, const double* src) {
    PF2_REQUIRE(F && src && which >= 0 && which < 8, PF2_BAD_INPUT, "bad field request");
    PF2_CUDA(cudaDeviceSynchronize());
    PF2_CUDA(cudaMemcpy(F->f[which].p, src, sizeof(double) * F->mesh->nv, cudaMemcpyHostToDevice));
    return PF2_OK;
}

// Checkpoint sections: sizes and step count, the eight node fields, the boundary values
// of the three Dirichlet sets, the particles, and the learned guess when there is one.
// The matrices, right-hand sides and solver work are rebuilt by the next step from these
// (assembly and solves are deterministic), so a run restarted from a checkpoint repeats
// the uninterrupted run bit for bit.
static pf2_status flow_checkpoint(pf2_flow* F, CkptFile& io, cudaStream_t st) {
    const pf2_mesh* M = F->mesh;
    long long meta[6] = { M->nv, M->nc, F->P.level, F->P.scheme, F->guess ? 1 : 0, F->steps_done };
    const long long want[5] = { meta[0], meta[1], meta[2], meta[3], meta[4] };
    PF2_TRY(io.host("fmeta", meta, sizeof(meta)));
    for (int k = 0; k < 5; ++k)
        PF2_REQUIRE(meta[k] == want[k], PF2_BAD_INPUT,
                    "checkpoint flow (nodes %lld, cells %lld, level %lld, scheme %lld, learned guess %lld) does "
                    "not match this engine (%lld, %lld, %lld, %lld, %lld)",
                    meta[0], meta[1], meta[2], meta[3], meta[4], want[0], want[1], want[2], want[3], want[4]);
    PF2_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < 8; ++k) {
        char tag[8];
        snprintf(tag, sizeof(tag), "field%d", k);
        PF2_TRY(io.device(tag, F->f[k].p, sizeof(double) * M->nv, st));
    }
    for (int k = 0; k < 3; ++k) {
        char tag[8];
        snprintf(tag, sizeof(tag), "bcval%d", k);
        PF2_TRY(io.device(tag, F->bc[k]->value.p, sizeof(double) * F->bc[k]->n_bc, st));
    }
    PF2_TRY(particles_checkpoint(F->ph, io, st));
    if (F->guess) PF2_TRY(guess_checkpoint(F->guess, io, st));
    if (!io.writing()) F->steps_done = meta[5];
    return PF2_OK;
}

pf2_status pf2_flow_save(pf2_flow* F, const char* path, void* stream) {
    PF2_REQUIRE(F && path, PF2_BAD_INPUT, "null argument");
    CkptFile io;
    PF2_TRY(io.open_write(path, CKPT_FLOW));
    PF2_TRY(flow_checkpoint(F, io, as_stream(stream)));
    return io.close();
}

pf2_status pf2_flow_load(pf2_flow* F, const char* path, void* stream) {
    PF2_REQUIRE(F && path, PF2_BAD_INPUT, "null argument");
    CkptFile io;
    PF2_TRY(io.open_read(path, CKPT_FLOW));
    PF2_TRY(flow_checkpoint(F, io, as_stream(stream)));
    return io.close();
}

pf2_status pf2_flow_set_boundary_values(pf2_flow* F, int which, const double* values, void* stream) {
    PF2_REQUIRE(F && which >= 0 && which < 3, PF2_BAD_INPUT, "bad boundary set");
    return pf2_bc_set_values(F->bc[which], values, stream);
}

pf2_status pf2_flow_system(pf2_flow* F, int which, pf2_csr** A, double** rhs) {
    PF2_REQUIRE(F && A && rhs && which >= 0 && which < 5, PF2_BAD_INPUT, "bad system request");
    *A = F->A[which];
    *rhs = F->b[which].p;
    return PF2_OK;
}

pf2_status pf2_flow_particles(pf2_flow* F, pf2_particles** ph) {
    PF2_REQUIRE(F && ph, PF2_BAD_INPUT, "null argument");
    *ph = F->ph;
    return PF2_OK;
}

pf2_status pf2_flow_step_info(pf2_flow* F, pf2_step_info* info) {
    PF2_REQUIRE(F && info, PF2_BAD_INPUT, "null argument");
    memset(info, 0, sizeof(*info));
    if (!F->stepped) return PF2_OK;
    PF2_CUDA(cudaEventSynchronize(F->done));
    PF2_TRY(particles_status(F->ph, nullptr));
    info->particles = F->h_np.p[0];
    info->converged = 1;
    info->status = PF2_OK;
    for (int it = 0; it < F->P.n_outer; ++it) {
        const SolveRecord* r = F->h_rec.p + 5 * it;
        info->it_prediction[0][it] = r[0].iterations;
        info->it_prediction[1][it] = r[1].iterations;
        info->it_pressure[it] = r[2].iterations;
        info->pressure_residual[it] = r[2].relres;
        info->it_correction[0][it] = r[3].iterations;
        info->it_correction[1][it] = r[4].iterations;
        for (int k = 0; k < 5; ++k) {
            if (!r[k].converged) info->converged = 0;
            if (r[k].err && info->status == PF2_OK) info->status = r[k].err;
        }
    }
    info->cx = F->h_loads.p[0];
    info->cy = F->h_loads.p[1];
    info->guess_used = F->guess ? F->h_guess_used.p[0] : 0;
    info->guess_residual[0] = F->h_guess_res.p[0];
    info->guess_residual[1] = F->h_guess_res.p[1];
    PF2_REQUIRE(info->status == PF2_OK, (pf2_status)info->status, "a device-side wait timed out during the step");
    return PF2_OK;
}

}  // extern "C"
