// guess.cu - the learned initial guess of the pressure solve (no reference counterpart).
//
// Before the first pressure solve of a step the network (mpnn.cu) sees, per node,
//   f = ((x - x0) / L, (y - y0) / L, b / s_b, p / s_p, (p - p_prev) / s_d)
// (b the pressure right-hand side, p the previous-step pressure, p_prev the one before;
// s_b = max |b|, s_p = max |p|, s_d = max |p - p_prev|) and predicts the increment
// p_new - p in units of s_d; the candidate start is
//   x0 = p + s_d y.
// The solver starts from x0 only if ||b - A x0|| < ||b - A p|| (both computed on the
// device); otherwise from p, the reference's start.  While training, after the step the
// target t = (p_new - p) / s_d drives one AdamW step on the same features.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "device.cuh"
#include "internal.cuh"

namespace pf2 {

struct Guess {
    const pf2_mesh* mesh = nullptr;
    pf2_mpnn* net = nullptr;
    int n = 0;
    double x0 = 0.0, y0 = 0.0, L = 1.0;
    DevBuf<float> feat, y, target;
    DevBuf<double> p_saved, p_prev, cand, part, res;
    DevBuf<unsigned long long> scale_bits;  // max |b|, max |p|, max |p - p_prev| as ordered bit patterns
    DevBuf<int> flag;
    int blocks = 0;
};

__device__ __forceinline__ void atomic_max_abs(unsigned long long* slot, double v) {
    atomicMax(slot, (unsigned long long)__double_as_longlong(fabs(v)));  // |v| >= 0: bits order as values
}

__global__ void k_guess_scales(int n, const double* __restrict__ b, const double* __restrict__ p,
                               const double* __restrict__ pp, unsigned long long* s) {
    double mb = 0.0, mp = 0.0, md = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        mb = fmax(mb, fabs(b[i]));
        mp = fmax(mp, fabs(p[i]));
        md = fmax(md, fabs(p[i] - pp[i]));
    }
    atomic_max_abs(&s[0], mb);
    atomic_max_abs(&s[1], mp);
    atomic_max_abs(&s[2], md);
}

__device__ __forceinline__ double scale_of(unsigned long long bits) {
    const double v = __longlong_as_double((long long)bits);
    return v > 1e-300 ? v : 1.0;
}

__global__ void k_guess_features(int n, const double2* __restrict__ xy, double x0, double y0, double invL,
                                 const double* __restrict__ b, const double* __restrict__ p,
                                 const double* __restrict__ pp, const unsigned long long* __restrict__ s, float* f,
                                 double* p_saved) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double sb = scale_of(s[0]), sp = scale_of(s[1]), sd = scale_of(s[2]);
    const double2 c = xy[i];
    f[5 * (size_t)i + 0] = (float)((c.x - x0) * invL);
    f[5 * (size_t)i + 1] = (float)((c.y - y0) * invL);
    f[5 * (size_t)i + 2] = (float)(b[i] / sb);
    f[5 * (size_t)i + 3] = (float)(p[i] / sp);
    f[5 * (size_t)i + 4] = (float)((p[i] - pp[i]) / sd);
    p_saved[i] = p[i];
}

__global__ void k_guess_candidate(int n, const double* __restrict__ p, const float* __restrict__ y,
                                  const unsigned long long* __restrict__ s, double* cand) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    cand[i] = p[i] + scale_of(s[2]) * (double)y[i];
}

// per-block partials of ||b - A p||^2 and ||b - A cand||^2
__global__ void k_guess_residuals(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                  const double* __restrict__ val, const double* __restrict__ b,
                                  const double* __restrict__ p, const double* __restrict__ cand, double* part) {
    __shared__ double sh[40];
    double r0 = 0.0, r1 = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double a0 = 0.0, a1 = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            a0 += val[k] * p[col[k]];
            a1 += val[k] * cand[col[k]];
        }
        const double e0 = b[i] - a0, e1 = b[i] - a1;
        r0 += e0 * e0;
        r1 += e1 * e1;
    }
    r0 = block_sum(r0, sh);
    r1 = block_sum(r1, sh);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = r0;
        part[2 * blockIdx.x + 1] = r1;
    }
}

__global__ void k_guess_decide(int nb, const double* __restrict__ part, double* res, int* flag) {
    double r0 = 0.0, r1 = 0.0;
    for (int k = 0; k < nb; ++k) {
        r0 += part[2 * k];
        r1 += part[2 * k + 1];
    }
    res[0] = sqrt(r0);
    res[1] = sqrt(r1);
    *flag = (r1 < r0) ? 1 : 0;
}

__global__ void k_guess_select(int n, const int* __restrict__ flag, const double* __restrict__ cand, double* x) {
    if (!*flag) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = cand[i];
}

__global__ void k_guess_target(int n, const double* __restrict__ pnew, const double* __restrict__ p,
                               const unsigned long long* __restrict__ s, float* t, double* pp_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    t[i] = (float)((pnew[i] - p[i]) / scale_of(s[2]));
    pp_out[i] = p[i];  // p becomes the previous pressure of the next step
}

pf2_status guess_create(const pf2_mesh* m, Guess** out) {
    Guess* G = new Guess();
    G->mesh = m;
    G->n = m->nv;
    auto fail = [&](pf2_status s) { guess_destroy(G); return s; };
    pf2_status s = pf2_mpnn_create(m, 0x5eedull, &G->net);
    if (s) return fail(s);
    double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
    for (int i = 0; i < m->nv; ++i) {
        xmin = std::min(xmin, m->h_xy[2 * i]);
        xmax = std::max(xmax, m->h_xy[2 * i]);
        ymin = std::min(ymin, m->h_xy[2 * i + 1]);
        ymax = std::max(ymax, m->h_xy[2 * i + 1]);
    }
    G->x0 = xmin;
    G->y0 = ymin;
    G->L = std::max(std::max(xmax - xmin, ymax - ymin), 1e-300);
    G->blocks = std::min((int)blocks_for(G->n), num_sms() * 4);
    const size_t n = G->n;
    if ((s = G->feat.alloc(5 * n)) || (s = G->y.alloc(n)) || (s = G->target.alloc(n)) || (s = G->p_saved.alloc(n)) ||
        (s = G->p_prev.alloc(n)) || (s = G->cand.alloc(n)) || (s = G->part.alloc(2 * (size_t)G->blocks)) ||
        (s = G->res.alloc(2)) || (s = G->scale_bits.alloc(3)) || (s = G->flag.alloc(1)))
        return fail(s);
    if (cudaMemset(G->p_prev.p, 0, sizeof(double) * n) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "cudaMemset", __FILE__, __LINE__));
    *out = G;
    return PF2_OK;
}

void guess_destroy(Guess* g) {
    if (!g) return;
    pf2_mpnn_destroy(g->net);
    delete g;
}

pf2_status guess_apply(Guess* G, const pf2_csr* A, const double* b, double* x, const double* /*unused*/,
                       double* res_out, int* used_out, cudaStream_t st) {
    const int n = G->n;
    PF2_CUDA(cudaMemsetAsync(G->scale_bits.p, 0, 3 * sizeof(unsigned long long), st));
    k_guess_scales<<<G->blocks, kThreads, 0, st>>>(n, b, x, G->p_prev.p, G->scale_bits.p);
    PF2_LAUNCH_CHECK();
    k_guess_features<<<blocks_for(n), kThreads, 0, st>>>(n, G->mesh->xy.p, G->x0, G->y0, 1.0 / G->L, b, x,
                                                         G->p_prev.p, G->scale_bits.p, G->feat.p, G->p_saved.p);
    PF2_LAUNCH_CHECK();
    PF2_TRY(pf2_mpnn_forward(G->net, G->feat.p, G->y.p, st));
    k_guess_candidate<<<blocks_for(n), kThreads, 0, st>>>(n, x, G->y.p, G->scale_bits.p, G->cand.p);
    PF2_LAUNCH_CHECK();
    k_guess_residuals<<<G->blocks, kThreads, 0, st>>>(n, A->mesh->rowptr.p, A->mesh->col.p, A->val.p, b, x,
                                                      G->cand.p, G->part.p);
    PF2_LAUNCH_CHECK();
    k_guess_decide<<<1, 1, 0, st>>>(G->blocks, G->part.p, G->res.p, G->flag.p);
    PF2_LAUNCH_CHECK();
    k_guess_select<<<blocks_for(n), kThreads, 0, st>>>(n, G->flag.p, G->cand.p, x);
    PF2_LAUNCH_CHECK();
    if (res_out) PF2_CUDA(cudaMemcpyAsync(res_out, G->res.p, 2 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (used_out) PF2_CUDA(cudaMemcpyAsync(used_out, G->flag.p, sizeof(int), cudaMemcpyDeviceToDevice, st));
    return PF2_OK;
}

pf2_status guess_train(Guess* G, const double* p_new, float lr, cudaStream_t st) {
    const int n = G->n;
    k_guess_target<<<blocks_for(n), kThreads, 0, st>>>(n, p_new, G->p_saved.p, G->scale_bits.p, G->target.p,
                                                       G->p_prev.p);
    PF2_LAUNCH_CHECK();
    if (lr > 0.0f) PF2_TRY(pf2_mpnn_train_step(G->net, G->feat.p, G->target.p, lr, 1, nullptr, st));
    return PF2_OK;
}

}  // namespace pf2
