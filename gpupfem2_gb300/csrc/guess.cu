// guess.cu - the learned initial guess of the pressure solve (no reference counterpart).
//
// Before the first pressure solve of a step the network (mpnn.cu) sees, per node,
//   f = ((x - x0) / L, (y - y0) / L, b / s_b, p / s_p, (p - p_prev) / s_d)
// (b the pressure right-hand side, p the previous-step pressure, p_prev the one before;
// s_b = max |b|, s_p = max |p|, s_d = max |p - p_prev|) and predicts the increment
// p_new - p in units of s_d: d1 = s_d y.  With d2 = p - p_prev, the last increment, the
// start is the Galerkin combination
//   x0 = p + c1 d1 + c2 d2,  (D^T A D) c = D^T (b - A p),  D = [d1 d2],
// the point of p + span{d1, d2} closest to the solution in the energy norm (A is SPD).
// It lowers the energy norm of the error by h^T c >= 0 (h = D^T r0); a direction that
// does not help gets a coefficient near 0, so the start is never worse than p in that
// norm, the norm CG minimises.  (The residual norm is a poor test here: the Laplacian
// amplifies any high-frequency error of a learned increment, so a useful increment can
// still raise ||b - A x0||.)  While training, after the step the target
// t = (p_new - p) / s_d drives one AdamW step on the same features.
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
    DevBuf<double> p_saved, p_prev, d1, d2, r0, a1, a2, coef, part, res;
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

__global__ void k_guess_dirs(int n, const double* __restrict__ p, const double* __restrict__ pp,
                             const float* __restrict__ y, const unsigned long long* __restrict__ s, double* d1,
                             double* d2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    d1[i] = scale_of(s[2]) * (double)y[i];
    d2[i] = p[i] - pp[i];
}

// One pass over A: r0 = b - A p, A d1, A d2 per row; per-block partials of
// d1.Ad1, d1.Ad2, d2.Ad2, d1.r0, d2.r0, r0.r0 (6 x blocks).
__global__ void k_guess_project(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                const double* __restrict__ val, const double* __restrict__ b,
                                const double* __restrict__ p, const double* __restrict__ d1,
                                const double* __restrict__ d2, double* r0, double* a1, double* a2, double* part) {
    __shared__ double sh[33 * 6];
    double acc[6] = { 0, 0, 0, 0, 0, 0 };
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double sp = 0.0, s1 = 0.0, s2 = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            const double v = val[k];
            const int c = col[k];
            sp += v * p[c];
            s1 += v * d1[c];
            s2 += v * d2[c];
        }
        const double ri = b[i] - sp;
        r0[i] = ri;
        a1[i] = s1;
        a2[i] = s2;
        acc[0] += d1[i] * s1;
        acc[1] += d1[i] * s2;
        acc[2] += d2[i] * s2;
        acc[3] += d1[i] * ri;
        acc[4] += d2[i] * ri;
        acc[5] += ri * ri;
    }
    block_sum_n<6>(acc, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; ++k) part[6 * blockIdx.x + k] = acc[k];
}

// Coefficients of the 2 x 2 Galerkin system (one thread, block partials in order);
// coef = {c1, c2}, res[0] = ||b - A p||.
__global__ void k_guess_solve(int nb, const double* __restrict__ part, double* coef, double* res, int* used) {
    double t[6] = { 0, 0, 0, 0, 0, 0 };
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < 6; ++k) t[k] += part[6 * b + k];
    const double g11 = t[0], g12 = t[1], g22 = t[2], h1 = t[3], h2 = t[4];
    double c1 = 0.0, c2 = 0.0;
    const double det = g11 * g22 - g12 * g12;
    if (g11 > 0.0 && g22 > 0.0 && det > 1e-12 * g11 * g22) {
        c1 = (g22 * h1 - g12 * h2) / det;
        c2 = (g11 * h2 - g12 * h1) / det;
    } else if (g11 > 0.0 && (g22 <= 0.0 || h1 * h1 / g11 >= h2 * h2 / g22)) {
        c1 = h1 / g11;  // one usable direction: the better of the two
    } else if (g22 > 0.0) {
        c2 = h2 / g22;
    }
    coef[0] = c1;
    coef[1] = c2;
    res[0] = sqrt(t[5]);
    *used = c1 != 0.0 ? 1 : 0;
}

// x0 = p + c1 d1 + c2 d2 (x holds p); per-block partials of ||r0 - c1 A d1 - c2 A d2||^2,
// the residual of the start.
__global__ void k_guess_combine(int n, const double* __restrict__ coef, const double* __restrict__ d1,
                                const double* __restrict__ d2, const double* __restrict__ r0,
                                const double* __restrict__ a1, const double* __restrict__ a2, double* x,
                                double* part) {
    __shared__ double sh[40];
    const double c1 = coef[0], c2 = coef[1];
    double rr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += c1 * d1[i] + c2 * d2[i];
        const double ri = r0[i] - c1 * a1[i] - c2 * a2[i];
        rr += ri * ri;
    }
    rr = block_sum(rr, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = rr;
}

__global__ void k_guess_res1(int nb, const double* __restrict__ part, double* res) {
    double t = 0.0;
    for (int b = 0; b < nb; ++b) t += part[b];
    res[1] = sqrt(t);
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
        (s = G->p_prev.alloc(n)) || (s = G->d1.alloc(n)) || (s = G->d2.alloc(n)) || (s = G->r0.alloc(n)) ||
        (s = G->a1.alloc(n)) || (s = G->a2.alloc(n)) || (s = G->coef.alloc(2)) ||
        (s = G->part.alloc(6 * (size_t)G->blocks)) ||
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
    k_guess_dirs<<<blocks_for(n), kThreads, 0, st>>>(n, x, G->p_prev.p, G->y.p, G->scale_bits.p, G->d1.p, G->d2.p);
    PF2_LAUNCH_CHECK();
    k_guess_project<<<G->blocks, kThreads, 0, st>>>(n, A->mesh->rowptr.p, A->mesh->col.p, A->val.p, b, x, G->d1.p,
                                                    G->d2.p, G->r0.p, G->a1.p, G->a2.p, G->part.p);
    PF2_LAUNCH_CHECK();
    k_guess_solve<<<1, 1, 0, st>>>(G->blocks, G->part.p, G->coef.p, G->res.p, G->flag.p);
    PF2_LAUNCH_CHECK();
    k_guess_combine<<<G->blocks, kThreads, 0, st>>>(n, G->coef.p, G->d1.p, G->d2.p, G->r0.p, G->a1.p, G->a2.p, x,
                                                    G->part.p);
    PF2_LAUNCH_CHECK();
    k_guess_res1<<<1, 1, 0, st>>>(G->blocks, G->part.p, G->res.p);
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
