// guess.cu - the learned initial guess of the pressure solve (no reference counterpart).
//
// Before the first pressure solve of a step the network (mpnn.cu) sees, per node,
//   f = ((x - x0) / L, (y - y0) / L, b / s_b, p / s_p, (p - p_prev) / s_d)
// (b the pressure right-hand side, p the previous-step pressure, p_prev the one before;
// s_b = max |b|, s_p = max |p|, s_d = max |p - p_prev|) and predicts the increment
// p_new - p in units of s_d: d0 = s_d y.  With the last kHistory pressure increments
// h_1 .. h_K of the run (and their images A h_k, kept when they are stored), the start
// is the Galerkin combination
//   x0 = p + D c,  (D^T A D) c = D^T (b - A p),  D = [d0 h_1 .. h_K],
// the point of p + span(D) closest to the solution in the energy norm (A is SPD).  It
// lowers the energy norm of the error by c^T D^T r0 >= 0; directions that do not help get
// coefficients near 0, so the start is never worse than p in that norm, the norm CG
// minimises.  (The residual norm is a poor test here: the Laplacian amplifies any
// high-frequency error of a learned increment, so a useful increment can still raise
// ||b - A x0||.)  While training, after the step the target t = (p_new - p) / s_d drives
// one AdamW step on the same features.  The history ring's state lives on the device, so
// a replayed step graph keeps it up to date.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "device.cuh"
#include "internal.cuh"

namespace pf2 {

constexpr int kHistory = 8;                 // pressure increments kept for the projection
constexpr int kDirs = kHistory + 1;         // the network's direction first
constexpr int kDots = 2 * kDirs + 1;        // D^T r0, D^T A d0, r0^T r0

struct Guess {
    const pf2_mesh* mesh = nullptr;
    pf2_mpnn* net = nullptr;
    int n = 0;
    double x0 = 0.0, y0 = 0.0, L = 1.0;
    DevBuf<float> feat, y, target;
    DevBuf<double> p_saved, p_prev, d0, r0, a0, coef, part, res;
    DevBuf<double> hist, ahist;             // kHistory x n increments and their images under A
    DevBuf<double> gram;                    // kHistory x kHistory, h_i^T A h_j
    DevBuf<int> ring;                       // {count, head}
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

__global__ void k_guess_dir(int n, const float* __restrict__ y, const unsigned long long* __restrict__ s,
                            double* d0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    d0[i] = scale_of(s[2]) * (double)y[i];
}

// y1 = b - A x1 (or A x1 when b is null) and y2 = A x2 (when x2 is not null), one pass over A.
__global__ void k_guess_spmv(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                             const double* __restrict__ val, const double* __restrict__ b,
                             const double* __restrict__ x1, const double* __restrict__ x2, double* y1, double* y2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double s1 = 0.0, s2 = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            const double v = val[k];
            const int c = col[k];
            s1 += v * x1[c];
            if (x2) s2 += v * x2[c];
        }
        y1[i] = b ? b[i] - s1 : s1;
        if (x2) y2[i] = s2;
    }
}

// Per-block partials of D_j . r0 and D_j . A d0 (j < kDirs; history slots beyond the
// ring's count give 0) and of r0 . r0.
__global__ void k_guess_dots(int n, const double* __restrict__ d0, const double* __restrict__ hist,
                             const int* __restrict__ ring, const double* __restrict__ r0,
                             const double* __restrict__ a0, double* part) {
    __shared__ double sh[33 * kDots];
    const int cnt = ring[0];
    double acc[kDots];
#pragma unroll
    for (int j = 0; j < kDots; ++j) acc[j] = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double r = r0[i], a = a0[i];
        const double d = d0[i];
        acc[0] += d * r;
        acc[kDirs] += d * a;
#pragma unroll
        for (int k = 0; k < kHistory; ++k)
            if (k < cnt) {
                const double h = hist[(size_t)k * n + i];
                acc[1 + k] += h * r;
                acc[kDirs + 1 + k] += h * a;
            }
        acc[2 * kDirs] += r * r;
    }
    block_sum_n<kDots>(acc, sh);
    if (threadIdx.x == 0)
        for (int j = 0; j < kDots; ++j) part[(size_t)kDots * blockIdx.x + j] = acc[j];
}

// The (kDirs x kDirs) Galerkin system by a Cholesky factorisation with a small relative
// diagonal shift, directions whose pivot vanishes dropped (one thread, partials summed
// in block order).  coef[j] for D_j, res[0] = ||b - A p||, used = the network's
// direction got a nonzero coefficient.
__global__ void k_guess_solve(int nb, const double* __restrict__ part, const double* __restrict__ gram,
                              const int* __restrict__ ring, double* coef, double* res, int* used) {
    double t[kDots];
    for (int j = 0; j < kDots; ++j) t[j] = 0.0;
    for (int b = 0; b < nb; ++b)
        for (int j = 0; j < kDots; ++j) t[j] += part[(size_t)kDots * b + j];
    const int cnt = ring[0];
    const int m = 1 + cnt;
    double G[kDirs][kDirs], h[kDirs], c[kDirs];
    for (int i = 0; i < kDirs; ++i) {
        h[i] = t[i];
        c[i] = 0.0;
        for (int j = 0; j < kDirs; ++j) G[i][j] = 0.0;
    }
    G[0][0] = t[kDirs];
    for (int k = 0; k < cnt; ++k) {
        G[0][1 + k] = G[1 + k][0] = t[kDirs + 1 + k];
        for (int l = 0; l < cnt; ++l) G[1 + k][1 + l] = gram[k * kHistory + l];
    }
    double dmax = 0.0;
    for (int i = 0; i < m; ++i) dmax = fmax(dmax, G[i][i]);
    bool keep[kDirs];
    // Cholesky G = R^T R in place (upper triangle), dropping near-dependent directions
    for (int i = 0; i < m; ++i) {
        keep[i] = false;
        if (!(dmax > 0.0)) continue;
        double d = G[i][i] + 1e-12 * dmax;
        for (int k = 0; k < i; ++k)
            if (keep[k]) d -= G[k][i] * G[k][i];
        if (!(d > 1e-10 * (G[i][i] + 1e-300))) continue;
        keep[i] = true;
        const double rii = sqrt(d);
        G[i][i] = rii;
        for (int j = i + 1; j < m; ++j) {
            double v = G[i][j];
            for (int k = 0; k < i; ++k)
                if (keep[k]) v -= G[k][i] * G[k][j];
            G[i][j] = v / rii;
        }
    }
    // R^T z = h, R c = z over the kept directions
    double z[kDirs];
    for (int i = 0; i < m; ++i) {
        z[i] = 0.0;
        if (!keep[i]) continue;
        double v = h[i];
        for (int k = 0; k < i; ++k)
            if (keep[k]) v -= G[k][i] * z[k];
        z[i] = v / G[i][i];
    }
    for (int i = m - 1; i >= 0; --i) {
        if (!keep[i]) continue;
        double v = z[i];
        for (int j = i + 1; j < m; ++j)
            if (keep[j]) v -= G[i][j] * c[j];
        c[i] = v / G[i][i];
    }
    for (int j = 0; j < kDirs; ++j) coef[j] = c[j];
    res[0] = sqrt(t[2 * kDirs]);
    *used = c[0] != 0.0 ? 1 : 0;
}

// x0 = p + sum_j c_j D_j (x holds p); per-block partials of ||b - A x0||^2 =
// ||r0 - c_0 A d0 - sum_k c_k A h_k||^2.
__global__ void k_guess_combine(int n, const double* __restrict__ coef, const double* __restrict__ d0,
                                const double* __restrict__ a0, const double* __restrict__ hist,
                                const double* __restrict__ ahist, const int* __restrict__ ring,
                                const double* __restrict__ r0, double* x, double* part) {
    __shared__ double sh[40];
    const int cnt = ring[0];
    double c[kDirs];
#pragma unroll
    for (int j = 0; j < kDirs; ++j) c[j] = coef[j];
    double rr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double dx = c[0] * d0[i], dr = c[0] * a0[i];
#pragma unroll
        for (int k = 0; k < kHistory; ++k)
            if (k < cnt) {
                dx += c[1 + k] * hist[(size_t)k * n + i];
                dr += c[1 + k] * ahist[(size_t)k * n + i];
            }
        x[i] += dx;
        const double ri = r0[i] - dr;
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

// After the step: the step's increment into the ring's head slot.
__global__ void k_guess_increment(int n, const double* __restrict__ pnew, const double* __restrict__ p,
                                  const int* __restrict__ ring, double* hist) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    hist[(size_t)ring[1] * n + i] = pnew[i] - p[i];
}

// Images under A of the head slot (pass 1 of the insertion): ahist[head] = A hist[head].
__global__ void k_guess_ahead(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                              const double* __restrict__ val, const int* __restrict__ ring,
                              const double* __restrict__ hist, double* ahist) {
    const double* h = hist + (size_t)ring[1] * n;
    double* ah = ahist + (size_t)ring[1] * n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) s += val[k] * h[col[k]];
        ah[i] = s;
    }
}

// Per-block partials of hist_k . A hist[head] for all k (pass 2 of the insertion).
__global__ void k_guess_gram_dots(int n, const double* __restrict__ hist, const double* __restrict__ ahist,
                                  const int* __restrict__ ring, double* part) {
    __shared__ double sh[33 * kHistory];
    const double* ah = ahist + (size_t)ring[1] * n;
    double acc[kHistory];
#pragma unroll
    for (int k = 0; k < kHistory; ++k) acc[k] = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double a = ah[i];
#pragma unroll
        for (int k = 0; k < kHistory; ++k) acc[k] += hist[(size_t)k * n + i] * a;
    }
    block_sum_n<kHistory>(acc, sh);
    if (threadIdx.x == 0)
        for (int k = 0; k < kHistory; ++k) part[(size_t)kHistory * blockIdx.x + k] = acc[k];
}

// Row and column of the head slot in the Gram matrix, then advance the ring (one thread).
// Slots not yet written hold zeros (the ring's buffers start zeroed), so their dots are 0.
__global__ void k_guess_insert(int nb, const double* __restrict__ part, double* gram, int* ring) {
    const int head = ring[1];
    for (int k = 0; k < kHistory; ++k) {
        double t = 0.0;
        for (int b = 0; b < nb; ++b) t += part[(size_t)kHistory * b + k];
        gram[head * kHistory + k] = t;
        gram[k * kHistory + head] = t;
    }
    ring[0] = min(ring[0] + 1, kHistory);
    ring[1] = (head + 1) % kHistory;
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
        (s = G->p_prev.alloc(n)) || (s = G->d0.alloc(n)) || (s = G->r0.alloc(n)) || (s = G->a0.alloc(n)) ||
        (s = G->coef.alloc(kDirs)) || (s = G->part.alloc((size_t)kDots * G->blocks)) ||
        (s = G->hist.alloc((size_t)kHistory * n)) || (s = G->ahist.alloc((size_t)kHistory * n)) ||
        (s = G->gram.alloc(kHistory * kHistory)) || (s = G->ring.alloc(2)) ||
        (s = G->res.alloc(2)) || (s = G->scale_bits.alloc(3)) || (s = G->flag.alloc(1)))
        return fail(s);
    if (cudaMemset(G->p_prev.p, 0, sizeof(double) * n) != cudaSuccess ||
        cudaMemset(G->hist.p, 0, G->hist.bytes()) != cudaSuccess ||
        cudaMemset(G->ahist.p, 0, G->ahist.bytes()) != cudaSuccess ||
        cudaMemset(G->gram.p, 0, G->gram.bytes()) != cudaSuccess || cudaMemset(G->ring.p, 0, G->ring.bytes()) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "cudaMemset", __FILE__, __LINE__));
    *out = G;
    return PF2_OK;
}

// Sections: the previous pressure, the increment history with its images under A, their
// Gram matrix and ring position, then the network.  The rest of the guess's buffers are
// written before they are read within a step.
pf2_status guess_checkpoint(Guess* G, CkptFile& io, cudaStream_t st) {
    int n = G->n;
    PF2_TRY(io.host("gmeta", &n, sizeof(n)));
    PF2_REQUIRE(n == G->n, PF2_BAD_INPUT, "checkpoint guess has %d nodes, this mesh %d", n, G->n);
    PF2_TRY(io.device("gpprev", G->p_prev.p, G->p_prev.bytes(), st));
    PF2_TRY(io.device("ghist", G->hist.p, G->hist.bytes(), st));
    PF2_TRY(io.device("gahist", G->ahist.p, G->ahist.bytes(), st));
    PF2_TRY(io.device("ggram", G->gram.p, G->gram.bytes(), st));
    PF2_TRY(io.device("gring", G->ring.p, G->ring.bytes(), st));
    return mpnn_checkpoint(G->net, io, st);
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
    k_guess_dir<<<blocks_for(n), kThreads, 0, st>>>(n, G->y.p, G->scale_bits.p, G->d0.p);
    PF2_LAUNCH_CHECK();
    const int* rp = A->mesh->rowptr.p;
    const int* cl = A->mesh->col.p;
    k_guess_spmv<<<G->blocks, kThreads, 0, st>>>(n, rp, cl, A->val.p, b, x, G->d0.p, G->r0.p, G->a0.p);
    PF2_LAUNCH_CHECK();
    k_guess_dots<<<G->blocks, kThreads, 0, st>>>(n, G->d0.p, G->hist.p, G->ring.p, G->r0.p, G->a0.p, G->part.p);
    PF2_LAUNCH_CHECK();
    k_guess_solve<<<1, 1, 0, st>>>(G->blocks, G->part.p, G->gram.p, G->ring.p, G->coef.p, G->res.p, G->flag.p);
    PF2_LAUNCH_CHECK();
    k_guess_combine<<<G->blocks, kThreads, 0, st>>>(n, G->coef.p, G->d0.p, G->a0.p, G->hist.p, G->ahist.p, G->ring.p,
                                                    G->r0.p, x, G->part.p);
    PF2_LAUNCH_CHECK();
    k_guess_res1<<<1, 1, 0, st>>>(G->blocks, G->part.p, G->res.p);
    PF2_LAUNCH_CHECK();
    if (res_out) PF2_CUDA(cudaMemcpyAsync(res_out, G->res.p, 2 * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (used_out) PF2_CUDA(cudaMemcpyAsync(used_out, G->flag.p, sizeof(int), cudaMemcpyDeviceToDevice, st));
    return PF2_OK;
}

pf2_status guess_train(Guess* G, const pf2_csr* A, const double* p_new, float lr, cudaStream_t st) {
    const int n = G->n;
    // the step's increment joins the history (before p_saved is consumed below)
    k_guess_increment<<<blocks_for(n), kThreads, 0, st>>>(n, p_new, G->p_saved.p, G->ring.p, G->hist.p);
    PF2_LAUNCH_CHECK();
    k_guess_ahead<<<G->blocks, kThreads, 0, st>>>(n, A->mesh->rowptr.p, A->mesh->col.p, A->val.p, G->ring.p,
                                                  G->hist.p, G->ahist.p);
    PF2_LAUNCH_CHECK();
    k_guess_gram_dots<<<G->blocks, kThreads, 0, st>>>(n, G->hist.p, G->ahist.p, G->ring.p, G->part.p);
    PF2_LAUNCH_CHECK();
    k_guess_insert<<<1, 1, 0, st>>>(G->blocks, G->part.p, G->gram.p, G->ring.p);
    PF2_LAUNCH_CHECK();
    k_guess_target<<<blocks_for(n), kThreads, 0, st>>>(n, p_new, G->p_saved.p, G->scale_bits.p, G->target.p,
                                                       G->p_prev.p);
    PF2_LAUNCH_CHECK();
    if (lr > 0.0f) PF2_TRY(pf2_mpnn_train_step(G->net, G->feat.p, G->target.p, lr, 1, nullptr, st));
    return PF2_OK;
}

}  // namespace pf2
