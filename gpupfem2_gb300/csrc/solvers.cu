// solvers.cu - CSR SpMV, preconditioned CG and GMRES, Jacobi / ILU(0) / IC(0).
//
// Reference: src/linear_algebra/linear_solver.cu (CG :301-376, GMRES :378-521),
// preconditioners.cu (Jacobi :3-46, ILU(0) :48-134, IC(0) :136-213), linear_algebra.h
// (cuSPARSE SpMV, csrilu02/csric02, SpSV; cuBLAS dot/nrm2/trsv/gemv).
//
// Each solve is one cooperative launch: every iteration, its dot products and its
// convergence test run on the device, with bounded grid barriers between phases, so
// the host never waits inside a solve (the reference copies the residual to the host
// every iteration).  Reductions are summed in a fixed order: repeated solves give
// identical bits.  The ILU(0)/IC(0) factorisation and triangular solves walk the rows
// in level order; a row waits (bounded) until the rows it depends on are done.
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "device.cuh"
#include "internal.cuh"

namespace pf2 {

constexpr int kSolverThreads = 512;
constexpr int kMaxGmresSmem = 1024;
constexpr int kShDoubles = 136;  // block_sum_n / grid_reduce scratch (33 x 4 doubles)
constexpr int kMaxOuter = 40;    // refinements of the mixed-precision solver
constexpr double kMixedInnerEta = 0.3;  // mixed CG refines when the iterated residual drops by this factor
constexpr int kBandRows = 12288;  // rows per range of the banded triangular solve (96 KB FP64 window)
constexpr int kBandMinLevels = 128;  // dependency chains at least this long use the banded solve
constexpr int kSolverBlocksPerSm = 2;  // cooperative solver blocks per SM (grid-barrier cost vs parallelism)

struct Csr {
    int n;
    const int* rowptr;
    const int* col;
    const double* val;
    const int* diag;  // position of a_ii
};

// by other blocks during the kernel, so it is read through L2.
// Row i of A times x, one thread per row (rows of ~7 entries: a thread per row keeps the
// most loads in flight); x may be written by other blocks during the kernel, so it is read
// through L2.
__device__ __forceinline__ double row_dot(const Csr& A, int row, const double* x) {
    const int s = __ldg(&A.rowptr[row]), e = __ldg(&A.rowptr[row + 1]);
    double sum = 0.0;
    for (int k = s; k < e; ++k) sum += __ldg(&A.val[k]) * __ldcg(&x[__ldg(&A.col[k])]);
    return sum;
}

__global__ void k_spmv(Csr A, const double* __restrict__ x, double* __restrict__ y) {
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n; row += gridDim.x * blockDim.x)
        y[row] = row_dot(A, row, x);
}

// ------------------------------------------------------------ triangular data
// The factors live on the pattern of B = P A P^T, where P is the identity (natural
// order, as the reference) or a multicolour ordering; perm maps a row of B to the row of
// A, iperm back.
// Banded triangular solve plan: the rows of B cut into P contiguous ranges, one block per
// range.  Per direction, each range's rows are grouped by their level counted over the
// dependencies inside the range only, levels cut into steps of at most one row per thread
// (range r owns steps rstep[r] .. rstep[r + 1], step s holds slots sptr[s] .. sptr[s + 1]).
// A slot is one row with everything its solve needs at fixed-stride positions: the row,
// the index of its right-hand side, K dependency columns (-1 padded) and, gathered after
// each factorisation, their factor values and the inverse of the dividing diagonal.
struct BandDir {
    const int* rstep;
    const int* sptr;
    const int* row;    // [slot]
    const int* rhs;    // [slot] right-hand side index (A's numbering forward, B's backward)
    const int* dep;    // [slot * K + k]
    double* val;       // [slot * K + k] factor values
    double* dinv;      // [slot] 1 / dividing diagonal (1 for ILU forward)
    float* val32;      // FP32 copies (mixed precision)
    float* dinv32;
    // sync-free solve: the slots' level groups (slots gstart[g] .. gstart[g + 1])
    int ngroups;
    const int* gstart;
};

struct Band {
    int P;             // ranges; 0 = sync-free row-per-lane solve instead
    int R;             // rows per range (the block's shared-memory window)
    int K;             // dependency slots per row
    const int* rs;     // P + 1 range starts
    BandDir f, b;
};

struct Tri {
    int kind;              // PF2_PRECOND_ILU or PF2_PRECOND_IC
    Band band;
    Csr B;                 // pattern of the factors (val unused)
    const int* perm;
    const int* iperm;
    const int* fwd_order;  // rows of B in forward level order
    const int* bwd_order;  // rows of B in backward level order
    const int* lt_off;     // IC: rows of L^T (strictly upper), (row k, position of l_ki)
    const int* lt_row;
    const int* lt_pos;
    double* fact;          // factor values on the pattern of B
    double* tmp;           // forward result (numbering of B)
    double* outB;          // backward result (numbering of B)
    float* fact32;         // mixed precision: FP32 copies of the three above
    float* tmp32;
    float* outB32;
    int* done_f;           // per-row epoch flags
    int* done_b;
    unsigned* tickets;     // one counter per (apply, direction)
    int* rec;              // where a wait gave up (GridBarrier::rec)
    // CG on B itself (orderings without the banded plan): A's values in B's
    // numbering, the factors as one array on B's pattern (row i: L to the left of the
    // diagonal, the upper factor to the right, 1 / dividing diagonal on it) and x in B's
    // numbering
    int csr;
    const double* bval;
    const double* fsym;
    double* xB;
    const float* bval32;   // mixed precision: FP32 copies of bval and fsym
    const float* fsym32;
    // B's rows in sweep groups: group g holds rows cstart[g] .. cstart[g + 1] (the colours
    // of a multicolour order, or all rows), swept one group after the other
    int ngroups;
    const int* cstart;
};

__device__ __forceinline__ bool wait_flag(const int* flag, int epoch, int* err, int* rec, int row, int dep) {
    long long polls = 0;
    while (*(volatile const int*)flag != epoch) {
        if (++polls > kFlagPolls) {
            atomicExch(err, (int)DEV_TIMEOUT);
            record_timeout(rec, 2, row, dep, epoch, *(volatile const int*)flag);
            return false;
        }
        if (*(volatile int*)err != 0) return false;
    }
    __threadfence();
    return true;
}

// "Not yet written" marker of the triangular-solve vectors: all bits set, a NaN that
// arithmetic never produces (the GPU returns its canonical NaN), so a byte memset of
// 0xff initialises a vector to it.
template <class V> struct Pending;
template <> struct Pending<double> {
    using Bits = unsigned long long;
    static constexpr Bits kBits = ~0ull;
    __device__ static Bits bits(double v) { return (Bits)__double_as_longlong(v); }
    __device__ static double marker() { return __longlong_as_double((long long)kBits); }
};
template <> struct Pending<float> {
    using Bits = unsigned int;
    static constexpr Bits kBits = ~0u;
    __device__ static Bits bits(float v) { return (Bits)__float_as_uint(v); }
    __device__ static float marker() { return __uint_as_float(kBits); }
};

// Value of row j of the vector being solved for, once its writer has stored it (bounded).
template <class V>
__device__ __forceinline__ bool wait_value(const V* dst, int j, V& out, int* err, int* rec, int row) {
    long long polls = 0;
    while (true) {
        const V v = *(volatile const V*)&dst[j];
        if (Pending<V>::bits(v) != Pending<V>::kBits) { out = v; return true; }
        if (++polls > kFlagPolls) {
            atomicExch(err, (int)DEV_TIMEOUT);
            record_timeout(rec, 2, row, j, 0, 0);
            return false;
        }
        if (*(volatile int*)err != 0) return false;
    }
}

// Sync-free triangular solve, one row per lane: warps take 32 rows at a time in level
// order from a shared ticket counter, so every row a lane waits on was taken earlier by a
// running lane.  The vector solved for starts as all "pending" markers and a row's value
// doubles as its completion flag (one 8-byte store, no fence, no separate flag).
// dir 0: forward  tmp = L^{-1} src (unit diagonal for ILU, l_ii for IC), src in A's numbering
// dir 1: backward dst = U^{-1} tmp (ILU) or L^{-T} tmp (IC); each row resets its tmp entry
// to pending after reading it, ready for the next forward solve.
// V is double (the FP64 preconditioner) or float (the FP32 apply of the mixed solver).
template <class V>
__device__ void tri_solve(const Tri& T, int dir, V* src, V* dst, const V* fact, unsigned* ticket, int* err) {
    const int lane = threadIdx.x & 31;
    const Csr& A = T.B;
    const int* order = dir == 0 ? T.fwd_order : T.bwd_order;
    const bool ic = T.kind == PF2_PRECOND_IC;
    while (true) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(ticket, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= (unsigned)A.n) break;
        const unsigned t = base + lane;
        if (t < (unsigned)A.n) {
            const int i = __ldg(&order[t]);
            int s, e;
            const int* cols;
            if (dir == 0) {
                s = __ldg(&A.rowptr[i]);
                e = __ldg(&A.diag[i]);
                cols = A.col;
            } else if (!ic) {
                s = __ldg(&A.diag[i]) + 1;
                e = __ldg(&A.rowptr[i + 1]);
                cols = A.col;
            } else {
                s = __ldg(&T.lt_off[i]);
                e = __ldg(&T.lt_off[i + 1]);
                cols = T.lt_row;
            }
            const V in = __ldcg(&src[dir == 0 ? __ldg(&T.perm[i]) : i]);
            const V d = (dir == 1 || ic) ? __ldcg(&fact[__ldg(&A.diag[i])]) : V(1);
            V sum = V(0);
            bool ok = true;
            for (int k = s; k < e; ++k) {
                const int j = __ldg(&cols[k]);
                const V f = __ldcg(&fact[(dir == 1 && ic) ? __ldg(&T.lt_pos[k]) : k]);
                V xj;
                if (!wait_value(dst, j, xj, err, T.rec, i)) { ok = false; break; }
                sum += f * xj;
            }
            if (ok) {
                V v = in - sum;
                if (dir == 1 || ic) v = v / d;
                __stcg(&dst[i], v);
                if (dir == 1) __stcg(&src[i], Pending<V>::marker());
            }
        }
        // warp-uniform exit: every lane reaches the next ticket broadcast or none does
        if (__any_sync(0xffffffffu, *(volatile int*)err != 0)) break;
    }
}

extern __shared__ __align__(16) unsigned char pf2_band_smem[];

// Banded triangular solve: block b takes ranges b, b + G, ... (forward in increasing,
// backward in decreasing order: a range waits only on ranges solved before it).  Steps
// of a range are separated by __syncthreads; values of the range come from the block's
// shared-memory window, values of other ranges are waited for as in tri_solve.  Each
// thread loads its next step's slot while it solves the current one, so a dependency
// chain costs one block barrier per step.  The diagonal division of tri_solve is a
// multiplication by the stored inverse here.
template <class V> struct BandVals;
template <> struct BandVals<double> {
    __device__ static const double* val(const BandDir& D) { return D.val; }
    __device__ static const double* dinv(const BandDir& D) { return D.dinv; }
};
template <> struct BandVals<float> {
    __device__ static const float* val(const BandDir& D) { return D.val32; }
    __device__ static const float* dinv(const BandDir& D) { return D.dinv32; }
};

constexpr int kBandMaxDeps = 8;

__device__ __forceinline__ void prefetch_l1(const void* p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// Pull slot t's fixed-stride record into L1 ahead of its step.
template <class V>
__device__ __forceinline__ void band_prefetch(const BandDir& D, int K, int t) {
    prefetch_l1(D.row + t);
    prefetch_l1(D.rhs + t);
    prefetch_l1(BandVals<V>::dinv(D) + t);
    prefetch_l1(D.dep + (size_t)t * K);
    prefetch_l1(D.dep + (size_t)t * K + K - 1);
    prefetch_l1(BandVals<V>::val(D) + (size_t)t * K);
    prefetch_l1(BandVals<V>::val(D) + (size_t)t * K + K - 1);
}

template <class V>
__device__ bool tri_solve_banded(const Tri& T, int dir, V* src, V* dst, int* err) {
    const Band& Bd = T.band;
    const BandDir& D = dir == 0 ? Bd.f : Bd.b;
    const int K = Bd.K;
    const V* vals = BandVals<V>::val(D);
    const V* dinv = BandVals<V>::dinv(D);
    V* xs = reinterpret_cast<V*>(pf2_band_smem);
    bool failed = false;
    const int tid = (int)threadIdx.x;
    const int nmine = blockIdx.x < Bd.P ? (Bd.P - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    for (int q = 0; q < nmine; ++q) {
        const int r = (int)blockIdx.x + (dir == 0 ? q : nmine - 1 - q) * (int)gridDim.x;
        const int r0 = __ldg(&Bd.rs[r]), r1 = __ldg(&Bd.rs[r + 1]);
        const int s0 = __ldg(&D.rstep[r]), s1 = __ldg(&D.rstep[r + 1]);
        // slot of this thread in the current and next step; the right-hand side of the
        // next step is loaded one step ahead, the rest of its record prefetched to L1
        int t = __ldg(&D.sptr[s0]) + tid, te = __ldg(&D.sptr[s0 + 1]);
        V in = V(0);
        if (t < te) in = __ldcg(&src[__ldg(&D.rhs[t])]);
        if (s0 + 1 < s1) {
            const int u = te + tid;
            if (u < __ldg(&D.sptr[s0 + 2])) band_prefetch<V>(D, K, u);
        }
        for (int st = s0; st < s1; ++st) {
            int tn = 0, tne = 0;
            V in_next = V(0);
            if (st + 1 < s1) {
                tn = te + tid;
                tne = __ldg(&D.sptr[st + 2]);
                if (tn < tne) in_next = __ldcg(&src[__ldg(&D.rhs[tn])]);
                if (st + 2 < s1) {
                    const int u = tne + tid;
                    if (u < __ldg(&D.sptr[st + 3])) band_prefetch<V>(D, K, u);
                }
            }
            if (t < te) {
                const int row = __ldg(&D.row[t]);
                const V di = __ldg(&dinv[t]);
                V sum = V(0);
                bool ok = true;
                for (int k = 0; k < K; ++k) {
                    const int j = __ldg(&D.dep[(size_t)t * K + k]);
                    if (j < 0) break;
                    const V f = __ldg(&vals[(size_t)t * K + k]);
                    V xj;
                    if (j >= r0 && j < r1) {
                        xj = xs[j - r0];
                    } else if (!wait_value(dst, j, xj, err, T.rec, row)) {
                        ok = false;
                        break;
                    }
                    sum += f * xj;
                }
                if (ok) {
                    const V v = (in - sum) * di;
                    xs[row - r0] = v;
                    __stcg(&dst[row], v);
                    if (dir == 1) __stcg(&src[row], Pending<V>::marker());
                } else {
                    failed = true;
                }
            }
            if (__syncthreads_or(failed)) return false;
            t = tn;
            te = tne;
            in = in_next;
        }
    }
    return true;
}

// Sync-free triangular solve on the slot records in level order, for orderings with few
// levels (multicolour): thread g solves slots g, g + T, ... (T threads in the grid) in
// increasing order.  In a cooperative launch every thread is resident, so the lowest
// unsolved slot always belongs to a thread that has reached it (its own earlier slots are
// lower and solved) and whose dependencies, in lower levels, are solved: no tickets.
// sum_k f_k x_{j_k} over a slot's dependencies, four at a time: the four value loads are
// issued together, then only the ones still pending are polled (one round trip instead
// of four when the dependencies are already solved).  Terms are added in slot order.
template <class V>
__device__ __forceinline__ bool slot_dot(const V* dst, const int* dep, const V* val, int K, int row, int* err,
                                         int* rec, V& sum) {
    sum = V(0);
    for (int k0 = 0; k0 < K; k0 += 4) {
        int j[4];
        V x[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) j[k] = k0 + k < K ? __ldg(&dep[k0 + k]) : -1;
#pragma unroll
        for (int k = 0; k < 4; ++k) x[k] = j[k] >= 0 ? *(volatile const V*)&dst[j[k]] : V(0);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (j[k] >= 0 && Pending<V>::bits(x[k]) == Pending<V>::kBits &&
                !wait_value(dst, j[k], x[k], err, rec, row))
                return false;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (j[k] >= 0) sum += __ldg(&val[k0 + k]) * x[k];
        if (j[3] < 0) break;
    }
    return true;
}

template <class V>
__device__ void tri_solve_slots(const Tri& T, int dir, V* src, V* dst, int* err) {
    const BandDir& D = dir == 0 ? T.band.f : T.band.b;
    const int K = T.band.K;
    const int n = T.B.n;
    const V* vals = BandVals<V>::val(D);
    const V* dinv = BandVals<V>::dinv(D);
    const int stride = gridDim.x * blockDim.x;
    (void)n;
    for (int gi = 0; gi < D.ngroups; ++gi)
    for (int t = __ldg(&D.gstart[gi]) + blockIdx.x * blockDim.x + threadIdx.x, g1 = __ldg(&D.gstart[gi + 1]); t < g1;
         t += stride) {
        const int row = __ldg(&D.row[t]);
        const V in = __ldcg(&src[__ldg(&D.rhs[t])]);
        const V di = __ldg(&dinv[t]);
        V sum;
        if (!slot_dot(dst, D.dep + (size_t)t * K, vals + (size_t)t * K, K, row, err, T.rec, sum)) return;
        __stcg(&dst[row], (in - sum) * di);
        if (dir == 1) __stcg(&src[row], Pending<V>::marker());
    }
}

// One CG iteration's preconditioner work on the slot path, fused with its vector
// updates (FP64 PCG, few-level orderings): the forward sweep updates x and r of its row
// (x += alpha p, r -= alpha q) before it solves with the new r, and resets the backward
// vector; the backward sweep writes z in A's numbering and the terms of r.z.  Rows are
// owned by slots here, not by block row ranges, so every vector crossing between the two
// is read through L2.  Returns this thread's r.r (forward) or r.z (backward) terms.
template <class V> struct SlotVecs;
template <> struct SlotVecs<double> {
    __device__ static double* tmp(const Tri& T) { return T.tmp; }
    __device__ static double* outB(const Tri& T) { return T.outB; }
};
template <> struct SlotVecs<float> {
    __device__ static float* tmp(const Tri& T) { return T.tmp32; }
    __device__ static float* outB(const Tri& T) { return T.outB32; }
};

// V = double for the FP64 PCG (x the solution), float for the mixed one (x the FP32
// update d); the thread's terms are summed in V and returned in FP64.
template <class V>
__device__ double slots_fwd_cg(const Tri& T, V alpha, V* r, const V* q, V* x, const V* p, int* err) {
    const BandDir& D = T.band.f;
    const int K = T.band.K;
    const int n = T.B.n;
    const int stride = gridDim.x * blockDim.x;
    const V* vals = BandVals<V>::val(D);
    const V* dinv = BandVals<V>::dinv(D);
    V* tmp = SlotVecs<V>::tmp(T);
    V* outB = SlotVecs<V>::outB(T);
    V rr = V(0);
    (void)n;
    for (int gi = 0; gi < D.ngroups; ++gi)
    for (int t = __ldg(&D.gstart[gi]) + blockIdx.x * blockDim.x + threadIdx.x, g1 = __ldg(&D.gstart[gi + 1]); t < g1;
         t += stride) {
        const int row = __ldg(&D.row[t]);
        const int ai = __ldg(&D.rhs[t]);  // the row in A's numbering
        const V ra = __ldcg(&r[ai]) - alpha * __ldcg(&q[ai]);
        __stcg(&r[ai], ra);
        __stcg(&x[ai], __ldcg(&x[ai]) + alpha * __ldcg(&p[ai]));
        rr += ra * ra;
        V sum;
        if (!slot_dot(tmp, D.dep + (size_t)t * K, vals + (size_t)t * K, K, row, err, T.rec, sum)) break;
        __stcg(&tmp[row], (ra - sum) * __ldg(&dinv[t]));
        __stcg(&outB[row], Pending<V>::marker());
    }
    return (double)rr;
}

template <class V>
__device__ double slots_bwd_cg(const Tri& T, const V* r, V* z, int* err) {
    const BandDir& D = T.band.b;
    const int K = T.band.K;
    const int n = T.B.n;
    const int stride = gridDim.x * blockDim.x;
    const V* vals = BandVals<V>::val(D);
    const V* dinv = BandVals<V>::dinv(D);
    V* tmp = SlotVecs<V>::tmp(T);
    V* outB = SlotVecs<V>::outB(T);
    V rz = V(0);
    (void)n;
    for (int gi = 0; gi < D.ngroups; ++gi)
    for (int t = __ldg(&D.gstart[gi]) + blockIdx.x * blockDim.x + threadIdx.x, g1 = __ldg(&D.gstart[gi + 1]); t < g1;
         t += stride) {
        const int row = __ldg(&D.row[t]);
        const V in = __ldcg(&tmp[row]);
        V sum;
        if (!slot_dot(outB, D.dep + (size_t)t * K, vals + (size_t)t * K, K, row, err, T.rec, sum)) break;
        const V v = (in - sum) * __ldg(&dinv[t]);
        __stcg(&outB[row], v);
        __stcg(&tmp[row], Pending<V>::marker());
        const int ai = __ldg(&T.perm[row]);
        __stcg(&z[ai], v);
        rz += __ldcg(&r[ai]) * v;
    }
    return (double)rz;
}

// Zero-fill factorisations on the CSR pattern (csrilu02 / csric02 semantics), one row
// per warp in level order, lane 0 working through the row.
__global__ void k_factor(Tri T, const int* __restrict__ order, unsigned* ticket, const int* epoch_ptr, int* err) {
    const Csr& A = T.B;
    const int lane = threadIdx.x & 31;
    const int epoch = *epoch_ptr + 1;
    double* a = T.fact;
    while (true) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(ticket, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= (unsigned)A.n) break;
        bool ok = true;
        const int i = order[t];
        if (lane == 0) {
            const int s = A.rowptr[i], d = A.diag[i], e = A.rowptr[i + 1];
            if (T.kind == PF2_PRECOND_ILU) {
                for (int kk = s; kk < d && ok; ++kk) {
                    const int k = A.col[kk];
                    if (!wait_flag(&T.done_f[k], epoch, err, T.rec, i, k)) { ok = false; break; }
                    const double aik = __ldcg(&a[kk]) / __ldcg(&a[A.diag[k]]);
                    __stcg(&a[kk], aik);
                    const int ks = A.diag[k] + 1, ke = A.rowptr[k + 1];
                    int q = ks;
                    for (int jj = kk + 1; jj < e; ++jj) {
                        const int j = A.col[jj];
                        while (q < ke && A.col[q] < j) ++q;
                        if (q < ke && A.col[q] == j) __stcg(&a[jj], __ldcg(&a[jj]) - aik * __ldcg(&a[q]));
                    }
                }
            } else {
                for (int kk = s; kk < d && ok; ++kk) {
                    const int k = A.col[kk];
                    if (!wait_flag(&T.done_f[k], epoch, err, T.rec, i, k)) { ok = false; break; }
                    double sum = __ldcg(&a[kk]);
                    int p = s, q = A.rowptr[k];
                    const int qe = A.diag[k];
                    while (p < kk && q < qe) {
                        const int cp = A.col[p], cq = A.col[q];
                        if (cp == cq) { sum -= __ldcg(&a[p]) * __ldcg(&a[q]); ++p; ++q; }
                        else if (cp < cq) ++p;
                        else ++q;
                    }
                    __stcg(&a[kk], sum / __ldcg(&a[A.diag[k]]));
                }
                if (ok) {
                    double dd = __ldcg(&a[d]);
                    for (int kk = s; kk < d; ++kk) { const double l = __ldcg(&a[kk]); dd -= l * l; }
                    __stcg(&a[d], sqrt(dd));
                }
            }
        }
        // lanes 1..31 wait here while lane 0 works through the row
        if (__any_sync(0xffffffffu, !ok)) return;
        if (lane == 0) {
            __threadfence();
            atomicExch(&T.done_f[i], epoch);
        }
    }
}

// ----------------------------------------------------------------- CG / GMRES
struct SolveOut {
    int iterations;
    int converged;
    double residual;
    int status;
    int pad;
    double relres;  // ||r|| / ||b|| at the end (the iterated residual; the true one for MIXED)
};

// ------------------------------------------------------------ partitioned CG
// CG with the rows cut into one part per block (a breadth-first recursive bisection of the
// matrix graph, one block per SM): a part's rows are consecutive in the part order Q (by
// part, then sweep group, then B's order), and their r, p, q, t, z live in the block's
// shared memory for the whole solve.  Only a part's boundary rows (rows with a neighbour in
// another part) go through global memory: their p (read by neighbours' SpMV after a grid
// barrier) and their forward and backward results t and z (read by neighbours' sweeps,
// polled on the pending marker as in the CSR sweeps).  Inside a part the sweep groups
// (colours) follow one another behind a __syncthreads.  Each row's arithmetic (SpMV entry
// order, sweep sums, vector updates) is that of k_pcg (Jacobi / none) and pcg_csr
// (ILU(0) / IC(0) on B); the reductions sum the blocks' rows in another order.
struct PartCg {
    int P;                    // parts (the grid's blocks)
    int R;                    // rows of the largest part (shared-memory vector length)
    int ng;                   // sweep groups per part (1 with Jacobi / none)
    const int* qs;            // group starts: part p group g holds rows qs[p ng + g] .. qs[p ng + g + 1]
    const int* rp;            // CSR in Q order, each row's entries in B's (or A's) order
    const int* col;
    const int* diag;
    const int* qa;            // Q row -> row of A
    const unsigned char* bnd; // 1: the row has a neighbour in another part
    const double* val;        // A's values in Q order (gathered per solve)
    const double* f;          // factors in Q order (B's fsym layout: L left, upper right, 1 / pivot on the diagonal)
    double* x;                // x in Q order (the solve's iterate)
    double* gp;               // boundary rows' p, t, z (t and z start as the pending marker)
    double* gt;
    double* gz;
    // mixed precision: FP32 values and factors in Q order, FP32 boundary copies
    const float* val32;
    const float* f32;
    float* gp32;
    float* gt32;
    float* gz32;
};

struct KArgs {
    Csr A;
    int precond;
    double* x;
    const double* b;
    double *r, *z, *p, *q, *invd;
    double* s;        // one-reduction CG: s = A p; BiCGStab: s = r - alpha v
    int variant;      // PF2_CG_*
    double *rhat, *y, *t;  // BiCGStab: shadow residual, M^{-1} p, A M^{-1} s
    double* partial;  // 4 arrays of gridDim doubles
    GridBarrier bar;
    Tri T;
    const int* epoch;  // device counter: this launch uses epochs *epoch + 1 ..
    double tol;
    int maxit;
    int criterion;
    SolveOut* out;
    // GMRES
    double* V;      // (m+1) x n
    double* H;      // m x m, column-major
    int m;          // Krylov dimension
    int gs;         // PF2_GS_MODIFIED or PF2_GS_CLASSICAL_TWICE
    double* vpart;  // (m + 1) x gridDim partial dots (classical Gram-Schmidt)
    double* vtot;   // m + 1 totals
    // mixed precision
    const float* val32;   // FP32 copy of the matrix values
    float *d32, *r32, *p32, *q32, *z32, *invd32;
    float* p32b;  // second direction array of the mixed CSR path
    int fuse_p;   // CSR paths: direction update inside the SpMV (1) or separate (0)
    double* pipe;  // pipelined CG: u, w, z and three m arrays (6 n)
    double inner_eta;     // inner solves stop at ||r_inner|| <= eta ||r_outer||
    int max_outer;
    PartCg part;  // partitioned CG (k_pcg_part)
};

__device__ __forceinline__ void row_range(int n, int& r0, int& r1) {
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    r0 = min(n, (int)blockIdx.x * chunk);
    r1 = min(n, r0 + chunk);
}

// Preconditioner apply z = M^{-1} r over the rows of this block (Jacobi) or the whole
// grid (ILU/IC; includes grid barriers).  `apply` counts the applies of this solve.
__device__ bool precond_apply(const KArgs& a, const double* src, double* dst, int r0, int r1, int apply,
                              int ep_base) {
    if (a.precond == PF2_PRECOND_ILU || a.precond == PF2_PRECOND_IC) {
        if (a.T.band.P) {
            tri_solve_banded<double>(a.T, 0, const_cast<double*>(src), a.T.tmp, a.bar.err);
            if (!grid_sync(a.bar, gridDim.x)) return false;
            tri_solve_banded<double>(a.T, 1, a.T.tmp, a.T.outB, a.bar.err);
        } else if (a.T.band.K) {
            tri_solve_slots<double>(a.T, 0, const_cast<double*>(src), a.T.tmp, a.bar.err);
            if (!grid_sync(a.bar, gridDim.x)) return false;
            tri_solve_slots<double>(a.T, 1, a.T.tmp, a.T.outB, a.bar.err);
        } else {
            tri_solve<double>(a.T, 0, const_cast<double*>(src), a.T.tmp, a.T.fact, &a.T.tickets[2 * apply],
                              a.bar.err);
            if (!grid_sync(a.bar, gridDim.x)) return false;
            tri_solve<double>(a.T, 1, a.T.tmp, a.T.outB, a.T.fact, &a.T.tickets[2 * apply + 1], a.bar.err);
        }
        if (!grid_sync(a.bar, gridDim.x)) return false;
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const int k = a.T.iperm[i];
            dst[i] = __ldcg(&a.T.outB[k]);
            __stcg(&a.T.outB[k], Pending<double>::marker());
        }
        __syncthreads();
        return true;
    }
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x)
        dst[i] = (a.precond == PF2_PRECOND_JACOBI) ? src[i] * a.invd[i] : src[i];
    return true;
}

// q = A p over the block's rows r0..r1 with this thread's p.q terms (values val, which
// may be A's or an FP32 copy): the thread's rows
// (r0 + tid + u * blockDim, u = 0..3) walked together, so the loads of four rows are in
// flight at once; each row sums its entries in order, as row_dot.
template <class V>
__device__ __forceinline__ V spmv_rows(const Csr& A, const V* __restrict__ val, const V* p, V* q, int r0, int r1) {
    V pq = V(0);
    for (int i0 = r0 + threadIdx.x; i0 < r1; i0 += 4 * blockDim.x) {
        int s[4], e[4];
        V acc[4] = { V(0), V(0), V(0), V(0) };
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = i0 + u * blockDim.x;
            s[u] = i < r1 ? __ldg(&A.rowptr[i]) : 0;
            e[u] = i < r1 ? __ldg(&A.rowptr[i + 1]) : 0;
        }
        int len = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) len = max(len, e[u] - s[u]);
        for (int k = 0; k < len; ++k) {
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (s[u] + k < e[u]) acc[u] += __ldg(&val[s[u] + k]) * __ldcg(&p[__ldg(&A.col[s[u] + k])]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = i0 + u * blockDim.x;
            if (i < r1) {
                __stcg(&q[i], acc[u]);
                pq += __ldcg(&p[i]) * acc[u];
            }
        }
    }
    return pq;
}

__device__ __forceinline__ double spmv_rows(const Csr& A, const double* p, double* q, int r0, int r1) {
    return spmv_rows<double>(A, A.val, p, q, r0, r1);
}

__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// The direction update fused into the SpMV: q = A pn with pn = z + beta po formed on the
// fly at every column (po and z are read-only in this phase), and the block's own rows of
// pn stored; each pn entry is one fma, so the stored pn and the values the SpMV used
// carry the same bits.  Saves the grid barrier between a separate direction update and
// the SpMV.  Returns the thread's pn.q terms.
template <class V>
__device__ __forceinline__ V spmv_rows_pz(const Csr& A, const V* __restrict__ val, const V* z, const V* po, V beta,
                                          V* pn, V* q, int r0, int r1) {
    V pq = V(0);
    for (int i0 = r0 + threadIdx.x; i0 < r1; i0 += 4 * blockDim.x) {
        int s[4], e[4];
        V acc[4] = { V(0), V(0), V(0), V(0) };
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = i0 + u * blockDim.x;
            s[u] = i < r1 ? __ldg(&A.rowptr[i]) : 0;
            e[u] = i < r1 ? __ldg(&A.rowptr[i + 1]) : 0;
        }
        int len = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) len = max(len, e[u] - s[u]);
        for (int k = 0; k < len; ++k) {
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (s[u] + k < e[u]) {
                    const int j = __ldg(&A.col[s[u] + k]);
                    acc[u] += __ldg(&val[s[u] + k]) * fma_rn(beta, __ldcg(&po[j]), __ldcg(&z[j]));
                }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = i0 + u * blockDim.x;
            if (i < r1) {
                const V pi = fma_rn(beta, __ldcg(&po[i]), __ldcg(&z[i]));
                __stcg(&pn[i], pi);
                __stcg(&q[i], acc[u]);
                pq += pi * acc[u];
            }
        }
    }
    return pq;
}

// p = z + beta p over the block's rows, four rows per pass with the loads first (z is
// written by other blocks' threads in the sweeps: read through L2).
template <class V>
__device__ __forceinline__ void p_update(V* p, const V* z, V beta, int r0, int r1) {
    for (int i0 = r0 + threadIdx.x; i0 < r1; i0 += 4 * blockDim.x) {
        V zv[4], pv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = i0 + u * blockDim.x;
            zv[u] = i < r1 ? __ldcg(&z[i]) : V(0);
            pv[u] = i < r1 ? __ldcg(&p[i]) : V(0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = i0 + u * blockDim.x;
            if (i < r1) __stcg(&p[i], zv[u] + beta * pv[u]);
        }
    }
}

// sum_k f_k x_{col_k} over the CSR entries [k0, k1) of a row whose x entries other
// threads of the same sweep are still writing: four entries loaded together, only the
// pending ones polled (bounded); terms added in entry order.
template <class V>
__device__ __forceinline__ bool csr_dot_wait(const V* x, const int* __restrict__ col, const V* __restrict__ f,
                                             int k0, int k1, int row, int* err, int* rec, V& sum) {
    sum = V(0);
    for (int k = k0; k < k1; k += 4) {
        int j[4];
        V v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) j[u] = k + u < k1 ? __ldg(&col[k + u]) : -1;
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = j[u] >= 0 ? *(volatile const V*)&x[j[u]] : V(0);
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (j[u] >= 0 && Pending<V>::bits(v[u]) == Pending<V>::kBits &&
                !wait_value(x, j[u], v[u], err, rec, row))
                return false;
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (j[u] >= 0) sum += __ldg(&f[k + u]) * v[u];
    }
    return true;
}

// Forward sweep of one CG iteration on B: group after group (a colour of a multicolour
// order, so a group's rows depend only on earlier groups), thread t taking rows
// g0 + t, g0 + t + T, ... of each.  Every thread's rows follow B's order and a row's
// dependencies are lower rows, so the lowest unsolved row always belongs to a thread
// that has reached it.  First the row's vector updates: MODE 1
// x += alpha p, r -= alpha q (q = A p); MODE 2 (one-reduction CG, q = A z) p = z + beta p,
// s = q + beta s, x += alpha p, r -= alpha s (first: p = z, s = q).  Writes the forward
// result and resets the row of z to the pending marker for the backward sweep.  Returns
// the thread's r.r terms (x; zero unless want_rr) and t.t terms of the forward result t
// (y): with IC(0), t = L^{-1} r and z = L^{-T} t, so r.z = t.t.
template <class V> struct CsrVecs;
template <> struct CsrVecs<double> {
    __device__ static double* tmp(const Tri& T) { return T.tmp; }
    __device__ static const double* fsym(const Tri& T) { return T.fsym; }
};
template <> struct CsrVecs<float> {
    __device__ static float* tmp(const Tri& T) { return T.tmp32; }
    __device__ static const float* fsym(const Tri& T) { return T.fsym32; }
};

template <int MODE, class V = double>
__device__ double2 csr_fwd(const Tri& T, V alpha, V beta, bool first, V* r, const V* q, V* x, V* p, V* sv, V* z,
                           int* err, bool want_rr = true) {
    V* tmp = CsrVecs<V>::tmp(T);
    const V* fsym = CsrVecs<V>::fsym(T);
    const int n = T.B.n;
    const int stride = gridDim.x * blockDim.x;
    const bool unit = T.kind != PF2_PRECOND_IC;  // ILU: L has a unit diagonal
    double rr = 0.0, tt = 0.0;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    (void)n;
    for (int gi = 0; gi < T.ngroups; ++gi) {
    const int g0 = __ldg(&T.cstart[gi]), g1 = __ldg(&T.cstart[gi + 1]);
    // each row's pattern bounds are loaded one row ahead
    int row = g0 + tid;
    int k0n = 0, dn = 0;
    if (row < g1) {
        k0n = __ldg(&T.B.rowptr[row]);
        dn = __ldg(&T.B.diag[row]);
    }
    for (; row < g1; row += stride) {
        const int k0 = k0n, d = dn;
        if (row + stride < g1) {
            k0n = __ldg(&T.B.rowptr[row + stride]);
            dn = __ldg(&T.B.diag[row + stride]);
        }
        V ra = __ldcg(&r[row]);
        if (MODE == 1) {
            ra -= alpha * __ldcg(&q[row]);
            __stcg(&r[row], ra);
            __stcg(&x[row], __ldcg(&x[row]) + alpha * __ldcg(&p[row]));
        } else if (MODE == 2) {
            const V zr = __ldcg(&z[row]), wr = __ldcg(&q[row]);
            const V pr = first ? zr : zr + beta * __ldcg(&p[row]);
            const V sr = first ? wr : wr + beta * __ldcg(&sv[row]);
            __stcg(&p[row], pr);
            __stcg(&sv[row], sr);
            __stcg(&x[row], __ldcg(&x[row]) + alpha * pr);
            ra -= alpha * sr;
            __stcg(&r[row], ra);
        }
        if (want_rr) rr += (double)ra * (double)ra;
        V sum;
        if (!csr_dot_wait(tmp, T.B.col, fsym, k0, d, row, err, T.rec, sum)) break;
        const V v = unit ? ra - sum : (ra - sum) * __ldg(&fsym[d]);
        __stcg(&tmp[row], v);
        __stcg(&z[row], Pending<V>::marker());
        tt += (double)v * (double)v;
    }
    }
    return make_double2(rr, tt);
}

// Backward sweep (groups and rows in reverse order): z = U^{-1} t, the forward result reset to the
// marker; with p_init the first direction p = z is stored too (PUPD: the direction update
// p = z + beta p instead, one fma per row).  Returns the r.z terms (none with PUPD).
template <class V = double, bool PUPD = false>
__device__ double csr_bwd(const Tri& T, const V* r, V* z, V* p_init, int* err, V beta = V(0)) {
    V* tmp = CsrVecs<V>::tmp(T);
    const V* fsym = CsrVecs<V>::fsym(T);
    const int n = T.B.n;
    const int stride = gridDim.x * blockDim.x;
    double rz = 0.0;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    (void)n;
    for (int gi = T.ngroups - 1; gi >= 0; --gi) {
    // rows g1 - 1 - t, g1 - 1 - t - stride, ... of the group, highest first
    const int g0 = __ldg(&T.cstart[gi]), g1 = __ldg(&T.cstart[gi + 1]);
    int row = g1 - 1 - tid;
    int dn = 0, k1n = 0;
    if (row >= g0) {
        dn = __ldg(&T.B.diag[row]);
        k1n = __ldg(&T.B.rowptr[row + 1]);
    }
    for (; row >= g0; row -= stride) {
        const int d = dn, k1 = k1n;
        if (row - stride >= g0) {
            dn = __ldg(&T.B.diag[row - stride]);
            k1n = __ldg(&T.B.rowptr[row - stride + 1]);
        }
        const V in = __ldcg(&tmp[row]);
        V sum;
        if (!csr_dot_wait(z, T.B.col, fsym, d + 1, k1, row, err, T.rec, sum)) break;
        const V v = (in - sum) * __ldg(&fsym[d]);
        __stcg(&z[row], v);
        if (PUPD)
            __stcg(&p_init[row], fma_rn(beta, __ldcg(&p_init[row]), v));
        else if (p_init)
            __stcg(&p_init[row], v);
        __stcg(&tmp[row], Pending<V>::marker());
        if (!PUPD) rz += (double)__ldcg(&r[row]) * (double)v;
    }
    }
    return rz;
}

// PCG in B's numbering (the ordering's permuted system B = P A P^T, with b and x
// permuted on the way in and out): the SpMV, the two sweeps and every vector run on
// B's CSR arrays, so the whole iteration reads one compact set of arrays (A's values on
// B's pattern, the factors, six vectors) that stays in L2 at a million rows.  ILU(0): the
// iteration of k_pcg, four barriers (p.q reduction, forward -> backward, r.z reduction,
// p update).  IC(0): three (p.q reduction, r.z = t.t and r.r reduction after the forward
// sweep, the backward sweep with the direction update).
__device__ void pcg_csr(const KArgs& a, double* sh) {
    const Tri& T = a.T;
    const int n = a.A.n;
    int r0, r1;
    row_range(n, r0, r1);
    const Csr B{ n, T.B.rowptr, T.B.col, T.bval, T.B.diag };
    double* xB = T.xB;
    const bool rel = a.criterion == PF2_CRITERION_REL;
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) __stcg(&xB[i], a.x[__ldg(&T.perm[i])]);
    if (!grid_sync(a.bar, gridDim.x)) return;
    double red[3] = { 0.0, 0.0, 0.0 };  // r.z, b.b, r.r
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const double bi = a.b[__ldg(&T.perm[i])];
        __stcg(&a.r[i], bi - row_dot(B, i, xB));
        red[1] += bi * bi;
    }
    if (!grid_sync(a.bar, gridDim.x)) return;
    red[2] = csr_fwd<0, double>(T, 0.0, 0.0, true, a.r, nullptr, nullptr, nullptr, nullptr, a.z, a.bar.err).x;
    if (!grid_sync(a.bar, gridDim.x)) return;
    const bool one = a.variant == PF2_CG_ONE_REDUCTION;
    red[0] = csr_bwd<double>(T, a.r, a.z, one ? nullptr : a.p, a.bar.err);
    double red4[4] = { red[0], red[1], red[2], 0.0 };
    if (one) {  // w = B z and z.w join the first reduction
        if (!grid_sync(a.bar, gridDim.x)) return;
        red4[3] = spmv_rows(B, a.z, a.q, r0, r1);
        if (!grid_reduce<4>(a.bar, red4, sh)) return;
    } else {
        if (!grid_reduce<3>(a.bar, red, sh)) return;
        red4[0] = red[0];
        red4[1] = red[1];
        red4[2] = red[2];
    }
    double gamma = red4[0];
    const double bnorm = sqrt(red4[1]);
    double rr = red4[2];
    const double tol2 = a.tol * a.tol;
    auto done_test = [&](double gm, double rr_) { return rel ? (sqrt(rr_) <= a.tol * bnorm) : (gm < tol2); };
    int it = 0;
    bool conv = done_test(gamma, rr);
    if (one) {
        // Chronopoulos-Gear: per iteration the forward sweep (with the p, s, x, r
        // updates), the backward sweep, w = B z with z.w, and one reduction of r.z, z.w, r.r
        double alpha = gamma / red4[3], beta = 0.0;
        bool first = true;
        while (!conv && it < a.maxit) {
            ++it;
            double g3[3] = { 0.0, 0.0, 0.0 };  // r.z, z.w, r.r
            g3[2] = csr_fwd<2, double>(T, alpha, beta, first, a.r, a.q, xB, a.p, a.s, a.z, a.bar.err).x;
            if (!grid_sync(a.bar, gridDim.x)) return;
            g3[0] = csr_bwd<double>(T, a.r, a.z, nullptr, a.bar.err);
            if (!grid_sync(a.bar, gridDim.x)) return;
            g3[1] = spmv_rows(B, a.z, a.q, r0, r1);
            if (!grid_reduce<3>(a.bar, g3, sh)) return;
            rr = g3[2];
            if (done_test(g3[0], rr)) { gamma = g3[0]; conv = true; break; }
            beta = g3[0] / gamma;
            alpha = g3[0] / (g3[1] - beta * g3[0] / alpha);
            gamma = g3[0];
            first = false;
        }
    }
    // with fuse_p three barriers per iteration: the direction update p = z + beta p runs
    // inside the next SpMV (spmv_rows_pz), alternating p between two arrays; else a
    // separate update and barrier
    double* pc = a.p;
    double* pa = a.s;
    double beta = 0.0;
    const bool ic = T.kind == PF2_PRECOND_IC;
    while (!conv && it < a.maxit) {
        double pq[1];
        if (it == 0 || !a.fuse_p) {
            pq[0] = spmv_rows(B, pc, a.q, r0, r1);
        } else {
            pq[0] = spmv_rows_pz<double>(B, T.bval, a.z, pc, beta, pa, a.q, r0, r1);
            double* t = pc;
            pc = pa;
            pa = t;
        }
        ++it;
        if (!grid_reduce<1>(a.bar, pq, sh)) return;
        const double alpha = gamma / pq[0];
        double g2[2] = { 0.0, 0.0 };
        if (ic && !a.fuse_p) {
            // IC(0): r.z = |L^{-1} r|^2 is known after the forward sweep, so one reduction
            // of r.z and r.r follows it and the backward sweep carries the direction update
            // (three barriers per iteration)
            // with the absolute criterion (a test of r.z alone) r.r is not formed per
            // iteration: one FP64 term per row and one reduced value fewer; it is
            // reduced once after the loop
            const double2 f = csr_fwd<1, double>(T, alpha, 0.0, false, a.r, a.q, xB, pc, nullptr, a.z, a.bar.err,
                                                 rel);
            double tt;
            if (rel) {
                double gt[2] = { f.y, f.x };
                if (!grid_reduce<2>(a.bar, gt, sh)) return;
                tt = gt[0];
                rr = gt[1];
            } else {
                double gt[1] = { f.y };
                if (!grid_reduce<1>(a.bar, gt, sh)) return;
                tt = gt[0];
            }
            if (done_test(tt, rr)) { gamma = tt; conv = true; break; }
            beta = tt / gamma;
            gamma = tt;
            csr_bwd<double, true>(T, nullptr, a.z, pc, a.bar.err, beta);
            if (!grid_sync(a.bar, gridDim.x)) return;
            continue;
        }
        g2[1] = csr_fwd<1, double>(T, alpha, 0.0, false, a.r, a.q, xB, pc, nullptr, a.z, a.bar.err, rel).x;
        if (!grid_sync(a.bar, gridDim.x)) return;
        g2[0] = csr_bwd<double>(T, a.r, a.z, nullptr, a.bar.err);
        if (rel) {
            if (!grid_reduce<2>(a.bar, g2, sh)) return;
            rr = g2[1];
        } else {
            double g1[1] = { g2[0] };
            if (!grid_reduce<1>(a.bar, g1, sh)) return;
            g2[0] = g1[0];
        }
        const double gnew = g2[0];
        if (done_test(gnew, rr)) { gamma = gnew; conv = true; break; }
        beta = gnew / gamma;
        gamma = gnew;
        if (!a.fuse_p) {
            p_update(pc, a.z, beta, r0, r1);
            if (!grid_sync(a.bar, gridDim.x)) return;
        }
    }
    // the absolute criterion left r.r out of the iterations: the final residual's norm
    if (!rel && !one && it > 0) {
        double f[1] = { 0.0 };
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const double ri = __ldcg(&a.r[i]);
            f[0] += ri * ri;
        }
        if (!grid_reduce<1>(a.bar, f, sh)) return;
        rr = f[0];
    }
    // every x update happened before the last reduction's barrier
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) a.x[__ldg(&T.perm[i])] = __ldcg(&xB[i]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->iterations = it;
        a.out->converged = conv ? 1 : 0;
        a.out->residual = rel ? sqrt(rr) / (bnorm > 0 ? bnorm : 1.0) : sqrt(gamma);
        a.out->relres = sqrt(rr) / (bnorm > 0 ? bnorm : 1.0);
        a.out->status = conv ? DEV_OK : DEV_NOT_CONVERGED;
    }
}

// One-reduction PCG (Chronopoulos-Gear) with the Jacobi or no preconditioner, on the
// block's rows: per iteration the vector updates (p = z + beta p, s = w + beta s,
// x += alpha p, r -= alpha s, z = M^{-1} r) with the r.z and r.r terms, one barrier, then
// w = A z with the z.w terms and one fused reduction of the three: two grid-wide steps
// instead of three.  alpha = gamma / (z.w - beta gamma / alpha_old).
__device__ void pcg_one_reduction(const KArgs& a, double* sh) {
    int r0, r1;
    row_range(a.A.n, r0, r1);
    const bool jac = a.precond == PF2_PRECOND_JACOBI;
    const bool rel = a.criterion == PF2_CRITERION_REL;
    if (jac)
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) a.invd[i] = 1.0 / a.A.val[a.A.diag[i]];
    double red[4] = { 0.0, 0.0, 0.0, 0.0 };  // r.z, b.b, r.r, z.w
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const double bi = a.b[i];
        const double ri = bi - row_dot(a.A, i, a.x);
        const double zi = jac ? ri * a.invd[i] : ri;
        a.r[i] = ri;
        __stcg(&a.z[i], zi);
        red[0] += ri * zi;
        red[1] += bi * bi;
        red[2] += ri * ri;
    }
    if (!grid_sync(a.bar, gridDim.x)) return;
    red[3] = spmv_rows(a.A, a.z, a.q, r0, r1);
    if (!grid_reduce<4>(a.bar, red, sh)) return;
    double gamma = red[0];
    const double bnorm = sqrt(red[1]);
    double rr = red[2];
    const double tol2 = a.tol * a.tol;
    auto done_test = [&](double gm, double rr_) { return rel ? (sqrt(rr_) <= a.tol * bnorm) : (gm < tol2); };
    int it = 0;
    bool conv = done_test(gamma, rr);
    double alpha = gamma / red[3], beta = 0.0;
    bool first = true;
    while (!conv && it < a.maxit) {
        ++it;
        double g3[3] = { 0.0, 0.0, 0.0 };  // r.z, z.w, r.r
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const double zi = __ldcg(&a.z[i]), wi = __ldcg(&a.q[i]);
            const double pi = first ? zi : zi + beta * a.p[i];
            const double si = first ? wi : wi + beta * a.s[i];
            a.p[i] = pi;
            a.s[i] = si;
            a.x[i] += alpha * pi;
            const double ri = a.r[i] - alpha * si;
            a.r[i] = ri;
            const double zn = jac ? ri * a.invd[i] : ri;
            __stcg(&a.z[i], zn);
            g3[0] += ri * zn;
            g3[2] += ri * ri;
        }
        if (!grid_sync(a.bar, gridDim.x)) return;
        g3[1] = spmv_rows(a.A, a.z, a.q, r0, r1);
        if (!grid_reduce<3>(a.bar, g3, sh)) return;
        rr = g3[2];
        if (done_test(g3[0], rr)) { gamma = g3[0]; conv = true; break; }
        beta = g3[0] / gamma;
        alpha = g3[0] / (g3[1] - beta * g3[0] / alpha);
        gamma = g3[0];
        first = false;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->iterations = it;
        a.out->converged = conv ? 1 : 0;
        a.out->residual = rel ? sqrt(rr) / (bnorm > 0 ? bnorm : 1.0) : sqrt(gamma);
        a.out->relres = sqrt(rr) / (bnorm > 0 ? bnorm : 1.0);
        a.out->status = conv ? DEV_OK : DEV_NOT_CONVERGED;
    }
}

// Right-preconditioned BiCGStab (van der Vorst 1992) with the Jacobi or no
// preconditioner, on the block's rows: per iteration two SpMVs, two barriers and three
// fused reductions.  Stops on ||M^{-1} r|| < tol (absolute: the preconditioned residual
// that the reference's GMRES tests, linear_solver.cu:500-505) or ||r|| <= tol ||b||
// (relative); a zero (rhat, v) ends the solve unconverged, and so does t.t = 0 unless
// the half step x += alpha y converged; a zero rhat.r with r != 0 restarts the shadow
// residual.  x changes every iteration (x += alpha y + omega z).
__global__ void __launch_bounds__(kSolverThreads, kSolverBlocksPerSm) k_bicgstab(KArgs a) {
    __shared__ double sh[kShDoubles];
    __shared__ double red_s[4 * kSolverThreads];  // grid_reduce_tree's block tree
    int r0, r1;
    row_range(a.A.n, r0, r1);
    const bool jac = a.precond == PF2_PRECOND_JACOBI;
    const bool rel = a.criterion == PF2_CRITERION_REL;
    if (jac)
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) a.invd[i] = 1.0 / a.A.val[a.A.diag[i]];
    // r = rhat = b - A x; p = v = 0
    double red[4] = { 0.0, 0.0, 0.0, 0.0 };  // rhat.r, r.r, |M^{-1} r|^2, b.b
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const double bi = a.b[i];
        const double ri = bi - row_dot(a.A, i, a.x);
        const double di = jac ? a.invd[i] : 1.0;
        a.r[i] = ri;
        a.rhat[i] = ri;
        a.p[i] = 0.0;
        a.q[i] = 0.0;
        red[0] += ri * ri;
        red[1] += ri * ri;
        red[2] += (ri * di) * (ri * di);
        red[3] += bi * bi;
    }
    // the iteration's scalars (divisions, square roots) by thread 0 (grid_reduce_tree)
    double bnorm = 0.0;
    auto test = [&](const double* t) { return rel ? sqrt(t[1]) <= a.tol * bnorm : sqrt(t[2]) < a.tol; };
    if (!grid_reduce_tree<kSolverThreads, 4>(a.bar, red, sh, red_s, [&](const double* t, double* o) {
            bnorm = sqrt(t[3]);
            o[0] = bnorm;
            o[1] = test(t);
            o[2] = (t[0] / 1.0) * (1.0 / 1.0);  // beta of the first iteration (rho_old = alpha = omega = 1)
        }))
        return;
    bnorm = sh[24];
    double alpha = 1.0, omega = 1.0;
    double rho = red[0], rr = red[1], mm = red[2];
    int it = 0;
    bool conv = sh[25] != 0.0;
    double beta = sh[26];
    while (!conv && it < a.maxit) {
        ++it;
        // p = r + beta (p - omega v); y = M^{-1} p
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const double pi = a.r[i] + beta * (a.p[i] - omega * a.q[i]);
            a.p[i] = pi;
            __stcg(&a.y[i], jac ? pi * a.invd[i] : pi);
        }
        if (!grid_sync(a.bar, gridDim.x)) return;
        // v = A y, rhat.v
        double rv[1] = { 0.0 };
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const double vi = row_dot(a.A, i, a.y);
            a.q[i] = vi;
            rv[0] += a.rhat[i] * vi;
        }
        if (!grid_reduce_tree<kSolverThreads, 1>(a.bar, rv, sh, red_s, [&](const double* t, double* o) {
                o[0] = t[0] == 0.0 ? 0.0 : rho / t[0];
            }))
            return;
        if (rv[0] == 0.0) break;  // breakdown: ends unconverged
        alpha = sh[24];
        // s = r - alpha v; z = M^{-1} s
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const double si = a.r[i] - alpha * a.q[i];
            a.s[i] = si;
            __stcg(&a.z[i], jac ? si * a.invd[i] : si);
        }
        if (!grid_sync(a.bar, gridDim.x)) return;
        // t = A z, t.s, t.t
        double ts[2] = { 0.0, 0.0 };
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const double ti = row_dot(a.A, i, a.z);
            a.t[i] = ti;
            ts[0] += ti * a.s[i];
            ts[1] += ti * ti;
        }
        // t = A M^{-1} s is zero only where s is: the half step alpha y already solves
        // the system, so take it (omega = 0: x += alpha y, r = s) and let the test below
        // decide; a nonzero s that A M^{-1} maps to zero ends the solve unconverged
        if (!grid_reduce_tree<kSolverThreads, 2>(a.bar, ts, sh, red_s, [&](const double* t, double* o) {
                o[0] = t[1] == 0.0 ? 0.0 : t[0] / t[1];
            }))
            return;
        omega = sh[24];
        // x += alpha y + omega z; r = s - omega t; rhat.r, r.r, |M^{-1} r|^2
        double g3[3] = { 0.0, 0.0, 0.0 };
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            a.x[i] += alpha * __ldcg(&a.y[i]) + omega * __ldcg(&a.z[i]);
            const double ri = a.s[i] - omega * a.t[i];
            const double di = jac ? a.invd[i] : 1.0;
            a.r[i] = ri;
            g3[0] += a.rhat[i] * ri;
            g3[1] += ri * ri;
            g3[2] += (ri * di) * (ri * di);
        }
        // the test and the next iteration's beta (after a shadow-residual restart: rho = r.r
        // with rho_old = alpha = omega = 1)
        if (!grid_reduce_tree<kSolverThreads, 3>(a.bar, g3, sh, red_s, [&](const double* t, double* o) {
                o[0] = test(t);
                o[1] = t[0] == 0.0 ? (t[1] / 1.0) * (1.0 / 1.0) : (t[0] / rho) * (alpha / omega);
            }))
            return;
        rho = g3[0];
        rr = g3[1];
        mm = g3[2];
        conv = sh[24] != 0.0;
        beta = sh[25];
        if (!conv && omega == 0.0) break;
        if (!conv && rho == 0.0) {
            // r orthogonal to rhat: with rhat = r0 supported on the Dirichlet rows alone
            // (the first step of a flow from rest), the first iteration zeroes r there.
            // Restart the shadow residual: rhat = r, p = v = 0 (each thread its own rows,
            // which it alone reads next)
            for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                a.rhat[i] = a.r[i];
                a.p[i] = 0.0;
                a.q[i] = 0.0;
            }
            rho = rr;
            alpha = 1.0;
            omega = 1.0;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->iterations = it;
        a.out->converged = conv ? 1 : 0;
        a.out->residual = rel ? sqrt(rr) / (bnorm > 0 ? bnorm : 1.0) : sqrt(mm);
        a.out->relres = sqrt(rr) / (bnorm > 0 ? bnorm : 1.0);
        a.out->status = conv ? DEV_OK : DEV_NOT_CONVERGED;
    }
}

// Pipelined PCG (Ghysels and Vanroose, "Hiding global synchronization latency in the
// preconditioned Conjugate Gradient algorithm", Parallel Computing 40 (2014), Algorithm 4)
// on B's CSR arrays, with ILU(0)/IC(0) on a few-level order: one grid-wide step per
// iteration.  The recurrences carry u = M^{-1} r, w = A u, m = M^{-1} w, n = A m and
// z, q, s, p beside x and r; in exact arithmetic the iterates equal PCG's.  Iteration i:
//  (1) rows in sweep order (group by group, thread t taking rows t, t + T, ...): with the
//      previous iteration's alpha, beta, n = (B m_{i-1})_row and the row's updates
//      z = n + beta z, q = m + beta q, s = w + beta s, p = u + beta p, x += alpha p,
//      r -= alpha s, u -= alpha q, w -= alpha z; the row's terms of r.u, w.u and r.r; then
//      the forward sweep on w over the same rows (the same thread handles a row in both
//      passes, so no barrier);
//  (2) the backward sweep into m_i, each row waiting for its own forward result (the value
//      is its flag) and its upper neighbours' m;
//  (3) one barrier fused with the reduction of r.u, w.u, r.r, which gives alpha, beta.
// m cycles through three arrays: m_i is written in (2), read by (1) of iteration i + 1,
// and the array for m_{i+1} is reset to the marker in (1) of iteration i, a barrier
// before its first write.  The forward results are reset by the backward sweep.
template <int kPipeW>  // rows of the update pass whose SpMV loads are in flight together
__global__ void __launch_bounds__(kSolverThreads, kSolverBlocksPerSm) k_pcg_pipe(KArgs a) {
    __shared__ double sh[kShDoubles];
    const Tri& T = a.T;
    const int n = a.A.n;
    int r0, r1;
    row_range(n, r0, r1);
    const Csr B{ n, T.B.rowptr, T.B.col, T.bval, T.B.diag };
    double* xB = T.xB;
    double* tmp = T.tmp;
    const double* fsym = T.fsym;
    double *r = a.r, *p = a.p, *q = a.q, *s = a.s;
    double* u = a.pipe;
    double* w = u + n;
    double* zv = w + n;
    double* m3 = zv + n;  // three arrays of n
    const bool unit = T.kind != PF2_PRECOND_IC;
    const bool rel = a.criterion == PF2_CRITERION_REL;
    int* err = a.bar.err;
    const double mk = Pending<double>::marker();
    // x and b in B's numbering, r = b - B x; z, q, s, p = 0; m_0 pending
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        __stcg(&xB[i], a.x[__ldg(&T.perm[i])]);
        __stcg(&zv[i], 0.0);
        __stcg(&q[i], 0.0);
        __stcg(&s[i], 0.0);
        __stcg(&p[i], 0.0);
        __stcg(&m3[i], mk);
    }
    if (!grid_sync(a.bar, gridDim.x)) return;
    double bb[1] = { 0.0 };
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const double bi = a.b[__ldg(&T.perm[i])];
        __stcg(&r[i], bi - row_dot(B, i, xB));
        bb[0] += bi * bi;
    }
    if (!grid_sync(a.bar, gridDim.x)) return;
    // u = M^{-1} r, w = B u
    csr_fwd<0, double>(T, 0.0, 0.0, true, r, nullptr, nullptr, nullptr, nullptr, u, err);
    if (!grid_sync(a.bar, gridDim.x)) return;
    csr_bwd<double>(T, r, u, nullptr, err);
    if (!grid_sync(a.bar, gridDim.x)) return;
    spmv_rows(B, u, w, r0, r1);
    if (!grid_reduce<1>(a.bar, bb, sh)) return;
    const double bnorm = sqrt(bb[0]);
    const double tol2 = a.tol * a.tol;
    const int stride = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    double alpha = 0.0, beta = 0.0, gamma = 0.0, gamma_old = 0.0, alpha_old = 0.0, rr = 0.0;
    int it = 0;
    bool conv = false;
    for (int i = 0;; ++i) {
        const double* mprev = m3 + (size_t)((i + 2) % 3) * n;  // m_{i-1}
        double* mcur = m3 + (size_t)(i % 3) * n;                // m_i
        double* mnext = m3 + (size_t)((i + 1) % 3) * n;         // reset for m_{i+1}
        double g[3] = { 0.0, 0.0, 0.0 };                        // r.u, w.u, r.r
        // (1) updates, rows in sweep order (no waits), then the forward sweep on w over the
        // same rows of the same thread, so the sweep's dependency chain carries no SpMV.
        // The update pass takes the thread's rows of kPipeW groups together (row j of
        // each), so the loads of kPipeW SpMV rows are in flight at once.
        for (int gb = 0; gb < T.ngroups; gb += kPipeW) {
            int lo[kPipeW], hi[kPipeW];
#pragma unroll
            for (int v = 0; v < kPipeW; ++v) {
                lo[v] = gb + v < T.ngroups ? __ldg(&T.cstart[gb + v]) : 0;
                hi[v] = gb + v < T.ngroups ? __ldg(&T.cstart[gb + v + 1]) : 0;
            }
            for (int j = tid;; j += stride) {
                int rw[kPipeW], ks[kPipeW], ke[kPipeW];
                bool any = false;
#pragma unroll
                for (int v = 0; v < kPipeW; ++v) {
                    rw[v] = lo[v] + j < hi[v] ? lo[v] + j : -1;
                    any = any || rw[v] >= 0;
                }
                if (!any) break;
                double nsum[kPipeW] = {};
                if (i > 0) {
                    int len = 0;
#pragma unroll
                    for (int v = 0; v < kPipeW; ++v) {
                        ks[v] = rw[v] >= 0 ? __ldg(&B.rowptr[rw[v]]) : 0;
                        ke[v] = rw[v] >= 0 ? __ldg(&B.rowptr[rw[v] + 1]) : 0;
                        len = max(len, ke[v] - ks[v]);
                    }
                    for (int k = 0; k < len; ++k) {
#pragma unroll
                        for (int v = 0; v < kPipeW; ++v)
                            if (ks[v] + k < ke[v])
                                nsum[v] += __ldg(&B.val[ks[v] + k]) * __ldcg(&mprev[__ldg(&B.col[ks[v] + k])]);
                    }
                }
#pragma unroll
                for (int v = 0; v < kPipeW; ++v) {
                    const int row = rw[v];
                    if (row < 0) continue;
                    double ri = __ldcg(&r[row]), ui = __ldcg(&u[row]), wi = __ldcg(&w[row]);
                    if (i > 0) {
                        const double zi = nsum[v] + beta * __ldcg(&zv[row]);
                        const double qi = __ldcg(&mprev[row]) + beta * __ldcg(&q[row]);
                        const double si = wi + beta * __ldcg(&s[row]);
                        const double pi = ui + beta * __ldcg(&p[row]);
                        __stcg(&zv[row], zi);
                        __stcg(&q[row], qi);
                        __stcg(&s[row], si);
                        __stcg(&p[row], pi);
                        __stcg(&xB[row], __ldcg(&xB[row]) + alpha * pi);
                        ri -= alpha * si;
                        ui -= alpha * qi;
                        wi -= alpha * zi;
                        __stcg(&r[row], ri);
                        __stcg(&u[row], ui);
                        __stcg(&w[row], wi);
                    }
                    g[0] += ri * ui;
                    g[1] += wi * ui;
                    g[2] += ri * ri;
                    __stcg(&mnext[row], mk);
                }
            }
        }
        for (int gi = 0; gi < T.ngroups; ++gi) {
            const int g0 = __ldg(&T.cstart[gi]), g1 = __ldg(&T.cstart[gi + 1]);
            for (int row = g0 + tid; row < g1; row += stride) {
                const int k0 = __ldg(&B.rowptr[row]), d = __ldg(&B.diag[row]);
                const double wi = __ldcg(&w[row]);
                double sum;
                if (!csr_dot_wait(tmp, B.col, fsym, k0, d, row, err, T.rec, sum)) break;
                __stcg(&tmp[row], unit ? wi - sum : (wi - sum) * __ldg(&fsym[d]));
            }
        }
        // (2) backward sweep into m_i
        for (int gi = T.ngroups - 1; gi >= 0; --gi) {
            const int g0 = __ldg(&T.cstart[gi]), g1 = __ldg(&T.cstart[gi + 1]);
            for (int row = g1 - 1 - tid; row >= g0; row -= stride) {
                const int d = __ldg(&B.diag[row]), k1 = __ldg(&B.rowptr[row + 1]);
                double in;
                if (!wait_value(tmp, row, in, err, T.rec, row)) break;
                double sum;
                if (!csr_dot_wait(mcur, B.col, fsym, d + 1, k1, row, err, T.rec, sum)) break;
                __stcg(&mcur[row], (in - sum) * __ldg(&fsym[d]));
                __stcg(&tmp[row], mk);
            }
        }
        // (3) the one grid-wide step
        if (!grid_reduce<3>(a.bar, g, sh)) return;
        gamma = g[0];
        rr = g[2];
        it = i;
        if (rel ? (sqrt(rr) <= a.tol * bnorm) : (gamma < tol2)) { conv = true; break; }
        if (i >= a.maxit) break;
        if (i == 0) {
            beta = 0.0;
            alpha = gamma / g[1];
        } else {
            beta = gamma / gamma_old;
            alpha = gamma / (g[1] - beta * gamma / alpha_old);
        }
        gamma_old = gamma;
        alpha_old = alpha;
    }
    // every x update happened before the last barrier
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) a.x[__ldg(&T.perm[i])] = __ldcg(&xB[i]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->iterations = it;
        a.out->converged = conv ? 1 : 0;
        a.out->residual = rel ? sqrt(rr) / (bnorm > 0 ? bnorm : 1.0) : sqrt(gamma);
        a.out->relres = sqrt(rr) / (bnorm > 0 ? bnorm : 1.0);
        a.out->status = conv ? DEV_OK : DEV_NOT_CONVERGED;
    }
}

// The part's shared memory: r, p, q and t of its rows in the solve's arithmetic type V
// (Jacobi / none: t = 1 / a_ii and a separate z; ILU / IC: z shares t's array, since a
// row's forward result is dead once the backward sweep has read it and the backward sweep
// reads only its own row's t), the mixed-precision solve's update d, the reduction scratch
// and (kPartMetaSmem) the rows' entry ranges, diagonal positions and boundary flags.  x
// stays in global memory: the smaller shared-memory carve-out leaves more of the SM's
// 256 KB to the L1 that caches the matrix and factor streams (measured: IC(0) CG at
// 499,288 rows 57.9 us per iteration with x in shared memory, 51.7 without).  The groups
// of a sweep follow one another behind a __syncthreads (measured against rows polling
// their own part's results in shared memory, with no barrier between the groups: 47 against
// 56 us per IC(0) iteration).
template <class V>
struct PartSm {
    V *r, *p, *q, *t, *z, *d;
    double* red;
    const int* rp;   // np + 1 absolute entry positions
    const int* dg;   // diagonal positions
    const unsigned char* bnd;
};

constexpr int kPartThreads = 1024;  // one block per SM
constexpr bool kPartMetaSmem = true;

__host__ __device__ constexpr size_t part_vec_bytes(int R, bool tri, size_t vsz, bool mixed) {
    return ((4 + (tri ? 0 : 1) + (mixed ? 1 : 0)) * (size_t)R * vsz + 15) / 16 * 16;
}

// Shared-memory bytes of a part of R rows (the layout of part_sm).
__host__ __device__ constexpr size_t part_smem_bytes(int R, bool tri, size_t vsz, bool mixed) {
    return part_vec_bytes(R, tri, vsz, mixed) + sizeof(double) * 2 * kPartThreads +
           (kPartMetaSmem ? sizeof(int) * (2 * (size_t)R + 1) + (size_t)R : 0);
}

template <class V>
__device__ __forceinline__ PartSm<V> part_sm(const PartCg& C, unsigned char* base, int R, bool tri, bool mixed,
                                             int p0) {
    PartSm<V> S;
    V* v = reinterpret_cast<V*>(base);
    S.r = v;
    S.p = v + R;
    S.q = v + 2 * R;
    S.t = v + 3 * R;
    S.z = tri ? S.t : v + 4 * R;
    S.d = mixed ? v + (tri ? 4 : 5) * R : nullptr;
    S.red = reinterpret_cast<double*>(base + part_vec_bytes(R, tri, sizeof(V), mixed));
    if (kPartMetaSmem) {
        int* rp = reinterpret_cast<int*>(S.red + 2 * kPartThreads);
        S.rp = rp;
        S.dg = rp + R + 1;
        S.bnd = reinterpret_cast<const unsigned char*>(rp + 2 * R + 1);
    } else {
        S.rp = C.rp + p0;
        S.dg = C.diag + p0;
        S.bnd = C.bnd + p0;
    }
    return S;
}

// The matrix, factor and boundary arrays of the solve's arithmetic type.
template <class V> struct PartVecs;
template <> struct PartVecs<double> {
    __device__ static const double* val(const PartCg& C) { return C.val; }
    __device__ static const double* f(const PartCg& C) { return C.f; }
    __device__ static double* gp(const PartCg& C) { return C.gp; }
    __device__ static double* gt(const PartCg& C) { return C.gt; }
    __device__ static double* gz(const PartCg& C) { return C.gz; }
};
template <> struct PartVecs<float> {
    __device__ static const float* val(const PartCg& C) { return C.val32; }
    __device__ static const float* f(const PartCg& C) { return C.f32; }
    __device__ static float* gp(const PartCg& C) { return C.gp32; }
    __device__ static float* gt(const PartCg& C) { return C.gt32; }
    __device__ static float* gz(const PartCg& C) { return C.gz32; }
};

// Grid-wide sums of NV <= 2 values for the partitioned kernels (grid_reduce_tree on
// kPartThreads threads; red: 2 x kPartThreads doubles of the part's shared memory).
template <int NV, class Post = NoPost>
__device__ __forceinline__ bool part_reduce(const GridBarrier& b, double (&v)[NV], double* sh, double* red,
                                            Post post = Post()) {
    static_assert(NV >= 1 && NV <= 2, "part_reduce sums one or two values");
    return grid_reduce_tree<kPartThreads, NV>(b, v, sh, red, post);
}

// v[j] for row j of a sweep: the part's own rows from shared memory, other parts' rows
// from the global copy, polled on the pending marker (bounded).  A failed wait records
// DEV_TIMEOUT and yields 0: the caller goes on to the next __syncthreads and the kernel
// returns at its next grid barrier.
template <class V>
__device__ __forceinline__ V part_dep(int j, int p0, int np, const V* sv, const V* gv, int* err, int* rec, int row) {
    if ((unsigned)(j - p0) < (unsigned)np) return sv[j - p0];
    V v = *(volatile const V*)&gv[j];
    if (Pending<V>::bits(v) == Pending<V>::kBits && !wait_value(gv, j, v, err, rec, row)) v = V(0);
    return v;
}

// q = A p over the part's rows (each row's entries in order, as spmv_rows); other parts'
// p from the global copy.  Returns the thread's p.q terms (in FP64).  reset_z: the
// boundary rows' backward results back to the pending marker.  This is the place for it:
// the SpMV follows the grid barrier that ends an iteration, so every part has finished
// the backward sweep that read them, and the next backward sweep (which may start before
// other parts end their forward sweep: it overlaps the t.t reduction) follows the p.q
// reduction's barrier.
template <class V>
__device__ __forceinline__ double part_spmv(const PartCg& C, const PartSm<V>& S, int p0, int np,
                                            bool reset_z = false) {
    const V* val = PartVecs<V>::val(C);
    const V* gp = PartVecs<V>::gp(C);
    V* gz = PartVecs<V>::gz(C);
    double pq = 0.0;
    for (int l = threadIdx.x; l < np; l += kPartThreads) {
        if (reset_z && S.bnd[l]) __stcg(&gz[p0 + l], Pending<V>::marker());
        const int s = S.rp[l], e = S.rp[l + 1];
        V acc = V(0);
        for (int k = s; k < e; ++k) {
            const int j = __ldg(&C.col[k]);
            const V pj = (unsigned)(j - p0) < (unsigned)np ? S.p[j - p0] : __ldcg(&gp[j]);
            acc += __ldg(&val[k]) * pj;
        }
        S.q[l] = acc;
        pq += (double)S.p[l] * (double)acc;
    }
    return pq;
}

// A sweep row's dependency entries and pivot pulled into L1 before the group's barrier
// (they do not depend on the earlier groups).
template <class V>
__device__ __forceinline__ void sweep_prefetch(const PartCg& C, int k0, int k1, int d) {
    const V* f = PartVecs<V>::f(C);
    if (k1 > k0) {
        prefetch_l1(&C.col[k0]);
        prefetch_l1(&f[k0]);
    }
    prefetch_l1(&f[d]);
}

// s - sum_k f_k v[col_k] over the dependency entries [k0, k1), in entry order, as a chain
// of fused multiply-adds from s (one FP64 instruction a row fewer than forming the sum and
// subtracting it; a sweep's rows are FP64-issue-bound on GB300); LOCAL (the
// partition-local factors, zero outside the part): the part's own entries only.
template <class V, bool LOCAL = false>
__device__ __forceinline__ V sweep_rest(const PartCg& C, int k0, int k1, int p0, int np, const V* sv, const V* gv,
                                        V s, int* err, int* rec, int row) {
    const V* f = PartVecs<V>::f(C);
    for (int k = k0; k < k1; ++k) {
        const int j = __ldg(&C.col[k]);
        if (LOCAL && (unsigned)(j - p0) >= (unsigned)np) continue;
        s = fma_rn(-__ldg(&f[k]), part_dep(j, p0, np, sv, gv, err, rec, row), s);
    }
    return s;
}

// Forward sweep over the part's groups (csr_fwd): first: t = L^{-1} r; else the updates
// r -= alpha q and (XUPD) x += alpha p (MIXED: the inner update d += alpha p) with it.
// Returns the r.r terms (want_rr) and the t.t terms, in FP64.  LOCAL: partition-local
// factors, no boundary copies.
template <bool IC, class V = double, bool MIXED = false, bool LOCAL = false, bool XUPD = true>
__device__ double2 part_fwd(const PartCg& C, const PartSm<V>& S, int p0, int np, bool first, V alpha, bool want_rr,
                            int* err, int* rec) {
    V* gt = PartVecs<V>::gt(C);
    const V* f = PartVecs<V>::f(C);
    double rr = 0.0, tt = 0.0;
    const int* qs = C.qs + blockIdx.x * C.ng;
    for (int g = 0; g < C.ng; ++g) {
        const int g0 = qs[g] - p0, g1 = qs[g + 1] - p0;
        if (g0 + (int)threadIdx.x < g1) {
            const int l = g0 + threadIdx.x;
            sweep_prefetch<V>(C, S.rp[l], S.dg[l], S.dg[l]);
        }
        __syncthreads();  // the part's earlier groups are done
        for (int l = g0 + threadIdx.x; l < g1; l += kPartThreads) {
            const int d = S.dg[l];
            V ra = S.r[l];
            if (!first) {
                ra -= alpha * S.q[l];
                S.r[l] = ra;
            }
            if (want_rr) rr += (double)ra * (double)ra;
            const V rest = sweep_rest<V, LOCAL>(C, S.rp[l], d, p0, np, S.t, gt, ra, err, rec, p0 + l);
            const V v = IC ? rest * __ldg(&f[d]) : rest;
            S.t[l] = v;
            if (!LOCAL && S.bnd[l]) __stcg(&gt[p0 + l], v);
            tt += (double)v * (double)v;
            // x += alpha p last: its global load is off the sweep's dependency chain
            if (XUPD && !first) {
                if (MIXED)
                    S.d[l] = S.d[l] + alpha * S.p[l];
                else
                    __stcg(&C.x[p0 + l], __ldcg(&C.x[p0 + l]) + (double)alpha * (double)S.p[l]);
            }
        }
    }
    return make_double2(rr, tt);
}

// Backward sweep over the part's groups in reverse (csr_bwd): z = U^{-1} t; PMODE 0: no
// direction, 1: p = z (the first), 2: p = z + beta p (IC's three-step iteration), 3: z
// alone (IC's iteration with the sweep overlapping the t.t reduction; the caller updates p
// and resets the boundary rows' t afterwards).  Returns the r.z terms (PMODE 0 and 1), in
// FP64.  LOCAL: partition-local factors.
template <int PMODE, class V = double, bool LOCAL = false>
__device__ double part_bwd(const PartCg& C, const PartSm<V>& S, int p0, int np, V beta, int* err, int* rec) {
    V* gp = PartVecs<V>::gp(C);
    V* gt = PartVecs<V>::gt(C);
    V* gz = PartVecs<V>::gz(C);
    const V* f = PartVecs<V>::f(C);
    double rz = 0.0;
    const int* qs = C.qs + blockIdx.x * C.ng;
    for (int g = C.ng - 1; g >= 0; --g) {
        const int g0 = qs[g] - p0, g1 = qs[g + 1] - p0;
        if (g0 + (int)threadIdx.x < g1) {
            const int l = g0 + threadIdx.x;
            sweep_prefetch<V>(C, S.dg[l] + 1, S.rp[l + 1], S.dg[l]);
        }
        __syncthreads();  // the part's later groups are done
        for (int l = g0 + threadIdx.x; l < g1; l += kPartThreads) {
            const int d = S.dg[l];
            const V in = S.t[l];
            const V v = sweep_rest<V, LOCAL>(C, d + 1, S.rp[l + 1], p0, np, S.z, gz, in, err, rec, p0 + l) *
                        __ldg(&f[d]);
            S.z[l] = v;
            V pn = V(0);
            if (PMODE == 1) pn = v;
            if (PMODE == 2) pn = fma_rn(beta, S.p[l], v);
            if (PMODE == 1 || PMODE == 2) S.p[l] = pn;
            if (S.bnd[l]) {
                if (!LOCAL) {
                    __stcg(&gz[p0 + l], v);
                    if (PMODE != 3) __stcg(&gt[p0 + l], Pending<V>::marker());
                }
                if (PMODE == 1 || PMODE == 2) __stcg(&gp[p0 + l], pn);
            }
            if (PMODE <= 1) rz += (double)S.r[l] * (double)v;
        }
    }
    return rz;
}

// IC's direction update after a backward sweep that overlapped the t.t reduction (PMODE
// 3): p = z + beta p (part_bwd's PUPD arithmetic) over the part's rows, boundary rows also
// to the global copy, and the boundary rows' forward results back to the marker (every
// part has passed its forward sweep: the reduction's barrier is behind).
template <class V>
__device__ __forceinline__ void part_p_after_bwd(const PartCg& C, const PartSm<V>& S, int p0, int np, V beta,
                                                 bool reset_t) {
    V* gp = PartVecs<V>::gp(C);
    V* gt = PartVecs<V>::gt(C);
    for (int l = threadIdx.x; l < np; l += kPartThreads) {
        const V pn = fma_rn(beta, S.p[l], S.z[l]);
        S.p[l] = pn;
        if (S.bnd[l]) {
            __stcg(&gp[p0 + l], pn);
            if (reset_t) __stcg(&gt[p0 + l], Pending<V>::marker());
        }
    }
}

// p = z + beta p over the part's rows (p_update), boundary rows also to the global copy.
template <class V>
__device__ __forceinline__ void part_p_update(const PartCg& C, const PartSm<V>& S, int p0, int np, V beta) {
    V* gp = PartVecs<V>::gp(C);
    for (int l = threadIdx.x; l < np; l += kPartThreads) {
        const V pn = S.z[l] + beta * S.p[l];
        S.p[l] = pn;
        if (S.bnd[l]) __stcg(&gp[p0 + l], pn);
    }
}

// The part's row metadata to shared memory and x (A's numbering) to the global iterate in
// Q order.
template <class V>
__device__ __forceinline__ void part_load(const KArgs& a, const PartSm<V>& S, int p0, int p1) {
    const PartCg& C = a.part;
    const int np = p1 - p0;
    for (int l = threadIdx.x; l < np; l += kPartThreads) {
        const int i = p0 + l;
        if (kPartMetaSmem) {
            const_cast<int*>(S.rp)[l] = __ldg(&C.rp[i]);
            const_cast<int*>(S.dg)[l] = __ldg(&C.diag[i]);
            const_cast<unsigned char*>(S.bnd)[l] = __ldg(&C.bnd[i]);
        }
        __stcg(&C.x[i], a.x[__ldg(&C.qa[i])]);
    }
    if (kPartMetaSmem && threadIdx.x == 0) const_cast<int*>(S.rp)[np] = __ldg(&C.rp[p1]);
}

// b - A x in FP64 for the part's row l (x from the global iterate in Q order).
__device__ __forceinline__ double part_residual(const KArgs& a, const int* rp, int p0, int l, double& bi) {
    const PartCg& C = a.part;
    bi = a.b[__ldg(&C.qa[p0 + l])];
    double v = 0.0;
    for (int k = rp[l]; k < rp[l + 1]; ++k) v += __ldg(&C.val[k]) * __ldcg(&C.x[__ldg(&C.col[k])]);
    return bi - v;
}

// MODE 0: Jacobi or no preconditioner (k_pcg's iteration: p.q reduction, x/r/z update
// with r.z, p update and barrier); 1: IC(0) (pcg_csr's three grid-wide steps); 2: ILU(0)
// (pcg_csr's four).
template <int MODE>
__device__ void pcg_part(const KArgs& a, double* sh, unsigned char* smem) {
    const PartCg& C = a.part;
    const int p0 = C.qs[blockIdx.x * C.ng], p1 = C.qs[(blockIdx.x + 1) * C.ng], np = p1 - p0;
    const PartSm<double> S = part_sm<double>(C, smem, C.R, MODE != 0, false, p0);
    const int tid = threadIdx.x;
    int* err = a.bar.err;
    int* rec = a.bar.rec;
    const bool rel = a.criterion == PF2_CRITERION_REL;
    const bool jac = a.precond == PF2_PRECOND_JACOBI;
    part_load(a, S, p0, p1);
    if (!grid_sync(a.bar, gridDim.x)) return;
    double red[3] = { 0.0, 0.0, 0.0 };  // r.z, b.b, r.r
    for (int l = tid; l < np; l += kPartThreads) {
        double bi;
        S.r[l] = part_residual(a, S.rp, p0, l, bi);
        red[1] += bi * bi;
        if (MODE == 0) S.t[l] = 1.0 / __ldg(&C.val[S.dg[l]]);
    }
    __syncthreads();
    if (MODE == 0) {
        for (int l = tid; l < np; l += kPartThreads) {
            const double ri = S.r[l];
            const double zi = jac ? ri * S.t[l] : ri;
            S.z[l] = zi;
            S.p[l] = zi;
            if (S.bnd[l]) __stcg(&C.gp[p0 + l], zi);
            red[0] += ri * zi;
            red[2] += ri * ri;
        }
    } else {
        red[2] = part_fwd<MODE == 1>(C, S, p0, np, true, 0.0, true, err, rec).x;
        if (!grid_sync(a.bar, gridDim.x)) return;
        red[0] = part_bwd<1>(C, S, p0, np, 0.0, err, rec);
    }
    double r2[2] = { red[0], red[1] }, r1[1] = { red[2] };
    if (!part_reduce<2>(a.bar, r2, sh, S.red)) return;
    // bnorm and the first test (thread 0; see part_reduce)
    if (!part_reduce<1>(a.bar, r1, sh, S.red, [&](const double* tot, double* out) {
            out[0] = sqrt(r2[1]);
            out[1] = rel ? (sqrt(tot[0]) <= a.tol * out[0]) : (r2[0] < a.tol * a.tol);
        }))
        return;
    double gamma = r2[0];
    const double bnorm = sh[24];
    double rr = r1[0];
    int it = 0;
    bool conv = sh[25] != 0.0;
    while (!conv && it < a.maxit) {
        ++it;
        double pq[1] = { part_spmv(C, S, p0, np, MODE != 0) };
        if (!part_reduce<1>(a.bar, pq, sh, S.red, [&](const double* tot, double* out) { out[0] = gamma / tot[0]; }))
            return;
        const double alpha = sh[24];
        // with the absolute criterion (a test of r.z alone) r.r is reduced once after the loop
        double g2[2] = { 0.0, 0.0 };  // r.z (IC: t.t), r.r
        if (MODE == 0) {
            for (int l = tid; l < np; l += kPartThreads) {
                __stcg(&C.x[p0 + l], __ldcg(&C.x[p0 + l]) + alpha * S.p[l]);
                const double ri = S.r[l] - alpha * S.q[l];
                const double zi = jac ? ri * S.t[l] : ri;
                S.r[l] = ri;
                S.z[l] = zi;
                g2[0] += ri * zi;
                if (rel) g2[1] += ri * ri;
            }
        } else if (MODE == 1) {
            // z = L^{-T} t does not depend on beta: the backward sweep runs between this
            // block's arrival at the t.t (and r.r) reduction and the wait for the others,
            // and the direction update p = z + beta p follows the wait
            // x += alpha p also waits for the arrival: the FP64 pipe is otherwise idle there
            const double2 f = part_fwd<true, double, false, false, false>(C, S, p0, np, false, alpha, rel, err, rec);
            bool done = false, ok;
            double beta = 0.0;
            auto x_update = [&]() {
                for (int l = tid; l < np; l += kPartThreads)
                    __stcg(&C.x[p0 + l], __ldcg(&C.x[p0 + l]) + alpha * S.p[l]);
            };
            if (rel) {
                double g[2] = { f.y, f.x };
                const unsigned tk = grid_reduce_tree_arrive<kPartThreads, 2>(a.bar, g, sh, S.red);
                part_bwd<3>(C, S, p0, np, 0.0, err, rec);
                x_update();
                ok = grid_reduce_tree_wait<kPartThreads, 2>(a.bar, tk, g, sh, [&](const double* tot, double* out) {
                    out[0] = sqrt(tot[1]) <= a.tol * bnorm;
                    out[1] = tot[0] / gamma;
                });
                g2[0] = g[0];
                rr = g[1];
            } else {
                double g[1] = { f.y };
                const unsigned tk = grid_reduce_tree_arrive<kPartThreads, 1>(a.bar, g, sh, S.red);
                part_bwd<3>(C, S, p0, np, 0.0, err, rec);
                x_update();
                ok = grid_reduce_tree_wait<kPartThreads, 1>(a.bar, tk, g, sh, [&](const double* tot, double* out) {
                    out[0] = tot[0] < a.tol * a.tol;
                    out[1] = tot[0] / gamma;
                });
                g2[0] = g[0];
            }
            if (!ok) return;
            done = sh[24] != 0.0;
            beta = sh[25];
            if (done) { gamma = g2[0]; conv = true; break; }
            gamma = g2[0];
            part_p_after_bwd(C, S, p0, np, beta, true);
            if (!grid_sync(a.bar, gridDim.x)) return;
            continue;
        } else {
            g2[1] = part_fwd<false>(C, S, p0, np, false, alpha, rel, err, rec).x;
            if (!grid_sync(a.bar, gridDim.x)) return;
            g2[0] = part_bwd<0>(C, S, p0, np, 0.0, err, rec);
        }
        // the test and beta = r.z / (previous r.z) (thread 0; see part_reduce)
        if (rel) {
            if (!part_reduce<2>(a.bar, g2, sh, S.red, [&](const double* tot, double* out) {
                    out[0] = sqrt(tot[1]) <= a.tol * bnorm;
                    out[1] = tot[0] / gamma;
                }))
                return;
            rr = g2[1];
        } else {
            double g1[1] = { g2[0] };
            if (!part_reduce<1>(a.bar, g1, sh, S.red, [&](const double* tot, double* out) {
                    out[0] = tot[0] < a.tol * a.tol;
                    out[1] = tot[0] / gamma;
                }))
                return;
            g2[0] = g1[0];
        }
        const double gnew = g2[0];
        if (sh[24] != 0.0) { gamma = gnew; conv = true; break; }
        const double beta = sh[25];
        gamma = gnew;
        part_p_update(C, S, p0, np, beta);
        if (!grid_sync(a.bar, gridDim.x)) return;
    }
    if (!rel && it > 0) {
        double f[1] = { 0.0 };
        for (int l = tid; l < np; l += kPartThreads) f[0] += S.r[l] * S.r[l];
        if (!part_reduce<1>(a.bar, f, sh, S.red)) return;
        rr = f[0];
    }
    for (int l = tid; l < np; l += kPartThreads) a.x[__ldg(&C.qa[p0 + l])] = __ldcg(&C.x[p0 + l]);
    if (blockIdx.x == 0 && tid == 0) {
        a.out->iterations = it;
        a.out->converged = conv ? 1 : 0;
        a.out->residual = rel ? sqrt(rr) / (bnorm > 0 ? bnorm : 1.0) : sqrt(gamma);
        a.out->relres = sqrt(rr) / (bnorm > 0 ? bnorm : 1.0);
        a.out->status = conv ? DEV_OK : DEV_NOT_CONVERGED;
    }
}

// Mixed-precision CG on the parts (pcg_csr_mixed's algorithm): FP32 SpMV, FP32 IC(0) or
// ILU(0) sweeps and FP32 vectors in shared memory, FP64-accumulated dot products, inside an
// FP64 iterative refinement: when the iterated residual has dropped by inner_eta (or
// below the target) the update d is added to x in FP64, r = b - A x is recomputed in FP64
// with A's FP64 values, and the relative test ||r|| <= tol ||b|| runs in FP64; CG then
// continues from the true residual, keeping its search direction.  LOCAL: the factors of
// each part's diagonal block alone (IC(0) / ILU(0) of A with the couplings between parts
// dropped, a block-Jacobi preconditioner with one block per part): the sweeps wait on no
// other part and run in shared memory only; the FP64 refinement keeps the solve's target.
template <bool IC, bool LOCAL>
__device__ void pcg_part_mixed(const KArgs& a, double* sh, unsigned char* smem) {
    const PartCg& C = a.part;
    const int p0 = C.qs[blockIdx.x * C.ng], p1 = C.qs[(blockIdx.x + 1) * C.ng], np = p1 - p0;
    const PartSm<float> S = part_sm<float>(C, smem, C.R, true, true, p0);
    const int tid = threadIdx.x;
    int* err = a.bar.err;
    int* rec = a.bar.rec;
    part_load(a, S, p0, p1);
    for (int l = tid; l < np; l += kPartThreads) S.d[l] = 0.0f;
    if (!grid_sync(a.bar, gridDim.x)) return;
    // r = b - A x in FP64; the refinement's form
    auto residual = [&](double& rr_, double* bb_) {
        for (int l = tid; l < np; l += kPartThreads) {
            double bi;
            const double ri = part_residual(a, S.rp, p0, l, bi);
            S.r[l] = (float)ri;
            rr_ += ri * ri;
            if (bb_) *bb_ += bi * bi;
        }
    };
    double red[2] = { 0.0, 0.0 };  // b.b, r.r
    residual(red[1], &red[0]);
    // square roots by thread 0 (see part_reduce)
    if (!part_reduce<2>(a.bar, red, sh, S.red, [&](const double* tot, double* out) {
            out[0] = sqrt(tot[0]);
            out[1] = sqrt(tot[1]);
        }))
        return;
    const double bnorm = sh[24];
    const double target = a.tol * bnorm;
    double rnorm = sh[25];
    double rlast = rnorm;
    int it = 0, refinements = 1;
    bool conv = rnorm <= target;
    if (!conv) {
        // z = M^{-1} r, p = z, gamma = r.z
        part_fwd<IC, float, true, LOCAL>(C, S, p0, np, true, 0.0f, false, err, rec);
        if (!grid_sync(a.bar, gridDim.x)) return;
        double g[1] = { part_bwd<1, float, LOCAL>(C, S, p0, np, 0.0f, err, rec) };
        if (!part_reduce<1>(a.bar, g, sh, S.red)) return;
        double gamma = g[0];
        while (it < a.maxit) {
            double pq[1] = { part_spmv(C, S, p0, np, !LOCAL) };
            ++it;
            if (!part_reduce<1>(a.bar, pq, sh, S.red, [&](const double* tot, double* out) {
                    out[0] = (double)(float)(gamma / tot[0]);
                }))
                return;
            const float alpha = (float)sh[24];
            double g2[2];  // r.z (IC: t.t), r.r
            // refinement test and beta (thread 0; see part_reduce)
            auto post = [&](const double* tot, double* out) {
                const double rit = sqrt(tot[1]);
                out[0] = rit <= a.inner_eta * rlast || rit <= target;
                out[1] = (double)(float)(tot[0] / gamma);
            };
            if (IC) {
                // the backward sweep (z alone) overlaps the reduction, as in pcg_part
                const double2 f = part_fwd<true, float, true, LOCAL>(C, S, p0, np, false, alpha, true, err, rec);
                g2[0] = f.y;
                g2[1] = f.x;
                const unsigned tk = grid_reduce_tree_arrive<kPartThreads, 2>(a.bar, g2, sh, S.red);
                part_bwd<3, float, LOCAL>(C, S, p0, np, 0.0f, err, rec);
                if (!grid_reduce_tree_wait<kPartThreads, 2>(a.bar, tk, g2, sh, post)) return;
            } else {
                g2[1] = part_fwd<false, float, true, LOCAL>(C, S, p0, np, false, alpha, true, err, rec).x;
                if (!LOCAL && !grid_sync(a.bar, gridDim.x)) return;
                g2[0] = part_bwd<0, float, LOCAL>(C, S, p0, np, 0.0f, err, rec);
                if (!part_reduce<2>(a.bar, g2, sh, S.red, post)) return;
            }
            bool refined = false;
            double gnew = g2[0];
            float beta = (float)sh[25];
            if (sh[24] != 0.0) {
                // refinement: x += d, r = b - A x and the test in FP64; the boundary rows'
                // forward results back to the marker for the forward sweep on the new r
                for (int l = tid; l < np; l += kPartThreads) {
                    __stcg(&C.x[p0 + l], __ldcg(&C.x[p0 + l]) + (double)S.d[l]);
                    S.d[l] = 0.0f;
                    if (!LOCAL && S.bnd[l]) __stcg(&C.gt32[p0 + l], Pending<float>::marker());
                }
                if (!grid_sync(a.bar, gridDim.x)) return;
                // (after the barrier: every part has ended the backward sweep that read them)
                if (!LOCAL)
                    for (int l = tid; l < np; l += kPartThreads)
                        if (S.bnd[l]) __stcg(&C.gz32[p0 + l], Pending<float>::marker());
                double rr[1] = { 0.0 };
                residual(rr[0], nullptr);
                if (!part_reduce<1>(a.bar, rr, sh, S.red, [&](const double* tot, double* out) {
                        out[0] = sqrt(tot[0]);
                    }))
                    return;
                ++refinements;
                rnorm = sh[24];
                if (rnorm <= target) { conv = true; break; }
                rlast = rnorm;
                // continue from the true residual, keeping the search direction
                double g3[1];
                if (IC) {
                    g3[0] = part_fwd<true, float, true, LOCAL>(C, S, p0, np, true, 0.0f, false, err, rec).y;
                } else {
                    part_fwd<false, float, true, LOCAL>(C, S, p0, np, true, 0.0f, false, err, rec);
                    if (!LOCAL && !grid_sync(a.bar, gridDim.x)) return;
                    g3[0] = part_bwd<0, float, LOCAL>(C, S, p0, np, 0.0f, err, rec);
                }
                if (!part_reduce<1>(a.bar, g3, sh, S.red, [&](const double* tot, double* out) {
                        out[0] = (double)(float)(tot[0] / gamma);
                    }))
                    return;
                gnew = g3[0];
                beta = (float)sh[24];
                refined = true;
            }
            gamma = gnew;
            if (IC && refined)  // the overlapped sweep used the old t
                part_bwd<2, float, LOCAL>(C, S, p0, np, beta, err, rec);
            else if (IC)
                part_p_after_bwd(C, S, p0, np, beta, !LOCAL);
            else
                part_p_update(C, S, p0, np, beta);
            if (!grid_sync(a.bar, gridDim.x)) return;
        }
        if (!conv)  // iteration limit: keep the accumulated update
            for (int l = tid; l < np; l += kPartThreads)
                __stcg(&C.x[p0 + l], __ldcg(&C.x[p0 + l]) + (double)S.d[l]);
    }
    for (int l = tid; l < np; l += kPartThreads) a.x[__ldg(&C.qa[p0 + l])] = __ldcg(&C.x[p0 + l]);
    if (blockIdx.x == 0 && tid == 0) {
        a.out->iterations = it;
        a.out->converged = conv ? 1 : 0;
        a.out->residual = rnorm / (bnorm > 0 ? bnorm : 1.0);
        a.out->relres = rnorm / (bnorm > 0 ? bnorm : 1.0);
        a.out->status = conv ? DEV_OK : DEV_NOT_CONVERGED;
        a.out->pad = refinements;
    }
}

template <int MODE>
__global__ void __launch_bounds__(kPartThreads, 1) k_pcg_part(KArgs a) {
    __shared__ double sh[kShDoubles];
    extern __shared__ __align__(16) unsigned char part_smem[];
    pcg_part<MODE>(a, sh, part_smem);
}

template <bool IC, bool LOCAL>
__global__ void __launch_bounds__(kPartThreads, 1) k_pcg_part_mixed(KArgs a) {
    __shared__ double sh[kShDoubles];
    extern __shared__ __align__(16) unsigned char part_smem[];
    pcg_part_mixed<IC, LOCAL>(a, sh, part_smem);
}


__global__ void __launch_bounds__(kSolverThreads, kSolverBlocksPerSm) k_pcg_one(KArgs a) {
    __shared__ double sh[kShDoubles];
    pcg_one_reduction(a, sh);
}

// SolverCG::solve (linear_solver.cu:440-515).  Per iteration: q = A p with p.q (one fused
// barrier-reduction), x/r update, z = M^{-1} r with r.z (and r.r) (one fused
// barrier-reduction), p = z + beta p (one barrier).
// CG with ILU(0)/IC(0) on B's CSR arrays (pcg_csr) as a kernel of its own: the
// iteration's code alone, so its loads can be batched without the other paths of k_pcg
// competing for the 64 registers a thread has at two 512-thread blocks per SM.
__global__ void __launch_bounds__(kSolverThreads, kSolverBlocksPerSm) k_pcg_csr(KArgs a) {
    __shared__ double sh[kShDoubles];
    pcg_csr(a, sh);
}

__global__ void __launch_bounds__(kSolverThreads, kSolverBlocksPerSm) k_pcg(KArgs a) {
    // read before the first barrier, so before the counter can advance
    const int ep_base = a.epoch ? *a.epoch : 0;
    __shared__ double sh[kShDoubles];
    int r0, r1;
    row_range(a.A.n, r0, r1);
    const bool global_pc = (a.precond == PF2_PRECOND_ILU || a.precond == PF2_PRECOND_IC);
    const bool fused = global_pc && a.T.band.P == 0 && a.T.band.K > 0;  // slot sweeps fused with the updates
    const bool rel = a.criterion == PF2_CRITERION_REL;
    if (global_pc && a.T.csr) {
        pcg_csr(a, sh);
        return;
    }
    // Jacobi: inverse diagonal (PreconditionerJacobi::initialize, preconditioners.cu:3-14)
    if (a.precond == PF2_PRECOND_JACOBI)
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) a.invd[i] = 1.0 / a.A.val[a.A.diag[i]];
    // r = b - A x
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const double v = row_dot(a.A, i, a.x);
        a.r[i] = a.b[i] - v;
    }
    __syncthreads();
    int apply = 0;
    if (global_pc && !grid_sync(a.bar, gridDim.x)) return;
    if (!precond_apply(a, a.r, a.z, r0, r1, apply++, ep_base)) return;
    __syncthreads();
    double red[3] = { 0.0, 0.0, 0.0 };  // r.z, b.b, r.r
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const double zi = __ldcg(&a.z[i]);
        const double ri = a.r[i];
        a.p[i] = zi;
        red[0] += ri * zi;
        red[1] += a.b[i] * a.b[i];
        red[2] += ri * ri;
    }
    if (!grid_reduce<3>(a.bar, red, sh)) return;
    double gamma = red[0];
    const double bnorm = sqrt(red[1]);
    double rr = red[2];
    const double tol2 = a.tol * a.tol;
    auto done_test = [&](double gm, double rr_) { return rel ? (sqrt(rr_) <= a.tol * bnorm) : (gm < tol2); };
    int it = 0;
    bool conv = done_test(gamma, rr);
    while (!conv && it < a.maxit) {
        ++it;
        double pq[1] = { spmv_rows(a.A, a.p, a.q, r0, r1) };
        if (!grid_reduce<1>(a.bar, pq, sh)) return;
        const double alpha = gamma / pq[0];
        double g2[2] = { 0.0, 0.0 };
        if (fused) {
            // 4 barriers per iteration: (p.q), forward -> backward, (r.z, r.r), p update
            g2[1] = slots_fwd_cg<double>(a.T, alpha, a.r, a.q, a.x, a.p, a.bar.err);
            if (!grid_sync(a.bar, gridDim.x)) return;
            g2[0] = slots_bwd_cg<double>(a.T, a.r, a.z, a.bar.err);
        } else if (global_pc) {
            for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                a.x[i] += alpha * a.p[i];
                a.r[i] -= alpha * a.q[i];
            }
            __syncthreads();
            if (!grid_sync(a.bar, gridDim.x)) return;
            if (!precond_apply(a, a.r, a.z, r0, r1, apply++, ep_base)) return;
            for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                const double ri = a.r[i];
                g2[0] += ri * __ldcg(&a.z[i]);
                if (rel) g2[1] += ri * ri;
            }
        } else {
            // two rows per pass, all loads issued before the stores
            const bool jac = a.precond == PF2_PRECOND_JACOBI;
            for (int i0 = r0 + threadIdx.x; i0 < r1; i0 += 2 * blockDim.x) {
                double xv[2], pv[2], rv[2], qv[2], dv[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int i = i0 + u * blockDim.x;
                    const bool in = i < r1;
                    xv[u] = in ? a.x[i] : 0.0;
                    pv[u] = in ? a.p[i] : 0.0;
                    rv[u] = in ? a.r[i] : 0.0;
                    qv[u] = in ? a.q[i] : 0.0;
                    dv[u] = in && jac ? a.invd[i] : 1.0;
                }
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int i = i0 + u * blockDim.x;
                    if (i >= r1) continue;
                    a.x[i] = xv[u] + alpha * pv[u];
                    const double ri = rv[u] - alpha * qv[u];
                    const double zi = jac ? ri * dv[u] : ri;
                    a.r[i] = ri;
                    a.z[i] = zi;
                    g2[0] += ri * zi;
                    if (rel) g2[1] += ri * ri;
                }
            }
        }
        // with the absolute criterion (a test of r.z alone) r.r is reduced once after
        // the loop, not per iteration
        if (rel || fused) {
            if (!grid_reduce<2>(a.bar, g2, sh)) return;
            rr = g2[1];
        } else {
            double g1[1] = { g2[0] };
            if (!grid_reduce<1>(a.bar, g1, sh)) return;
            g2[0] = g1[0];
        }
        const double gnew = g2[0];
        if (done_test(gnew, rr)) { gamma = gnew; conv = true; break; }
        const double beta = gnew / gamma;
        gamma = gnew;
        p_update(a.p, a.z, beta, r0, r1);
        if (!grid_sync(a.bar, gridDim.x)) return;
    }
    if (!rel && !fused && it > 0) {
        double f[1] = { 0.0 };
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const double ri = __ldcg(&a.r[i]);
            f[0] += ri * ri;
        }
        if (!grid_reduce<1>(a.bar, f, sh)) return;
        rr = f[0];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->iterations = it;
        a.out->converged = conv ? 1 : 0;
        a.out->residual = rel ? sqrt(rr) / (bnorm > 0 ? bnorm : 1.0) : sqrt(gamma);
        a.out->relres = sqrt(rr) / (bnorm > 0 ? bnorm : 1.0);
        a.out->status = conv ? DEV_OK : DEV_NOT_CONVERGED;
    }
}

// out[i] = this block's part of w . V_i (rows r0..r1), i < K; warp q takes i = q, q + 8, ...
__device__ __forceinline__ void block_dots(const double* V, int n, int K, const double* w, int r0, int r1,
                                           double* out, bool with_norm = false) {
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = wq; i < K; i += nw) {
        const double* vi = V + (size_t)i * n;
        // four independent partial sums keep four loads of each stream in flight
        double d0 = 0.0, d1 = 0.0, d2 = 0.0, d3 = 0.0;
        int j = r0 + lane;
        for (; j + 96 < r1; j += 128) {
            d0 += w[j] * vi[j];
            d1 += w[j + 32] * vi[j + 32];
            d2 += w[j + 64] * vi[j + 64];
            d3 += w[j + 96] * vi[j + 96];
        }
        for (; j < r1; j += 32) d0 += w[j] * vi[j];
        double d = (d0 + d1) + (d2 + d3);
        d = warp_sum(d);
        if (lane == 0) out[i] = d;
    }
    if (with_norm && wq == K % nw) {  // out[K] = w . w
        double d = 0.0;
        for (int j = r0 + lane; j < r1; j += 32) d += w[j] * w[j];
        d = warp_sum(d);
        if (lane == 0) out[K] = d;
    }
    __syncthreads();
}

// Grid-wide sums of K per-block values (vals, shared memory), in two barriers: every
// block stores its K partials, block b adds up values b, b + G, ... over the blocks in
// block order, then every block reads the K totals back into vals.
__device__ bool grid_reduce_vec(const KArgs& a, double* vals, int K, double* sh) {
    const int G = gridDim.x;
    for (int k = threadIdx.x; k < K; k += blockDim.x) __stcg(&a.vpart[(size_t)k * G + blockIdx.x], vals[k]);
    if (!grid_sync(a.bar, G)) return false;
    for (int k = blockIdx.x; k < K; k += G) {
        double t = 0.0;
        for (int q = threadIdx.x; q < G; q += blockDim.x) t += __ldcg(&a.vpart[(size_t)k * G + q]);
        t = block_sum(t, sh);
        if (threadIdx.x == 0) __stcg(&a.vtot[k], t);
    }
    if (!grid_sync(a.bar, G)) return false;
    for (int k = threadIdx.x; k < K; k += blockDim.x) vals[k] = __ldcg(&a.vtot[k]);
    __syncthreads();
    return true;
}

// SolverGMRES::solve (linear_solver.cu:560-660): left-preconditioned GMRES, the
// projections taken one after another on the updated vector, Givens rotations
// (updateHcolumn :40-66), stop on |beta_k| < tol; x changes only on convergence.  With
// m < maxit the Krylov space restarts every m iterations.
__global__ void __launch_bounds__(kSolverThreads, kSolverBlocksPerSm) k_gmres(KArgs a) {
    // read before the first barrier, so before the counter can advance
    const int ep_base = a.epoch ? *a.epoch : 0;
    __shared__ double sh[kShDoubles];
    __shared__ double cs[kMaxGmresSmem], sn[kMaxGmresSmem], beta[kMaxGmresSmem + 1], hcol[kMaxGmresSmem + 1];
    __shared__ double h2[kMaxGmresSmem + 1];
    int r0, r1;
    row_range(a.A.n, r0, r1);
    const int n = a.A.n;
    const bool global_pc = (a.precond == PF2_PRECOND_ILU || a.precond == PF2_PRECOND_IC);
    if (a.precond == PF2_PRECOND_JACOBI)
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) a.invd[i] = 1.0 / a.A.val[a.A.diag[i]];
    int apply = 0, total_it = 0;
    bool conv = false;
    double res = 0.0;
    const int m = a.m;
    while (true) {
        // v0 = M^{-1}(b - A x), beta0 = ||v0||
        double* v0 = a.V;
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const double v = row_dot(a.A, i, a.x);
            a.r[i] = a.b[i] - v;
        }
        __syncthreads();
        if (global_pc && !grid_sync(a.bar, gridDim.x)) return;
        if (!precond_apply(a, a.r, v0, r0, r1, apply++, ep_base)) return;
        __syncthreads();
        double s2[1] = { 0.0 };
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const double vi = __ldcg(&v0[i]);
            s2[0] += vi * vi;
        }
        if (!grid_reduce<1>(a.bar, s2, sh)) return;
        const double b0 = sqrt(s2[0]);
        res = b0;
        if (b0 < a.tol) { conv = true; break; }
        if (total_it >= a.maxit) break;
        if (threadIdx.x == 0) beta[0] = b0;
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) v0[i] = __ldcg(&v0[i]) / b0;
        if (!grid_sync(a.bar, gridDim.x)) return;
        int k = 0;
        bool inner_conv = false;
        while (k < m && total_it < a.maxit) {
            ++total_it;
            double* vk = a.V + (size_t)k * n;
            double* vkp = a.V + (size_t)(k + 1) * n;
            for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                const double v = row_dot(a.A, i, vk);
                a.q[i] = v;
            }
            __syncthreads();
            if (global_pc && !grid_sync(a.bar, gridDim.x)) return;
            if (!precond_apply(a, a.q, vkp, r0, r1, apply++, ep_base)) return;
            __syncthreads();
            if (a.gs == PF2_GS_CLASSICAL_TWICE) {
                // h = V^T v_{k+1}, v_{k+1} -= V h; a second pass (its h added) unless the
                // first kept ||v_{k+1}|| above 0.7 of its value (the DGKS test: then one
                // pass is already orthogonal to working accuracy)
                for (int pass = 0; pass < 2; ++pass) {
                    double* hv = pass == 0 ? hcol : h2;
                    block_dots(a.V, n, k + 1, vkp, r0, r1, hv, pass == 0);
                    if (!grid_reduce_vec(a, hv, pass == 0 ? k + 2 : k + 1, sh)) return;
                    for (int j = r0 + threadIdx.x; j < r1; j += blockDim.x) {
                        double v = vkp[j];
                        for (int i = 0; i <= k; ++i) v -= hv[i] * a.V[(size_t)i * n + j];
                        vkp[j] = v;
                    }
                    __syncthreads();
                    if (pass == 0) {
                        double hh = 0.0;
                        for (int i = 0; i <= k; ++i) hh += hv[i] * hv[i];
                        const double ww = hv[k + 1];
                        if (ww - hh > 0.49 * ww) {  // uniform: every block holds the same totals
                            for (int i = threadIdx.x; i <= k; i += blockDim.x) h2[i] = 0.0;
                            __syncthreads();
                            break;
                        }
                    }
                }
                for (int i = threadIdx.x; i <= k; i += blockDim.x) hcol[i] += h2[i];
                __syncthreads();
            } else {
                // h_ik = v_{k+1} . v_i, then v_{k+1} -= h_ik v_i, i = 0..k (the reference's order)
                for (int i = 0; i <= k; ++i) {
                    const double* vi = a.V + (size_t)i * n;
                    double d[1] = { 0.0 };
                    for (int j = r0 + threadIdx.x; j < r1; j += blockDim.x) d[0] += __ldcg(&vkp[j]) * vi[j];
                    if (!grid_reduce<1>(a.bar, d, sh)) return;
                    const double h = d[0];
                    if (threadIdx.x == 0) hcol[i] = h;
                    for (int j = r0 + threadIdx.x; j < r1; j += blockDim.x) vkp[j] = __ldcg(&vkp[j]) - h * vi[j];
                    __syncthreads();
                }
            }
            double nn[1] = { 0.0 };
            for (int j = r0 + threadIdx.x; j < r1; j += blockDim.x) {
                const double v = __ldcg(&vkp[j]);
                nn[0] += v * v;
            }
            if (!grid_reduce<1>(a.bar, nn, sh)) return;
            const double aux = sqrt(nn[0]);
            for (int j = r0 + threadIdx.x; j < r1; j += blockDim.x) vkp[j] = __ldcg(&vkp[j]) / aux;
            if (threadIdx.x == 0) {
                double* h = hcol;
                for (int i = 0; i < k; ++i) {
                    const double tmp = cs[i] * h[i] + sn[i] * h[i + 1];
                    h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
                    h[i] = tmp;
                }
                const double coeff = rsqrt(h[k] * h[k] + aux * aux);
                cs[k] = h[k] * coeff;
                sn[k] = aux * coeff;
                h[k] = cs[k] * h[k] + sn[k] * aux;
                beta[k + 1] = -sn[k] * beta[k];
                beta[k] *= cs[k];
                if (blockIdx.x == 0)
                    for (int i = 0; i <= k; ++i) a.H[(size_t)m * k + i] = h[i];
            }
            __syncthreads();
            res = fabs(beta[k + 1]);
            ++k;
            if (!grid_sync(a.bar, gridDim.x)) return;
            if (res < a.tol) { inner_conv = true; break; }
        }
        // y = H^{-1} beta (upper triangular), x += V y (own rows)
        if (threadIdx.x == 0) {
            for (int i = k - 1; i >= 0; --i) {
                double s = beta[i];
                for (int j = i + 1; j < k; ++j) s -= __ldcg(&a.H[i + (size_t)m * j]) * hcol[j];
                hcol[i] = s / __ldcg(&a.H[i + (size_t)m * i]);
            }
        }
        __syncthreads();
        const bool update = inner_conv || (k == m && m < a.maxit);
        if (update)
            for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                double s = 0.0;
                for (int j = 0; j < k; ++j) s += __ldcg(&a.V[(size_t)j * n + i]) * hcol[j];
                a.x[i] = s + a.x[i];
            }
        if (!grid_sync(a.bar, gridDim.x)) return;
        if (inner_conv) { conv = true; break; }
        if (!update || total_it >= a.maxit) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->iterations = total_it;
        a.out->converged = conv ? 1 : 0;
        a.out->residual = res;
        a.out->relres = 0.0;  // GMRES tracks the preconditioned residual only
        a.out->status = conv ? DEV_OK : DEV_NOT_CONVERGED;
    }
}

// FP32 SpMV row (FP32 products summed in FP32 within the row; values read through L2
// only where other blocks write them during the kernel).
__device__ __forceinline__ float row_dot32(const Csr& A, const float* __restrict__ val32, int row, const float* x) {
    const int s = __ldg(&A.rowptr[row]), e = __ldg(&A.rowptr[row + 1]);
    float sum = 0.0f;
    for (int k = s; k < e; ++k) sum += __ldg(&val32[k]) * __ldcg(&x[__ldg(&A.col[k])]);
    return sum;
}

// FP32 preconditioner apply of the mixed solver: ILU(0)/IC(0) with the factors rounded
// to FP32 (grid-wide, includes grid barriers) or Jacobi / none on this block's rows.
__device__ bool precond_apply32(const KArgs& a, const float* src, float* dst, int r0, int r1, int apply,
                                int ep_base) {
    if (a.precond == PF2_PRECOND_ILU || a.precond == PF2_PRECOND_IC) {
        if (a.T.band.P) {
            tri_solve_banded<float>(a.T, 0, const_cast<float*>(src), a.T.tmp32, a.bar.err);
            if (!grid_sync(a.bar, gridDim.x)) return false;
            tri_solve_banded<float>(a.T, 1, a.T.tmp32, a.T.outB32, a.bar.err);
        } else if (a.T.band.K) {
            tri_solve_slots<float>(a.T, 0, const_cast<float*>(src), a.T.tmp32, a.bar.err);
            if (!grid_sync(a.bar, gridDim.x)) return false;
            tri_solve_slots<float>(a.T, 1, a.T.tmp32, a.T.outB32, a.bar.err);
        } else {
            tri_solve<float>(a.T, 0, const_cast<float*>(src), a.T.tmp32, a.T.fact32, &a.T.tickets[2 * apply],
                             a.bar.err);
            if (!grid_sync(a.bar, gridDim.x)) return false;
            tri_solve<float>(a.T, 1, a.T.tmp32, a.T.outB32, a.T.fact32, &a.T.tickets[2 * apply + 1], a.bar.err);
        }
        if (!grid_sync(a.bar, gridDim.x)) return false;
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const int k = a.T.iperm[i];
            dst[i] = __ldcg(&a.T.outB32[k]);
            __stcg(&a.T.outB32[k], Pending<float>::marker());
        }
        __syncthreads();
        return true;
    }
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) dst[i] = src[i] * a.invd32[i];
    __syncthreads();
    return true;
}

// Mixed-precision CG with reliable updates (no reference counterpart).  The iteration
// (SpMV, preconditioner, vector updates) runs in FP32; each thread's few dot-product
// terms are summed in FP32 and the block and grid sums in FP64.  The solution lives in
// FP64: the FP32 iterates accumulate the update d, and at a refinement point (the
// iterated residual fell below kReliableDrop of its value at the last refinement, or
// below the target) x += d, r = b - A x and the test ||r|| <= tol ||b|| run in FP64, and
// the iteration continues from the true residual with its search direction kept, so the
// Krylov space is not restarted.  On GB300 the FP32 iteration also stays off the small
// FP64 pipe.  a.inner_eta is the refinement trigger (the drop of the iterated residual).
// Mixed-precision PCG in B's numbering (the CSR path of pcg_csr with the inner iteration
// in FP32): the SpMV on an FP32 copy of B's values, the sweeps on an FP32 copy of the
// factors, FP32 vectors; the update d is folded into x (FP64, B's numbering) and the
// residual recomputed in FP64 from B's FP64 values whenever the iterated residual fell by
// the inner factor since the last refinement, as in k_pcg_mixed.
__device__ void pcg_csr_mixed(const KArgs& a, double* sh) {
    const Tri& T = a.T;
    const int n = a.A.n;
    int r0, r1;
    row_range(n, r0, r1);
    const Csr B{ n, T.B.rowptr, T.B.col, T.bval, T.B.diag };
    double* xB = T.xB;
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        __stcg(&xB[i], a.x[__ldg(&T.perm[i])]);
        __stcg(&a.d32[i], 0.0f);
    }
    if (!grid_sync(a.bar, gridDim.x)) return;
    double red[2] = { 0.0, 0.0 };  // b.b, r.r
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const double bi = a.b[__ldg(&T.perm[i])];
        const double ri = bi - row_dot(B, i, xB);
        __stcg(&a.r32[i], (float)ri);
        red[0] += bi * bi;
        red[1] += ri * ri;
    }
    if (!grid_reduce<2>(a.bar, red, sh)) return;
    const double bnorm = sqrt(red[0]);
    const double target = a.tol * bnorm;
    double rnorm = sqrt(red[1]);
    double rlast = rnorm;
    int it = 0, refinements = 1;
    bool conv = rnorm <= target;
    if (!conv) {
        // z = M^{-1} r, p = z, gamma = r.z
        csr_fwd<0, float>(T, 0.0f, 0.0f, true, a.r32, nullptr, nullptr, nullptr, nullptr, a.z32, a.bar.err);
        if (!grid_sync(a.bar, gridDim.x)) return;
        double g[1] = { csr_bwd<float>(T, a.r32, a.z32, a.p32, a.bar.err) };
        if (!grid_reduce<1>(a.bar, g, sh)) return;
        double gamma = g[0];
        // IC(0): three barriers per iteration with r.z = t.t (below); ILU(0) (fuse_p): the
        // direction update inside the next SpMV (spmv_rows_pz), p alternating between two
        // arrays
        float* pc = a.p32;
        float* pa = a.p32b;
        float beta = 0.0f;
        const bool ic = T.kind == PF2_PRECOND_IC;
        while (it < a.maxit) {
            double pq[1];
            if (it == 0 || !a.fuse_p) {
                pq[0] = (double)spmv_rows<float>(B, T.bval32, pc, a.q32, r0, r1);
            } else {
                pq[0] = (double)spmv_rows_pz<float>(B, T.bval32, a.z32, pc, beta, pa, a.q32, r0, r1);
                float* t = pc;
                pc = pa;
                pa = t;
            }
            ++it;
            if (!grid_reduce<1>(a.bar, pq, sh)) return;
            const float alpha = (float)(gamma / pq[0]);
            if (ic && !a.fuse_p) {
                // IC(0) in three barriers (as pcg_csr): r.z = t.t after the forward sweep,
                // the backward sweep with the direction update
                const double2 f =
                    csr_fwd<1, float>(T, alpha, 0.0f, false, a.r32, a.q32, a.d32, pc, nullptr, a.z32, a.bar.err);
                double gt[2] = { f.y, f.x };
                if (!grid_reduce<2>(a.bar, gt, sh)) return;
                double gnew = gt[0];
                const double rit = sqrt(gt[1]);
                if (rit <= a.inner_eta * rlast || rit <= target) {
                    // refinement; the forward results are reset to the marker for the
                    // forward sweep on the new residual
                    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                        __stcg(&xB[i], __ldcg(&xB[i]) + (double)__ldcg(&a.d32[i]));
                        __stcg(&a.d32[i], 0.0f);
                        __stcg(&T.tmp32[i], Pending<float>::marker());
                    }
                    if (!grid_sync(a.bar, gridDim.x)) return;
                    double rr[1] = { 0.0 };
                    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                        const double ri = a.b[__ldg(&T.perm[i])] - row_dot(B, i, xB);
                        __stcg(&a.r32[i], (float)ri);
                        rr[0] += ri * ri;
                    }
                    if (!grid_reduce<1>(a.bar, rr, sh)) return;
                    ++refinements;
                    rnorm = sqrt(rr[0]);
                    if (rnorm <= target) { conv = true; break; }
                    rlast = rnorm;
                    double g3[1] = { csr_fwd<0, float>(T, 0.0f, 0.0f, true, a.r32, nullptr, nullptr, nullptr, nullptr,
                                                       a.z32, a.bar.err).y };
                    if (!grid_reduce<1>(a.bar, g3, sh)) return;
                    gnew = g3[0];
                }
                beta = (float)(gnew / gamma);
                gamma = gnew;
                csr_bwd<float, true>(T, nullptr, a.z32, pc, a.bar.err, beta);
                if (!grid_sync(a.bar, gridDim.x)) return;
                continue;
            }
            // d += alpha p, r -= alpha q and the forward sweep; the backward sweep with r.z
            double g2[2] = { 0.0, 0.0 };
            g2[1] = csr_fwd<1, float>(T, alpha, 0.0f, false, a.r32, a.q32, a.d32, pc, nullptr, a.z32, a.bar.err).x;
            if (!grid_sync(a.bar, gridDim.x)) return;
            g2[0] = csr_bwd<float>(T, a.r32, a.z32, nullptr, a.bar.err);
            if (!grid_reduce<2>(a.bar, g2, sh)) return;
            double gnew = g2[0];
            const double rit = sqrt(g2[1]);
            if (rit <= a.inner_eta * rlast || rit <= target) {
                // refinement: x += d, r = b - B x and the convergence test in FP64
                for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                    __stcg(&xB[i], __ldcg(&xB[i]) + (double)__ldcg(&a.d32[i]));
                    __stcg(&a.d32[i], 0.0f);
                }
                if (!grid_sync(a.bar, gridDim.x)) return;
                double rr[1] = { 0.0 };
                for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                    const double ri = a.b[__ldg(&T.perm[i])] - row_dot(B, i, xB);
                    __stcg(&a.r32[i], (float)ri);
                    rr[0] += ri * ri;
                }
                if (!grid_reduce<1>(a.bar, rr, sh)) return;
                ++refinements;
                rnorm = sqrt(rr[0]);
                if (rnorm <= target) { conv = true; break; }
                rlast = rnorm;
                // continue from the true residual, keeping the search direction
                csr_fwd<0, float>(T, 0.0f, 0.0f, true, a.r32, nullptr, nullptr, nullptr, nullptr, a.z32, a.bar.err);
                if (!grid_sync(a.bar, gridDim.x)) return;
                double g3[1] = { csr_bwd<float>(T, a.r32, a.z32, nullptr, a.bar.err) };
                if (!grid_reduce<1>(a.bar, g3, sh)) return;
                gnew = g3[0];
            }
            beta = (float)(gnew / gamma);
            gamma = gnew;
            if (!a.fuse_p) {
                p_update<float>(pc, a.z32, beta, r0, r1);
                if (!grid_sync(a.bar, gridDim.x)) return;
            }
        }
        if (!conv)  // iteration limit: keep the accumulated update
            for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x)
                __stcg(&xB[i], __ldcg(&xB[i]) + (double)__ldcg(&a.d32[i]));
    }
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) a.x[__ldg(&T.perm[i])] = __ldcg(&xB[i]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->iterations = it;
        a.out->converged = conv ? 1 : 0;
        a.out->residual = rnorm / (bnorm > 0 ? bnorm : 1.0);
        a.out->relres = rnorm / (bnorm > 0 ? bnorm : 1.0);
        a.out->status = conv ? DEV_OK : DEV_NOT_CONVERGED;
        a.out->pad = refinements;
    }
}

__global__ void __launch_bounds__(kSolverThreads, kSolverBlocksPerSm) k_pcg_mixed(KArgs a) {
    // read before the first barrier, so before the counter can advance
    const int ep_base = a.epoch ? *a.epoch : 0;
    __shared__ double sh[kShDoubles];
    if (a.T.csr) {
        pcg_csr_mixed(a, sh);
        return;
    }
    int r0, r1;
    row_range(a.A.n, r0, r1);
    const bool global_pc = (a.precond == PF2_PRECOND_ILU || a.precond == PF2_PRECOND_IC);
    const bool fused = global_pc && a.T.band.P == 0 && a.T.band.K > 0;  // slot sweeps fused with the updates
    // r = b - A x (FP64), r32 = r, d = 0, inverse diagonal
    double red[2] = { 0.0, 0.0 };  // b.b, r.r
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        a.invd32[i] = (a.precond == PF2_PRECOND_JACOBI) ? (float)(1.0 / a.A.val[a.A.diag[i]]) : 1.0f;
        const double ri = a.b[i] - row_dot(a.A, i, a.x);
        a.r32[i] = (float)ri;
        a.d32[i] = 0.0f;
        red[0] += a.b[i] * a.b[i];
        red[1] += ri * ri;
    }
    if (!grid_reduce<2>(a.bar, red, sh)) return;
    const double bnorm = sqrt(red[0]);
    const double target = a.tol * bnorm;
    double rnorm = sqrt(red[1]);       // true (FP64) residual at the last refinement
    double rlast = rnorm;              // iterated residual norm at the last refinement
    int it = 0, refinements = 1, apply = 0;
    bool conv = rnorm <= target;
    if (!conv) {
        // z = M^{-1} r32, p = z, gamma = r.z
        if (global_pc && !grid_sync(a.bar, gridDim.x)) return;
        if (!precond_apply32(a, a.r32, a.z32, r0, r1, apply++, ep_base)) return;
        float gl = 0.0f;
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
            const float zi = a.z32[i];
            a.p32[i] = zi;
            gl = fmaf(a.r32[i], zi, gl);
        }
        double g[1] = { (double)gl };
        if (!grid_reduce<1>(a.bar, g, sh)) return;
        double gamma = g[0];
        while (it < a.maxit) {
            ++it;
            // q = A p, p.q
            float pql = 0.0f;
            for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                const float v = row_dot32(a.A, a.val32, i, a.p32);
                a.q32[i] = v;
                pql = fmaf(a.p32[i], v, pql);
            }
            double pq[1] = { (double)pql };
            if (!grid_reduce<1>(a.bar, pq, sh)) return;
            const float alpha = (float)(gamma / pq[0]);
            // d += alpha p, r -= alpha q, z = M^{-1} r, r.z and r.r
            float gl2 = 0.0f, rl2 = 0.0f;
            double g2[2] = { 0.0, 0.0 };
            if (fused) {
                g2[1] = slots_fwd_cg<float>(a.T, alpha, a.r32, a.q32, a.d32, a.p32, a.bar.err);
                if (!grid_sync(a.bar, gridDim.x)) return;
                g2[0] = slots_bwd_cg<float>(a.T, a.r32, a.z32, a.bar.err);
            } else if (global_pc) {
                for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                    a.d32[i] = fmaf(alpha, a.p32[i], a.d32[i]);
                    const float ri = fmaf(-alpha, a.q32[i], a.r32[i]);
                    a.r32[i] = ri;
                    rl2 = fmaf(ri, ri, rl2);
                }
                __syncthreads();
                if (!grid_sync(a.bar, gridDim.x)) return;
                if (!precond_apply32(a, a.r32, a.z32, r0, r1, apply++, ep_base)) return;
                for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) gl2 = fmaf(a.r32[i], a.z32[i], gl2);
            } else {
                for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                    a.d32[i] = fmaf(alpha, a.p32[i], a.d32[i]);
                    const float ri = fmaf(-alpha, a.q32[i], a.r32[i]);
                    const float zi = ri * a.invd32[i];
                    a.r32[i] = ri;
                    a.z32[i] = zi;
                    gl2 = fmaf(ri, zi, gl2);
                    rl2 = fmaf(ri, ri, rl2);
                }
            }
            if (!fused) {
                g2[0] = (double)gl2;
                g2[1] = (double)rl2;
            }
            if (!grid_reduce<2>(a.bar, g2, sh)) return;
            double gnew = g2[0];
            const double rit = sqrt(g2[1]);
            if (rit <= a.inner_eta * rlast || rit <= target) {
                // refinement: x += d (own rows), r = b - A x and the convergence test in FP64
                for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                    a.x[i] += (double)__ldcg(&a.d32[i]);  // d may come from other blocks' slots
                    __stcg(&a.d32[i], 0.0f);
                }
                if (!grid_sync(a.bar, gridDim.x)) return;
                double rr[1] = { 0.0 };
                for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
                    const double ri = a.b[i] - row_dot(a.A, i, a.x);
                    a.r32[i] = (float)ri;
                    rr[0] += ri * ri;
                }
                if (!grid_reduce<1>(a.bar, rr, sh)) return;
                ++refinements;
                rnorm = sqrt(rr[0]);
                if (rnorm <= target) { conv = true; break; }
                rlast = rnorm;
                // continue from the true residual, keeping the search direction
                if (global_pc && !grid_sync(a.bar, gridDim.x)) return;
                if (!precond_apply32(a, a.r32, a.z32, r0, r1, apply++, ep_base)) return;
                float gl3 = 0.0f;
                for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) gl3 = fmaf(a.r32[i], __ldcg(&a.z32[i]), gl3);
                double g3[1] = { (double)gl3 };
                if (!grid_reduce<1>(a.bar, g3, sh)) return;
                gnew = g3[0];
            }
            const float beta = (float)(gnew / gamma);
            gamma = gnew;
            for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) a.p32[i] = fmaf(beta, a.p32[i], __ldcg(&a.z32[i]));
            if (!grid_sync(a.bar, gridDim.x)) return;
        }
        if (!conv) {
            // iteration limit: keep the accumulated update
            for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) a.x[i] += (double)__ldcg(&a.d32[i]);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->iterations = it;
        a.out->converged = conv ? 1 : 0;
        a.out->residual = rnorm / (bnorm > 0 ? bnorm : 1.0);
        a.out->relres = rnorm / (bnorm > 0 ? bnorm : 1.0);
        a.out->status = conv ? DEV_OK : DEV_NOT_CONVERGED;
        a.out->pad = refinements;
    }
}

__global__ void k_to_float(long long n, const double* __restrict__ a, float* __restrict__ b) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

__global__ void k_precond_apply(KArgs a) {
    const int ep_base = a.epoch ? *a.epoch : 0;
    int r0, r1;
    row_range(a.A.n, r0, r1);
    precond_apply(a, a.r, a.z, r0, r1, 0, ep_base);
}

}  // namespace pf2

using namespace pf2;

struct BandHost {
    DevBuf<int> rstep, sptr, row, rhs, dep, pos, dpos, gstart;
    int ngroups = 0;
    DevBuf<double> val, dinv;
    DevBuf<float> val32, dinv32;
};

struct pf2_solver {
    pf2_solver_options opt{};
    const pf2_mesh* mesh = nullptr;
    int n = 0, nnz = 0, blocks = 0, m = 0;
    long long barrier_polls = 0;  // PF2_BARRIER_POLLS (tests): a grid-barrier wait's poll limit
    DevBuf<double> r, z, p, q, s, invd, partial, V, H, vpart, rhat, yv, tv;
    DevBuf<unsigned> bar;  // count, gen
    DevBuf<int> err;
    DevBuf<int> rec;  // where a device wait gave up (5 ints)
    DevBuf<SolveOut> out;
    PinnedBuf<SolveOut> h_out;
    // ILU / IC
    DevBuf<double> fact, tmp;
    // mixed precision
    DevBuf<float> val32, d32, r32, p32, q32, z32, invd32, p32b;
    DevBuf<int> fwd_order, bwd_order, lt_off, lt_row, lt_pos, done_f, done_b;
    DevBuf<unsigned> tickets;
    DevBuf<int> epoch;  // device counter of the row flags' epochs (graph replays stay valid)
    DevBuf<int> brp, bcol, bdiag, bmap, perm, iperm;  // pattern of the factors and the ordering
    DevBuf<int> band_rs;
    BandHost band[2];  // banded solve plan, forward and backward
    int band_P = 0, band_R = 0, band_K = 0;
    size_t smem = 0;  // dynamic shared memory of the solver kernels (banded window)
    DevBuf<double> outB;
    DevBuf<float> fact32, tmp32, outB32;  // mixed precision with ILU/IC
    // FP64 CG on B (Tri::csr): A's values and the factors on B's pattern, x in B's
    // numbering, and per entry of B the factor entry it takes (lower and ILU upper: its
    // own; IC upper (i, j): l_ji; diagonal: -1 - position, stored as its inverse)
    bool csr = false;
    DevBuf<double> bval, fsym, xB;
    DevBuf<float> bval32, fsym32;  // mixed precision on the CSR path
    DevBuf<double> pipe;           // pipelined CG: u, w, z, three m arrays
    DevBuf<int> tpos;
    int ngroups = 0;
    DevBuf<int> cstart;
    int levels_fwd = 0, levels_bwd = 0, colors = 0;
    // partitioned CG (k_pcg_part): group starts per part, CSR in the part order Q with the
    // positions of its entries in A (values) and in B (factors), Q -> A rows, boundary
    // flags, x in Q order and the boundary rows' global copies of p, t, z
    bool part = false;
    bool part_local = false;  // mixed precision: partition-local factors (A's values through bmap_local)
    DevBuf<int> bmap_local;   // bmap with the entries that couple two parts set to -1
    const char* part_why = "not planned";  // why the partitioned kernel does not apply
    int part_P = 0, part_R = 0, part_ng = 0;
    size_t part_smem = 0;
    long long part_boundary_rows = 0;
    DevBuf<int> q_s, q_rp, q_col, q_diag, q_a, q_amap, q_fmap;
    DevBuf<unsigned char> q_bnd;
    DevBuf<double> q_val, q_f, q_x, q_gp, q_gt, q_gz;
    DevBuf<float> q_val32, q_f32, q_gp32, q_gt32, q_gz32;  // mixed precision
    bool factored = false;
    const pf2_csr* last = nullptr;  // matrix of the last setup / solve
};

// Greedy colouring leaves a thin tail of high colours (on the cylinder meshes 306 of
// 499,288 nodes in colours 4 and 5), and each colour is one more dependency level of
// both triangular sweeps.  Each tail node is moved below K (the first colour whose tail
// holds under 0.2 % of the nodes) by a Kempe-chain swap: for colours a, b < K, swap a and
// b in the (a, b)-components of v's a-coloured neighbours, provided none of those
// components reaches a b-coloured neighbour of v; v then takes a.  Swaps keep the
// colouring proper.  Nodes that no swap frees keep their colour; the search stops after
// 64 n visited nodes.  Returns the number of colours.
static int kempe_trim(int n, const std::vector<int>& rp, const std::vector<int>& col, std::vector<int>& color,
                      int nc) {
    std::vector<long long> size(nc, 0);
    for (int i = 0; i < n; ++i) size[color[i]]++;
    int K = nc;
    long long tail = 0;
    while (K > 1 && tail + size[K - 1] < std::max(1LL, (long long)n / 500)) tail += size[--K];
    if (K == nc) return nc;
    std::vector<int> mark(n, -1), comp, queue;
    long long budget = 64LL * n;
    int stamp = 0;
    auto fix = [&](int v) {
        for (int a = 0; a < K; ++a) {
            bool has_a = false;
            for (int k = rp[v]; k < rp[v + 1]; ++k) has_a |= col[k] != v && color[col[k]] == a;
            if (!has_a) {
                color[v] = a;
                return true;
            }
            for (int b = 0; b < K; ++b) {
                if (b == a) continue;
                ++stamp;
                comp.clear();
                queue.clear();
                for (int k = rp[v]; k < rp[v + 1]; ++k)
                    if (col[k] != v && color[col[k]] == a && mark[col[k]] != stamp) {
                        mark[col[k]] = stamp;
                        queue.push_back(col[k]);
                    }
                bool ok = true;
                for (size_t h = 0; h < queue.size() && ok; ++h) {
                    const int x = queue[h];
                    comp.push_back(x);
                    if (--budget < 0) return false;
                    for (int k = rp[x]; k < rp[x + 1]; ++k) {
                        const int y = col[k];
                        if (y == x || y == v || mark[y] == stamp) continue;
                        if (color[y] != a && color[y] != b) continue;
                        // a b-coloured neighbour of v inside the component: the swap would
                        // give v an a-coloured neighbour again
                        bool nb_of_v = false;
                        for (int q = rp[v]; q < rp[v + 1]; ++q) nb_of_v |= col[q] == y;
                        if (nb_of_v && color[y] == b) { ok = false; break; }
                        mark[y] = stamp;
                        queue.push_back(y);
                    }
                }
                if (!ok) continue;
                for (int x : comp) color[x] = color[x] == a ? b : a;
                color[v] = a;
                return true;
            }
        }
        return false;
    };
    // a few passes: a swap for one node can free another node's colour
    for (int pass = 0; pass < 4 && budget > 0; ++pass) {
        int left = 0, fixed = 0;
        for (int v = 0; v < n && budget > 0; ++v)
            if (color[v] >= K) {
                if (fix(v)) ++fixed;
                else ++left;
            }
        if (left == 0 || fixed == 0) break;
    }
    int m = 0;
    for (int i = 0; i < n; ++i) m = std::max(m, color[i] + 1);
    return m;
}

// Multicolour permutation of a symmetric pattern: greedy colouring in row order, then
// (kempe) the thin tail of high colours moved down by kempe_trim.  perm[r] is the row of
// A at position r of B (colour by colour, rows of a colour ascending); groups receives
// the sweep groups (the colour starts and n), where without kempe the tail colours are
// merged into the group before them.  Returns the number of colours.
static int multicolour_order(int n, const int* rp, const int* col, bool kempe, std::vector<int>& perm,
                             std::vector<int>& groups) {
    std::vector<int> color(n, -1);
    int nc = 0;
    std::vector<char> used;
    for (int i = 0; i < n; ++i) {
        used.assign(nc + 1, 0);
        for (int k = rp[i]; k < rp[i + 1]; ++k)
            if (col[k] < i) used[color[col[k]]] = 1;
        int c = 0;
        while (used[c]) ++c;
        color[i] = c;
        nc = std::max(nc, c + 1);
    }
    const int nc_greedy = nc;
    if (kempe) {
        const std::vector<int> rpv(rp, rp + n + 1), colv(col, col + rp[n]);
        nc = kempe_trim(n, rpv, colv, color, nc);
    }
    std::vector<int> cnt(nc + 1, 0);
    for (int i = 0; i < n; ++i) cnt[color[i] + 1]++;
    for (int c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
    groups = cnt;
    if (!kempe) {  // merge the thin tail (under 0.2 % of the rows) into the group before it
        int g = nc_greedy;
        long long tail = 0;
        while (g > 1 && tail + (cnt[g] - cnt[g - 1]) < std::max(1, n / 500)) {
            tail += cnt[g] - cnt[g - 1];
            --g;
        }
        groups.assign(cnt.begin(), cnt.begin() + g);
        groups.push_back(n);
    }
    perm.assign(n, 0);
    for (int i = 0; i < n; ++i) perm[cnt[color[i]]++] = i;
    return nc;
}

// Recursive bisection of the graph of a symmetric pattern into P parts whose sizes differ
// by at most one row per level: a subset is ordered breadth-first from a pseudo-peripheral
// node (the last node a breadth-first search from the subset's first node reaches; a
// disconnected subset continues from its next unreached node) and cut after the rows of
// its first P / 2 parts.  part[i] receives the part of row i.
static void graph_parts(int n, const std::vector<int>& rp, const std::vector<int>& col, int P, std::vector<int>& part) {
    part.assign(n, 0);
    std::vector<int> order(n), tmp(n), subset(n, -1), seen(n, -1);
    for (int i = 0; i < n; ++i) order[i] = i;
    struct Job { int lo, hi, P, first; };
    std::vector<Job> jobs{ { 0, n, P, 0 } };
    int sid = 0, stamp = 0;
    auto bfs = [&](int lo, int hi, int start) {
        ++stamp;
        int w = lo, next = lo;
        tmp[w++] = start;
        seen[start] = stamp;
        for (int h = lo; h < hi; ++h) {
            if (h == w) {  // the reached component is exhausted: the subset's next unreached row
                while (seen[order[next]] == stamp) ++next;
                tmp[w++] = order[next];
                seen[order[next]] = stamp;
            }
            const int v = tmp[h];
            for (int k = rp[v]; k < rp[v + 1]; ++k) {
                const int u = col[k];
                if (subset[u] == sid && seen[u] != stamp) {
                    seen[u] = stamp;
                    tmp[w++] = u;
                }
            }
        }
        return tmp[hi - 1];
    };
    while (!jobs.empty()) {
        const Job j = jobs.back();
        jobs.pop_back();
        if (j.P <= 1 || j.hi - j.lo <= 1) {
            for (int q = j.lo; q < j.hi; ++q) part[order[q]] = j.first;
            continue;
        }
        ++sid;
        for (int q = j.lo; q < j.hi; ++q) subset[order[q]] = sid;
        const int far = bfs(j.lo, j.hi, order[j.lo]);
        bfs(j.lo, j.hi, far);
        std::copy(tmp.begin() + j.lo, tmp.begin() + j.hi, order.begin() + j.lo);
        const int P1 = j.P / 2;
        const int mid = j.lo + (int)((long long)(j.hi - j.lo) * P1 / j.P);
        jobs.push_back({ mid, j.hi, j.P - P1, j.first + P1 });
        jobs.push_back({ j.lo, mid, P1, j.first });
    }
}

// The partitioned CG plan (k_pcg_part) for the pattern of B = P A P^T (brp, bcol; bmap:
// position in A of each entry of B; bdiag; perm: row of A at each row of B) with sweep
// groups `groups` of B's rows: parts from graph_parts on A's pattern (rp, col), one per SM
// (at least kPartMinRows rows each), the part order Q, the CSR arrays in Q order and the
// boundary flags.  Leaves S->part false where the plan does not apply: a group whose rows
// depend on one another, or a part too large for the shared-memory vectors.
constexpr int kPartMinRows = 512;
static pf2_status build_part_plan(pf2_solver* S, const std::vector<int>& rp, const std::vector<int>& col,
                                  const std::vector<int>& brp, const std::vector<int>& bcol,
                                  const std::vector<int>& bmap, const std::vector<int>& bdiag,
                                  const std::vector<int>& perm, const std::vector<int>& groups, bool tri) {
    S->part = false;
    const int n = S->n, nnz = S->nnz;
    const int ng = (int)groups.size() - 1;
    std::vector<int> grp(n);
    for (int g = 0; g < ng; ++g)
        for (int r = groups[g]; r < groups[g + 1]; ++r) grp[r] = g;
    if (tri)  // the rows of a group must depend only on earlier groups
        for (int r = 0; r < n; ++r)
            for (int k = brp[r]; k < bdiag[r]; ++k)
                if (grp[bcol[k]] >= grp[r]) {
                    S->part_why = "a sweep group's rows depend on one another";
                    return PF2_OK;
                }
    int P = std::max(1, std::min(num_sms(), n / kPartMinRows));
    if (const char* e = getenv("PF2_CG_PARTS")) P = std::max(1, std::min(num_sms(), atoi(e)));  // tests, tuning
    std::vector<int> part;
    graph_parts(n, rp, col, P, part);
    // boundary rows (a neighbour in another part), in A's numbering
    std::vector<unsigned char> bnd_a(n, 0);
    for (int i = 0; i < n; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k)
            if (part[col[k]] != part[i]) bnd_a[i] = 1;
    // Q: by part, then group, then the group's boundary rows before its interior rows (the
    // threads that wait on other parts' values share warps with as few others as possible),
    // then B's order
    std::vector<int> cls((size_t)P * ng * 2 + 1, 0);
    auto cell = [&](int r) { return ((size_t)part[perm[r]] * ng + grp[r]) * 2 + (bnd_a[perm[r]] ? 0 : 1); };
    for (int r = 0; r < n; ++r) cls[cell(r) + 1]++;
    for (size_t c = 0; c + 1 < cls.size(); ++c) cls[c + 1] += cls[c];
    std::vector<int> qs((size_t)P * ng + 1);
    for (size_t c = 0; c < qs.size(); ++c) qs[c] = cls[2 * c];
    std::vector<int> fill(cls.begin(), cls.end() - 1), bq(n), qa(n), qb(n);
    for (int r = 0; r < n; ++r) {
        const int q = fill[cell(r)]++;
        bq[r] = q;
        qb[q] = r;
        qa[q] = perm[r];
    }
    int R = 0;
    for (int p = 0; p < P; ++p) R = std::max(R, qs[(size_t)(p + 1) * ng] - qs[(size_t)p * ng]);
    int optin = 0;
    PF2_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, 0));
    const bool mixed = S->opt.precision == PF2_PRECISION_MIXED;
    const size_t smem = (part_smem_bytes(R, tri, mixed ? sizeof(float) : sizeof(double), mixed) + 15) / 16 * 16;
    if (smem + 2048 > (size_t)optin) {
        S->part_why = "a part's vectors exceed the shared memory of a block";
        return PF2_OK;
    }
    std::vector<int> qrp(n + 1, 0), qcol(std::max(nnz, 1)), qdiag(n), qamap(std::max(nnz, 1)),
        qfmap(std::max(nnz, 1));
    std::vector<unsigned char> bnd(n, 0);
    long long nb = 0;
    for (int q = 0; q < n; ++q) {
        const int r = qb[q];
        const int len = brp[r + 1] - brp[r];
        qrp[q + 1] = qrp[q] + len;
        const int pr = part[perm[r]];
        for (int e = 0; e < len; ++e) {
            const int kb = brp[r] + e, kq = qrp[q] + e;
            qcol[kq] = bq[bcol[kb]];
            qamap[kq] = bmap[kb];
            qfmap[kq] = kb;
            if (part[perm[bcol[kb]]] != pr) bnd[q] = 1;
        }
        qdiag[q] = qrp[q] + (bdiag[r] - brp[r]);
        nb += bnd[q];
    }
    auto up = [&](auto& d, const auto& h) -> pf2_status {
        PF2_TRY(d.alloc(h.size()));
        PF2_CUDA(cudaMemcpy(d.p, h.data(), sizeof(h[0]) * h.size(), cudaMemcpyHostToDevice));
        return PF2_OK;
    };
    PF2_TRY(up(S->q_s, qs));
    PF2_TRY(up(S->q_rp, qrp));
    PF2_TRY(up(S->q_col, qcol));
    PF2_TRY(up(S->q_diag, qdiag));
    PF2_TRY(up(S->q_a, qa));
    PF2_TRY(up(S->q_amap, qamap));
    PF2_TRY(up(S->q_bnd, bnd));
    PF2_TRY(S->q_val.alloc(std::max(nnz, 1)));
    if (tri) {
        PF2_TRY(up(S->q_fmap, qfmap));
        PF2_TRY(S->q_f.alloc(std::max(nnz, 1)));
    }
    PF2_TRY(S->q_x.alloc(n));
    PF2_TRY(S->q_gp.alloc(n));
    PF2_TRY(S->q_gt.alloc(n));
    PF2_TRY(S->q_gz.alloc(n));
    // mixed precision, PF2_CG_PART_LOCAL=1: partition-local factors (block-Jacobi IC(0) /
    // ILU(0), one block per part).  Not the default: at 499,288 rows (152 parts) the sweeps
    // get 17 % cheaper but the solve takes twice the iterations (1,428 against 712 to 1e-8)
    S->part_local = false;
    if (mixed && tri) {
        const char* e = getenv("PF2_CG_PART_LOCAL");
        if (e && atoi(e) != 0) {
            std::vector<int> bl(std::max(nnz, 1));
            for (int r = 0; r < n; ++r)
                for (int k = brp[r]; k < brp[r + 1]; ++k)
                    bl[k] = part[perm[bcol[k]]] == part[perm[r]] ? bmap[k] : -1;
            PF2_TRY(up(S->bmap_local, bl));
            S->part_local = true;
        }
    }
    if (mixed) {
        PF2_TRY(S->q_val32.alloc(std::max(nnz, 1)));
        PF2_TRY(S->q_f32.alloc(std::max(nnz, 1)));
        PF2_TRY(S->q_gp32.alloc(n));
        PF2_TRY(S->q_gt32.alloc(n));
        PF2_TRY(S->q_gz32.alloc(n));
    }
    S->part = true;
    S->part_P = P;
    S->part_R = R;
    S->part_ng = ng;
    S->part_smem = smem;
    S->part_boundary_rows = nb;
    return PF2_OK;
}

// Whether a solve with these options may run on the parts: standard CG, FP64 (k_pcg_part)
// or, with ILU(0) / IC(0), mixed precision (k_pcg_part_mixed); PF2_CG_PART=0 keeps the
// other kernels (tuning, comparisons).
static bool part_eligible(const pf2_solver* S) {
    if (const char* e = getenv("PF2_CG_PART"))
        if (atoi(e) == 0) return false;
    const bool tri = S->opt.precond == PF2_PRECOND_ILU || S->opt.precond == PF2_PRECOND_IC;
    return S->opt.kind == PF2_SOLVER_CG && S->opt.cg_variant == PF2_CG_STANDARD &&
           (S->opt.precision == PF2_PRECISION_FP64 || (S->opt.precision == PF2_PRECISION_MIXED && tri));
}

// The partitioned CG kernel of the solver's preconditioner.
static void* part_kernel(const pf2_solver* S) {
    if (S->opt.precision == PF2_PRECISION_MIXED) {
        if (S->part_local)
            return S->opt.precond == PF2_PRECOND_IC ? (void*)k_pcg_part_mixed<true, true>
                                                    : (void*)k_pcg_part_mixed<false, true>;
        return S->opt.precond == PF2_PRECOND_IC ? (void*)k_pcg_part_mixed<true, false>
                                                : (void*)k_pcg_part_mixed<false, false>;
    }
    if (S->opt.precond == PF2_PRECOND_IC) return (void*)k_pcg_part<1>;
    if (S->opt.precond == PF2_PRECOND_ILU) return (void*)k_pcg_part<2>;
    return (void*)k_pcg_part<0>;
}

static pf2_status build_tri_plan(pf2_solver* S) {
    const pf2_mesh* M = S->mesh;
    const int n = M->nv, nnz = M->nnz;
    std::vector<int> rp(n + 1), col(nnz);
    PF2_CUDA(cudaMemcpy(rp.data(), M->rowptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
    PF2_CUDA(cudaMemcpy(col.data(), M->col.p, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
    // ordering: natural (the reference's) or greedy multicolour in natural order, rows
    // of a colour kept in natural order
    std::vector<int> perm(n), iperm(n);
    std::vector<int> groups{ 0, n };  // sweep groups of the CSR path: the colours, or all rows
    if (S->opt.ordering == PF2_ORDERING_MULTICOLOR) {
        // PF2_KEMPE=0 (tuning): keep the greedy colours and sweep the tail colours with the
        // last main colour (same permutation as greedy, fewer sweep groups)
        const char* ke = getenv("PF2_KEMPE");
        S->colors = multicolour_order(n, rp.data(), col.data(), !ke || atoi(ke) != 0, perm, groups);
    } else {
        for (int i = 0; i < n; ++i) perm[i] = i;
    }
    for (int r = 0; r < n; ++r) iperm[perm[r]] = r;
    // pattern of B = P A P^T with the position in A of each entry
    std::vector<int> brp(n + 1, 0), bcol(nnz), bmap(nnz), bdiag(n);
    std::vector<std::pair<int, int>> row;
    for (int r = 0; r < n; ++r) {
        const int o = perm[r];
        row.clear();
        for (int k = rp[o]; k < rp[o + 1]; ++k) row.emplace_back(iperm[col[k]], k);
        std::sort(row.begin(), row.end());
        brp[r + 1] = brp[r] + (int)row.size();
        for (size_t q = 0; q < row.size(); ++q) {
            bcol[brp[r] + q] = row[q].first;
            bmap[brp[r] + q] = row[q].second;
            if (row[q].first == r) bdiag[r] = brp[r] + (int)q;
        }
    }
    // forward levels: 1 + max over the strictly lower entries
    std::vector<int> lev(n, 0);
    int nl = 0;
    for (int i = 0; i < n; ++i) {
        int l = 0;
        for (int k = brp[i]; k < bdiag[i]; ++k) l = std::max(l, lev[bcol[k]] + 1);
        lev[i] = l;
        nl = std::max(nl, l + 1);
    }
    S->levels_fwd = nl;
    std::vector<int> level_groups[2];
    level_groups[0].assign(nl + 1, 0);
    for (int i = 0; i < n; ++i) level_groups[0][lev[i] + 1]++;
    for (int l = 0; l < nl; ++l) level_groups[0][l + 1] += level_groups[0][l];
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return lev[a] < lev[b]; });
    PF2_TRY(S->fwd_order.alloc(n));
    PF2_CUDA(cudaMemcpy(S->fwd_order.p, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    const std::vector<int> fwd_h = order;
    // backward levels: 1 + max over the strictly upper entries (the pattern is symmetric)
    std::fill(lev.begin(), lev.end(), 0);
    nl = 0;
    for (int i = n - 1; i >= 0; --i) {
        int l = 0;
        for (int k = bdiag[i] + 1; k < brp[i + 1]; ++k) l = std::max(l, lev[bcol[k]] + 1);
        lev[i] = l;
        nl = std::max(nl, l + 1);
    }
    S->levels_bwd = nl;
    level_groups[1].assign(nl + 1, 0);
    for (int i = 0; i < n; ++i) level_groups[1][lev[i] + 1]++;
    for (int l = 0; l < nl; ++l) level_groups[1][l + 1] += level_groups[1][l];
    for (int i = 0; i < n; ++i) order[i] = n - 1 - i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return lev[a] < lev[b]; });
    PF2_TRY(S->bwd_order.alloc(n));
    PF2_CUDA(cudaMemcpy(S->bwd_order.p, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    const std::vector<int> bwd_h = order;
    // rows of L^T: for each k, the entries l_ik with i > k as (row i, position in B)
    std::vector<int> off(n + 1, 0);
    for (int i = 0; i < n; ++i)
        for (int k = brp[i]; k < bdiag[i]; ++k) off[bcol[k] + 1]++;
    for (int i = 0; i < n; ++i) off[i + 1] += off[i];
    std::vector<int> lrow(std::max(off[n], 1)), lpos(std::max(off[n], 1)), fill(off.begin(), off.end() - 1);
    for (int i = 0; i < n; ++i)
        for (int k = brp[i]; k < bdiag[i]; ++k) {
            const int c = bcol[k];
            lrow[fill[c]] = i;
            lpos[fill[c]] = k;
            fill[c]++;
        }
    auto up = [&](DevBuf<int>& d, const std::vector<int>& h) -> pf2_status {
        PF2_TRY(d.alloc(h.size()));
        PF2_CUDA(cudaMemcpy(d.p, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice));
        return PF2_OK;
    };
    PF2_TRY(up(S->lt_off, off));
    PF2_TRY(up(S->lt_row, lrow));
    PF2_TRY(up(S->lt_pos, lpos));
    PF2_TRY(up(S->brp, brp));
    PF2_TRY(up(S->bcol, bcol));
    PF2_TRY(up(S->bdiag, bdiag));
    PF2_TRY(up(S->bmap, bmap));
    PF2_TRY(up(S->perm, perm));
    PF2_TRY(up(S->iperm, iperm));
    PF2_TRY(S->fact.alloc(nnz));
    PF2_TRY(S->tmp.alloc(n));
    PF2_TRY(S->outB.alloc(n));
    PF2_TRY(S->done_f.alloc(n));
    PF2_TRY(S->done_b.alloc(n));
    PF2_TRY(S->epoch.alloc(1));
    PF2_CUDA(cudaMemset(S->epoch.p, 0, sizeof(int)));
    PF2_CUDA(cudaMemset(S->done_f.p, 0, sizeof(int) * n));
    PF2_CUDA(cudaMemset(S->done_b.p, 0, sizeof(int) * n));
    // long dependency chains (the natural order of a mesh numbered column by column):
    // banded solve, ranges of kBandRows rows, levels counted inside each range
    // PF2_BAND_ROWS / PF2_BAND_MIN_LEVELS override the range size and the threshold
    // (tuning and tests)
    int band_rows = kBandRows, band_min = kBandMinLevels;
    if (const char* e = getenv("PF2_BAND_ROWS")) band_rows = std::max(32, std::min(kBandRows, atoi(e)));
    if (const char* e = getenv("PF2_BAND_MIN_LEVELS")) band_min = std::max(1, atoi(e));
    S->band_P = 0;
    const bool ic = S->opt.precond == PF2_PRECOND_IC;
    // dependencies of row i in a direction: (column, factor position)
    auto deps = [&](int dir, int i, auto&& f) {
        if (dir == 0) {
            for (int k = brp[i]; k < bdiag[i]; ++k) f(bcol[k], k);
        } else if (!ic) {
            for (int k = bdiag[i] + 1; k < brp[i + 1]; ++k) f(bcol[k], k);
        } else {
            for (int k = off[i]; k < off[i + 1]; ++k) f(lrow[k], lpos[k]);
        }
    };
    int K = 1;
    for (int dir = 0; dir < 2; ++dir)
        for (int i = 0; i < n; ++i) {
            int c = 0;
            deps(dir, i, [&](int, int) { ++c; });
            K = std::max(K, c);
        }
    // slot records (rows with at most kBandMaxDeps dependencies): in (range, step) order for
    // the banded solve, in level order for the sync-free one
    const bool banded = K <= kBandMaxDeps && std::max(S->levels_fwd, S->levels_bwd) >= band_min;
    // CG with few levels: the whole iteration on B's CSR arrays (pcg_csr, pcg_csr_mixed)
    S->csr = std::max(S->levels_fwd, S->levels_bwd) < band_min && S->opt.kind == PF2_SOLVER_CG;
    if (const char* e = getenv("PF2_CG_SLOTS")) S->csr = S->csr && atoi(e) == 0;  // tuning: keep the slot sweeps
    if (S->csr) {
        std::vector<int> tpos(std::max(nnz, 1));
        for (int r = 0; r < n; ++r)
            for (int k = brp[r]; k < brp[r + 1]; ++k) tpos[k] = (k == bdiag[r]) ? -1 - k : k;
        if (ic)  // upper entry (i, j) of row i takes l_ji, the lower entry (j, i) of row j
            for (int j = 0; j < n; ++j)
                for (int k = brp[j]; k < bdiag[j]; ++k) {
                    const int i = bcol[k];
                    const int* b0 = bcol.data() + bdiag[i] + 1;
                    const int* b1 = bcol.data() + brp[i + 1];
                    const int* f = std::lower_bound(b0, b1, j);
                    if (f == b1 || *f != j) {
                        set_error("pattern of B is not symmetric at (%d, %d)", i, j);
                        return PF2_BAD_INPUT;
                    }
                    tpos[f - bcol.data()] = k;
                }
        PF2_TRY(up(S->tpos, tpos));
        PF2_TRY(up(S->cstart, groups));
        S->ngroups = (int)groups.size() - 1;
        PF2_TRY(S->bval.alloc(nnz));
        PF2_TRY(S->fsym.alloc(nnz));
        PF2_TRY(S->xB.alloc(n));
        if (S->opt.precision == PF2_PRECISION_MIXED) {
            PF2_TRY(S->bval32.alloc(nnz));
            PF2_TRY(S->fsym32.alloc(nnz));
        }
        if (S->opt.ordering == PF2_ORDERING_MULTICOLOR && part_eligible(S))
            PF2_TRY(build_part_plan(S, rp, col, brp, bcol, bmap, bdiag, perm, groups, true));
        else
            S->part_why = "ILU(0) / IC(0) in the natural order";
    }
    if (K <= kBandMaxDeps) {
        const int R = banded ? std::min(n, band_rows) : n;
        const int P = banded ? (n + R - 1) / R : 0;
        std::vector<int> rs(P + 1);
        for (int r = 0; r <= P; ++r) rs[r] = std::min(n, r * R);
        for (int dir = 0; dir < 2; ++dir) {
            BandHost& H = S->band[dir];
            std::vector<int> rstep(P + 1, 0), sptr, srow;
            srow.reserve(n);
            std::vector<int> loc(n, 0);
            if (!banded) {
                srow = dir == 0 ? fwd_h : bwd_h;
                PF2_TRY(up(H.gstart, level_groups[dir]));
                H.ngroups = (int)level_groups[dir].size() - 1;
            }
            for (int r = 0; r < P; ++r) {
                const int r0 = rs[r], r1 = rs[r + 1];
                int nl = 0;
                for (int q = 0; q < r1 - r0; ++q) {
                    const int i = dir == 0 ? r0 + q : r1 - 1 - q;
                    int l = 0;
                    deps(dir, i, [&](int j, int) {
                        if (j >= r0 && j < r1) l = std::max(l, loc[j] + 1);
                    });
                    loc[i] = l;
                    nl = std::max(nl, l + 1);
                }
                // rows grouped by level (processing order inside a level), levels cut into
                // steps of at most one row per thread
                std::vector<int> cnt(nl + 1, 0);
                for (int i = r0; i < r1; ++i) cnt[loc[i] + 1]++;
                for (int l = 0; l < nl; ++l) cnt[l + 1] += cnt[l];
                const int base = (int)srow.size();
                srow.resize(base + (r1 - r0));
                std::vector<int> fill(cnt.begin(), cnt.end() - 1);
                for (int q = 0; q < r1 - r0; ++q) {
                    const int i = dir == 0 ? r0 + q : r1 - 1 - q;
                    srow[base + fill[loc[i]]++] = i;
                }
                rstep[r] = (int)sptr.size();
                for (int l = 0; l < nl; ++l)
                    for (int t = cnt[l]; t < cnt[l + 1]; t += kSolverThreads) sptr.push_back(base + t);
            }
            rstep[P] = (int)sptr.size();
            sptr.push_back(n);
            std::vector<int> rhs(n), dep((size_t)n * K, -1), pos((size_t)n * K, -1), dpos(n, -1);
            for (int t = 0; t < n; ++t) {
                const int i = srow[t];
                rhs[t] = dir == 0 ? perm[i] : i;
                int c = 0;
                deps(dir, i, [&](int j, int k) {
                    dep[(size_t)t * K + c] = j;
                    pos[(size_t)t * K + c] = k;
                    ++c;
                });
                dpos[t] = (dir == 1 || ic) ? bdiag[i] : -1;
            }
            PF2_TRY(up(H.rstep, rstep));
            PF2_TRY(up(H.sptr, sptr));
            PF2_TRY(up(H.row, srow));
            PF2_TRY(up(H.rhs, rhs));
            PF2_TRY(up(H.dep, dep));
            PF2_TRY(up(H.pos, pos));
            PF2_TRY(up(H.dpos, dpos));
            PF2_TRY(H.val.alloc((size_t)n * K));
            PF2_TRY(H.dinv.alloc(n));
            if (S->opt.precision == PF2_PRECISION_MIXED) {
                PF2_TRY(H.val32.alloc((size_t)n * K));
                PF2_TRY(H.dinv32.alloc(n));
            }
        }
        PF2_TRY(up(S->band_rs, rs));
        S->band_P = P;
        S->band_R = banded ? R : 0;
        S->band_K = K;
    }
    return PF2_OK;
}

static Csr csr_of(const pf2_csr* A) {
    return Csr{ A->n, A->mesh->rowptr.p, A->mesh->col.p, A->val.p, A->mesh->diag.p };
}

static Tri tri_of(pf2_solver* S) {
    auto dir = [&](BandHost& H) {
        return BandDir{ H.rstep.p, H.sptr.p, H.row.p, H.rhs.p, H.dep.p, H.val.p, H.dinv.p, H.val32.p, H.dinv32.p,
                        H.ngroups, H.gstart.p };
    };
    const Band band{ S->band_P, S->band_R, S->band_K, S->band_rs.p, dir(S->band[0]), dir(S->band[1]) };
    return Tri{ S->opt.precond, band, Csr{ S->n, S->brp.p, S->bcol.p, nullptr, S->bdiag.p }, S->perm.p, S->iperm.p,
                S->fwd_order.p, S->bwd_order.p, S->lt_off.p, S->lt_row.p, S->lt_pos.p, S->fact.p, S->tmp.p,
                S->outB.p, S->fact32.p, S->tmp32.p, S->outB32.p, S->done_f.p, S->done_b.p, S->tickets.p,
                S->rec.p, S->csr ? 1 : 0, S->bval.p, S->fsym.p, S->xB.p, S->bval32.p, S->fsym32.p, S->ngroups,
                S->cstart.p };
}

static bool uses_tri(const pf2_solver* S) {
    return S->opt.precond == PF2_PRECOND_ILU || S->opt.precond == PF2_PRECOND_IC;
}

// Preconditioner::initialize(A): ILU/IC factorise a copy of A's values.
__global__ void k_epoch_advance(int* epoch, int delta) { *epoch += delta; }

// out[k] = val[map[k]] (0 where map[k] < 0).
__global__ void k_gather_values(long long nnz, const double* __restrict__ val, const int* __restrict__ map,
                                double* __restrict__ out) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nnz; k += (long long)gridDim.x * blockDim.x) {
        const int m = map[k];
        out[k] = m >= 0 ? val[m] : 0.0;
    }
}

__global__ void k_inv_diag(int n, const double* __restrict__ val, const int* __restrict__ diag, double* invd) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) invd[i] = 1.0 / val[diag[i]];
}

// Factor values and inverse diagonals of the banded plan's slots (after a factorisation).
__global__ void k_band_values(long long nk, int n, const int* __restrict__ pos, const int* __restrict__ dpos,
                              const double* __restrict__ fact, double* val, double* dinv, float* val32,
                              float* dinv32) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nk; q += stride) {
        const int p = pos[q];
        const double v = p >= 0 ? fact[p] : 0.0;
        val[q] = v;
        if (val32) val32[q] = (float)v;
    }
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += stride) {
        const int d = dpos[t];
        dinv[t] = d >= 0 ? 1.0 / fact[d] : 1.0;
        if (dinv32) dinv32[t] = d >= 0 ? 1.0f / (float)fact[d] : 1.0f;
    }
}

// The factors on B's pattern for the CSR sweeps (pf2_solver::tpos).
__global__ void k_fsym(long long nnz, const int* __restrict__ tpos, const double* __restrict__ fact, double* fsym) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nnz; k += (long long)gridDim.x * blockDim.x) {
        const int t = tpos[k];
        fsym[k] = t >= 0 ? fact[t] : 1.0 / fact[-1 - t];
    }
}

static pf2_status factorize(pf2_solver* S, const pf2_csr* A, cudaStream_t st) {
    S->last = A;
    const bool mixed = S->opt.precision == PF2_PRECISION_MIXED;
    if (mixed) {
        k_to_float<<<std::min((int)blocks_for(S->nnz), num_sms() * 8), kThreads, 0, st>>>(S->nnz, A->val.p,
                                                                                        S->val32.p);
        PF2_LAUNCH_CHECK();
    }
    if (S->opt.precond == PF2_PRECOND_JACOBI) {
        k_inv_diag<<<blocks_for(S->n), kThreads, 0, st>>>(S->n, A->val.p, A->mesh->diag.p, S->invd.p);
        PF2_LAUNCH_CHECK();
        return PF2_OK;
    }
    if (!uses_tri(S)) return PF2_OK;
    // (partition-local factors: the entries coupling two parts factor as zeros)
    k_gather_values<<<std::min((int)blocks_for(S->nnz), num_sms() * 8), kThreads, 0, st>>>(
        S->nnz, A->val.p, S->part_local ? S->bmap_local.p : S->bmap.p, S->fact.p);
    PF2_LAUNCH_CHECK();
    PF2_CUDA(cudaMemsetAsync(S->tickets.p, 0, sizeof(unsigned), st));
    PF2_CUDA(cudaMemsetAsync(S->err.p, 0, sizeof(int), st));
    PF2_CUDA(cudaMemsetAsync(S->rec.p, 0, 5 * sizeof(int), st));
    Tri T = tri_of(S);
    const int nb = std::min(num_sms() * 8, (int)blocks_for(S->n, kSolverThreads / 32));
    k_factor<<<std::max(nb, 1), kSolverThreads, 0, st>>>(T, S->fwd_order.p, S->tickets.p, S->epoch.p, S->err.p);
    PF2_LAUNCH_CHECK();
    k_epoch_advance<<<1, 1, 0, st>>>(S->epoch.p, 1);
    PF2_LAUNCH_CHECK();
    if (S->band_K) {
        const long long nk = (long long)S->n * S->band_K;
        for (BandHost& H : S->band) {
            k_band_values<<<std::min((int)blocks_for(nk), num_sms() * 8), kThreads, 0, st>>>(
                nk, S->n, H.pos.p, H.dpos.p, S->fact.p, H.val.p, H.dinv.p, H.val32.p, H.dinv32.p);
            PF2_LAUNCH_CHECK();
        }
    }
    if (S->csr) {
        k_fsym<<<std::min((int)blocks_for(S->nnz), num_sms() * 8), kThreads, 0, st>>>(S->nnz, S->tpos.p, S->fact.p,
                                                                                    S->fsym.p);
        PF2_LAUNCH_CHECK();
        if (S->part) {
            k_gather_values<<<std::min((int)blocks_for(S->nnz), num_sms() * 8), kThreads, 0, st>>>(
                S->nnz, S->fsym.p, S->q_fmap.p, S->q_f.p);
            PF2_LAUNCH_CHECK();
            if (S->q_f32.p) {
                k_to_float<<<std::min((int)blocks_for(S->nnz), num_sms() * 8), kThreads, 0, st>>>(S->nnz, S->q_f.p,
                                                                                                S->q_f32.p);
                PF2_LAUNCH_CHECK();
            }
        }
        if (mixed) {
            k_to_float<<<std::min((int)blocks_for(S->nnz), num_sms() * 8), kThreads, 0, st>>>(S->nnz, S->fsym.p,
                                                                                            S->fsym32.p);
            PF2_LAUNCH_CHECK();
        }
    }
    if (mixed) {
        k_to_float<<<std::min((int)blocks_for(S->nnz), num_sms() * 8), kThreads, 0, st>>>(S->nnz, S->fact.p,
                                                                                        S->fact32.p);
        PF2_LAUNCH_CHECK();
    }
    S->factored = true;
    return PF2_OK;
}

// Upper bound of the preconditioner applies of one solve (each uses two tickets and two
// row-flag epochs): CG one per iteration plus the first; mixed CG one per inner
// iteration plus one per refinement; GMRES one per iteration plus two per restart.
static int max_applies(const pf2_solver* S) {
    const int it = S->opt.max_iterations;
    if (S->opt.kind == PF2_SOLVER_GMRES) return it + 2 * (it / std::max(S->m, 1)) + 4;
    if (S->opt.precision == PF2_PRECISION_MIXED) return it + kMaxOuter + 2;
    return it + 2;
}

// The kernel of a solve: GMRES, mixed CG, the one-reduction CG with a local (Jacobi or
// no) preconditioner, k_pcg_csr (ILU/IC on B's CSR arrays, either variant) or k_pcg (the
// standard iteration otherwise).
static void* solve_kernel(const pf2_solver_options& o, bool csr) {
    if (o.kind == PF2_SOLVER_GMRES) return (void*)k_gmres;
    if (o.kind == PF2_SOLVER_BICGSTAB) return (void*)k_bicgstab;
    if (o.precision == PF2_PRECISION_MIXED) return (void*)k_pcg_mixed;
    const bool tri = o.precond == PF2_PRECOND_ILU || o.precond == PF2_PRECOND_IC;
    if (o.cg_variant == PF2_CG_ONE_REDUCTION && !tri) return (void*)k_pcg_one;
    if (tri && csr) return (void*)k_pcg_csr;
    return (void*)k_pcg;
}

// The pipelined CG kernel: PF2_PIPE_W=1/2/4 picks the rows its update pass walks together
// (tuning; 2 measured fastest at 1M rows)
static void* pipe_kernel() {
    int w = 2;
    if (const char* e = getenv("PF2_PIPE_W")) w = atoi(e);
    return w >= 4 ? (void*)k_pcg_pipe<4> : w == 2 ? (void*)k_pcg_pipe<2> : (void*)k_pcg_pipe<1>;
}

static pf2_status launch_solver(pf2_solver* S, const pf2_csr* A, double* x, const double* b, cudaStream_t st,
                                bool precond_only = false) {
    KArgs a{};
    a.A = csr_of(A ? A : S->last);
    a.precond = S->opt.precond;
    a.x = x;
    a.b = b;
    a.r = S->r.p;
    a.z = S->z.p;
    a.p = S->p.p;
    a.q = S->q.p;
    a.s = S->s.p;
    a.pipe = S->pipe.p;
    a.variant = S->opt.cg_variant;
    a.rhat = S->rhat.p;
    a.y = S->yv.p;
    a.t = S->tv.p;
    a.invd = S->invd.p;
    a.partial = S->partial.p;
    a.bar = GridBarrier{ S->bar.p, S->err.p, S->partial.p, S->rec.p, S->barrier_polls };
    a.T = tri_of(S);
    a.tol = S->opt.tolerance;
    a.maxit = S->opt.max_iterations;
    a.criterion = S->opt.criterion;
    a.out = S->out.p;
    a.V = S->V.p;
    a.H = S->H.p;
    a.m = S->m;
    a.gs = S->opt.orthogonalization;
    a.vpart = S->vpart.p;
    a.vtot = S->vpart.p ? S->vpart.p + (size_t)(S->m + 1) * S->blocks : nullptr;
    const bool mixed = S->opt.precision == PF2_PRECISION_MIXED && !precond_only;
    // CSR paths: the direction update inside the SpMV (saves a barrier, gathers z and p);
    // PF2_CG_FUSED_P=0/1 overrides the default (tuning)
    a.fuse_p = mixed && S->opt.precond != PF2_PRECOND_IC ? 1 : 0;
    if (const char* e = getenv("PF2_CG_FUSED_P")) a.fuse_p = atoi(e) != 0;
    if (mixed) {
        a.val32 = S->val32.p;
        a.d32 = S->d32.p;
        a.r32 = S->r32.p;
        a.p32 = S->p32.p;
        a.q32 = S->q32.p;
        a.z32 = S->z32.p;
        a.invd32 = S->invd32.p;
        a.p32b = S->p32b.p;
        a.inner_eta = kMixedInnerEta;
        if (const char* e = getenv("PF2_MIXED_INNER_ETA")) a.inner_eta = std::max(1e-12, atof(e));  // tuning
        a.max_outer = kMaxOuter;
    }
    const int applies = max_applies(S);
    if (S->part && !precond_only) {
        // A's values in Q order for this solve's matrix; t and z start as pending markers
        k_gather_values<<<std::min((int)blocks_for(S->nnz), num_sms() * 8), kThreads, 0, st>>>(
            S->nnz, a.A.val, S->q_amap.p, S->q_val.p);
        PF2_LAUNCH_CHECK();
        if (uses_tri(S)) {
            PF2_CUDA(cudaMemsetAsync(S->q_gt.p, 0xff, S->q_gt.bytes(), st));
            PF2_CUDA(cudaMemsetAsync(S->q_gz.p, 0xff, S->q_gz.bytes(), st));
        }
        if (S->q_val32.p) {
            k_to_float<<<std::min((int)blocks_for(S->nnz), num_sms() * 8), kThreads, 0, st>>>(S->nnz, S->q_val.p,
                                                                                            S->q_val32.p);
            PF2_LAUNCH_CHECK();
            PF2_CUDA(cudaMemsetAsync(S->q_gt32.p, 0xff, S->q_gt32.bytes(), st));
            PF2_CUDA(cudaMemsetAsync(S->q_gz32.p, 0xff, S->q_gz32.bytes(), st));
        }
        a.part = PartCg{ S->part_P, S->part_R, S->part_ng, S->q_s.p, S->q_rp.p, S->q_col.p, S->q_diag.p, S->q_a.p,
                         S->q_bnd.p, S->q_val.p, S->q_f.p, S->q_x.p, S->q_gp.p, S->q_gt.p, S->q_gz.p,
                         S->q_val32.p, S->q_f32.p, S->q_gp32.p, S->q_gt32.p, S->q_gz32.p };
        PF2_CUDA(cudaMemsetAsync(S->bar.p, 0, 2 * sizeof(unsigned), st));
        PF2_CUDA(cudaMemsetAsync(S->err.p, 0, sizeof(int), st));
        PF2_CUDA(cudaMemsetAsync(S->rec.p, 0, 5 * sizeof(int), st));
        void* args[] = { &a };
        PF2_COOP_LAUNCH(part_kernel(S), dim3(S->part_P), dim3(kPartThreads), args, S->part_smem, st);
        return PF2_OK;
    }
    if (S->csr && !precond_only) {  // A's values in B's numbering, for this solve's matrix
        k_gather_values<<<std::min((int)blocks_for(S->nnz), num_sms() * 8), kThreads, 0, st>>>(
            S->nnz, a.A.val, S->bmap.p, S->bval.p);
        PF2_LAUNCH_CHECK();
        if (mixed) {
            k_to_float<<<std::min((int)blocks_for(S->nnz), num_sms() * 8), kThreads, 0, st>>>(S->nnz, S->bval.p,
                                                                                            S->bval32.p);
            PF2_LAUNCH_CHECK();
        }
    }
    if (uses_tri(S)) {
        PF2_CUDA(cudaMemsetAsync(S->tickets.p, 0, sizeof(unsigned) * S->tickets.n, st));
        // triangular-solve vectors start as "pending" (all bits set)
        PF2_CUDA(cudaMemsetAsync(S->tmp.p, 0xff, S->tmp.bytes(), st));
        PF2_CUDA(cudaMemsetAsync(S->outB.p, 0xff, S->outB.bytes(), st));
        if (S->tmp32.p) {
            PF2_CUDA(cudaMemsetAsync(S->tmp32.p, 0xff, S->tmp32.bytes(), st));
            PF2_CUDA(cudaMemsetAsync(S->outB32.p, 0xff, S->outB32.bytes(), st));
        }
        a.epoch = S->epoch.p;
    }
    PF2_CUDA(cudaMemsetAsync(S->bar.p, 0, 2 * sizeof(unsigned), st));
    PF2_CUDA(cudaMemsetAsync(S->err.p, 0, sizeof(int), st));
    PF2_CUDA(cudaMemsetAsync(S->rec.p, 0, 5 * sizeof(int), st));
    void* args[] = { &a };
    if (precond_only) {
        PF2_COOP_LAUNCH((void*)k_precond_apply, dim3(S->blocks), dim3(kSolverThreads), args, S->smem, st);
        if (uses_tri(S)) {
            k_epoch_advance<<<1, 1, 0, st>>>(S->epoch.p, 4);
            PF2_LAUNCH_CHECK();
        }
        return PF2_OK;
    }
    void* fn = mixed ? (void*)k_pcg_mixed : solve_kernel(S->opt, S->csr);
    // pipelined CG on B's CSR arrays (ILU(0)/IC(0) on a few-level order); the standard
    // iteration elsewhere
    if (!mixed && S->opt.kind == PF2_SOLVER_CG && S->opt.cg_variant == PF2_CG_PIPELINED && S->csr)
        fn = pipe_kernel();
    PF2_COOP_LAUNCH(fn, dim3(S->blocks), dim3(kSolverThreads), args, S->smem, st);
    if (uses_tri(S)) {
        k_epoch_advance<<<1, 1, 0, st>>>(S->epoch.p, 2 * applies + 2);
        PF2_LAUNCH_CHECK();
    }
    return PF2_OK;
}

// The partitioned CG plan of a Jacobi / no-preconditioner solve: B = A, one group.
static pf2_status build_part_plan_local(pf2_solver* S) {
    const pf2_mesh* M = S->mesh;
    const int n = S->n, nnz = S->nnz;
    std::vector<int> rp(n + 1), col(nnz), dg(n), ident(n), kmap(nnz);
    PF2_CUDA(cudaMemcpy(rp.data(), M->rowptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
    PF2_CUDA(cudaMemcpy(col.data(), M->col.p, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
    PF2_CUDA(cudaMemcpy(dg.data(), M->diag.p, sizeof(int) * n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i) ident[i] = i;
    for (int k = 0; k < nnz; ++k) kmap[k] = k;
    const std::vector<int> groups{ 0, n };
    return build_part_plan(S, rp, col, rp, col, kmap, dg, ident, groups, false);
}

extern "C" {

pf2_status pf2_multicolour_order(int n, const int* rowptr, const int* col, int kempe, int* perm, int* ncolours,
                                 int* nstarts, int* starts) {
    PF2_REQUIRE(n > 0 && rowptr && col && perm && ncolours && nstarts, PF2_BAD_INPUT, "null argument");
    for (int i = 0; i < n; ++i)
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
            PF2_REQUIRE(col[k] >= 0 && col[k] < n, PF2_BAD_INPUT, "column %d of row %d out of range", col[k], i);
    std::vector<int> p, groups;
    *ncolours = multicolour_order(n, rowptr, col, kempe != 0, p, groups);
    std::copy(p.begin(), p.end(), perm);
    *nstarts = (int)groups.size();
    if (starts) std::copy(groups.begin(), groups.end(), starts);
    return PF2_OK;
}

pf2_status pf2_graph_parts(int n, const int* rowptr, const int* col, int parts, int* part) {
    PF2_REQUIRE(n > 0 && rowptr && col && part, PF2_BAD_INPUT, "null argument");
    PF2_REQUIRE(parts >= 1, PF2_BAD_INPUT, "parts %d < 1", parts);
    for (int i = 0; i < n; ++i)
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
            PF2_REQUIRE(col[k] >= 0 && col[k] < n, PF2_BAD_INPUT, "column %d of row %d out of range", col[k], i);
    std::vector<int> p;
    graph_parts(n, std::vector<int>(rowptr, rowptr + n + 1), std::vector<int>(col, col + rowptr[n]), parts, p);
    std::copy(p.begin(), p.end(), part);
    return PF2_OK;
}

pf2_status pf2_solver_create(const pf2_csr* A, const pf2_solver_options* opt, pf2_solver** out) {
    PF2_REQUIRE(A && opt && out, PF2_BAD_INPUT, "null argument");
    *out = nullptr;
    PF2_REQUIRE(opt->kind == PF2_SOLVER_CG || opt->kind == PF2_SOLVER_GMRES || opt->kind == PF2_SOLVER_BICGSTAB,
                PF2_BAD_INPUT, "unknown solver kind %d", opt->kind);
    PF2_REQUIRE(opt->kind != PF2_SOLVER_BICGSTAB ||
                    (opt->precond != PF2_PRECOND_ILU && opt->precond != PF2_PRECOND_IC &&
                     opt->precision == PF2_PRECISION_FP64),
                PF2_BAD_INPUT, "BiCGStab takes the Jacobi or no preconditioner, in FP64");
    PF2_REQUIRE(opt->precond >= PF2_PRECOND_NONE && opt->precond <= PF2_PRECOND_IC, PF2_BAD_INPUT,
                "unknown preconditioner %d", opt->precond);
    PF2_REQUIRE(opt->max_iterations >= 0 && opt->tolerance >= 0, PF2_BAD_INPUT, "bad tolerance or iteration limit");
    PF2_REQUIRE(opt->ordering == PF2_ORDERING_NATURAL || opt->ordering == PF2_ORDERING_MULTICOLOR, PF2_BAD_INPUT,
                "unknown ordering %d", opt->ordering);
    PF2_REQUIRE(opt->orthogonalization == PF2_GS_MODIFIED || opt->orthogonalization == PF2_GS_CLASSICAL_TWICE,
                PF2_BAD_INPUT, "unknown orthogonalization %d", opt->orthogonalization);
    PF2_REQUIRE(opt->cg_variant == PF2_CG_STANDARD || opt->cg_variant == PF2_CG_ONE_REDUCTION ||
                    opt->cg_variant == PF2_CG_PIPELINED,
                PF2_BAD_INPUT,
                "unknown CG variant %d", opt->cg_variant);
    PF2_REQUIRE(opt->precision == PF2_PRECISION_FP64 || (opt->precision == PF2_PRECISION_MIXED && opt->kind == PF2_SOLVER_CG),
                PF2_BAD_INPUT, "unknown precision %d for this solver", opt->precision);
    pf2_solver* S = new pf2_solver();
    S->opt = *opt;
    S->mesh = A->mesh;
    S->n = A->n;
    S->nnz = A->nnz;
    auto fail = [&](pf2_status s) { delete S; return s; };
    // SolverGMRES::init clamps the iteration limit to the matrix size (linear_solver.cu:396-399)
    if (opt->kind == PF2_SOLVER_GMRES && S->opt.max_iterations > S->n) S->opt.max_iterations = S->n;
    int occ = 0;
    pf2_status s;
    const bool mixed = opt->precision == PF2_PRECISION_MIXED;
    if (uses_tri(S) && (s = build_tri_plan(S))) return fail(s);
    if (!uses_tri(S) && part_eligible(S) && (s = build_part_plan_local(S))) return fail(s);
    if (S->part) {
        int occ_p = 0;
        void* pf = part_kernel(S);
        if (cudaFuncSetAttribute(pf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S->part_smem) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_p, pf, kPartThreads, S->part_smem) != cudaSuccess)
            return fail(cuda_fail(cudaGetLastError(), "partitioned CG attributes", __FILE__, __LINE__));
        if (occ_p < 1) {  // the other kernels then
            S->part = false;
            S->part_why = "no block of the partitioned kernel fits on an SM";
        }
    }
    // PF2_CG_PART=2 (tests): require the partitioned kernel
    if (const char* e = getenv("PF2_CG_PART"))
        if (atoi(e) == 2 && !S->part) {
            set_error("the partitioned CG kernel does not apply: %s", part_eligible(S) ? S->part_why :
                      "solver kind, variant, precision or preconditioner");
            return fail(PF2_BAD_INPUT);
        }
    // the banded triangular solve keeps a range of the solution in shared memory
    S->smem = S->band_P ? sizeof(double) * (size_t)S->band_R : 0;
    void* fn = solve_kernel(*opt, S->csr);
    if (S->smem) {
        if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S->smem) != cudaSuccess ||
            cudaFuncSetAttribute((void*)k_precond_apply, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)S->smem) != cudaSuccess)
            return fail(cuda_fail(cudaGetLastError(), "shared-memory attribute", __FILE__, __LINE__));
    }
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kSolverThreads, S->smem) != cudaSuccess || occ < 1)
        return fail(cuda_fail(cudaGetLastError(), "occupancy query", __FILE__, __LINE__));
    int occ_pc = occ;
    if (uses_tri(S) &&
        (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_pc, (void*)k_precond_apply, kSolverThreads, S->smem) !=
             cudaSuccess ||
         occ_pc < 1))
        return fail(cuda_fail(cudaGetLastError(), "occupancy query", __FILE__, __LINE__));
    // blocks per SM: fewer blocks make cheaper grid barriers (one arrival atomic per block);
    // PF2_SOLVER_BLOCKS_PER_SM overrides the default of kSolverBlocksPerSm (tuning)
    int bps = kSolverBlocksPerSm;
    // tests: a short grid-barrier poll limit, so that a bounded wait runs out and the
    // solve returns PF2_TIMEOUT with the place it gave up
    if (const char* e = getenv("PF2_BARRIER_POLLS")) S->barrier_polls = std::max(1LL, atoll(e));
    if (const char* e = getenv("PF2_SOLVER_BLOCKS_PER_SM")) bps = std::max(1, atoi(e));
    if (opt->kind == PF2_SOLVER_CG && opt->cg_variant == PF2_CG_PIPELINED) {
        int occ_pp = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_pp, pipe_kernel(), kSolverThreads, S->smem) !=
                cudaSuccess ||
            occ_pp < 1)
            return fail(cuda_fail(cudaGetLastError(), "occupancy query", __FILE__, __LINE__));
        occ = std::min(occ, occ_pp);
    }
    const int maxb = std::min(std::min(occ, occ_pc), bps) * num_sms();
    // at least ~512 rows per block keeps the barrier count per unit of work low
    S->blocks = std::max(1, std::min(maxb, (int)((S->n + 511) / 512)));
    if ((s = S->r.alloc(S->n)) || (s = S->z.alloc(S->n)) || (s = S->p.alloc(S->n)) || (s = S->q.alloc(S->n)) ||
        (opt->kind == PF2_SOLVER_CG && (s = S->s.alloc(S->n))) ||
        (opt->kind == PF2_SOLVER_CG && opt->cg_variant == PF2_CG_PIPELINED && (s = S->pipe.alloc(6 * S->n))) ||
        (opt->kind == PF2_SOLVER_BICGSTAB && ((s = S->s.alloc(S->n)) || (s = S->rhat.alloc(S->n)) ||
                                               (s = S->yv.alloc(S->n)) || (s = S->tv.alloc(S->n)))) ||
        (s = S->invd.alloc(S->n)) || (s = S->partial.alloc(8 * (size_t)std::max(S->blocks, S->part_P))) || (s = S->bar.alloc(2)) ||
        (s = S->err.alloc(1)) || (s = S->rec.alloc(5)) || (s = S->out.alloc(1)) || (s = S->h_out.alloc(1)))
        return fail(s);
    if (mixed && ((s = S->val32.alloc(S->nnz)) || (s = S->d32.alloc(S->n)) || (s = S->r32.alloc(S->n)) ||
                  (s = S->p32.alloc(S->n)) || (s = S->q32.alloc(S->n)) || (s = S->z32.alloc(S->n)) ||
                  (s = S->invd32.alloc(S->n)) || (s = S->p32b.alloc(S->n))))
        return fail(s);
    if (opt->kind == PF2_SOLVER_GMRES) {
        int m = opt->restart > 0 ? opt->restart : S->opt.max_iterations;
        m = std::max(1, std::min(m, std::min(S->opt.max_iterations, kMaxGmresSmem - 1)));
        S->m = m;
        if ((s = S->V.alloc((size_t)(m + 1) * S->n)) || (s = S->H.alloc((size_t)m * m))) return fail(s);
        if (opt->orthogonalization == PF2_GS_CLASSICAL_TWICE &&
            (s = S->vpart.alloc((size_t)(m + 1) * (S->blocks + 1))))
            return fail(s);
    }
    if (uses_tri(S)) {
        if ((s = S->tickets.alloc(2 * (size_t)max_applies(S) + 2))) return fail(s);
        if (mixed && ((s = S->fact32.alloc(S->nnz)) || (s = S->tmp32.alloc(S->n)) || (s = S->outB32.alloc(S->n))))
            return fail(s);
    }
    *out = S;
    return PF2_OK;
}

pf2_status pf2_solver_destroy(pf2_solver* s) {
    delete s;
    return PF2_OK;
}

pf2_status pf2_solver_setup(pf2_solver* S, const pf2_csr* A, void* stream) {
    PF2_REQUIRE(S && A, PF2_BAD_INPUT, "null argument");
    PF2_REQUIRE(A->mesh == S->mesh, PF2_BAD_INPUT, "matrix pattern differs from the solver's");
    return factorize(S, A, as_stream(stream));
}

}  // extern "C"

namespace pf2 {

__global__ void k_record(const SolveOut* out, const int* err, SolveRecord* rec) {
    rec->iterations = out->iterations;
    rec->converged = out->converged;
    rec->residual = out->residual;
    rec->relres = out->relres;
    rec->status = out->status;
    rec->err = *err;
}

pf2_status solver_solve_async(pf2_solver* S, const pf2_csr* A, double* x, const double* b, SolveRecord* rec,
                              cudaStream_t st, bool refactor) {
    if (refactor || S->last != A) PF2_TRY(factorize(S, A, st));
    PF2_TRY(launch_solver(S, A, x, b, st));
    if (rec) {
        k_record<<<1, 1, 0, st>>>(S->out.p, S->err.p, rec);
        PF2_LAUNCH_CHECK();
    }
    return PF2_OK;
}

}  // namespace pf2

extern "C" {

pf2_status pf2_solver_solve(pf2_solver* S, const pf2_csr* A, double* x, const double* b, pf2_solve_info* info,
                            void* stream) {
    PF2_REQUIRE(S && A && x && b, PF2_BAD_INPUT, "null argument");
    PF2_REQUIRE(A->mesh == S->mesh, PF2_BAD_INPUT, "matrix pattern differs from the solver's");
    cudaStream_t st = as_stream(stream);
    PF2_TRY(factorize(S, A, st));
    PF2_TRY(launch_solver(S, A, x, b, st));
    if (!info) return PF2_OK;
    int err = 0, rec[5] = { 0, 0, 0, 0, 0 };
    PF2_CUDA(cudaMemcpyAsync(S->h_out.p, S->out.p, sizeof(SolveOut), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaMemcpyAsync(&err, S->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaMemcpyAsync(rec, S->rec.p, sizeof(rec), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaStreamSynchronize(st));
    info->iterations = S->h_out.p->iterations;
    info->converged = S->h_out.p->converged;
    info->residual = S->h_out.p->residual;
    info->outer_iterations = S->opt.precision == PF2_PRECISION_MIXED ? S->h_out.p->pad : 1;
    info->status = err ? err : S->h_out.p->status;
    PF2_REQUIRE(err == 0, (pf2_status)err,
                rec[0] == 1   ? "grid barrier timed out in the solver (block %d, barrier %d, arrivals %d)"
                : rec[0] == 2 ? "row wait timed out in the solver (row %d waited for row %d, epoch %d, flag %d)"
                              : "device-side wait timed out in the solver",
                rec[1], rec[2], rec[3], rec[4]);
    if (!info->converged) {
        set_error("solver did not converge in %d iterations (residual %g)", info->iterations, info->residual);
        return PF2_NOT_CONVERGED;
    }
    return PF2_OK;
}

pf2_status pf2_precond_apply(pf2_solver* S, double* dst, const double* src, void* stream) {
    PF2_REQUIRE(S && dst && src, PF2_BAD_INPUT, "null argument");
    cudaStream_t st = as_stream(stream);
    if (S->opt.precond == PF2_PRECOND_NONE) {
        PF2_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * S->n, cudaMemcpyDeviceToDevice, st));
        return PF2_OK;
    }
    PF2_REQUIRE(S->last && (S->factored || S->opt.precond == PF2_PRECOND_JACOBI), PF2_BAD_INPUT,
                "preconditioner not initialised: call pf2_solver_setup or pf2_solver_solve first");
    PF2_CUDA(cudaMemcpyAsync(S->r.p, src, sizeof(double) * S->n, cudaMemcpyDeviceToDevice, st));
    PF2_TRY(launch_solver(S, nullptr, nullptr, nullptr, st, true));
    PF2_CUDA(cudaMemcpyAsync(dst, S->z.p, sizeof(double) * S->n, cudaMemcpyDeviceToDevice, st));
    return PF2_OK;
}

pf2_status pf2_spmv(const pf2_csr* A, const double* x, double* y, void* stream) {
    PF2_REQUIRE(A && x && y, PF2_BAD_INPUT, "null argument");
    const int blocks = std::min((int)blocks_for((long long)A->n), num_sms() * 8);
    k_spmv<<<std::max(blocks, 1), kThreads, 0, as_stream(stream)>>>(csr_of(A), x, y);
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

}  // extern "C"

// ------------------------------------------------- allocation-free Jacobi-PCG
namespace pf2 {

constexpr int kStaticMaxRows = PF2_STATIC_MAX_ROWS;
constexpr int kStaticMaxBlocks = 512;
// r, z, p, q and the inverse diagonal (kStaticMaxRows each), 2 x 4 partial sums per block,
// the solve record (4 doubles)
constexpr size_t kStaticDoubles = 5ull * kStaticMaxRows + 8ull * kStaticMaxBlocks + 4;
static __device__ __align__(256) double g_static_work[kStaticDoubles];
// barrier count, (unused), error word, timeout record (5): all zeroed per call
static __device__ __align__(256) unsigned g_static_words[8];

struct StaticWork {
    double* work = nullptr;
    unsigned* words = nullptr;
};
static std::mutex g_static_mu;
static StaticWork g_static[64];  // per device ordinal

static pf2_status static_work(StaticWork& out) {
    int dev = 0;
    PF2_CUDA(cudaGetDevice(&dev));
    PF2_REQUIRE(dev >= 0 && dev < 64, PF2_BAD_INPUT, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_static_mu);
    StaticWork& w = g_static[dev];
    if (!w.work) {
        void* p = nullptr;
        void* q = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_work);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(work)", __FILE__, __LINE__);
        e = cudaGetSymbolAddress(&q, g_static_words);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(words)", __FILE__, __LINE__);
        w.work = static_cast<double*>(p);
        w.words = static_cast<unsigned*>(q);
    }
    out = w;
    return PF2_OK;
}

}  // namespace pf2

extern "C" pf2_status pf2_pcg_jacobi_static(const pf2_csr* A, double* x, const double* b, double tolerance,
                                            int max_iterations, int criterion, pf2_solve_info* info,
                                            void* stream) {
    PF2_REQUIRE(A && x && b, PF2_BAD_INPUT, "null argument");
    PF2_REQUIRE(A->n <= kStaticMaxRows, PF2_BAD_INPUT,
                "pf2_pcg_jacobi_static: %d rows exceed its static work storage (%d rows); use pf2_solver_create",
                A->n, kStaticMaxRows);
    PF2_REQUIRE(max_iterations >= 0 && tolerance >= 0, PF2_BAD_INPUT, "bad tolerance or iteration limit");
    PF2_REQUIRE(criterion == PF2_CRITERION_ABS || criterion == PF2_CRITERION_REL, PF2_BAD_INPUT,
                "unknown criterion %d", criterion);
    StaticWork w;
    PF2_TRY(static_work(w));
    cudaStream_t st = as_stream(stream);
    // the block count of a pf2_solver_create Jacobi-CG solver (same partition, same bits)
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (void*)k_pcg, kSolverThreads, 0) != cudaSuccess ||
        occ < 1)
        return cuda_fail(cudaGetLastError(), "occupancy query", __FILE__, __LINE__);
    int bps = kSolverBlocksPerSm;
    if (const char* e = getenv("PF2_SOLVER_BLOCKS_PER_SM")) bps = std::max(1, atoi(e));
    const int maxb = std::min(occ, bps) * num_sms();
    const int blocks = std::max(1, std::min(std::min(maxb, kStaticMaxBlocks), (A->n + 511) / 512));
    double* base = w.work;
    KArgs a{};
    a.A = csr_of(A);
    a.precond = PF2_PRECOND_JACOBI;
    a.x = x;
    a.b = b;
    a.r = base;
    a.z = base + (size_t)kStaticMaxRows;
    a.p = base + 2 * (size_t)kStaticMaxRows;
    a.q = base + 3 * (size_t)kStaticMaxRows;
    a.invd = base + 4 * (size_t)kStaticMaxRows;
    a.partial = base + 5 * (size_t)kStaticMaxRows;
    int* err = reinterpret_cast<int*>(w.words + 2);
    a.bar = GridBarrier{ w.words, err, a.partial, reinterpret_cast<int*>(w.words + 3), 0 };
    a.tol = tolerance;
    a.maxit = max_iterations;
    a.criterion = criterion;
    a.out = reinterpret_cast<SolveOut*>(base + 5 * (size_t)kStaticMaxRows + 8 * (size_t)kStaticMaxBlocks);
    PF2_CUDA(cudaMemsetAsync(w.words, 0, 8 * sizeof(unsigned), st));
    // the solve record of the previous call must not stand in for this one's: a kernel
    // that gives up on a wait returns before writing it
    PF2_CUDA(cudaMemsetAsync(a.out, 0, sizeof(SolveOut), st));
    void* args[] = { &a };
    PF2_COOP_LAUNCH((void*)k_pcg, dim3(blocks), dim3(kSolverThreads), args, 0, st);
    if (!info) return PF2_OK;
    SolveOut o{};
    int e = 0, rec[5] = { 0, 0, 0, 0, 0 };
    PF2_CUDA(cudaMemcpyAsync(&o, a.out, sizeof(SolveOut), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaMemcpyAsync(rec, w.words + 3, sizeof(rec), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaStreamSynchronize(st));
    info->iterations = o.iterations;
    info->converged = o.converged;
    info->residual = o.residual;
    info->outer_iterations = 1;
    info->status = e ? e : o.status;
    PF2_REQUIRE(e == 0, (pf2_status)e,
                rec[0] == 1 ? "grid barrier timed out in the solver (block %d, barrier %d, arrivals %d)"
                            : "device-side wait timed out in the solver",
                rec[1], rec[2], rec[3]);
    if (!info->converged) {
        set_error("solver did not converge in %d iterations (residual %g)", info->iterations, info->residual);
        return PF2_NOT_CONVERGED;
    }
    return PF2_OK;
}
