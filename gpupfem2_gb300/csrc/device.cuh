// device.cuh - device helpers shared by the kernels.
//
// Arithmetic whose result must match the reference bit for bit (cell geometry,
// global->local transforms, advection, interpolation) is written with explicit
// __fma_rn/__dmul_rn/__dadd_rn/__dsub_rn/__ddiv_rn intrinsics, which the compiler never
// re-associates or fuses, at exactly the places where nvcc contracts the reference's
// expressions into fused multiply-adds.  The CPU oracle calls fma() at the same places.
#pragma once

#include <type_traits>
#include <cuda_runtime.h>

#include "common.cuh"

namespace pf2 {

// Sorts buf[0, m) ascending in place and drops repeats; returns the unique count.
__device__ __forceinline__ int sort_unique(int* buf, int m) {
    for (int a = 1; a < m; ++a) {
        const int x = buf[a];
        int b = a - 1;
        while (b >= 0 && buf[b] > x) { buf[b + 1] = buf[b]; --b; }
        buf[b + 1] = x;
    }
    int u = 0;
    for (int q = 0; q < m; ++q)
        if (q == 0 || buf[q] != buf[q - 1]) buf[u++] = buf[q];
    return u;
}

// Row-major invJ {d0, d1, d2, d3}.  shapeFuncGrad(i) mapped by invJ
// (numerical_integrator_2d.cuh:8-20 with Matrix2x2::operator*, cuda_math.cuh:146-153):
// grad N0 = (d0, d2), grad N1 = (d1, d3), grad N2 = (-d0 - d1, -d2 - d3).
__device__ __forceinline__ void shape_grads(const double4_32a J, double2 g[3]) {
    g[0] = make_double2(J.x, J.z);
    g[1] = make_double2(J.y, J.w);
    g[2] = make_double2(__dsub_rn(-J.x, J.y), __dsub_rn(-J.z, J.w));
}

// GEOMETRY::transformGlobalToLocal (geometry.cuh:14-23)
__device__ __forceinline__ void global_to_local(double x, double y, const double4_32a J, const double2 v3, double& l0,
                                                double& l1, double& l2) {
    const double dx = __dsub_rn(x, v3.x), dy = __dsub_rn(y, v3.y);
    l0 = __fma_rn(J.x, dx, __dmul_rn(J.z, dy));
    l1 = __fma_rn(J.y, dx, __dmul_rn(J.w, dy));
    l2 = __dsub_rn(__dsub_rn(1.0, l0), l1);
}

// GEOMETRY::isPointInsideUnitTriangle (geometry.cuh:37-46): every coordinate in
// [-2e-6, 1 + 2e-6].  The comparisons run on the IEEE bit patterns with integer
// instructions (GB300 issues FP64 compares on its small FP64 pipe): for a double v,
// v > hi (hi > 0) iff bits(v) > bits(hi) as signed 64-bit integers, and v < lo (lo < 0)
// iff v is negative with |v| > |lo|, i.e. bits(v) < 0 and (bits(v) & ~sign) >
// bits(|lo|).  Same result as the floating-point test for every non-NaN v (a NaN
// coordinate, which only a degenerate cell produces, counts as outside here).
__device__ __forceinline__ bool in_band(double v) {
    const long long b = __double_as_longlong(v);
    const long long hi = __double_as_longlong(1.0 + kDoubleMin);
    const long long lo_mag = __double_as_longlong(kDoubleMin);
    if (b >= 0) return b <= hi;
    return (b & 0x7fffffffffffffffll) <= lo_mag;
}

__device__ __forceinline__ bool inside_unit(double l0, double l1, double l2) {
    return in_band(l0) && in_band(l1) && in_band(l2);
}

// Conservative single-precision test used to skip cells: false only when the point is
// outside the cell by more than 0.01 in some barycentric coordinate.  Position, vertex
// and inverse Jacobian are FP32 roundings (relative error 6e-8 each): for coordinates
// below ~8 the barycentric error is below 1e-6 / h, so for cells larger than ~1e-4 it
// never rejects a cell the exact FP64 test would accept.  Pure FP32 arithmetic keeps
// the candidates off GB300's small FP64 pipe.
__device__ __forceinline__ bool maybe_inside_f32(float x, float y, const float4 J, const float2 v3) {
    const float dx = x - v3.x, dy = y - v3.y;
    const float l0 = J.x * dx + J.z * dy;
    const float l1 = J.y * dx + J.w * dy;
    const float l2 = 1.0f - l0 - l1;
    const float m = 0.01f;
    return l0 > -m && l0 < 1.0f + m && l1 > -m && l1 < 1.0f + m && l2 > -m && l2 < 1.0f + m;
}

// sum_i L_i u(node_i) accumulated from 0.0 (particle_handler_2d.cu:62-66)
__device__ __forceinline__ double interp3(double l0, double l1, double l2, double u0, double u1, double u2) {
    double s = __fma_rn(l0, u0, 0.0);
    s = __fma_rn(l1, u1, s);
    return __fma_rn(l2, u2, s);
}

// transformLocalToGlobal (geometry.cuh:6-8)
__device__ __forceinline__ double local_to_global(double L0, double L1, double L2, double a, double b, double c) {
    return __fma_rn(c, L2, __fma_rn(a, L0, __dmul_rn(b, L1)));
}

// determineSubcell (particle_handler_2d.cu:10-33); may return >= n*n (no clamping)
__device__ __forceinline__ int determine_subcell(int n, double step, double l0, double l1, double l2) {
    const int i = (int)__dmul_rn(__dsub_rn(1.0, l1), (double)n);
    int res = i * i;  // sum_{row<i} (2 row + 1)
    const int j = (int)__dmul_rn(l0, (double)n);
    res += 2 * j;
    if (j != i) {
        const double x = __dmul_rn(step, (double)(j + 1));
        const double y = __fma_rn(-step, (double)(i + 1), 1.0);
        const double z = __dsub_rn(__dsub_rn(1.0, x), y);
        if (l2 < z) ++res;
    }
    return res;
}

// --------------------------------------------------------------- reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum (any blockDim multiple of 32, <= 1024); the result is returned to every
// thread.  Fixed order, so repeated runs give identical bits.
__device__ __forceinline__ double block_sum(double v, double* sh /* >= 33 doubles */) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        double t = lane < nw ? sh[lane] : 0.0;
        t = warp_sum(t);
        if (lane == 0) sh[32] = t;
    }
    __syncthreads();
    return sh[32];
}

// Block-wide sums of NV values at once (fixed order); every thread gets the results.
// sh holds at least 33 * NV doubles.
template <int NV>
__device__ __forceinline__ void block_sum_n(double (&v)[NV], double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = warp_sum(v[j]);
    __syncthreads();
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < NV; ++j) sh[32 * j + w] = v[j];
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            double t = lane < nw ? sh[32 * j + lane] : 0.0;
            t = warp_sum(t);
            if (lane == 0) sh[32 * NV + j] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = sh[32 * NV + j];
}

// ------------------------------------------------------------ grid barrier
// Barrier over all blocks of a cooperative launch (all blocks co-resident).  Arrivals add
// to one counter that only grows during a launch (zeroed before each launch): barrier k
// is complete once the counter reaches (k + 1) * gridDim, so a block that arrives with the
// counter at c waits for (c / gridDim + 1) * gridDim.  Thread 0 arrives with a gpu-scope
// release after the block's __syncthreads and waits with gpu-scope acquire loads, which
// orders every thread's writes before the barrier against every thread's reads after it.
// The wait is bounded: after `kBarrierPolls` polls it records DEV_TIMEOUT in *err (and
// where it gave up in rec) and returns, and callers check the result after every barrier,
// so no block waits forever.
struct GridBarrier {
    unsigned int* count;  // zero-initialised before each launch
    int* err;
    double* part;  // 2 x 4 x gridDim per-block partial sums (grid_reduce)
    int* rec;      // where a wait gave up: {kind, a, b, c, d}, kind 0 = none
    long long max_polls;  // polls of a barrier wait before it gives up; 0 = kBarrierPolls
};

constexpr long long kBarrierPolls = 1ll << 22;
constexpr long long kFlagPolls = 1ll << 21;

// First timeout of a launch records its place (kind 1: grid barrier, 2: row flag).
__device__ __forceinline__ void record_timeout(int* rec, int kind, int a, int b, int c, int d) {
    if (rec && atomicCAS(&rec[0], 0, kind) == 0) {
        rec[1] = a;
        rec[2] = b;
        rec[3] = c;
        rec[4] = d;
        __threadfence();
    }
}

__device__ __forceinline__ unsigned ld_relaxed_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void arrive_release_gpu(unsigned* p) {
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" : : "l"(p) : "memory");
}

// Thread 0 arrives at barrier k (the counter read before arriving, c0, lies in
// [k G, (k + 1) G)) and waits for the other blocks.  False on a timeout or an error.
__device__ __forceinline__ bool barrier_wait(const GridBarrier& b, unsigned c0, unsigned nblocks) {
    const unsigned target = (c0 / nblocks + 1) * nblocks;
    const long long limit = b.max_polls > 0 ? b.max_polls : kBarrierPolls;
    long long polls = 0;
    unsigned c;
    while ((int)((c = ld_acquire_gpu(b.count)) - target) < 0) {
        if (++polls > limit) {
            atomicExch(b.err, (int)DEV_TIMEOUT);
            record_timeout(b.rec, 1, (int)blockIdx.x, (int)(c0 / nblocks), (int)c, 0);
            return false;
        }
        if ((polls & 255) == 0 && *(volatile int*)b.err != 0) return false;
    }
    return *(volatile int*)b.err == 0;
}

__device__ __forceinline__ bool arrive_and_wait(const GridBarrier& b, unsigned c0, unsigned nblocks) {
    arrive_release_gpu(b.count);
    return barrier_wait(b, c0, nblocks);
}

// The counter is read before the block's __syncthreads, whose wait hides the load: the
// value is at least k G (this thread saw it reach k G at the last barrier) and below
// (k + 1) G (barrier k cannot complete before this block arrives).  The error word is
// read once per block (thread 0) so that every thread of a block takes the same branch
// afterwards.
__device__ __forceinline__ bool grid_sync(const GridBarrier& b, unsigned nblocks) {
    __shared__ int s_ok;
    unsigned c0 = 0;
    if (threadIdx.x == 0) c0 = ld_relaxed_gpu(b.count);
    __syncthreads();
    if (threadIdx.x == 0) s_ok = arrive_and_wait(b, c0, nblocks) ? 1 : 0;
    __syncthreads();
    return s_ok != 0;
}

// Barrier fused with grid-wide sums of NV (<= 4) values.  The block sums (warp
// butterflies, then warp 0 over the warp sums) are stored by thread 0 in one of two
// partial arrays (chosen by the parity of the barrier index) before it arrives; once
// released, warp 0 of every block adds all blocks' partials in the same fixed order
// (lane l: partials l, l + 32, ... in increasing order, then a butterfly; lane 0's
// total), so all blocks get the same bits whatever the arrival order.  Two arrays
// suffice: a block can be at most one barrier ahead of the slowest reader of
// the other array.  On return v holds the totals in every thread.  sh holds at least 33 * NV
// doubles; part holds 2 x 4 x gridDim doubles.
template <int NV>
__device__ __forceinline__ bool grid_reduce(const GridBarrier& b, double (&v)[NV], double* sh) {
    __shared__ int s_ok;
    const unsigned G = gridDim.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned c0 = 0;
    if (threadIdx.x == 0) c0 = ld_relaxed_gpu(b.count);
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = warp_sum(v[j]);
    __syncthreads();  // the previous call's readers of sh are done
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < NV; ++j) sh[32 * j + w] = v[j];
    }
    __syncthreads();
    if (w == 0) {
        double t[NV];
#pragma unroll
        for (int j = 0; j < NV; ++j) t[j] = warp_sum(lane < nw ? sh[32 * j + lane] : 0.0);
        const unsigned k = __shfl_sync(0xffffffffu, c0, 0) / G;
        double* part = b.part + (size_t)(k & 1u) * 4 * G;
        int ok = 1;
        if (lane == 0) {
#pragma unroll
            for (int j = 0; j < NV; ++j) __stcg(&part[j * G + blockIdx.x], t[j]);
            ok = arrive_and_wait(b, c0, G) ? 1 : 0;
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        __syncwarp();  // lane 0's acquire orders the other lanes' reads of the partials
#pragma unroll
        for (int j = 0; j < NV; ++j) t[j] = 0.0;
        for (unsigned q = lane; q < G; q += 32) {
#pragma unroll
            for (int j = 0; j < NV; ++j) t[j] += __ldcg(&part[j * G + q]);
        }
#pragma unroll
        for (int j = 0; j < NV; ++j) t[j] = warp_sum(t[j]);
        if (lane == 0) {
#pragma unroll
            for (int j = 0; j < NV; ++j) sh[32 * NV + j] = t[j];
            s_ok = ok;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = sh[32 * NV + j];
    return s_ok != 0;
}

struct NoPost {
    __device__ void operator()(const double*, double*) const {}
};

// Grid-wide sums of NV <= 4 values fused with the grid barrier, for blocks of BT threads
// (BT a multiple of 128, at most 1024), with few FP64 instructions: on GB300 an SM issues
// one FP64 warp instruction per ~19 clocks (~64 per sub-partition), so warp butterflies
// in every warp (five FP64 additions per value per warp) cost microseconds per reduction.
// The block's values go to red (NV x BT doubles of shared memory) and a fixed tree adds
// them: a quarter of the threads per value add 4 values each, a sixteenth add 4 of those,
// one warp per value adds up to 2 and finishes with a butterfly.  Thread 0 stores the block
// sums in one of two partial arrays (by the barrier's parity) and arrives on the grid
// barrier; after the release warp j adds value j's partials in block order (lane l:
// partials l, l + 32, ...; butterfly).  The order depends on no arrival order: the sums
// are reproducible bit for bit.  Post (not NoPost): thread 0 alone then derives the
// iteration's scalars from the totals (post(totals, out), out = sh + 24, up to 8 doubles),
// which every thread reads after the call: an FP64 division or square root is tens of
// FP64 instructions and would cost microseconds computed by every warp.  sh holds at least
// 32 doubles.
// The first half of grid_reduce_tree: the block tree, the block sums stored and the
// arrival.  Returns the barrier ticket (thread 0's counter read; meaningful in thread 0
// only) for grid_reduce_tree_wait; work that needs no other block's contribution to this
// reduction may run in between (the wait is split from the arrival so that it overlaps).
template <int BT, int NV>
__device__ __forceinline__ unsigned grid_reduce_tree_arrive(const GridBarrier& b, const double (&v)[NV], double* sh,
                                                            double* red) {
    static_assert(NV >= 1 && NV <= 4, "grid_reduce_tree sums one to four values");
    static_assert(BT % 128 == 0 && BT <= 1024, "block size of the tree");
    const unsigned G = gridDim.x;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    unsigned c0 = 0;
    if (tid == 0) c0 = ld_relaxed_gpu(b.count);
    __syncthreads();  // the previous call's readers of red and sh are done
#pragma unroll
    for (int j = 0; j < NV; ++j) red[j * BT + tid] = v[j];
    __syncthreads();
    for (int t = tid; t < NV * (BT / 4); t += BT) {
        const int j = t / (BT / 4), u = t % (BT / 4);
        double* c = red + j * BT + u;
        c[0] = ((c[0] + c[BT / 4]) + c[BT / 2]) + c[3 * BT / 4];
    }
    __syncthreads();
    if (tid < NV * (BT / 16)) {
        const int j = tid / (BT / 16), u = tid % (BT / 16);
        double* c = red + j * BT + u;
        c[0] = ((c[0] + c[BT / 16]) + c[BT / 8]) + c[3 * BT / 16];
    }
    __syncthreads();
    if (w < NV) {
        const double s = warp_sum(red[w * BT + lane] + (lane + 32 < BT / 16 ? red[w * BT + lane + 32] : 0.0));
        if (lane == 0) sh[w] = s;
    }
    __syncthreads();
    if (tid == 0) {
        double* part = b.part + (size_t)((c0 / G) & 1u) * 4 * G;
#pragma unroll
        for (int j = 0; j < NV; ++j) __stcg(&part[j * G + blockIdx.x], sh[j]);
        arrive_release_gpu(b.count);
    }
    return c0;
}

// The second half: thread 0 waits for the other blocks (bounded), warp j adds value j's
// partials in block order, thread 0 runs post, and every thread gets the totals in v.
template <int BT, int NV, class Post = NoPost>
__device__ __forceinline__ bool grid_reduce_tree_wait(const GridBarrier& b, unsigned c0, double (&v)[NV], double* sh,
                                                      Post post = Post()) {
    __shared__ int s_ok, s_par;
    const unsigned G = gridDim.x;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) {
        s_ok = barrier_wait(b, c0, G) ? 1 : 0;
        s_par = (int)((c0 / G) & 1u);
    }
    __syncthreads();
    if (w < NV) {
        const double* part = b.part + (size_t)s_par * 4 * G + w * G;
        double t = 0.0;
        for (unsigned q = lane; q < G; q += 32) t += __ldcg(&part[q]);
        t = warp_sum(t);
        if (lane == 0) sh[16 + w] = t;
    }
    __syncthreads();
    if (!std::is_same<Post, NoPost>::value) {
        if (tid == 0) post(sh + 16, sh + 24);
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = sh[16 + j];
    return s_ok != 0;
}

template <int BT, int NV, class Post = NoPost>
__device__ __forceinline__ bool grid_reduce_tree(const GridBarrier& b, double (&v)[NV], double* sh, double* red,
                                                 Post post = Post()) {
    const unsigned c0 = grid_reduce_tree_arrive<BT, NV>(b, v, sh, red);
    return grid_reduce_tree_wait<BT, NV>(b, c0, v, sh, post);
}

}  // namespace pf2
