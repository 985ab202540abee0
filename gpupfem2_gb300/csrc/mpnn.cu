// mpnn.cu - the learned initial guess of the pressure solve (no reference counterpart).
//
// A message-passing network over the mesh graph (nodes; edges = off-diagonal CSR
// entries, symmetric) with 5 input features, 64 hidden units and 3 layers:
//   h0 = relu(W0 f + c0)
//   l = 1..3:  m_i = mean_{j in N(i)} h_j ;  h = h + relu(W_l [h ; m] + c_l)
//   y  = w4 . h + c4
// Master parameters are FP32; the per-node MLPs run on the tensor cores with BF16
// weights and activations and FP32 accumulation on tcgen05 (accumulators in tensor
// memory, 128 nodes per CTA); the mma.sync m16n8k16 kernels stay as the
// PF2_MPNN_MMA=sync path.  Training
// (backward and AdamW) runs on the device; gradients are summed in a fixed order.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "device.cuh"
#include "internal.cuh"

namespace pf2 {

constexpr int MH = 64;      // hidden width
constexpr int MIN = 5;      // input features
constexpr int ML = 3;       // message-passing layers
constexpr int MK = 2 * MH;  // layer input width [h ; m]
constexpr int kTile = 64;   // nodes per CTA tile
constexpr int kMpnnThreads = 128;
constexpr int kPad = 8;     // bf16 row padding against bank conflicts

constexpr int kParamW0 = 0;
constexpr int kParamC0 = kParamW0 + MH * MIN;
constexpr int kParamLayer0 = kParamC0 + MH;
constexpr int kLayerSize = MH * MK + MH;
constexpr int kParamW4 = kParamLayer0 + ML * kLayerSize;
constexpr int kParamC4 = kParamW4 + MH;
constexpr int kParams = kParamC4 + 1;

__device__ __forceinline__ unsigned pack_bf16(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<unsigned*>(&v);
}

// D = A(16x16, row) * B(16x8, col) + D, bf16 inputs, f32 accumulate
__device__ __forceinline__ void mma16816(float d[4], const unsigned a[4], const unsigned b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// One warp: acc[16 x 8NT] += A[16 x 16KT] (smem row-major, stride sa) * B, with B given as
// rows of n (smem [n][k], stride sb).
template <int KT, int NT>
__device__ __forceinline__ void warp_gemm(const __nv_bfloat16* A, int sa, const __nv_bfloat16* B, int sb,
                                          float acc[NT][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
        const int k0 = kt * 16 + 2 * t;
        unsigned a[4];
        a[0] = *reinterpret_cast<const unsigned*>(A + g * sa + k0);
        a[1] = *reinterpret_cast<const unsigned*>(A + (g + 8) * sa + k0);
        a[2] = *reinterpret_cast<const unsigned*>(A + g * sa + k0 + 8);
        a[3] = *reinterpret_cast<const unsigned*>(A + (g + 8) * sa + k0 + 8);
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const __nv_bfloat16* Bn = B + (nt * 8 + g) * sb + k0;
            unsigned b[2];
            b[0] = *reinterpret_cast<const unsigned*>(Bn);
            b[1] = *reinterpret_cast<const unsigned*>(Bn + 8);
            mma16816(acc[nt], a, b);
        }
    }
}

struct Graph {
    int n;
    const int* rowptr;
    const int* col;
    const float* deg_inv;  // 1 / #neighbours (0 for an isolated node)
};

// ---------------------------------------------------------------- forward
__global__ void k_mpnn_encoder(Graph G, const float* __restrict__ feat, const float* __restrict__ P, float* H0,
                               unsigned long long* mask0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= G.n) return;
    float f[MIN];
#pragma unroll
    for (int k = 0; k < MIN; ++k) f[k] = feat[(size_t)i * MIN + k];
    unsigned long long mk = 0ull;
    for (int o = 0; o < MH; ++o) {
        float s = P[kParamC0 + o];
#pragma unroll
        for (int k = 0; k < MIN; ++k) s += P[kParamW0 + o * MIN + k] * f[k];
        if (s > 0.0f) mk |= 1ull << o;
        H0[(size_t)i * MH + o] = s > 0.0f ? s : 0.0f;
    }
    mask0[i] = mk;
}

// mean of the neighbours' h (fixed order: ascending column)
__device__ __forceinline__ void gather_mean(const Graph& G, const float* __restrict__ H, int i, int o, float& out) {
    float s = 0.0f;
    for (int k = G.rowptr[i]; k < G.rowptr[i + 1]; ++k) {
        const int j = G.col[k];
        if (j != i) s += H[(size_t)j * MH + o];
    }
    out = s * G.deg_inv[i];
}

// One layer: h_out = h_in + relu(W [h_in ; m] + c); stores m (for the backward pass)
// and the relu mask.  CTA = 4 warps x 16 nodes.
__global__ void __launch_bounds__(kMpnnThreads) k_mpnn_layer(Graph G, const float* __restrict__ Hin,
                                                             const __nv_bfloat16* __restrict__ Wb,
                                                             const float* __restrict__ c, float* Hout, float* M,
                                                             unsigned long long* mask) {
    __shared__ __align__(16) __nv_bfloat16 sA[kTile][MK + kPad];
    __shared__ __align__(16) __nv_bfloat16 sW[MH][MK + kPad];
    const int base = blockIdx.x * kTile;
    for (int q = threadIdx.x; q < MH * MK; q += blockDim.x) sW[q / MK][q % MK] = Wb[q];
    for (int q = threadIdx.x; q < kTile * MH; q += blockDim.x) {
        const int r = q / MH, o = q % MH, i = base + r;
        float h = 0.0f, m = 0.0f;
        if (i < G.n) {
            h = Hin[(size_t)i * MH + o];
            gather_mean(G, Hin, i, o, m);
            M[(size_t)i * MH + o] = m;
        }
        sA[r][o] = __float2bfloat16_rn(h);
        sA[r][MH + o] = __float2bfloat16_rn(m);
    }
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float acc[MH / 8][4];
#pragma unroll
    for (int nt = 0; nt < MH / 8; ++nt)
        for (int k = 0; k < 4; ++k) acc[nt][k] = 0.0f;
    warp_gemm<MK / 16, MH / 8>(&sA[w * 16][0], MK + kPad, &sW[0][0], MK + kPad, acc);
    // epilogue: rows g, g+8 of this warp's 16 nodes; columns nt*8 + 2t, +1
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const int i = base + w * 16 + g + 8 * half;
        const bool valid = i < G.n;
        unsigned long long bits = 0ull;
#pragma unroll
        for (int nt = 0; nt < MH / 8; ++nt)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int o = nt * 8 + 2 * t + e;
                const float z = acc[nt][2 * half + e] + c[o];
                if (z > 0.0f) bits |= 1ull << o;
                if (valid) Hout[(size_t)i * MH + o] = Hin[(size_t)i * MH + o] + (z > 0.0f ? z : 0.0f);
            }
        // the four threads of a quad own disjoint columns of the row: combine their bits
        // (every lane takes part in the shuffles; only the store is guarded)
        bits |= __shfl_xor_sync(0xffffffffu, bits, 1);
        bits |= __shfl_xor_sync(0xffffffffu, bits, 2);
        if (valid && t == 0) mask[i] = bits;
    }
}

// ------------------------------------------------ fifth-generation tensor cores
// The layer GEMM on tcgen05: one thread issues tcgen05.mma (kind::f16, BF16 operands from
// shared memory, FP32 accumulator in tensor memory), the CTA reads the accumulator back
// with tcgen05.ld.  Operands sit in shared memory in the canonical K-major layout without
// swizzle: 8-row x 16-byte core matrices, element (r, k) of an R-row tile at byte
//   ((k / 8) * (R / 8) + r / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// so core matrices adjacent in K are R * 16 bytes apart (the descriptor's leading byte
// offset) and those adjacent in rows 128 bytes apart (its stride byte offset).
constexpr int kTcTile = 128;  // nodes per CTA: the MMA's M (accumulator lanes 0..127)
constexpr long long kTcPolls = 1ll << 24;
// Dynamic shared memory of k_mpnn_layer_tc: A (32 KB) in a 64 KB region, W (16 KB) in a
// 24 KB region.  The MMAs read A within [start, start + 32 KB) and W within 16 KB; the
// regions are larger so that the descriptors' reads stay inside the CTA's shared memory
// whichever way the two offsets are read.
constexpr int kTcRegionA = 64 * 1024;
constexpr int kTcRegionB = 24 * 1024;
constexpr int kTcSmem = kTcRegionA + kTcRegionB;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ int tc_offset(int r, int k, int rows) {
    return ((k >> 3) * (rows >> 3) + (r >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Shared-memory matrix descriptor (no swizzle, version 1): start, leading byte offset
// (between core matrices adjacent in K), stride byte offset (adjacent in rows).
__device__ __forceinline__ unsigned long long tc_desc(unsigned addr, unsigned lbo, unsigned sbo) {
    return (unsigned long long)((addr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
           ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major,
// N and M as given.
__host__ __device__ constexpr unsigned tc_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(n >> 3) << 17) | ((unsigned)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(unsigned tmem_d, unsigned long long a, unsigned long long b, unsigned idesc,
                                       int accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :
        : "r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(unsigned mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" : : "r"(mbar)
                 : "memory");
}

// Bounded wait for phase `parity` of an mbarrier; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(unsigned mbar, unsigned parity) {
    for (long long i = 0; i < kTcPolls; ++i) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 32 consecutive accumulator columns of this warp's 32 lanes: register j of lane l holds
// row (lane base + l), column (col + j).
__device__ __forceinline__ void tc_ld32(unsigned taddr, float (&v)[32]) {
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
        "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// One layer as k_mpnn_layer, 128 nodes per CTA on tcgen05: h_out = h_in + relu(W [h ; m]
// + c), m (for the backward pass) and the relu mask stored.  CTA = 4 warps; warp 0 holds
// the 64 accumulator columns of tensor memory; thread 0 issues the eight K = 16 MMAs
// (M = 128, N = 64); warp w reads back the rows 32 w .. 32 w + 31, one row per thread.
// A wait that runs out sets *err and skips the outputs.
__global__ void __launch_bounds__(128) k_mpnn_layer_tc(Graph G, const float* __restrict__ Hin,
                                                       const __nv_bfloat16* __restrict__ Wb,
                                                       const float* __restrict__ c, float* Hout, float* M,
                                                       unsigned long long* mask, int* err) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char* sA = tc_smem;               // [node][in], canonical layout
    unsigned char* sB = tc_smem + kTcRegionA;  // W [out][in], canonical layout
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ unsigned tmem_slot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int base = blockIdx.x * kTcTile;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(MH));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    for (int q = threadIdx.x; q < MH * MK; q += blockDim.x) {
        const int o = q / MK, k = q % MK;
        *reinterpret_cast<__nv_bfloat16*>(sB + tc_offset(o, k, MH)) = Wb[q];
    }
    for (int q = threadIdx.x; q < kTcTile * MH; q += blockDim.x) {
        const int r = q / MH, o = q % MH, i = base + r;
        float h = 0.0f, m = 0.0f;
        if (i < G.n) {
            h = Hin[(size_t)i * MH + o];
            gather_mean(G, Hin, i, o, m);
            M[(size_t)i * MH + o] = m;
        }
        *reinterpret_cast<__nv_bfloat16*>(sA + tc_offset(r, o, kTcTile)) = __float2bfloat16_rn(h);
        *reinterpret_cast<__nv_bfloat16*>(sA + tc_offset(r, MH + o, kTcTile)) = __float2bfloat16_rn(m);
    }
    // the operands written by threads become visible to the tensor cores' async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tmem_slot;
    if (threadIdx.x == 0) {
        const unsigned a0 = smem_u32(sA), b0 = smem_u32(sB);
        constexpr unsigned idesc = tc_idesc(kTcTile, MH);
#pragma unroll
        for (int ks = 0; ks < MK / 16; ++ks) {
            const unsigned long long da = tc_desc(a0 + ks * 2 * (kTcTile * 16), kTcTile * 16, 128);
            const unsigned long long db = tc_desc(b0 + ks * 2 * (MH * 16), MH * 16, 128);
            tc_mma(tmem, da, db, idesc, ks > 0);
        }
        tc_commit(smem_u32(&mbar));
    }
    // every thread polls; the outcome is made block-uniform (the reads below are
    // warp-collective)
    const bool ok = __syncthreads_and(mbar_wait(smem_u32(&mbar), 0));
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(err, (int)DEV_TIMEOUT);
        mbar_wait(smem_u32(&mbar), 0);  // bounded: the MMAs may still be writing
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        const int r = warp * 32 + lane, i = base + r;
        unsigned long long bits = 0ull;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            float acc[32];
            tc_ld32(tmem + ((unsigned)(warp * 32) << 16) + half * 32, acc);
            if (i < G.n) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int o = half * 32 + j;
                    const float z = acc[j] + c[o];
                    if (z > 0.0f) bits |= 1ull << o;
                    Hout[(size_t)i * MH + o] = Hin[(size_t)i * MH + o] + (z > 0.0f ? z : 0.0f);
                }
            }
        }
        if (i < G.n) mask[i] = bits;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(MH));
}

// The CTA's tensor-memory columns (warp 0 allocates; power of two >= 32).
__device__ __forceinline__ void tc_alloc(unsigned* slot, int cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tc_dealloc(unsigned tmem, int cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols));
}

__device__ __forceinline__ void tc_sync_in() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Backward node part on tcgen05: [dself ; dm] = dz W for 128 nodes per CTA (M = 128,
// N = 128 inputs, K = 64 outputs in four MMAs); dz = dh * mask; dm scaled by 1 / d_i.
// Operand regions of 48 KB each (16 KB used), as k_mpnn_layer_tc.
constexpr int kTcBnRegion = 48 * 1024;
constexpr int kTcBnSmem = 2 * kTcBnRegion;
__global__ void __launch_bounds__(128) k_mpnn_layer_back_nodes_tc(Graph G, const float* __restrict__ dH,
                                                                  const unsigned long long* __restrict__ mask,
                                                                  const __nv_bfloat16* __restrict__ Wb, float* dSelf,
                                                                  float* dMs, int* err) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char* sA = tc_smem;                // dz [node][out]
    unsigned char* sB = tc_smem + kTcBnRegion;  // W^T [in][out]
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ unsigned tmem_slot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int base = blockIdx.x * kTcTile;
    if (warp == 0) tc_alloc(&tmem_slot, MK);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    for (int q = threadIdx.x; q < MH * MK; q += blockDim.x) {
        const int o = q / MK, k = q % MK;
        *reinterpret_cast<__nv_bfloat16*>(sB + tc_offset(k, o, MK)) = Wb[q];
    }
    for (int q = threadIdx.x; q < kTcTile * MH; q += blockDim.x) {
        const int r = q / MH, o = q % MH, i = base + r;
        float v = 0.0f;
        if (i < G.n && ((mask[i] >> o) & 1ull)) v = dH[(size_t)i * MH + o];
        *reinterpret_cast<__nv_bfloat16*>(sA + tc_offset(r, o, kTcTile)) = __float2bfloat16_rn(v);
    }
    tc_sync_in();
    const unsigned tmem = tmem_slot;
    if (threadIdx.x == 0) {
        const unsigned a0 = smem_u32(sA), b0 = smem_u32(sB);
        constexpr unsigned idesc = tc_idesc(kTcTile, MK);
#pragma unroll
        for (int ks = 0; ks < MH / 16; ++ks)
            tc_mma(tmem, tc_desc(a0 + ks * 2 * (kTcTile * 16), kTcTile * 16, 128),
                   tc_desc(b0 + ks * 2 * (MK * 16), MK * 16, 128), idesc, ks > 0);
        tc_commit(smem_u32(&mbar));
    }
    const bool ok = __syncthreads_and(mbar_wait(smem_u32(&mbar), 0));
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(err, (int)DEV_TIMEOUT);
        mbar_wait(smem_u32(&mbar), 0);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        const int r = warp * 32 + lane, i = base + r;
        const float di = i < G.n ? G.deg_inv[i] : 0.0f;
#pragma unroll
        for (int q = 0; q < MK / 32; ++q) {
            float acc[32];
            tc_ld32(tmem + ((unsigned)(warp * 32) << 16) + q * 32, acc);
            if (i < G.n) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int k = q * 32 + j;
                    if (k < MH) dSelf[(size_t)i * MH + k] = acc[j];
                    else dMs[(size_t)i * MH + (k - MH)] = acc[j] * di;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, MK);
}

// Backward weight part on tcgen05: per-CTA partial dW[out][in] = sum over the CTA's node
// tiles of [h ; m]^T dz (M = 128 inputs, N = 64 outputs, K = 128 nodes per tile,
// accumulated in tensor memory across the tiles) and dc on the CUDA cores.  A tile's
// operands are overwritten only after its MMAs completed (mbarrier phase per tile).
// Operand regions as k_mpnn_layer_tc.
__global__ void __launch_bounds__(128) k_mpnn_layer_back_weights_tc(Graph G, const float* __restrict__ Hin,
                                                                    const float* __restrict__ M,
                                                                    const float* __restrict__ dH,
                                                                    const unsigned long long* __restrict__ mask,
                                                                    float* part, int* err) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char* sA = tc_smem;               // [h ; m]^T [in][node]
    unsigned char* sB = tc_smem + kTcRegionA;  // dz^T [out][node]
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ unsigned tmem_slot;
    __shared__ float sC[MH];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) tc_alloc(&tmem_slot, MH);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    for (int o = threadIdx.x; o < MH; o += blockDim.x) sC[o] = 0.0f;
    const int ntiles = (G.n + kTcTile - 1) / kTcTile;
    unsigned phase = 0;
    bool ok = true, issued = false;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int base = tile * kTcTile;
        if (issued) {  // the previous tile's MMAs have read the operands
            ok = __syncthreads_and(mbar_wait(smem_u32(&mbar), phase));
            phase ^= 1u;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (!ok) break;
        }
        for (int q = threadIdx.x; q < kTcTile * MH; q += blockDim.x) {
            const int r = q / MH, o = q % MH, i = base + r;
            float h = 0.0f, m = 0.0f, z = 0.0f;
            if (i < G.n) {
                h = Hin[(size_t)i * MH + o];
                m = M[(size_t)i * MH + o];
                if ((mask[i] >> o) & 1ull) z = dH[(size_t)i * MH + o];
            }
            *reinterpret_cast<__nv_bfloat16*>(sA + tc_offset(o, r, MK)) = __float2bfloat16_rn(h);
            *reinterpret_cast<__nv_bfloat16*>(sA + tc_offset(MH + o, r, MK)) = __float2bfloat16_rn(m);
            *reinterpret_cast<__nv_bfloat16*>(sB + tc_offset(o, r, MH)) = __float2bfloat16_rn(z);
        }
        tc_sync_in();
        // dc: the outputs' sums of the rounded dz over the tile's nodes
        for (int o = threadIdx.x; o < MH; o += blockDim.x) {
            float s = 0.0f;
            for (int r = 0; r < kTcTile; ++r)
                s += __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(sB + tc_offset(o, r, MH)));
            sC[o] += s;
        }
        if (threadIdx.x == 0) {
            const unsigned a0 = smem_u32(sA), b0 = smem_u32(sB);
            constexpr unsigned idesc = tc_idesc(MK, MH);
#pragma unroll
            for (int ks = 0; ks < kTcTile / 16; ++ks)
                tc_mma(tmem_slot, tc_desc(a0 + ks * 2 * (MK * 16), MK * 16, 128),
                       tc_desc(b0 + ks * 2 * (MH * 16), MH * 16, 128), idesc, (issued || ks > 0) ? 1 : 0);
            tc_commit(smem_u32(&mbar));
        }
        issued = true;
        __syncthreads();  // sC complete before the next tile overwrites sB
    }
    if (issued && ok) {
        ok = __syncthreads_and(mbar_wait(smem_u32(&mbar), phase));
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(err, (int)DEV_TIMEOUT);
        if (issued) mbar_wait(smem_u32(&mbar), phase);
    }
    float* P = part + (size_t)blockIdx.x * (MH * MK + MH);
    const unsigned tmem = tmem_slot;
    const int in = warp * 32 + lane;  // accumulator lane = input row of dW^T
#pragma unroll
    for (int q = 0; q < MH / 32; ++q) {
        float acc[32];
        if (issued && ok) tc_ld32(tmem + ((unsigned)(warp * 32) << 16) + q * 32, acc);
        else
#pragma unroll
            for (int j = 0; j < 32; ++j) acc[j] = 0.0f;
#pragma unroll
        for (int j = 0; j < 32; ++j) P[(q * 32 + j) * MK + in] = acc[j];
    }
    __syncthreads();
    for (int o = threadIdx.x; o < MH; o += blockDim.x) P[MH * MK + o] = sC[o];
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, MH);
}

// y = w4 . h + c4; optionally loss partials and dy = 2 (y - t) / n
__global__ void k_mpnn_decoder(int n, const float* __restrict__ H, const float* __restrict__ P, float* y,
                               const float* __restrict__ target, float* dy, double* loss_part) {
    __shared__ double sh[40];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (i < n) {
        float s = P[kParamC4];
        for (int o = 0; o < MH; ++o) s += P[kParamW4 + o] * H[(size_t)i * MH + o];
        y[i] = s;
        if (target) {
            const float r = s - target[i];
            dy[i] = 2.0f * r / (float)n;
            l = (double)r * r;
        }
    }
    if (target) {
        l = block_sum(l, sh);
        if (threadIdx.x == 0) loss_part[blockIdx.x] = l;
    }
}

// ---------------------------------------------------------------- backward
// dh = dy w4, and per-block partials of (dw4, dc4)
__global__ void k_mpnn_decoder_back(int n, const float* __restrict__ H, const float* __restrict__ P,
                                    const float* __restrict__ dy, float* dH, float* part /* [grid][MH+1] */) {
    __shared__ float sp[MH + 1][kMpnnThreads / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const float d = (i < n) ? dy[i] : 0.0f;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 0; o <= MH; ++o) {
        float v = 0.0f;
        if (i < n) {
            if (o < MH) {
                v = d * H[(size_t)i * MH + o];
                dH[(size_t)i * MH + o] = d * P[kParamW4 + o];
            } else {
                v = d;
            }
        }
        v = warp_sumf(v);
        if (lane == 0) sp[o][w] = v;
    }
    __syncthreads();
    for (int o = threadIdx.x; o <= MH; o += blockDim.x) {
        float s = 0.0f;
        for (int k = 0; k < kMpnnThreads / 32; ++k) s += sp[o][k];
        part[(size_t)blockIdx.x * (MH + 1) + o] = s;
    }
}

// One layer backward, node part: dz = dh * mask; [dself ; dm] = dz W (tensor cores);
// writes dself and dm / d_i.
__global__ void __launch_bounds__(kMpnnThreads) k_mpnn_layer_back_nodes(Graph G, const float* __restrict__ dH,
                                                                        const unsigned long long* __restrict__ mask,
                                                                        const __nv_bfloat16* __restrict__ Wb,
                                                                        float* dSelf, float* dMs) {
    __shared__ __align__(16) __nv_bfloat16 sZ[kTile][MH + kPad];
    __shared__ __align__(16) __nv_bfloat16 sWT[MK][MH + kPad];  // W^T: [in][out]
    const int base = blockIdx.x * kTile;
    for (int q = threadIdx.x; q < MH * MK; q += blockDim.x) {
        const int o = q / MK, k = q % MK;
        sWT[k][o] = Wb[q];
    }
    for (int q = threadIdx.x; q < kTile * MH; q += blockDim.x) {
        const int r = q / MH, o = q % MH, i = base + r;
        float v = 0.0f;
        if (i < G.n && ((mask[i] >> o) & 1ull)) v = dH[(size_t)i * MH + o];
        sZ[r][o] = __float2bfloat16_rn(v);
    }
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float acc[MK / 8][4];
#pragma unroll
    for (int nt = 0; nt < MK / 8; ++nt)
        for (int k = 0; k < 4; ++k) acc[nt][k] = 0.0f;
    warp_gemm<MH / 16, MK / 8>(&sZ[w * 16][0], MH + kPad, &sWT[0][0], MH + kPad, acc);
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const int i = base + w * 16 + g + 8 * half;
        if (i >= G.n) continue;
        const float di = G.deg_inv[i];
#pragma unroll
        for (int nt = 0; nt < MK / 8; ++nt)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int k = nt * 8 + 2 * t + e;
                const float v = acc[nt][2 * half + e];
                if (k < MH) dSelf[(size_t)i * MH + k] = v;
                else dMs[(size_t)i * MH + (k - MH)] = v * di;
            }
    }
}

// dh_prev_i = dh_i + dself_i + sum_{k in N(i)} dm_k / d_k (the graph is symmetric)
__global__ void k_mpnn_agg_back(Graph G, const float* __restrict__ dH, const float* __restrict__ dSelf,
                                const float* __restrict__ dMs, float* dHprev) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)G.n * MH) return;
    const int i = (int)(q / MH), o = (int)(q % MH);
    float s = dH[q] + dSelf[q];
    for (int k = G.rowptr[i]; k < G.rowptr[i + 1]; ++k) {
        const int j = G.col[k];
        if (j != i) s += dMs[(size_t)j * MH + o];
    }
    dHprev[q] = s;
}

// One layer backward, weight part: per-CTA partial dW (= [h ; m]^T dz, tensor cores) and
// dc, over the node tiles this CTA visits.
__global__ void __launch_bounds__(kMpnnThreads) k_mpnn_layer_back_weights(Graph G, const float* __restrict__ Hin,
                                                                          const float* __restrict__ M,
                                                                          const float* __restrict__ dH,
                                                                          const unsigned long long* __restrict__ mask,
                                                                          float* part /* [grid][MH*MK + MH] */) {
    __shared__ __align__(16) __nv_bfloat16 sAT[MK][kTile + kPad];  // [in][node]
    __shared__ __align__(16) __nv_bfloat16 sZT[MH][kTile + kPad];  // [out][node]
    __shared__ float sC[MH];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    // warp w owns rows (inputs) w*32 .. w*32+31: two m tiles
    float acc[2][MH / 8][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < MH / 8; ++nt)
            for (int k = 0; k < 4; ++k) acc[mt][nt][k] = 0.0f;
    for (int o = threadIdx.x; o < MH; o += blockDim.x) sC[o] = 0.0f;
    const int ntiles = (G.n + kTile - 1) / kTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int base = tile * kTile;
        __syncthreads();
        for (int q = threadIdx.x; q < kTile * MH; q += blockDim.x) {
            const int r = q / MH, o = q % MH, i = base + r;
            float h = 0.0f, m = 0.0f, z = 0.0f;
            if (i < G.n) {
                h = Hin[(size_t)i * MH + o];
                m = M[(size_t)i * MH + o];
                if ((mask[i] >> o) & 1ull) z = dH[(size_t)i * MH + o];
            }
            sAT[o][r] = __float2bfloat16_rn(h);
            sAT[MH + o][r] = __float2bfloat16_rn(m);
            sZT[o][r] = __float2bfloat16_rn(z);
        }
        __syncthreads();
        for (int o = threadIdx.x; o < MH; o += blockDim.x) {
            float s = 0.0f;
            for (int r = 0; r < kTile; ++r) s += __bfloat162float(sZT[o][r]);
            sC[o] += s;
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
            warp_gemm<kTile / 16, MH / 8>(&sAT[w * 32 + mt * 16][0], kTile + kPad, &sZT[0][0], kTile + kPad, acc[mt]);
    }
    __syncthreads();
    // dW[out][in] = acc[in][out]
    float* P = part + (size_t)blockIdx.x * (MH * MK + MH);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int in = w * 32 + mt * 16 + g + 8 * half;
#pragma unroll
            for (int nt = 0; nt < MH / 8; ++nt)
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int o = nt * 8 + 2 * t + e;
                    P[o * MK + in] = acc[mt][nt][2 * half + e];
                }
        }
    for (int o = threadIdx.x; o < MH; o += blockDim.x) P[MH * MK + o] = sC[o];
}

// Encoder backward: per-block partials of (dW0, dc0)
__global__ void k_mpnn_encoder_back(int n, const float* __restrict__ feat, const float* __restrict__ dH,
                                    const unsigned long long* __restrict__ mask0, float* part /* [grid][MH*MIN+MH] */) {
    __shared__ float sp[MH * (MIN + 1)];
    for (int q = threadIdx.x; q < MH * (MIN + 1); q += blockDim.x) sp[q] = 0.0f;
    __syncthreads();
    const int nper = (n + gridDim.x - 1) / gridDim.x;
    const int i0 = blockIdx.x * nper, i1 = min(n, i0 + nper);
    // thread (o, k): sums dz_o * f_k (k < MIN) or dz_o (k == MIN) over this block's nodes
    for (int q = threadIdx.x; q < MH * (MIN + 1); q += blockDim.x) {
        const int o = q / (MIN + 1), k = q % (MIN + 1);
        float s = 0.0f;
        for (int i = i0; i < i1; ++i) {
            if (!((mask0[i] >> o) & 1ull)) continue;
            const float dz = dH[(size_t)i * MH + o];
            s += (k < MIN) ? dz * feat[(size_t)i * MIN + k] : dz;
        }
        sp[q] = s;
    }
    __syncthreads();
    float* P = part + (size_t)blockIdx.x * (MH * MIN + MH);
    for (int q = threadIdx.x; q < MH * (MIN + 1); q += blockDim.x) {
        const int o = q / (MIN + 1), k = q % (MIN + 1);
        if (k < MIN) P[o * MIN + k] = sp[q];
        else P[MH * MIN + o] = sp[q];
    }
}

// grad[off + j] = sum_b part[b * width + j], fixed order, FP64 accumulation
__global__ void k_reduce_cols(const float* __restrict__ part, int nb, int width, float* grad, int off) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= width) return;
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += part[(size_t)b * width + j];
    grad[off + j] = (float)s;
}

__global__ void k_adamw(int np, float* P, const float* __restrict__ g, float* m, float* v, float c1, float c2,
                        float lr, float b1, float b2, float eps, float wd) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.0f - b1) * gk;
    const float vk = b2 * v[k] + (1.0f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    P[k] -= lr * (mk / c1 / (sqrtf(vk / c2) + eps) + wd * P[k]);
}

__global__ void k_weights_bf16(const float* __restrict__ P, __nv_bfloat16* Wb) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ML * MH * MK) return;
    const int l = q / (MH * MK), r = q % (MH * MK);
    Wb[q] = __float2bfloat16_rn(P[kParamLayer0 + l * kLayerSize + r]);
}

__global__ void k_deg_inv(int n, const int* __restrict__ rowptr, const int* __restrict__ col, float* dinv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int d = 0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) d += (col[k] != i);
    dinv[i] = d ? 1.0f / (float)d : 0.0f;
}

}  // namespace pf2

using namespace pf2;

struct pf2_mpnn {
    int n = 0;
    const pf2_mesh* mesh = nullptr;
    DevBuf<float> P, grad, am, av, dinv, feat, y, dy, H, M, dH, dH2, dSelf, dMs, part, target;
    DevBuf<unsigned long long> mask;
    DevBuf<__nv_bfloat16> Wb;
    DevBuf<double> loss_part;
    DevBuf<int> err;  // a tcgen05 wait that ran out (DEV_TIMEOUT)
    int step = 0;
    int wgrid = 0;
    bool tc = true;  // the layer GEMMs on tcgen05 (PF2_MPNN_MMA=sync: mma.sync)
    Graph graph() const { return Graph{ n, mesh->rowptr.p, mesh->col.p, dinv.p }; }
    float* Hl(int l) { return H.p + (size_t)l * n * MH; }
    float* Ml(int l) { return M.p + (size_t)l * n * MH; }
    unsigned long long* maskl(int l) { return mask.p + (size_t)l * n; }
};

namespace pf2 {

// Sections: the parameter count, the FP32 parameters, the AdamW moments and step count.
// The BF16 weight copies follow from the parameters and are rebuilt on reading.
pf2_status mpnn_checkpoint(pf2_mpnn* N, CkptFile& io, cudaStream_t st) {
    int meta[2] = { kParams, N->step };
    PF2_TRY(io.host("nmeta", meta, sizeof(meta)));
    PF2_REQUIRE(meta[0] == kParams, PF2_BAD_INPUT, "checkpoint network has %d parameters, this one %d", meta[0],
                kParams);
    PF2_TRY(io.device("nparams", N->P.p, sizeof(float) * kParams, st));
    PF2_TRY(io.device("nadam_m", N->am.p, sizeof(float) * kParams, st));
    PF2_TRY(io.device("nadam_v", N->av.p, sizeof(float) * kParams, st));
    if (!io.writing()) {
        N->step = meta[1];
        k_weights_bf16<<<blocks_for(ML * MH * MK), kThreads, 0, st>>>(N->P.p, N->Wb.p);
        PF2_LAUNCH_CHECK();
        PF2_CUDA(cudaStreamSynchronize(st));
    }
    return PF2_OK;
}

static pf2_status mpnn_forward(pf2_mpnn* N, cudaStream_t st) {
    const Graph G = N->graph();
    k_mpnn_encoder<<<blocks_for(N->n), kThreads, 0, st>>>(G, N->feat.p, N->P.p, N->Hl(0), N->maskl(0));
    PF2_LAUNCH_CHECK();
    const unsigned tiles = blocks_for(N->n, kTile);
    for (int l = 0; l < ML; ++l) {
        if (N->tc)
            k_mpnn_layer_tc<<<blocks_for(N->n, kTcTile), 128, kTcSmem, st>>>(
                G, N->Hl(l), N->Wb.p + (size_t)l * MH * MK, N->P.p + kParamLayer0 + l * kLayerSize + MH * MK,
                N->Hl(l + 1), N->Ml(l), N->maskl(l + 1), N->err.p);
        else
            k_mpnn_layer<<<tiles, kMpnnThreads, 0, st>>>(G, N->Hl(l), N->Wb.p + (size_t)l * MH * MK,
                                                         N->P.p + kParamLayer0 + l * kLayerSize + MH * MK,
                                                         N->Hl(l + 1), N->Ml(l), N->maskl(l + 1));
        PF2_LAUNCH_CHECK();
    }
    return PF2_OK;
}

static pf2_status mpnn_backward(pf2_mpnn* N, cudaStream_t st) {
    const Graph G = N->graph();
    const unsigned nb = blocks_for(N->n, kMpnnThreads);
    k_mpnn_decoder_back<<<nb, kMpnnThreads, 0, st>>>(N->n, N->Hl(ML), N->P.p, N->dy.p, N->dH.p, N->part.p);
    PF2_LAUNCH_CHECK();
    k_reduce_cols<<<blocks_for(MH + 1), kThreads, 0, st>>>(N->part.p, (int)nb, MH + 1, N->grad.p, kParamW4);
    PF2_LAUNCH_CHECK();
    const unsigned tiles = blocks_for(N->n, kTile);
    float* dh = N->dH.p;
    float* dh2 = N->dH2.p;
    for (int l = ML - 1; l >= 0; --l) {
        const __nv_bfloat16* W = N->Wb.p + (size_t)l * MH * MK;
        if (N->tc)
            k_mpnn_layer_back_weights_tc<<<N->wgrid, 128, kTcSmem, st>>>(G, N->Hl(l), N->Ml(l), dh, N->maskl(l + 1),
                                                                         N->part.p, N->err.p);
        else
            k_mpnn_layer_back_weights<<<N->wgrid, kMpnnThreads, 0, st>>>(G, N->Hl(l), N->Ml(l), dh,
                                                                         N->maskl(l + 1), N->part.p);
        PF2_LAUNCH_CHECK();
        k_reduce_cols<<<blocks_for(kLayerSize), kThreads, 0, st>>>(N->part.p, N->wgrid, kLayerSize, N->grad.p,
                                                                   kParamLayer0 + l * kLayerSize);
        PF2_LAUNCH_CHECK();
        if (N->tc)
            k_mpnn_layer_back_nodes_tc<<<blocks_for(N->n, kTcTile), 128, kTcBnSmem, st>>>(
                G, dh, N->maskl(l + 1), W, N->dSelf.p, N->dMs.p, N->err.p);
        else
            k_mpnn_layer_back_nodes<<<tiles, kMpnnThreads, 0, st>>>(G, dh, N->maskl(l + 1), W, N->dSelf.p,
                                                                    N->dMs.p);
        PF2_LAUNCH_CHECK();
        k_mpnn_agg_back<<<blocks_for((long long)N->n * MH), kThreads, 0, st>>>(G, dh, N->dSelf.p, N->dMs.p, dh2);
        PF2_LAUNCH_CHECK();
        std::swap(dh, dh2);
    }
    k_mpnn_encoder_back<<<N->wgrid, kThreads, 0, st>>>(N->n, N->feat.p, dh, N->maskl(0), N->part.p);
    PF2_LAUNCH_CHECK();
    k_reduce_cols<<<blocks_for(MH * MIN + MH), kThreads, 0, st>>>(N->part.p, N->wgrid, MH * MIN + MH, N->grad.p,
                                                                  kParamW0);
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

}  // namespace pf2

extern "C" {

pf2_status pf2_mpnn_create(const pf2_mesh* mesh, unsigned long long seed, pf2_mpnn** out) {
    PF2_REQUIRE(mesh && out, PF2_BAD_INPUT, "null argument");
    *out = nullptr;
    pf2_mpnn* N = new pf2_mpnn();
    N->mesh = mesh;
    N->n = mesh->nv;
    const size_t n = N->n;
    auto fail = [&](pf2_status s) { delete N; return s; };
    N->wgrid = std::max(1, std::min((int)blocks_for(N->n, kTile), num_sms() * 2));
    const size_t part = std::max<size_t>((size_t)N->wgrid * (MH * MK + MH),
                                         (size_t)blocks_for(N->n, kMpnnThreads) * (MH + 1));
    pf2_status s;
    if ((s = N->P.alloc(kParams)) || (s = N->grad.alloc(kParams)) || (s = N->am.alloc(kParams)) ||
        (s = N->av.alloc(kParams)) || (s = N->dinv.alloc(n)) || (s = N->feat.alloc(n * MIN)) ||
        (s = N->y.alloc(n)) || (s = N->dy.alloc(n)) || (s = N->target.alloc(n)) ||
        (s = N->H.alloc((ML + 1) * n * MH)) || (s = N->M.alloc(ML * n * MH)) || (s = N->dH.alloc(n * MH)) ||
        (s = N->dH2.alloc(n * MH)) || (s = N->dSelf.alloc(n * MH)) || (s = N->dMs.alloc(n * MH)) ||
        (s = N->part.alloc(part)) || (s = N->mask.alloc((ML + 1) * n)) || (s = N->Wb.alloc(ML * MH * MK)) ||
        (s = N->loss_part.alloc(blocks_for(N->n))) || (s = N->err.alloc(1)))
        return fail(s);
    if (const char* e = getenv("PF2_MPNN_MMA")) N->tc = strcmp(e, "sync") != 0;
    if (cudaMemset(N->err.p, 0, sizeof(int)) != cudaSuccess ||
        cudaFuncSetAttribute((void*)k_mpnn_layer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem) !=
            cudaSuccess ||
        cudaFuncSetAttribute((void*)k_mpnn_layer_back_nodes_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kTcBnSmem) != cudaSuccess ||
        cudaFuncSetAttribute((void*)k_mpnn_layer_back_weights_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kTcSmem) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "mpnn set-up", __FILE__, __LINE__));
    // He-style initialisation from a splitmix64 stream (deterministic for a seed);
    // the output layer starts at zero so the untrained guess is the extrapolation alone
    std::vector<float> h(kParams, 0.0f);
    unsigned long long st = seed;
    auto next = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        unsigned long long z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    };
    for (int k = 0; k < MH * MIN; ++k) h[kParamW0 + k] = (float)(next() * std::sqrt(6.0 / MIN));
    for (int l = 0; l < ML; ++l)
        for (int k = 0; k < MH * MK; ++k)
            h[kParamLayer0 + l * kLayerSize + k] = (float)(next() * std::sqrt(6.0 / MK) * 0.5);
    if (cudaMemcpy(N->P.p, h.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(N->am.p, 0, sizeof(float) * kParams) != cudaSuccess ||
        cudaMemset(N->av.p, 0, sizeof(float) * kParams) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "mpnn init", __FILE__, __LINE__));
    k_deg_inv<<<blocks_for(N->n), kThreads>>>(N->n, mesh->rowptr.p, mesh->col.p, N->dinv.p);
    k_weights_bf16<<<blocks_for(ML * MH * MK), kThreads>>>(N->P.p, N->Wb.p);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(cuda_fail(cudaGetLastError(), "mpnn init", __FILE__, __LINE__));
    *out = N;
    return PF2_OK;
}

pf2_status pf2_mpnn_destroy(pf2_mpnn* N) {
    delete N;
    return PF2_OK;
}

int pf2_mpnn_param_count(void) { return kParams; }

pf2_status pf2_mpnn_save(const pf2_mpnn* N, const char* path) {
    PF2_REQUIRE(N && path, PF2_BAD_INPUT, "null argument");
    CkptFile io;
    PF2_TRY(io.open_write(path, CKPT_MPNN));
    PF2_TRY(mpnn_checkpoint(const_cast<pf2_mpnn*>(N), io, nullptr));
    return io.close();
}

pf2_status pf2_mpnn_load(pf2_mpnn* N, const char* path) {
    PF2_REQUIRE(N && path, PF2_BAD_INPUT, "null argument");
    CkptFile io;
    PF2_TRY(io.open_read(path, CKPT_MPNN));
    PF2_TRY(mpnn_checkpoint(N, io, nullptr));
    return io.close();
}

pf2_status pf2_mpnn_set_params(pf2_mpnn* N, const float* params_host) {
    PF2_REQUIRE(N && params_host, PF2_BAD_INPUT, "null argument");
    PF2_CUDA(cudaMemcpy(N->P.p, params_host, sizeof(float) * kParams, cudaMemcpyHostToDevice));
    k_weights_bf16<<<blocks_for(ML * MH * MK), kThreads>>>(N->P.p, N->Wb.p);
    PF2_LAUNCH_CHECK();
    PF2_CUDA(cudaDeviceSynchronize());
    return PF2_OK;
}

pf2_status pf2_mpnn_get_params(const pf2_mpnn* N, float* params_host, float* grad_host) {
    PF2_REQUIRE(N, PF2_BAD_INPUT, "null argument");
    PF2_CUDA(cudaDeviceSynchronize());
    int e = 0;
    PF2_CUDA(cudaMemcpy(&e, N->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    PF2_REQUIRE(e == 0, (pf2_status)e, "a tensor-core wait timed out in the network's forward pass");
    if (params_host) PF2_CUDA(cudaMemcpy(params_host, N->P.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
    if (grad_host) PF2_CUDA(cudaMemcpy(grad_host, N->grad.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
    return PF2_OK;
}

pf2_status pf2_mpnn_forward(pf2_mpnn* N, const float* feat_dev, float* y_dev, void* stream) {
    PF2_REQUIRE(N && feat_dev && y_dev, PF2_BAD_INPUT, "null argument");
    cudaStream_t st = as_stream(stream);
    PF2_CUDA(cudaMemcpyAsync(N->feat.p, feat_dev, sizeof(float) * MIN * (size_t)N->n, cudaMemcpyDeviceToDevice, st));
    PF2_TRY(mpnn_forward(N, st));
    k_mpnn_decoder<<<blocks_for(N->n), kThreads, 0, st>>>(N->n, N->Hl(ML), N->P.p, y_dev, nullptr, nullptr, nullptr);
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

pf2_status pf2_mpnn_train_step(pf2_mpnn* N, const float* feat_dev, const float* target_dev, float lr, int apply,
                               double* loss_host, void* stream) {
    PF2_REQUIRE(N && feat_dev && target_dev, PF2_BAD_INPUT, "null argument");
    cudaStream_t st = as_stream(stream);
    PF2_CUDA(cudaMemcpyAsync(N->feat.p, feat_dev, sizeof(float) * MIN * (size_t)N->n, cudaMemcpyDeviceToDevice, st));
    PF2_CUDA(cudaMemcpyAsync(N->target.p, target_dev, sizeof(float) * (size_t)N->n, cudaMemcpyDeviceToDevice, st));
    PF2_TRY(mpnn_forward(N, st));
    k_mpnn_decoder<<<blocks_for(N->n), kThreads, 0, st>>>(N->n, N->Hl(ML), N->P.p, N->y.p, N->target.p, N->dy.p,
                                                         N->loss_part.p);
    PF2_LAUNCH_CHECK();
    PF2_TRY(mpnn_backward(N, st));
    if (apply) {
        ++N->step;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.0f - std::pow(b1, (float)N->step), c2 = 1.0f - std::pow(b2, (float)N->step);
        k_adamw<<<blocks_for(kParams), kThreads, 0, st>>>(kParams, N->P.p, N->grad.p, N->am.p, N->av.p, c1, c2, lr,
                                                          b1, b2, 1e-8f, 0.01f);
        PF2_LAUNCH_CHECK();
        k_weights_bf16<<<blocks_for(ML * MH * MK), kThreads, 0, st>>>(N->P.p, N->Wb.p);
        PF2_LAUNCH_CHECK();
    }
    if (loss_host) {
        std::vector<double> lp(blocks_for(N->n));
        PF2_CUDA(cudaMemcpyAsync(lp.data(), N->loss_part.p, sizeof(double) * lp.size(), cudaMemcpyDeviceToHost, st));
        PF2_CUDA(cudaStreamSynchronize(st));
        double s = 0.0;
        for (double v : lp) s += v;
        *loss_host = s / N->n;
    }
    return PF2_OK;
}

}  // extern "C"
