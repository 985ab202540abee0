// particles.cu - ParticleHandler2D on the device.
//
// Reference: src/particles/particle_handler_2d.cu.  The state is SoA (x, y, l0, l1, u,
// v: double; a cell word: int) and is kept ordered by cell.  One step of
// advectParticles becomes:
//   k_advect   - every substep of every particle in registers: advection, location
//                (own cell, then neighbours in ascending order), deletion mark; then a
//                per-cell particle count (atomic rank) and sub-cell occupancy bits;
//   scan       - segment of each cell = particles + empty sub-cells (reseeds);
//   k_scatter  - old index of each particle into its cell's segment;
//   k_gather   - per cell: restore the old order inside the segment (stable sort),
//                move the particles, append reseeded particles in sub-cell order, and
//                form the cell's projection partial sums.
// projectVelocityOntoGrid then only gathers the partial sums of the cells around each
// node (k_project_nodes): no atomics, and the result does not depend on timing.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "device.cuh"
#include "internal.cuh"

namespace pf2 {

struct Centers {
    double c[kMaxPerCell][3];
};

struct PState {
    double *x, *y, *l0, *l1, *u, *v;
    int* cw;
};

__device__ __forceinline__ double third_coord(int cw, double l0, double l1, const Centers& C) {
    const unsigned f = ((unsigned)cw) >> kCellBits;
    return f ? C.c[f - 1][2] : __dsub_rn(__dsub_rn(1.0, l0), l1);
}

// ParticleHandler2D::seedParticles / kSeedParticlesIntoCell (:35-52, :304-320)
__global__ void k_seed(int nc, int ppc, Centers C, const double2* __restrict__ xy, const int4* __restrict__ tri,
                       PState P, int* seg) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long long)nc * ppc) return;
    const int c = (int)(g / ppc), k = (int)(g % ppc);
    const int4 t = tri[c];
    const double2 A = xy[t.x], B = xy[t.y], D = xy[t.z];
    P.x[g] = local_to_global(C.c[k][0], C.c[k][1], C.c[k][2], A.x, B.x, D.x);
    P.y[g] = local_to_global(C.c[k][0], C.c[k][1], C.c[k][2], A.y, B.y, D.y);
    P.l0[g] = C.c[k][0];
    P.l1[g] = C.c[k][1];
    P.u[g] = 0.0;
    P.v[g] = 0.0;
    P.cw[g] = c | ((k + 1) << kCellBits);
    if (k == 0) seg[c] = (int)g;
    if (g == 0) seg[nc] = nc * ppc;
}

struct MeshRefs {
    const int4* tri;
    const double4_32a* invJ;
    const double2* v3;
    const float4* invJf;
    const float2* v3f;
    const int* nb_off;
    const int* nb_idx;
    const double2* xy;
    int nc;
};

// Per-warp scratch of the warp-cooperative cell location in k_advect.
constexpr int kSearchCap = 64;  // candidate cells a warp tests together per substep
struct SearchBuf {
    double x[32], y[32];          // the searching lanes' positions
    double l[kSearchCap][3];      // a candidate's barycentric coordinates, when it holds the point
    int nb[kSearchCap];           // candidate cell
    int k[kSearchCap];            // its position in its lane's neighbour list
    int owner[kSearchCap];        // the lane searching it
    int best[32];                 // per lane: the lowest position that holds the point
    int win[32];                  // per lane: the candidate at that position
    int count;
};

// kAdvectParticles (:54-70) for every substep, the location of sortParticlesInCells
// (:363-395, kernels :117-162) after each, and kCountParticlesInSubcells (:173-181).
// Warps stride over the particles together so that the ranks of particles that land in
// the same cell come from one atomic per cell and warp (the order of ranks is free: the
// gather restores the old order).  The lanes of a warp take the substeps together: after
// each, the particles that left their cell are located by the whole warp.  Each such lane
// walks its cell's neighbours in order through the FP32 pre-filter (FP32 pipe) and
// appends the survivors to the warp's list; then every lane tests one candidate with the
// FP64 transform, so one pass of FP64 instructions serves up to 32 candidates of any
// lanes (a lane searching alone through its neighbours would issue the FP64 transform for
// each of its candidates with the other 31 lanes idle: GB300 issues an FP64 warp
// instruction at the same cost whatever its active lanes).  A lane's cell is its
// lowest-positioned candidate that holds the point: the first one the reference's
// sequential search finds, with the same FP64 arithmetic, so the result is bit-identical.
// A lane whose candidates do not fit the list searches sequentially.
__global__ void __launch_bounds__(256) k_advect(const int* __restrict__ np_ptr, int substeps, double dts, Centers C,
                                                MeshRefs M, const double* __restrict__ ux,
                                                const double* __restrict__ uy, PState P, int* count, int* mask,
                                                int* rank, int level, double step) {
    __shared__ SearchBuf sbuf[8];
    SearchBuf& B = sbuf[threadIdx.x >> 5];
    const int np = *np_ptr;
    const int ppc = level * level;
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long wb = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31); wb < np; wb += stride) {
        const int p = (int)(wb + lane);
        int key = -1;  // cell the particle ends in, -1 if none
        int sub = 0;
        const int cw = p < np ? P.cw[p] : -1;
        const bool valid = cw >= 0;
        int c = cw & kCellMask;
        double l0 = 0.0, l1 = 0.0, l2 = 0.0, x = 0.0, y = 0.0;
        if (valid) {
            l0 = P.l0[p];
            l1 = P.l1[p];
            l2 = third_coord(cw, l0, l1, C);
            x = P.x[p];
            y = P.y[p];
        }
        bool lost = false;
        for (int s = 0; s < substeps; ++s) {
            const bool act = valid && !lost;
            double n0 = 0.0, n1 = 0.0, n2 = 0.0;
            bool need = false;
            if (act) {
                const int4 t = M.tri[c];
                const double vx = interp3(l0, l1, l2, __ldg(&ux[t.x]), __ldg(&ux[t.y]), __ldg(&ux[t.z]));
                const double vy = interp3(l0, l1, l2, __ldg(&uy[t.x]), __ldg(&uy[t.y]), __ldg(&uy[t.z]));
                x = __fma_rn(vx, dts, x);
                y = __fma_rn(vy, dts, y);
                global_to_local(x, y, M.invJ[c], M.v3[c], n0, n1, n2);
                need = !inside_unit(n0, n1, n2);
            }
            if (__ballot_sync(0xffffffffu, need)) {
                if (lane == 0) B.count = 0;
                B.best[lane] = INT_MAX;
                __syncwarp();
                bool overflow = false;
                int o = 0, e = 0;
                if (need) {
                    B.x[lane] = x;
                    B.y[lane] = y;
                    o = M.nb_off[c];
                    e = M.nb_off[c + 1];
                    const float xf = (float)x, yf = (float)y;
                    for (int k = o; k < e; ++k) {
                        const int nb = M.nb_idx[k];
                        if (!maybe_inside_f32(xf, yf, M.invJf[nb], M.v3f[nb])) continue;
                        const int slot = atomicAdd(&B.count, 1);
                        if (slot < kSearchCap) {
                            B.nb[slot] = nb;
                            B.k[slot] = k;
                            B.owner[slot] = lane;
                        } else {
                            overflow = true;
                        }
                    }
                }
                __syncwarp();
                const int total = min(B.count, kSearchCap);
                for (int base = 0; base < total; base += 32) {
                    const int i = base + lane;
                    if (i < total) {
                        const int ow = B.owner[i], nb = B.nb[i];
                        double m0, m1, m2;
                        global_to_local(B.x[ow], B.y[ow], M.invJ[nb], M.v3[nb], m0, m1, m2);
                        if (inside_unit(m0, m1, m2)) {
                            B.l[i][0] = m0;
                            B.l[i][1] = m1;
                            B.l[i][2] = m2;
                            atomicMin(&B.best[ow], B.k[i]);
                        }
                    }
                }
                __syncwarp();
                for (int base = 0; base < total; base += 32) {
                    const int i = base + lane;
                    if (i < total && B.k[i] == B.best[B.owner[i]]) B.win[B.owner[i]] = i;
                }
                __syncwarp();
                if (need) {
                    if (overflow) {
                        // more candidates than the list holds: this lane's own search, in order
                        const float xf = (float)x, yf = (float)y;
                        int found = -1;
                        for (int k = o; k < e; ++k) {
                            const int nb = M.nb_idx[k];
                            if (!maybe_inside_f32(xf, yf, M.invJf[nb], M.v3f[nb])) continue;
                            global_to_local(x, y, M.invJ[nb], M.v3[nb], n0, n1, n2);
                            if (inside_unit(n0, n1, n2)) { found = nb; break; }
                        }
                        if (found < 0) lost = true;
                        else c = found;
                    } else if (B.best[lane] == INT_MAX) {
                        lost = true;
                    } else {
                        const int i = B.win[lane];
                        c = B.nb[i];
                        n0 = B.l[i][0];
                        n1 = B.l[i][1];
                        n2 = B.l[i][2];
                    }
                }
                __syncwarp();  // the list is rebuilt at the next substep
            }
            if (act && !lost) {
                l0 = n0;
                l1 = n1;
                l2 = n2;
            }
        }
        if (valid) {
            P.x[p] = x;
            P.y[p] = y;
            P.l0[p] = l0;
            P.l1[p] = l1;
            if (lost) {
                P.cw[p] = -1;
            } else {
                // a located particle loses its centroid flag; with no substeps it keeps it
                P.cw[p] = substeps > 0 ? c : cw;
                key = c;
                sub = determine_subcell(level, step, l0, l1, l2);
            }
        }
        // one atomic per (warp, cell); each lane's rank = group base + lanes below it
        const unsigned grp = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(grp) - 1;
        int base = 0;
        if (lane == leader && key >= 0) base = atomicAdd(&count[key], __popc(grp));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (p < np) rank[p] = key >= 0 ? base + __popc(grp & ((1u << lane) - 1u)) : -1;
        if (key >= 0) {
            const int tc = key + sub / ppc;
            if (tc < M.nc) atomicOr(&mask[tc], 1 << (sub % ppc));
        }
    }
}

// Count and rank of an arbitrary particle order (upload, or a sort without advection).
__global__ void k_rank_only(const int* __restrict__ np_ptr, const int* __restrict__ cw, int* count, int* rank) {
    const int np = *np_ptr;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int w = cw[p];
        rank[p] = (w < 0) ? -1 : atomicAdd(&count[w & kCellMask], 1);
    }
}

__global__ void k_seg_sizes(int nc, const int* __restrict__ count, const int* __restrict__ mask, int ppc, int reseed,
                            int* sz) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const unsigned full = (ppc >= 32) ? 0xffffffffu : ((1u << ppc) - 1u);
    sz[c] = count[c] + (reseed ? ppc - __popc((unsigned)mask[c] & full) : 0);
}

__global__ void k_set_count(const int* __restrict__ seg, int nc, long long cap, int* cnt, int* err) {
    const int total = seg[nc];
    if (total > cap) {
        atomicExch(err, (int)DEV_OVERFLOW);
        cnt[1] = (int)cap;
    } else {
        cnt[1] = total;
    }
}

__global__ void k_scatter(const int* __restrict__ np_ptr, const int* __restrict__ cw, const int* __restrict__ rank,
                          const int* __restrict__ seg, int* perm, long long cap) {
    const int np = *np_ptr;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int w = cw[p];
        if (w < 0) continue;
        const long long slot = (long long)seg[w & kCellMask] + rank[p];
        if (slot < cap) perm[slot] = p;
    }
}

struct Partials {
    double* s;  // 9 arrays of nc: (sum L u, sum L v, sum L) for local vertices 0, 1, 2
    int nc;
};

// The nine projection partial sums of a block's eight cells c0 .. c0 + 7, cell i holding
// slots [bs[i], bs[i] + bn[i]) of S (bn[i] < 0: the cell is skipped, no sums written):
// for each cell (sum L0 u, sum L0 v, sum L0, the same for L1 and L2), the sums of
// kProjectParticleVelocityOntoGrid (particle_handler_2d.cu:90-107) gathered per cell.  Thread
// t < 216 forms one value over one third of one cell's slots, in slot order, one fused
// multiply-add per slot (by 1.0 for the coordinate alone), and the three thirds are
// added in order: all lanes of seven warps stay busy however many particles a cell has
// (a warp per cell with lane j taking slots j, j + 32, ... idles most lanes of its
// second pass at ~36 particles per cell, and every FP64 instruction costs the same
// issue slot whatever its active lanes).  The cells' slots are contiguous; when they
// fit kStageSlots they are first staged in shared memory by coalesced loads, L2 formed
// once per slot, else the threads read them from S (same arithmetic, same bits).  Every
// thread of the block calls it; S must be written before the call by this block or an
// earlier kernel.  k_gather and k_partials both go through here, so a projection gives
// the same bits whichever formed its sums.
constexpr int kStageSlots = 512;
struct PartialStage {
    double l[3][kStageSlots];
    double u[kStageSlots], v[kStageSlots];
    double third[216];
    int bs[8], bn[8];
};

__device__ __forceinline__ void block_partials(PartialStage& G, int c0, int nc, PState S, const Centers& C,
                                               Partials part) {
    const int t = threadIdx.x;
    __syncthreads();  // bs, bn and the block's slots are in place
    const int S0 = G.bs[0];
    int total = 0;
    bool contiguous = true;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        if (c0 + i >= nc) break;
        if (G.bn[i] < 0 || G.bs[i] != S0 + total) contiguous = false;
        total += max(G.bn[i], 0);
    }
    const bool staged = contiguous && total <= kStageSlots;  // uniform over the block
    if (staged) {
        for (int k = t; k < total; k += blockDim.x) {
            const int o = S0 + k;
            const int w = S.cw[o];
            const double l0 = S.l0[o], l1 = S.l1[o];
            G.l[0][k] = l0;
            G.l[1][k] = l1;
            G.l[2][k] = third_coord(w, l0, l1, C);
            G.u[k] = S.u[o];
            G.v[k] = S.v[o];
        }
    }
    __syncthreads();
    // thread t: coordinate a (grouped so that the L2 threads of the unstaged path share
    // warps), cell i, factor j (u, v, 1), third q
    const int a = t / 72, rem = t % 72, i = rem / 9, j = (rem % 9) / 3, q = rem % 3;
    double acc = 0.0;
    if (t < 216) {
        const int n = G.bn[i];
        if (c0 + i < nc && n > 0) {
            const int lo = q * n / 3, hi = (q + 1) * n / 3;
            if (staged) {
                const int base = G.bs[i] - S0;
                const double* L = G.l[a] + base;
                const double* W = (j == 0 ? G.u : G.v) + base;
                for (int k = lo; k < hi; ++k) acc = __fma_rn(L[k], j < 2 ? W[k] : 1.0, acc);
            } else {
                const int base = G.bs[i];
                const double* W = j == 0 ? S.u : S.v;
                for (int k = lo; k < hi; ++k) {
                    const int o = base + k;
                    const double l0 = S.l0[o], l1 = S.l1[o];
                    const double lv = a == 0 ? l0 : (a == 1 ? l1 : third_coord(S.cw[o], l0, l1, C));
                    acc = __fma_rn(lv, j < 2 ? W[o] : 1.0, acc);
                }
            }
        }
        G.third[t] = acc;
    }
    __syncthreads();
    if (t < 216 && q == 0 && c0 + i < nc && G.bn[i] >= 0)
        part.s[(size_t)(3 * a + j) * part.nc + c0 + i] =
            __dadd_rn(__dadd_rn(G.third[t], G.third[t + 1]), G.third[t + 2]);
}

// Per cell, one warp: stable order, move, reseed (kAddParticlesToCell :197-236); then the
// block's partial sums.  The cell's particles arrive in perm[s, s + n) in the order the
// atomics handed out ranks; each lane ranks its particle by old index against all n (the
// old order is the order the cell keeps), moves it to slot s + rank, then lanes fill the
// missing sub-cells after them.  The partial sums are formed over the slots after the
// moves, so they do not depend on the atomics' order.
__global__ void __launch_bounds__(256, 5) k_gather(int nc, const int* __restrict__ seg, int* count, int* mask,
                                                const int* __restrict__ perm, PState S, PState D, Centers C,
                                                int level, int reseed, const double2* __restrict__ xy,
                                                const int4* __restrict__ tri, const double* __restrict__ ux,
                                                const double* __restrict__ uy, Partials part, long long cap,
                                                int* cnt) {
    __shared__ PartialStage G;
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const int c0 = blockIdx.x * 8;
    const int c = c0 + wi;
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt[0] = cnt[1];
    const int ppc = level * level;
    int s = 0, n = 0, nadd = 0;
    unsigned m = 0;
    bool fits = false;
    if (c < nc) {  // uniform over the warp
        s = seg[c];
        n = count[c];
        m = (unsigned)mask[c];
        __syncwarp();
        if (lane == 0) {
            count[c] = 0;
            mask[c] = 0;
        }
        const unsigned full = (1u << ppc) - 1u;
        nadd = reseed ? ppc - __popc(m & full) : 0;
        fits = (long long)s + n + nadd <= cap;
    }
    if (lane == 0) {
        G.bs[wi] = s;
        G.bn[wi] = fits ? n + nadd : -1;
    }
    if (fits) {
        // existing particles: lane handles entries base + lane of perm[s, s + n)
        for (int base = 0; base < n; base += 32) {
            const int i = base + lane;
            const int v = i < n ? perm[s + i] : 0x7fffffff;
            int r = 0;
            for (int cb = 0; cb < n; cb += 32) {
                const int w = cb + lane < n ? perm[s + cb + lane] : 0x7fffffff;
                const int lim = min(32, n - cb);
                for (int j = 0; j < lim; ++j) r += (__shfl_sync(0xffffffffu, w, j) < v) ? 1 : 0;
            }
            if (i < n) {
                const int o = s + r;
                D.x[o] = S.x[v];
                D.y[o] = S.y[v];
                D.l0[o] = S.l0[v];
                D.l1[o] = S.l1[v];
                D.u[o] = S.u[v];
                D.v[o] = S.v[v];
                D.cw[o] = S.cw[v];
            }
        }
        // reseed: the q-th missing sub-cell goes to slot s + n + q
        if (nadd) {
            const int4 t = tri[c];
            const double2 A = xy[t.x], B = xy[t.y], E = xy[t.z];
            const double u0 = ux[t.x], u1 = ux[t.y], u2 = ux[t.z];
            const double w0 = uy[t.x], w1 = uy[t.y], w2 = uy[t.z];
            const unsigned missing = ~m & ((1u << ppc) - 1u);
            for (int q = lane; q < nadd; q += 32) {
                const int k = (int)__fns(missing, 0, q + 1);
                const int o = s + n + q;
                const double L0 = C.c[k][0], L1 = C.c[k][1], L2 = C.c[k][2];
                D.x[o] = local_to_global(L0, L1, L2, A.x, B.x, E.x);
                D.y[o] = local_to_global(L0, L1, L2, A.y, B.y, E.y);
                D.l0[o] = L0;
                D.l1[o] = L1;
                D.u[o] = interp3(L0, L1, L2, u0, u1, u2);
                D.v[o] = interp3(L0, L1, L2, w0, w1, w2);
                D.cw[o] = c | ((k + 1) << kCellBits);
            }
        }
    }
    block_partials(G, c0, nc, D, C, part);
}

// Partial sums of every cell from the current (cell-ordered) particles, eight cells per
// block as in k_gather, so a projection gives the same bits whether its partial sums
// came from the sort or from here.
__global__ void __launch_bounds__(256) k_partials(int nc, const int* __restrict__ seg, PState S, Centers C,
                                                  Partials part) {
    __shared__ PartialStage G;
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const int c0 = blockIdx.x * 8;
    const int c = c0 + wi;
    if (lane == 0) {
        G.bs[wi] = c < nc ? seg[c] : 0;
        G.bn[wi] = c < nc ? seg[c + 1] - seg[c] : -1;
    }
    block_partials(G, c0, nc, S, C, part);
}

// kFinalizeVelocityProjection (:109-115): u_i = sum L v / sum L over the cells around
// node i; optionally also the copy u -> u_old of the step (Cylinder2D/main.cu:805-806).
__global__ void k_project_nodes(int nv, const int* __restrict__ inc_off, const int* __restrict__ inc, Partials part,
                                double* ux, double* uy, double* uxo, double* uyo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    double sx = 0.0, sy = 0.0, w = 0.0;
    for (int q = inc_off[i]; q < inc_off[i + 1]; ++q) {
        const int e = inc[q], c = e >> 2, lv = e & 3;
        sx += part.s[(size_t)(3 * lv) * part.nc + c];
        sy += part.s[(size_t)(3 * lv + 1) * part.nc + c];
        w += part.s[(size_t)(3 * lv + 2) * part.nc + c];
    }
    const double a = sx / w, b = sy / w;
    ux[i] = a;
    uy[i] = b;
    if (uxo) { uxo[i] = a; uyo[i] = b; }
}

// kCorrectParticleVelocity (:72-88); old == nullptr gives initParticleVelocity.
__global__ void k_correct(const int* __restrict__ np_ptr, PState P, Centers C, const int4* __restrict__ tri,
                          const double* __restrict__ ux, const double* __restrict__ uy,
                          const double* __restrict__ uxo, const double* __restrict__ uyo) {
    const int np = *np_ptr;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int w = P.cw[p];
        if (w < 0) continue;
        const int4 t = tri[w & kCellMask];
        const double l0 = P.l0[p], l1 = P.l1[p], l2 = third_coord(w, l0, l1, C);
        double dx0 = ux[t.x], dx1 = ux[t.y], dx2 = ux[t.z];
        double dy0 = uy[t.x], dy1 = uy[t.y], dy2 = uy[t.z];
        if (uxo) {
            dx0 = __dsub_rn(dx0, uxo[t.x]); dx1 = __dsub_rn(dx1, uxo[t.y]); dx2 = __dsub_rn(dx2, uxo[t.z]);
            dy0 = __dsub_rn(dy0, uyo[t.x]); dy1 = __dsub_rn(dy1, uyo[t.y]); dy2 = __dsub_rn(dy2, uyo[t.z]);
        }
        P.u[p] = __dadd_rn(P.u[p], interp3(l0, l1, l2, dx0, dx1, dx2));
        P.v[p] = __dadd_rn(P.v[p], interp3(l0, l1, l2, dy0, dy1, dy2));
    }
}

}  // namespace pf2

using namespace pf2;

struct pf2_particles {
    const pf2_mesh* mesh = nullptr;
    int level = 0, ppc = 0;
    double step = 0.0;
    long long cap = 0;
    Centers C{};
    DevBuf<double> buf[2][6];
    DevBuf<int> cw[2];
    int cur = 0;
    DevBuf<int> rank, perm, count, mask, seg, segsz, scratch, cnt, err;
    DevBuf<double> part;
    PinnedBuf<int> h_cnt;
    bool partials_valid = false;
    bool seeded = false;

    PState state(int k) {
        return PState{ buf[k][0].p, buf[k][1].p, buf[k][2].p, buf[k][3].p, buf[k][4].p, buf[k][5].p, cw[k].p };
    }
};

namespace pf2 {

// ParticleHandler2D::ParticleHandler2D (:238-294): sub-triangle centroids of a cell
// divided into level^2 triangles, rows from the top; computed on the host as there.
static void subcell_centers(int n, Centers& C) {
    const double dx = 1.0 / n;
    int k = 0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 2 * i + 1; ++j) {
            const double xmin = (j / 2) * dx, xmax = xmin + dx;
            const double ymin = (n - 1 - i) * dx, ymax = ymin + dx;
            const double v0[3] = { xmin, ymax, 1.0 - xmin - ymax };
            double v1[3];
            v1[0] = (j % 2 == 0) ? xmin : xmax;
            v1[1] = (j % 2 == 0) ? ymin : ymax;
            v1[2] = 1.0 - v1[0] - v1[1];
            const double v2[3] = { xmax, ymin, 1.0 - xmax - ymin };
            for (int a = 0; a < 3; ++a) C.c[k][a] = 0.3333333333333333 * ((v0[a] + v1[a]) + v2[a]);
            ++k;
        }
}

static MeshRefs mesh_refs(const pf2_mesh* m) {
    return MeshRefs{ m->tri4.p, m->invJ.p, m->v3.p, m->invJf.p, m->v3f.p, m->nb_off.p, m->nb_idx.p, m->xy.p, m->nc };
}

static unsigned particle_grid() { return (unsigned)(num_sms() * 8); }

// Sort (and optionally reseed) the particles of buffer `cur` into the other buffer.
// `ranked`: counts and ranks are already set (by k_advect).
static pf2_status sort_cells(pf2_particles* H, bool ranked, bool reseed, const double* ux, const double* uy,
                             cudaStream_t st) {
    const pf2_mesh* M = H->mesh;
    const int nc = M->nc;
    if (!ranked) {
        k_rank_only<<<particle_grid(), kThreads, 0, st>>>(H->cnt.p, H->cw[H->cur].p, H->count.p, H->rank.p);
        PF2_LAUNCH_CHECK();
    }
    k_seg_sizes<<<blocks_for(nc), kThreads, 0, st>>>(nc, H->count.p, H->mask.p, H->ppc, reseed ? 1 : 0, H->segsz.p);
    PF2_LAUNCH_CHECK();
    PF2_TRY(exclusive_scan(H->segsz.p, H->seg.p, nc, H->scratch.p, st));
    k_set_count<<<1, 1, 0, st>>>(H->seg.p, nc, H->cap, H->cnt.p, H->err.p);
    PF2_LAUNCH_CHECK();
    k_scatter<<<particle_grid(), kThreads, 0, st>>>(H->cnt.p, H->cw[H->cur].p, H->rank.p, H->seg.p, H->perm.p, H->cap);
    PF2_LAUNCH_CHECK();
    const int nxt = 1 - H->cur;
    k_gather<<<blocks_for((long long)nc * 32, 256), 256, 0, st>>>(nc, H->seg.p, H->count.p, H->mask.p, H->perm.p,
                                                                 H->state(H->cur),
                                                  H->state(nxt), H->C, H->level, reseed ? 1 : 0, M->xy.p, M->tri4.p,
                                                  ux, uy, Partials{ H->part.p, nc }, H->cap, H->cnt.p);
    PF2_LAUNCH_CHECK();
    H->cur = nxt;
    H->partials_valid = true;
    return PF2_OK;
}

pf2_status particles_advect(pf2_particles* H, const double* ux, const double* uy, double dt, int substeps,
                            cudaStream_t st) {
    const pf2_mesh* M = H->mesh;
    const double dts = dt / substeps;  // particleAdvectionTimeStep, :330
    k_advect<<<particle_grid(), 256, 0, st>>>(H->cnt.p, substeps, dts, H->C, mesh_refs(M), ux, uy, H->state(H->cur),
                                              H->count.p, H->mask.p, H->rank.p, H->level, H->step);
    PF2_LAUNCH_CHECK();
    return sort_cells(H, true, true, ux, uy, st);
}

pf2_status particles_project(pf2_particles* H, double* ux, double* uy, double* uxo, double* uyo, cudaStream_t st) {
    const pf2_mesh* M = H->mesh;
    if (!H->partials_valid) {
        k_partials<<<blocks_for((long long)M->nc * 32, 256), 256, 0, st>>>(M->nc, H->seg.p, H->state(H->cur),
                                                                         H->C, Partials{ H->part.p, M->nc });
        PF2_LAUNCH_CHECK();
        H->partials_valid = true;
    }
    k_project_nodes<<<blocks_for(M->nv), kThreads, 0, st>>>(M->nv, M->inc_off.p, M->inc.p, Partials{ H->part.p, M->nc },
                                                            ux, uy, uxo, uyo);
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

pf2_status particles_correct(pf2_particles* H, const double* ux, const double* uy, const double* uxo,
                             const double* uyo, cudaStream_t st) {
    k_correct<<<particle_grid(), kThreads, 0, st>>>(H->cnt.p, H->state(H->cur), H->C, H->mesh->tri4.p, ux, uy, uxo,
                                                    uyo);
    PF2_LAUNCH_CHECK();
    H->partials_valid = false;
    return PF2_OK;
}

pf2_status particles_seed(pf2_particles* H, cudaStream_t st) {
    const pf2_mesh* M = H->mesh;
    const long long np = (long long)M->nc * H->ppc;
    PF2_REQUIRE(np <= H->cap, PF2_OVERFLOW, "seeding %lld particles exceeds the capacity %lld", np, H->cap);
    k_seed<<<blocks_for(np), kThreads, 0, st>>>(M->nc, H->ppc, H->C, M->xy.p, M->tri4.p, H->state(H->cur), H->seg.p);
    PF2_LAUNCH_CHECK();
    const int h[2] = { (int)np, (int)np };
    PF2_CUDA(cudaMemcpyAsync(H->cnt.p, h, sizeof(h), cudaMemcpyHostToDevice, st));
    PF2_CUDA(cudaStreamSynchronize(st));
    H->partials_valid = false;
    H->seeded = true;
    return PF2_OK;
}

pf2_status particles_status(pf2_particles* H, cudaStream_t st) {
    int e = 0;
    PF2_CUDA(cudaMemcpyAsync(&e, H->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaStreamSynchronize(st));
    PF2_REQUIRE(e == 0, (pf2_status)e, "particle buffer capacity (%lld) exceeded", H->cap);
    return PF2_OK;
}

const int* particles_count_ptr(const pf2_particles* H) { return H->cnt.p; }
int particles_parity(const pf2_particles* H) { return H->cur; }
long long particles_capacity(const pf2_particles* H) { return H->cap; }

// Larger particle buffers with the current particles copied over (the reference
// reallocates its particle vector when reseeding outgrows it).  The second buffer of
// the pair, the ranks and the permutation are scratch and are not copied.
pf2_status particles_reserve(pf2_particles* H, long long cap, cudaStream_t st) {
    if (cap <= H->cap) return PF2_OK;
    PF2_REQUIRE(cap <= (long long)INT32_MAX - 1, PF2_OVERFLOW, "particle capacity %lld too large", cap);
    int n = 0;
    PF2_CUDA(cudaMemcpyAsync(&n, H->cnt.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaStreamSynchronize(st));
    DevBuf<double> nb[2][6];
    DevBuf<int> ncw[2], nrank, nperm;
    for (int b = 0; b < 2; ++b) {
        for (int k = 0; k < 6; ++k) PF2_TRY(nb[b][k].alloc(cap));
        PF2_TRY(ncw[b].alloc(cap));
    }
    PF2_TRY(nrank.alloc(cap));
    PF2_TRY(nperm.alloc(cap));
    const int c = H->cur;
    if (n > 0) {
        for (int k = 0; k < 6; ++k)
            PF2_CUDA(cudaMemcpyAsync(nb[c][k].p, H->buf[c][k].p, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        PF2_CUDA(cudaMemcpyAsync(ncw[c].p, H->cw[c].p, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
    }
    PF2_CUDA(cudaStreamSynchronize(st));
    for (int b = 0; b < 2; ++b) {
        for (int k = 0; k < 6; ++k) H->buf[b][k] = std::move(nb[b][k]);
        H->cw[b] = std::move(ncw[b]);
    }
    H->rank = std::move(nrank);
    H->perm = std::move(nperm);
    H->cap = cap;
    return PF2_OK;
}
void particles_set_parity(pf2_particles* H, int parity) { H->cur = parity; }

// Sections: sizes {cells, level, count, seeded}, the SoA arrays and cell words of the
// current buffer, and the cell segments of the last sort (read by a projection that
// comes before the next advection).  Between steps that is the whole particle state:
// the per-cell counts and masks are zero and the other buffer is scratch.
pf2_status particles_checkpoint(pf2_particles* H, CkptFile& io, cudaStream_t st) {
    const int nc = H->mesh->nc;
    int meta[4] = { nc, H->level, 0, H->seeded ? 1 : 0 };
    if (io.writing()) {
        PF2_TRY(particles_status(H, st));
        PF2_CUDA(cudaMemcpyAsync(&meta[2], H->cnt.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        PF2_CUDA(cudaStreamSynchronize(st));
    }
    PF2_TRY(io.host("pmeta", meta, sizeof(meta)));
    if (!io.writing()) {
        PF2_REQUIRE(meta[0] == nc && meta[1] == H->level, PF2_BAD_INPUT,
                    "checkpoint particles: %d cells at level %d, these particles: %d cells at level %d", meta[0],
                    meta[1], nc, H->level);
        PF2_REQUIRE(meta[2] >= 0 && meta[2] <= H->cap, PF2_OVERFLOW,
                    "checkpoint holds %d particles, the capacity is %lld", meta[2], H->cap);
    }
    const size_t n = (size_t)meta[2];
    static const char* const tags[6] = { "px", "py", "pl0", "pl1", "pu", "pv" };
    for (int k = 0; k < 6; ++k) PF2_TRY(io.device(tags[k], H->buf[H->cur][k].p, n * sizeof(double), st));
    PF2_TRY(io.device("pcell", H->cw[H->cur].p, n * sizeof(int), st));
    PF2_TRY(io.device("pseg", H->seg.p, (size_t)(nc + 1) * sizeof(int), st));
    if (!io.writing()) {
        const int h[2] = { meta[2], meta[2] };
        PF2_CUDA(cudaMemcpyAsync(H->cnt.p, h, sizeof(h), cudaMemcpyHostToDevice, st));
        PF2_CUDA(cudaStreamSynchronize(st));
        H->partials_valid = false;
        H->seeded = meta[3] != 0;
    }
    return PF2_OK;
}

}  // namespace pf2

extern "C" {

pf2_status pf2_particles_create(const pf2_mesh* m, int level, double capacity_factor, pf2_particles** out) {
    PF2_REQUIRE(m && out, PF2_BAD_INPUT, "null argument");
    *out = nullptr;
    PF2_REQUIRE(m->nnb > 0 || m->nc == 1, PF2_BAD_INPUT, "the mesh was built without neighbour lists");
    pf2_particles* H = new pf2_particles();
    H->mesh = m;
    H->level = std::max(std::min(level, kMaxLevel), 1);  // :241
    H->ppc = H->level * H->level;
    H->step = 1.0 / H->level;
    subcell_centers(H->level, H->C);
    const double f = std::max(capacity_factor, 1.1);
    H->cap = (long long)std::ceil(f * (double)m->nc * H->ppc);
    auto fail = [&](pf2_status s) { delete H; return s; };
    if (H->cap > (long long)INT32_MAX - 1) return fail((set_error("particle capacity too large"), PF2_BAD_INPUT));
    pf2_status s;
    for (int b = 0; b < 2; ++b) {
        for (int k = 0; k < 6; ++k)
            if ((s = H->buf[b][k].alloc(H->cap))) return fail(s);
        if ((s = H->cw[b].alloc(H->cap))) return fail(s);
    }
    const int nc = m->nc;
    if ((s = H->rank.alloc(H->cap)) || (s = H->perm.alloc(H->cap)) || (s = H->count.alloc(nc + 1)) ||
        (s = H->mask.alloc(nc + 1)) || (s = H->seg.alloc(nc + 1)) || (s = H->segsz.alloc(nc + 1)) ||
        (s = H->scratch.alloc(scan_scratch_ints(nc))) || (s = H->cnt.alloc(2)) || (s = H->err.alloc(1)) ||
        (s = H->part.alloc(9 * (size_t)nc)) || (s = H->h_cnt.alloc(2)))
        return fail(s);
    if (cudaMemset(H->count.p, 0, sizeof(int) * (nc + 1)) != cudaSuccess ||
        cudaMemset(H->mask.p, 0, sizeof(int) * (nc + 1)) != cudaSuccess ||
        cudaMemset(H->seg.p, 0, sizeof(int) * (nc + 1)) != cudaSuccess ||
        cudaMemset(H->cnt.p, 0, sizeof(int) * 2) != cudaSuccess || cudaMemset(H->err.p, 0, sizeof(int)) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "cudaMemset", __FILE__, __LINE__));
    *out = H;
    return PF2_OK;
}

pf2_status pf2_particles_destroy(pf2_particles* H) {
    delete H;
    return PF2_OK;
}

pf2_status pf2_particles_seed(pf2_particles* H, void* stream) {
    PF2_REQUIRE(H, PF2_BAD_INPUT, "null particles");
    return particles_seed(H, as_stream(stream));
}

pf2_status pf2_particles_init_velocity(pf2_particles* H, const double* ux, const double* uy, void* stream) {
    PF2_REQUIRE(H && ux && uy, PF2_BAD_INPUT, "null argument");
    return particles_correct(H, ux, uy, nullptr, nullptr, as_stream(stream));
}

pf2_status pf2_particles_advect(pf2_particles* H, const double* ux, const double* uy, double dt, int substeps,
                                void* stream) {
    PF2_REQUIRE(H && ux && uy, PF2_BAD_INPUT, "null argument");
    PF2_REQUIRE(substeps >= 1, PF2_BAD_INPUT, "substeps must be >= 1");
    cudaStream_t st = as_stream(stream);
    PF2_TRY(particles_advect(H, ux, uy, dt, substeps, st));
    return PF2_OK;
}

pf2_status pf2_particles_correct(pf2_particles* H, const double* ux, const double* uy, const double* uxo,
                                 const double* uyo, void* stream) {
    PF2_REQUIRE(H && ux && uy && uxo && uyo, PF2_BAD_INPUT, "null argument");
    return particles_correct(H, ux, uy, uxo, uyo, as_stream(stream));
}

pf2_status pf2_particles_project(pf2_particles* H, double* ux, double* uy, void* stream) {
    PF2_REQUIRE(H && ux && uy, PF2_BAD_INPUT, "null argument");
    return particles_project(H, ux, uy, nullptr, nullptr, as_stream(stream));
}

pf2_status pf2_particles_count(const pf2_particles* H, int* count) {
    PF2_REQUIRE(H && count, PF2_BAD_INPUT, "null argument");
    PF2_CUDA(cudaDeviceSynchronize());
    int e = 0;
    PF2_CUDA(cudaMemcpy(&e, H->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    PF2_CUDA(cudaMemcpy(count, H->cnt.p, sizeof(int), cudaMemcpyDeviceToHost));
    PF2_REQUIRE(e == 0, (pf2_status)e, "particle buffer capacity (%lld) exceeded", H->cap);
    return PF2_OK;
}

pf2_status pf2_particles_download(const pf2_particles* Hc, double* x, double* y, double* l0, double* l1, double* l2,
                                  double* u, double* v, int* cell) {
    PF2_REQUIRE(Hc, PF2_BAD_INPUT, "null particles");
    pf2_particles* H = const_cast<pf2_particles*>(Hc);
    int n = 0;
    PF2_TRY(pf2_particles_count(H, &n));
    double* dst[6] = { x, y, l0, l1, u, v };
    for (int k = 0; k < 6; ++k)
        if (dst[k]) PF2_CUDA(cudaMemcpy(dst[k], H->buf[H->cur][k].p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (cell || l2) {
        std::vector<int> w(n);
        std::vector<double> a(l2 && !l0 ? n : 0), b(l2 && !l1 ? n : 0);
        PF2_CUDA(cudaMemcpy(w.data(), H->cw[H->cur].p, sizeof(int) * n, cudaMemcpyDeviceToHost));
        const double* L0 = l0;
        const double* L1 = l1;
        if (l2 && !l0) { PF2_CUDA(cudaMemcpy(a.data(), H->buf[H->cur][2].p, sizeof(double) * n, cudaMemcpyDeviceToHost)); L0 = a.data(); }
        if (l2 && !l1) { PF2_CUDA(cudaMemcpy(b.data(), H->buf[H->cur][3].p, sizeof(double) * n, cudaMemcpyDeviceToHost)); L1 = b.data(); }
        for (int p = 0; p < n; ++p) {
            if (cell) cell[p] = w[p] < 0 ? -1 : (w[p] & kCellMask);
            if (l2) {
                const unsigned f = ((unsigned)w[p]) >> kCellBits;
                l2[p] = (w[p] >= 0 && f) ? H->C.c[f - 1][2] : (1.0 - L0[p]) - L1[p];
            }
        }
    }
    return PF2_OK;
}

pf2_status pf2_particles_reserve(pf2_particles* H, long long capacity) {
    PF2_REQUIRE(H, PF2_BAD_INPUT, "null particles");
    PF2_CUDA(cudaDeviceSynchronize());
    return particles_reserve(H, capacity, nullptr);
}

pf2_status pf2_particles_save(const pf2_particles* Hc, const char* path) {
    PF2_REQUIRE(Hc && path, PF2_BAD_INPUT, "null argument");
    pf2_particles* H = const_cast<pf2_particles*>(Hc);  // only read
    CkptFile io;
    PF2_TRY(io.open_write(path, CKPT_PARTICLES));
    PF2_TRY(particles_checkpoint(H, io, nullptr));
    return io.close();
}

pf2_status pf2_particles_load(pf2_particles* H, const char* path) {
    PF2_REQUIRE(H && path, PF2_BAD_INPUT, "null argument");
    CkptFile io;
    PF2_TRY(io.open_read(path, CKPT_PARTICLES));
    PF2_TRY(particles_checkpoint(H, io, nullptr));
    return io.close();
}

pf2_status pf2_particles_upload(pf2_particles* H, int n, const double* x, const double* y, const double* l0,
                                const double* l1, const double* l2, const double* u, const double* v,
                                const int* cell) {
    PF2_REQUIRE(H && x && y && l0 && l1 && u && v && cell, PF2_BAD_INPUT, "null argument");
    PF2_REQUIRE(n >= 0 && n <= H->cap, PF2_OVERFLOW, "%d particles exceed the capacity %lld", n, H->cap);
    std::vector<int> w(n);
    for (int p = 0; p < n; ++p) {
        PF2_REQUIRE(cell[p] >= 0 && cell[p] < H->mesh->nc, PF2_BAD_INPUT, "particle %d: cell %d out of range", p, cell[p]);
        int word = cell[p];
        if (l2 && l2[p] != (1.0 - l0[p]) - l1[p]) {
            int k = -1;
            for (int q = 0; q < H->ppc; ++q)
                if (H->C.c[q][0] == l0[p] && H->C.c[q][1] == l1[p] && H->C.c[q][2] == l2[p]) { k = q; break; }
            PF2_REQUIRE(k >= 0, PF2_BAD_INPUT,
                        "particle %d: l2 differs from 1 - l0 - l1 and is not a sub-cell centroid", p);
            word |= (k + 1) << kCellBits;
        }
        w[p] = word;
    }
    const int c = H->cur;
    const double* src[6] = { x, y, l0, l1, u, v };
    for (int k = 0; k < 6; ++k)
        if (n) PF2_CUDA(cudaMemcpy(H->buf[c][k].p, src[k], sizeof(double) * n, cudaMemcpyHostToDevice));
    if (n) PF2_CUDA(cudaMemcpy(H->cw[c].p, w.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    const int h[2] = { n, n };
    PF2_CUDA(cudaMemcpy(H->cnt.p, h, sizeof(h), cudaMemcpyHostToDevice));
    PF2_TRY(sort_cells(H, false, false, nullptr, nullptr, nullptr));
    H->partials_valid = false;
    H->seeded = true;
    PF2_CUDA(cudaDeviceSynchronize());
    return particles_status(H, nullptr);
}

}  // extern "C"
