// assembly.cu - finite element assembly of the CSR systems and the Dirichlet rule.
//
// Every kernel is row-centric: thread i owns CSR row i, walks the cells around node i
// (ascending cell order, so sums are deterministic), adds row "local vertex of i" of
// each cell's 3x3 matrix and rhs into a per-thread row buffer, applies the Dirichlet
// rule to the finished row and writes it once.  No atomics and no clearing pass are
// needed, and the result does not depend on thread timing.
//
// The cell integrals are the reference's 3-point Gauss rule evaluated in closed form
// (the rule is exact for the P1 products involved): sum_q N_m N_j w_q = (1 + d_mj)/12,
// sum_q N_m w_q = 1/3, sum_q w_q = 1 (quadrature_formula_2d.cu:17-24).  The Poisson
// right-hand side keeps the point evaluation of f at the three Gauss points.
#include <cmath>

#include "common.cuh"
#include "device.cuh"
#include "internal.cuh"

namespace pf2 {

struct RowMesh {
    const int* rowptr;
    const int* col;
    const int* inc_off;
    const int* inc;
    const int* inc_pos;
    const int4* tri4;
    const double4_32a* invJ;
    const double* area;
    const double2* xy;
    const int* edge_ids;
};

static RowMesh row_mesh(const pf2_mesh* m) {
    return RowMesh{ m->rowptr.p, m->col.p, m->inc_off.p, m->inc.p, m->inc_pos.p, m->tri4.p,
                    m->invJ.p, m->area.p, m->xy.p, m->edge_ids.p };
}

struct BcView {
    const int* node_to_bc;  // nullptr: no boundary conditions
    const double* value;
};

static BcView bc_view(const pf2_bc* b) {
    return b ? BcView{ b->node_to_bc.p, b->value.p } : BcView{ nullptr, nullptr };
}

__device__ __forceinline__ int vtx(const int4& t, int k) { return k == 0 ? t.x : (k == 1 ? t.y : t.z); }

// Dirichlet rule of DirichletBCs::applyBCs (Dirichlet_bcs.cu:3-51) on a finished row
// that is not itself a boundary row: unless |first off-diagonal| < 2e-6, every
// boundary column d moves to the rhs (rhs -= a_id * g_d) and is zeroed.  Columns are
// visited in ascending order.
__device__ __forceinline__ void eliminate_row(int i, int s, int len, const int* __restrict__ col, double* v,
                                              double& rhs, const BcView& bc) {
    if (!bc.node_to_bc) return;
    const int first = (col[s] == i) ? 1 : 0;
    if (first >= len || fabs(v[first]) < kDoubleMin) return;
    for (int k = 0; k < len; ++k) {
        const int j = col[s + k];
        if (j == i) continue;
        const int b = bc.node_to_bc[j];
        if (b >= 0) {
            rhs = __dadd_rn(rhs, __dmul_rn(v[k], -bc.value[b]));
            v[k] = 0.0;
        }
    }
}

// True when some column of row i (other than i) is a boundary node of bc: only such rows
// need their matrix values in a right-hand-side-only assembly (for the elimination).
__device__ __forceinline__ bool has_bc_column(int i, int s, int len, const int* __restrict__ col, const BcView& bc) {
    if (!bc.node_to_bc) return false;
    for (int k = 0; k < len; ++k) {
        const int j = col[s + k];
        if (j != i && bc.node_to_bc[j] >= 0) return true;
    }
    return false;
}

__device__ __forceinline__ bool boundary_row(int i, int s, int len, const int* __restrict__ col, double* __restrict__ val,
                                             double* __restrict__ rhs, const BcView& bc, bool matrix = true) {
    if (!bc.node_to_bc) return false;
    const int b = bc.node_to_bc[i];
    if (b < 0) return false;
    if (matrix)
        for (int k = 0; k < len; ++k) val[s + k] = (col[s + k] == i) ? 1.0 : 0.0;
    rhs[i] = bc.value[b];
    return true;
}

// ------------------------------------------------------------- Poisson
__device__ __forceinline__ double rhs_f(int kind, double x, double y) {
    if (kind == PF2_RHS_SINSIN) {
        const double pi = 3.14159265358979323846;
        return 2.0 * pi * pi * sin(pi * x) * sin(pi * y);
    }
    return exp(-(x * x + 10 * y * y));
}

// cases/Poisson2D/main.cu:28-68
__global__ void k_poisson(int nv, RowMesh M, int kind, double lambda, double* __restrict__ val,
                          double* __restrict__ rhs, BcView bc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int s = M.rowptr[i], len = M.rowptr[i + 1] - s;
    if (boundary_row(i, s, len, M.col, val, rhs, bc)) return;
    // 3-point rule of quadrature_formula_2d.cu:17-24 (z = 1 - x - y as there)
    const double q1 = 0.1666666666666667, q2 = 0.6666666666666667;
    const double QL[3][3] = { { q1, q1, 1.0 - q1 - q1 }, { q2, q1, 1.0 - q2 - q1 }, { q1, q2, 1.0 - q1 - q2 } };
    const double w = 0.3333333333333333;
    double v[kMaxRow];
    for (int k = 0; k < len; ++k) v[k] = 0.0;
    double r = 0.0;
    for (int q = M.inc_off[i]; q < M.inc_off[i + 1]; ++q) {
        const int e = M.inc[q], c = e >> 2, m = e & 3, pos = M.inc_pos[q];
        const double4_32a J = M.invJ[c];
        const double A = M.area[c];
        double2 g[3];
        shape_grads(J, g);
        const int4 t = M.tri4[c];
        const double2 P0 = M.xy[t.x], P1 = M.xy[t.y], P2 = M.xy[t.z];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int p = (pos >> (10 * j)) & 1023;
            v[p] += lambda * (g[m].x * g[j].x + g[m].y * g[j].y) * A;
        }
        double rr = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double x = QL[k][0] * P0.x + QL[k][1] * P1.x + QL[k][2] * P2.x;
            const double y = QL[k][0] * P0.y + QL[k][1] * P1.y + QL[k][2] * P2.y;
            rr += rhs_f(kind, x, y) * QL[k][m] * w;
        }
        r += rr * A;
    }
    eliminate_row(i, s, len, M.col, v, r, bc);
    for (int k = 0; k < len; ++k) val[s + k] = v[k];
    rhs[i] = r;
}

// ------------------------------------------------------------- flow systems
// `matrix` is a runtime flag, not a template parameter: the matrix values that feed the
// elimination of a right-hand-side-only assembly then come from the same machine code
// as a full assembly's, so both give the same bits (separate instantiations may fuse
// the products differently).

// kIntegrateVelocityPrediction, cases/Cylinder2D/main.cu:72-167.  Outlet edge term on
// boundary id 1 with n = (1, 0); like the cell terms it is scaled by the cell area
// (addLocalToGlobal).  Along an edge, sum_q w_q N_m(q) = 1 for both edge vertices.
__global__ void k_prediction(bool matrix, int nv, RowMesh M, FlowCoef P, const double* __restrict__ ux,
                             const double* __restrict__ uy, const double* __restrict__ uxo,
                             const double* __restrict__ uyo, const double* __restrict__ pold,
                             double* __restrict__ valx, double* __restrict__ valy, double* __restrict__ rhsx,
                             double* __restrict__ rhsy, BcView bcx, BcView bcy) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int s = M.rowptr[i], len = M.rowptr[i + 1] - s;
    const bool bx = boundary_row(i, s, len, M.col, valx, rhsx, bcx, matrix);
    const bool by = boundary_row(i, s, len, M.col, valy, rhsy, bcy, matrix);
    if (bx && by) return;
    // the matrix rows are needed when written, or for the elimination of boundary columns
    const bool need = matrix || has_bc_column(i, s, len, M.col, bcx) || has_bc_column(i, s, len, M.col, bcy);
    double v0[kMaxRow], v1[kMaxRow];
    if (need)
        for (int k = 0; k < len; ++k) { v0[k] = 0.0; v1[k] = 0.0; }
    double r0 = 0.0, r1 = 0.0;
    const double visc = P.mu * P.dt;
    const double third = 1.0 / 3.0;
    for (int q = M.inc_off[i]; q < M.inc_off[i + 1]; ++q) {
        const int e = M.inc[q], c = e >> 2, m = e & 3, pos = M.inc_pos[q];
        const double A = M.area[c];
        double2 g[3];
        shape_grads(M.invJ[c], g);
        const int4 t = M.tri4[c];
        double c0 = 0.0, c1 = 0.0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int nj = vtx(t, j), p = (pos >> (10 * j)) & 1023;
            const double mass = P.rho * ((j == m) ? (1.0 / 6.0) : (1.0 / 12.0));
            const double xx = g[m].x * g[j].x, yy = g[m].y * g[j].y;
            const double xy_ = g[m].y * g[j].x, yx = g[m].x * g[j].y;
            if (need) {
                v0[p] += (mass + visc * (yy + 4.0 / 3.0 * xx)) * A;
                v1[p] += (mass + visc * (xx + 4.0 / 3.0 * yy)) * A;
            }
            c0 += mass * uxo[nj] - visc * (xy_ - 2.0 / 3.0 * yx) * uy[nj];
            c1 += mass * uyo[nj] - visc * (yx - 2.0 / 3.0 * xy_) * ux[nj];
            if (pold) {
                const double a = third * pold[nj] * P.dt;
                c0 -= a * g[j].x;
                c1 -= a * g[j].y;
            }
        }
        // outlet edges (id 1) that contain local vertex m
        const int e0 = M.edge_ids[3 * c], e1 = M.edge_ids[3 * c + 1], e2 = M.edge_ids[3 * c + 2];
        const int ids[3] = { e0, e1, e2 };
#pragma unroll
        for (int ed = 0; ed < 3; ++ed) {
            if (ids[ed] != 1) continue;
            if (m != ed && m != (ed + 1) % 3) continue;
            const double2 S = M.xy[vtx(t, ed)], E = M.xy[vtx(t, (ed + 1) % 3)];
            const double half = 0.5 * sqrt((S.x - E.x) * (S.x - E.x) + (S.y - E.y) * (S.y - E.y));
            const double w = visc * half;
            const double nx = 1.0, ny = 0.0;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int nj = vtx(t, j), p = (pos >> (10 * j)) & 1023;
                if (need) {
                    v0[p] -= w * ((4.0 / 3.0) * g[j].x * nx + g[j].y * ny) * A;
                    v1[p] -= w * (g[j].x * nx + (4.0 / 3.0) * g[j].y * ny) * A;
                }
                c0 += w * uy[nj] * ((-2.0 / 3.0) * g[j].y * nx + g[j].x * ny);
                c1 += w * ux[nj] * (g[j].y * nx + (-2.0 / 3.0) * g[j].x * ny);
            }
        }
        r0 += c0 * A;
        r1 += c1 * A;
    }
    if (!bx) {
        if (need) eliminate_row(i, s, len, M.col, v0, r0, bcx);
        if (matrix)
            for (int k = 0; k < len; ++k) valx[s + k] = v0[k];
        rhsx[i] = r0;
    }
    if (!by) {
        if (need) eliminate_row(i, s, len, M.col, v1, r1, bcy);
        if (matrix)
            for (int k = 0; k < len; ++k) valy[s + k] = v1[k];
        rhsy[i] = r1;
    }
}

// kIntegratePressureEquation, cases/Cylinder2D/main.cu:169-211
__global__ void k_pressure(bool matrix, int nv, RowMesh M, FlowCoef P, const double* __restrict__ px,
                           const double* __restrict__ py, const double* __restrict__ pold, double* __restrict__ val,
                           double* __restrict__ rhs, BcView bc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int s = M.rowptr[i], len = M.rowptr[i + 1] - s;
    if (boundary_row(i, s, len, M.col, val, rhs, bc, matrix)) return;
    const bool need = matrix || has_bc_column(i, s, len, M.col, bc);
    double v[kMaxRow];
    if (need)
        for (int k = 0; k < len; ++k) v[k] = 0.0;
    double r = 0.0;
    const double fdiv = -P.rho / P.dt / 3.0;
    for (int q = M.inc_off[i]; q < M.inc_off[i + 1]; ++q) {
        const int e = M.inc[q], c = e >> 2, m = e & 3, pos = M.inc_pos[q];
        const double A = M.area[c];
        double2 g[3];
        shape_grads(M.invJ[c], g);
        const int4 t = M.tri4[c];
        double cr = 0.0, div = 0.0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int nj = vtx(t, j), p = (pos >> (10 * j)) & 1023;
            const double K = g[m].x * g[j].x + g[m].y * g[j].y;
            if (need) v[p] += K * A;
            if (pold) cr += K * pold[nj];
            div += g[j].x * px[nj] + g[j].y * py[nj];
        }
        r += (cr + fdiv * div) * A;
    }
    if (need) eliminate_row(i, s, len, M.col, v, r, bc);
    if (matrix)
        for (int k = 0; k < len; ++k) val[s + k] = v[k];
    rhs[i] = r;
}

// kIntegrateVelocityCorrection, cases/Cylinder2D/main.cu:213-259
__global__ void k_correction(bool matrix, int nv, RowMesh M, FlowCoef P, const double* __restrict__ px,
                             const double* __restrict__ py, const double* __restrict__ pres,
                             const double* __restrict__ pold, double* __restrict__ valx, double* __restrict__ valy,
                             double* __restrict__ rhsx, double* __restrict__ rhsy, BcView bcx, BcView bcy) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int s = M.rowptr[i], len = M.rowptr[i + 1] - s;
    const bool bx = boundary_row(i, s, len, M.col, valx, rhsx, bcx, matrix);
    const bool by = boundary_row(i, s, len, M.col, valy, rhsy, bcy, matrix);
    if (bx && by) return;
    const bool need = matrix || has_bc_column(i, s, len, M.col, bcx) || has_bc_column(i, s, len, M.col, bcy);
    double v[kMaxRow];
    if (need)
        for (int k = 0; k < len; ++k) v[k] = 0.0;
    double r0 = 0.0, r1 = 0.0;
    const double gdt = P.dt / 3.0;
    for (int q = M.inc_off[i]; q < M.inc_off[i + 1]; ++q) {
        const int e = M.inc[q], c = e >> 2, m = e & 3, pos = M.inc_pos[q];
        const double A = M.area[c];
        double2 g[3];
        shape_grads(M.invJ[c], g);
        const int4 t = M.tri4[c];
        double c0 = 0.0, c1 = 0.0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int nj = vtx(t, j), p = (pos >> (10 * j)) & 1023;
            const double mass = P.rho * ((j == m) ? (1.0 / 6.0) : (1.0 / 12.0));
            if (need) v[p] += mass * A;
            const double dp = pold ? (pres[nj] - pold[nj]) : pres[nj];
            c0 += mass * px[nj] - gdt * g[j].x * dp;
            c1 += mass * py[nj] - gdt * g[j].y * dp;
        }
        r0 += c0 * A;
        r1 += c1 * A;
    }
    double w[kMaxRow];
    if (need)
        for (int k = 0; k < len; ++k) w[k] = v[k];
    if (!bx) {
        if (need) eliminate_row(i, s, len, M.col, v, r0, bcx);
        if (matrix)
            for (int k = 0; k < len; ++k) valx[s + k] = v[k];
        rhsx[i] = r0;
    }
    if (!by) {
        if (need) eliminate_row(i, s, len, M.col, w, r1, bcy);
        if (matrix)
            for (int k = 0; k < len; ++k) valy[s + k] = w[k];
        rhsy[i] = r1;
    }
}

// Standalone DirichletBCs::applyBCs on an assembled system: the same rule per row.
__global__ void k_apply_bc(int nv, const int* __restrict__ rowptr, const int* __restrict__ col,
                           double* __restrict__ val, double* __restrict__ rhs, BcView bc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int s = rowptr[i], len = rowptr[i + 1] - s;
    if (boundary_row(i, s, len, col, val, rhs, bc)) return;
    const int first = (col[s] == i) ? 1 : 0;
    if (first >= len || fabs(val[s + first]) < kDoubleMin) return;
    double r = rhs[i];
    bool changed = false;
    for (int k = 0; k < len; ++k) {
        const int j = col[s + k];
        if (j == i) continue;
        const int b = bc.node_to_bc[j];
        if (b >= 0) {
            r = __dadd_rn(r, __dmul_rn(val[s + k], -bc.value[b]));
            val[s + k] = 0.0;
            changed = true;
        }
    }
    if (changed) rhs[i] = r;
}

// kAccumulatePressureGradient + kFinalizePredictionBC (Cylinder2D/main.cu:261-297):
// one thread per boundary node gathers over its cells (ascending).
__global__ void k_prediction_bc(int nbc, const int* __restrict__ node, const double* __restrict__ src,
                                double* __restrict__ dst, RowMesh M, FlowCoef P, const double* __restrict__ pres,
                                const double* __restrict__ pold, int comp) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbc) return;
    const int d = node[b];
    double num = 0.0, den = 0.0;
    for (int q = M.inc_off[d]; q < M.inc_off[d + 1]; ++q) {
        const int c = M.inc[q] >> 2;
        const int4 t = M.tri4[c];
        const double dp0 = pres[t.x] - (pold ? pold[t.x] : 0.0);
        const double dp1 = pres[t.y] - (pold ? pold[t.y] : 0.0);
        const double dp2 = pres[t.z] - (pold ? pold[t.z] : 0.0);
        const double gx = dp0 - dp2, gy = dp1 - dp2;
        const double4_32a J = M.invJ[c];
        const double cg = comp == 0 ? (J.x * gx + J.y * gy) : (J.z * gx + J.w * gy);
        const double A = M.area[c];
        num += A * cg;
        den += A;
    }
    dst[b] = src[b] + P.dt / P.rho * num / den;
}

// kCountBodyEdges + kCalculateBodyForces + reduceVector (Cylinder2D/main.cu:299-376,
// :414-428): kLoadBlocks blocks, block b over the cells [b * chunk, (b + 1) * chunk), its
// threads striding over them and taking the first body edge of each cell (the scan of
// the cells' edge ids is the kernel's work: a million cells hold a few hundred body
// edges).  Each block's fixed-order sums go to out[2 ...]; the last block to finish
// (a ticket after out's partials) adds the blocks' sums in block order, writes the two
// coefficients and rewinds the ticket.  No block waits for another.
__global__ void __launch_bounds__(256) k_body_loads(int nc, RowMesh M, FlowCoef P, int body_id, double thickness,
                                                    double umean, double cx, double cy,
                                                    const double* __restrict__ ux, const double* __restrict__ uy,
                                                    const double* __restrict__ pres, double* out) {
    __shared__ double sh[33 * 4];
    __shared__ int last;
    const double gq[2] = { -0.577350269189626, 0.577350269189626 };  // quadrature_formula_1d.cu:15-18
    double F[4] = { 0, 0, 0, 0 };
    const int chunk = (nc + kLoadBlocks - 1) / kLoadBlocks;
    const long long lo = (long long)blockIdx.x * chunk;
    const int c1 = (int)std::min<long long>(nc, lo + chunk);
    for (int c = (int)std::min<long long>(lo, nc) + threadIdx.x; c < c1; c += blockDim.x) {
        int e = -1;
        for (int k = 0; k < 3; ++k)
            if (M.edge_ids[3 * c + k] == body_id) { e = k; break; }
        if (e < 0) continue;
        const int4 t = M.tri4[c];
        const double4_32a J = M.invJ[c];
        const double2 S = M.xy[vtx(t, e)], E = M.xy[vtx(t, (e + 1) % 3)], V3 = M.xy[t.z];
        double nx = 0.5 * (S.x + E.x) - cx, ny = 0.5 * (S.y + E.y) - cy;
        const double il = 1.0 / sqrt(nx * nx + ny * ny);
        nx *= il;
        ny *= il;
        const double half = 0.5 * sqrt((S.x - E.x) * (S.x - E.x) + (S.y - E.y) * (S.y - E.y));
        const double tx = ny, ty = -nx;
        double2 g[3];
        shape_grads(J, g);
        const double dvn0 = ux[t.x] * tx + uy[t.x] * ty, dvn1 = ux[t.y] * tx + uy[t.y] * ty,
                     dvn2 = ux[t.z] * tx + uy[t.z] * ty;
        const double dvt = dvn0 * (g[0].x * nx + g[0].y * ny) + dvn1 * (g[1].x * nx + g[1].y * ny) +
                           dvn2 * (g[2].x * nx + g[2].y * ny);
        for (int q = 0; q < 2; ++q) {
            const double qx = 0.5 * (gq[q] * (E.x - S.x) + (S.x + E.x));
            const double qy = 0.5 * (gq[q] * (E.y - S.y) + (S.y + E.y));
            const double dx = qx - V3.x, dy = qy - V3.y;
            const double L0 = J.x * dx + J.z * dy, L1 = J.y * dx + J.w * dy, L2 = 1.0 - L0 - L1;
            const double pq = pres[t.x] * L0 + pres[t.y] * L1 + pres[t.z] * L2;
            const double w = half;
            F[0] -= pq * nx * w;
            F[1] -= pq * ny * w;
            F[2] += P.mu * dvt * tx * w;
            F[3] += P.mu * dvt * ty * w;
        }
    }
    block_sum_n<4>(F, sh);
    double* part = out + 2;
    unsigned* ticket = reinterpret_cast<unsigned*>(out + 2 + 4 * kLoadBlocks);
    if (threadIdx.x == 0) {
        for (int k = 0; k < 4; ++k) __stcg(&part[k * kLoadBlocks + blockIdx.x], F[k]);
        __threadfence();
        last = atomicAdd(ticket, 1u) == kLoadBlocks - 1;
    }
    __syncthreads();
    if (!last) return;  // uniform over the block
    __threadfence();
    double tot[4] = { 0, 0, 0, 0 };
    for (int b = threadIdx.x; b < kLoadBlocks; b += blockDim.x)
        for (int k = 0; k < 4; ++k) tot[k] += __ldcg(&part[k * kLoadBlocks + b]);
    block_sum_n<4>(tot, sh);
    if (threadIdx.x == 0) {
        const double coeff = 2.0 / (P.rho * umean * umean * thickness);
        out[0] = (tot[0] + tot[2]) * coeff;
        out[1] = (tot[1] + tot[3]) * coeff;
        *ticket = 0u;
    }
}

// ------------------------------------------------------------- launchers
pf2_status launch_prediction(const pf2_mesh* m, const FlowCoef& P, bool matrix, const double* ux, const double* uy,
                             const double* uxo, const double* uyo, const double* pold, double* valx, double* valy,
                             double* rhsx, double* rhsy, const pf2_bc* bcx, const pf2_bc* bcy, cudaStream_t st) {
    k_prediction<<<blocks_for(m->nv), kThreads, 0, st>>>(matrix, m->nv, row_mesh(m), P, ux, uy, uxo, uyo, pold, valx,
                                                         valy, rhsx, rhsy, bc_view(bcx), bc_view(bcy));
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

pf2_status launch_pressure(const pf2_mesh* m, const FlowCoef& P, bool matrix, const double* px, const double* py,
                           const double* pold, double* val, double* rhs, const pf2_bc* bc, cudaStream_t st) {
    k_pressure<<<blocks_for(m->nv), kThreads, 0, st>>>(matrix, m->nv, row_mesh(m), P, px, py, pold, val, rhs,
                                                       bc_view(bc));
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

pf2_status launch_correction(const pf2_mesh* m, const FlowCoef& P, bool matrix, const double* px, const double* py,
                             const double* pres, const double* pold, double* valx, double* valy, double* rhsx,
                             double* rhsy, const pf2_bc* bcx, const pf2_bc* bcy, cudaStream_t st) {
    k_correction<<<blocks_for(m->nv), kThreads, 0, st>>>(matrix, m->nv, row_mesh(m), P, px, py, pres, pold, valx, valy,
                                                         rhsx, rhsy, bc_view(bcx), bc_view(bcy));
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

pf2_status launch_prediction_bc(const pf2_mesh* m, const FlowCoef& P, const pf2_bc* src, pf2_bc* dst,
                                const double* pres, const double* pold, int comp, cudaStream_t st) {
    if (dst->n_bc == 0) return PF2_OK;
    k_prediction_bc<<<blocks_for(dst->n_bc), kThreads, 0, st>>>(dst->n_bc, dst->node.p, src->value.p, dst->value.p,
                                                                row_mesh(m), P, pres, pold, comp);
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

pf2_status launch_body_loads(const pf2_mesh* m, const FlowCoef& P, int body_id, double thickness, double umean,
                             double cx, double cy, const double* ux, const double* uy, const double* pres,
                             double* out_dev, cudaStream_t st) {
    k_body_loads<<<kLoadBlocks, 256, 0, st>>>(m->nc, row_mesh(m), P, body_id, thickness, umean, cx, cy, ux, uy,
                                              pres, out_dev);
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

}  // namespace pf2

using namespace pf2;

static pf2_status check_csr(const pf2_mesh* m, const pf2_csr* A) {
    PF2_REQUIRE(m && A, PF2_BAD_INPUT, "null mesh or matrix");
    PF2_REQUIRE(A->mesh == m, PF2_BAD_INPUT, "matrix was not created for this mesh");
    return PF2_OK;
}

static pf2_status check_bc(const pf2_mesh* m, const pf2_bc* b) {
    if (!b) return PF2_OK;
    PF2_REQUIRE(b->n_nodes == m->nv, PF2_BAD_INPUT, "boundary set built for %d nodes, mesh has %d", b->n_nodes, m->nv);
    return PF2_OK;
}

extern "C" {

pf2_status pf2_params_default(pf2_params* p) {
    PF2_REQUIRE(p, PF2_BAD_INPUT, "null params");
    // SimulationParameters::setDefaultParameters (parameters.cuh:30-50)
    p->rho = 1.0;
    p->mu = 1.0;
    p->dt = 0.01;
    p->tolerance = 1e-8;
    p->max_iterations = 1000;
    p->scheme = 0;
    p->substeps = 3;
    p->level = 2;
    p->n_outer = 2;
    p->pressure_precond = PF2_PRECOND_JACOBI;
    p->calculate_loads = 0;
    p->body_boundary_id = -1;
    p->thickness = 1.0;
    p->mean_velocity = 1.0;
    p->body_cx = 0.2;
    p->body_cy = 0.2;
    p->pressure_precision = PF2_PRECISION_FP64;
    p->pressure_x0 = PF2_X0_GIVEN;
    p->gmres_restart = 0;
    p->pressure_criterion = PF2_CRITERION_ABS;
    p->pressure_tolerance = 0.0;
    p->pressure_max_iterations = 0;
    p->learn_steps = 500;
    p->learn_rate = 1e-3f;
    p->pressure_ordering = PF2_ORDERING_NATURAL;
    p->gmres_orthogonalization = PF2_GS_MODIFIED;
    p->cg_variant = PF2_CG_STANDARD;
    p->prediction_solver = PF2_SOLVER_GMRES;
    return PF2_OK;
}

pf2_status pf2_assemble_poisson(const pf2_mesh* m, pf2_csr* A, double* rhs, int kind, double lambda, const pf2_bc* bc,
                                void* stream) {
    PF2_TRY(check_csr(m, A));
    PF2_TRY(check_bc(m, bc));
    PF2_REQUIRE(rhs, PF2_BAD_INPUT, "null rhs");
    k_poisson<<<blocks_for(m->nv), kThreads, 0, as_stream(stream)>>>(m->nv, row_mesh(m), kind, lambda, A->val.p, rhs,
                                                                      bc_view(bc));
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

pf2_status pf2_assemble_velocity_prediction(const pf2_mesh* m, const pf2_params* p, const double* ux,
                                            const double* uy, const double* uxo, const double* uyo,
                                            const double* pold, pf2_csr* Ax, pf2_csr* Ay, double* rx, double* ry,
                                            const pf2_bc* bcx, const pf2_bc* bcy, void* stream) {
    PF2_TRY(check_csr(m, Ax));
    PF2_TRY(check_csr(m, Ay));
    PF2_TRY(check_bc(m, bcx));
    PF2_TRY(check_bc(m, bcy));
    PF2_REQUIRE(p && ux && uy && uxo && uyo && rx && ry, PF2_BAD_INPUT, "null argument");
    return launch_prediction(m, FlowCoef{ p->rho, p->mu, p->dt }, true, ux, uy, uxo, uyo, pold, Ax->val.p, Ay->val.p,
                             rx, ry, bcx, bcy, as_stream(stream));
}

pf2_status pf2_assemble_pressure(const pf2_mesh* m, const pf2_params* p, const double* px, const double* py,
                                 const double* pold, pf2_csr* A, double* rhs, const pf2_bc* bc, void* stream) {
    PF2_TRY(check_csr(m, A));
    PF2_TRY(check_bc(m, bc));
    PF2_REQUIRE(p && px && py && rhs, PF2_BAD_INPUT, "null argument");
    return launch_pressure(m, FlowCoef{ p->rho, p->mu, p->dt }, true, px, py, pold, A->val.p, rhs, bc,
                           as_stream(stream));
}

pf2_status pf2_assemble_velocity_correction(const pf2_mesh* m, const pf2_params* p, const double* px,
                                            const double* py, const double* pres, const double* pold, pf2_csr* Ax,
                                            pf2_csr* Ay, double* rx, double* ry, const pf2_bc* bcx,
                                            const pf2_bc* bcy, void* stream) {
    PF2_TRY(check_csr(m, Ax));
    PF2_TRY(check_csr(m, Ay));
    PF2_TRY(check_bc(m, bcx));
    PF2_TRY(check_bc(m, bcy));
    PF2_REQUIRE(p && px && py && pres && rx && ry, PF2_BAD_INPUT, "null argument");
    return launch_correction(m, FlowCoef{ p->rho, p->mu, p->dt }, true, px, py, pres, pold, Ax->val.p, Ay->val.p, rx,
                             ry, bcx, bcy, as_stream(stream));
}

pf2_status pf2_prediction_bc_values(const pf2_mesh* m, const pf2_params* p, const pf2_bc* src, pf2_bc* dst,
                                    const double* pres, const double* pold, int comp, void* stream) {
    PF2_REQUIRE(m && p && src && dst && pres, PF2_BAD_INPUT, "null argument");
    PF2_REQUIRE(src->n_bc == dst->n_bc, PF2_BAD_INPUT, "source and target boundary sets differ in size");
    PF2_REQUIRE(comp == 0 || comp == 1, PF2_BAD_INPUT, "component must be 0 or 1");
    return launch_prediction_bc(m, FlowCoef{ p->rho, p->mu, p->dt }, src, dst, pres, pold, comp, as_stream(stream));
}

pf2_status pf2_body_loads(const pf2_mesh* m, const pf2_params* p, double cx, double cy, const double* ux,
                          const double* uy, const double* pres, double* cxcy, void* stream) {
    PF2_REQUIRE(m && p && ux && uy && pres && cxcy, PF2_BAD_INPUT, "null argument");
    cudaStream_t st = as_stream(stream);
    DevBuf<double> out;
    PF2_TRY(out.alloc(kBodyLoadsDoubles));
    PF2_CUDA(cudaMemsetAsync(out.p, 0, sizeof(double) * kBodyLoadsDoubles, st));
    PF2_TRY(launch_body_loads(m, FlowCoef{ p->rho, p->mu, p->dt }, p->body_boundary_id, p->thickness,
                              p->mean_velocity, cx, cy, ux, uy, pres, out.p, st));
    PF2_CUDA(cudaMemcpyAsync(cxcy, out.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaStreamSynchronize(st));
    return PF2_OK;
}

// ------------------------------------------------------------ CSR and BCs
pf2_status pf2_csr_create(const pf2_mesh* m, pf2_csr** out) {
    PF2_REQUIRE(m && out, PF2_BAD_INPUT, "null argument");
    *out = nullptr;
    pf2_csr* A = new pf2_csr();
    A->mesh = m;
    A->n = m->nv;
    A->nnz = m->nnz;
    pf2_status s = A->val.alloc(m->nnz);
    if (s == PF2_OK && cudaMemset(A->val.p, 0, sizeof(double) * m->nnz) != cudaSuccess) s = PF2_CUDA_ERROR;
    if (s != PF2_OK) { delete A; return s; }
    *out = A;
    return PF2_OK;
}

pf2_status pf2_csr_destroy(pf2_csr* A) {
    delete A;
    return PF2_OK;
}

pf2_status pf2_csr_sizes(const pf2_csr* A, int* rows, int* nnz) {
    PF2_REQUIRE(A, PF2_BAD_INPUT, "null matrix");
    if (rows) *rows = A->n;
    if (nnz) *nnz = A->nnz;
    return PF2_OK;
}

pf2_status pf2_csr_view(const pf2_csr* A, const int** rp, const int** col, double** val) {
    PF2_REQUIRE(A, PF2_BAD_INPUT, "null matrix");
    if (rp) *rp = A->mesh->rowptr.p;
    if (col) *col = A->mesh->col.p;
    if (val) *val = A->val.p;
    return PF2_OK;
}

pf2_status pf2_csr_clear_values(pf2_csr* A, void* stream) {
    PF2_REQUIRE(A, PF2_BAD_INPUT, "null matrix");
    PF2_CUDA(cudaMemsetAsync(A->val.p, 0, sizeof(double) * A->nnz, as_stream(stream)));
    return PF2_OK;
}

pf2_status pf2_csr_download(const pf2_csr* A, int* rp, int* col, double* val) {
    PF2_REQUIRE(A, PF2_BAD_INPUT, "null matrix");
    PF2_CUDA(cudaDeviceSynchronize());
    if (rp) PF2_CUDA(cudaMemcpy(rp, A->mesh->rowptr.p, sizeof(int) * (A->n + 1), cudaMemcpyDeviceToHost));
    if (col) PF2_CUDA(cudaMemcpy(col, A->mesh->col.p, sizeof(int) * A->nnz, cudaMemcpyDeviceToHost));
    if (val) PF2_CUDA(cudaMemcpy(val, A->val.p, sizeof(double) * A->nnz, cudaMemcpyDeviceToHost));
    return PF2_OK;
}

pf2_status pf2_csr_upload_values(pf2_csr* A, const double* val) {
    PF2_REQUIRE(A && val, PF2_BAD_INPUT, "null argument");
    PF2_CUDA(cudaMemcpy(A->val.p, val, sizeof(double) * A->nnz, cudaMemcpyHostToDevice));
    return PF2_OK;
}

pf2_status pf2_bc_create(int n_nodes, int n_bc, const pf2_dirichlet_node* nodes, pf2_bc** out) {
    PF2_REQUIRE(out && n_nodes > 0 && n_bc >= 0 && (n_bc == 0 || nodes), PF2_BAD_INPUT, "bad boundary set arguments");
    *out = nullptr;
    std::vector<int> node(n_bc), map(n_nodes, -1);
    std::vector<double> val(n_bc);
    for (int b = 0; b < n_bc; ++b) {
        PF2_REQUIRE(nodes[b].node < (unsigned)n_nodes, PF2_BAD_INPUT, "boundary node %u out of range",
                    nodes[b].node);
        node[b] = (int)nodes[b].node;
        val[b] = nodes[b].value;
        map[node[b]] = b;  // setupNodeMap: the last entry of a repeated node wins
    }
    pf2_bc* B = new pf2_bc();
    B->n_nodes = n_nodes;
    B->n_bc = n_bc;
    B->h_node = node;
    pf2_status s = B->node.alloc(n_bc);
    if (s == PF2_OK) s = B->value.alloc(n_bc);
    if (s == PF2_OK) s = B->node_to_bc.alloc(n_nodes);
    if (s == PF2_OK && n_bc &&
        (cudaMemcpy(B->node.p, node.data(), sizeof(int) * n_bc, cudaMemcpyHostToDevice) != cudaSuccess ||
         cudaMemcpy(B->value.p, val.data(), sizeof(double) * n_bc, cudaMemcpyHostToDevice) != cudaSuccess))
        s = PF2_CUDA_ERROR;
    if (s == PF2_OK &&
        cudaMemcpy(B->node_to_bc.p, map.data(), sizeof(int) * n_nodes, cudaMemcpyHostToDevice) != cudaSuccess)
        s = PF2_CUDA_ERROR;
    if (s != PF2_OK) {
        delete B;
        if (s == PF2_CUDA_ERROR) set_error("pf2_bc_create: device copy failed");
        return s;
    }
    *out = B;
    return PF2_OK;
}

pf2_status pf2_bc_destroy(pf2_bc* b) {
    delete b;
    return PF2_OK;
}

pf2_status pf2_bc_size(const pf2_bc* b, int* n) {
    PF2_REQUIRE(b && n, PF2_BAD_INPUT, "null argument");
    *n = b->n_bc;
    return PF2_OK;
}

pf2_status pf2_bc_set_values(pf2_bc* b, const double* values, void* stream) {
    PF2_REQUIRE(b && (values || b->n_bc == 0), PF2_BAD_INPUT, "null argument");
    if (b->n_bc)
        PF2_CUDA(cudaMemcpyAsync(b->value.p, values, sizeof(double) * b->n_bc, cudaMemcpyDeviceToDevice,
                                 as_stream(stream)));
    return PF2_OK;
}

pf2_status pf2_bc_get_values(const pf2_bc* b, double* values, void* stream) {
    PF2_REQUIRE(b && (values || b->n_bc == 0), PF2_BAD_INPUT, "null argument");
    if (b->n_bc)
        PF2_CUDA(cudaMemcpyAsync(values, b->value.p, sizeof(double) * b->n_bc, cudaMemcpyDeviceToDevice,
                                 as_stream(stream)));
    return PF2_OK;
}

pf2_status pf2_bc_apply(const pf2_bc* b, pf2_csr* A, double* rhs, void* stream) {
    PF2_REQUIRE(b && A && rhs, PF2_BAD_INPUT, "null argument");
    PF2_REQUIRE(b->n_nodes == A->n, PF2_BAD_INPUT, "boundary set and matrix sizes differ");
    k_apply_bc<<<blocks_for(A->n), kThreads, 0, as_stream(stream)>>>(A->n, A->mesh->rowptr.p, A->mesh->col.p,
                                                                      A->val.p, rhs, bc_view(b));
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

}  // extern "C"
