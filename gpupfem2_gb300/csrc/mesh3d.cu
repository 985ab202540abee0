// mesh3d.cu - Mesh3D and the Poisson3D integrator on the device: tetrahedron geometry,
// node incidence, the node graph's CSR pattern, face-sharing neighbour lists and the
// row-centric assembly of the Poisson system.
//
// Reference: src/mesh_3d.cu (volume and inverse Jacobian :12-35, all-pairs neighbour
// kernel :37-82, DAT reader :84-147), sparse_matrix.cu:56-97 (CSR pattern) and
// cases/Poisson3D/main.cu:22-85 (rhs function and kIntegrateOverCell).  The neighbour
// lists and the pattern come from the node incidence in O(N) instead of all pairs; the
// assembly gives each matrix row to one thread, which sums the contributions of the
// row's cells in ascending cell order, so no atomics are needed and the result does not
// depend on timing.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <vector>

#include "common.cuh"
#include "device.cuh"

namespace pf2 {

namespace {

constexpr int kMaxNodeDegree3 = 64;  // cells around one node
constexpr int kMaxRow3 = 128;        // CSR entries of one row (positions fit 8 bits)

// createCellQuadratureFormula(1) (quadrature_formula_3d.cu, case 1): six points with
// barycentric (x, y, z), w = 1 - x - y - z formed as there, and their weights (which
// sum to 1; the integral is weight x volume).
constexpr int kQ3 = 6;
constexpr double kQ3xyz[kQ3][3] = { { 0.0701026973651683, 0.166660699730426, 0.596575741463645 },
                                    { 0.168695371477743, 0.584652626698847, 0.168695218708539 },
                                    { 0.418175789241166, 0.0803037256707293, 0.418101348156118 },
                                    { 0.596576288848820, 0.166672635105983, 0.0700786026978242 },
                                    { 0.164808547352848, 0.0851134715186107, 0.164808684755350 },
                                    { 0.0731475667668616, 0.440339136918213, 0.0731570614497775 } };
constexpr double kQ3w[kQ3] = { 0.180396407632724, 0.193316294293662, 0.133594798870359,
                               0.180371079146698, 0.201016720944591, 0.111304699111967 };

struct Quad3 {
    double L[kQ3][4];
    double w[kQ3];
};

Quad3 quad3() {
    Quad3 q{};
    for (int k = 0; k < kQ3; ++k) {
        for (int a = 0; a < 3; ++a) q.L[k][a] = kQ3xyz[k][a];
        q.L[k][3] = ((1.0 - kQ3xyz[k][0]) - kQ3xyz[k][1]) - kQ3xyz[k][2];
        q.w[k] = kQ3w[k];
    }
    return q;
}

}  // namespace

__global__ void k_tet4(int nc, const int* __restrict__ tet, int4* tet4, int nv, int* err) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int v[4] = { tet[4 * c], tet[4 * c + 1], tet[4 * c + 2], tet[4 * c + 3] };
    bool ok = true;
    for (int a = 0; a < 4; ++a) {
        ok = ok && v[a] >= 0 && v[a] < nv;
        for (int b = a + 1; b < 4; ++b) ok = ok && v[a] != v[b];
    }
    if (!ok) atomicExch(err, (int)DEV_BAD_INPUT);
    tet4[c] = make_int4(v[0], v[1], v[2], v[3]);
}

// kCalculateCellVolume / kCalculateInvJacobi (mesh_3d.cu:12-35): with e_k = v_k - v_3,
// volume = |e_0 . (e_1 x e_2)| / 6 and invJ = J^-1 for J with rows e_0, e_1, e_2, by the
// adjugate; as GenericMatrix3x3::inverse (matrix3x3.cuh) a cell with |det J| < 2e-6 gets
// the zero matrix.
__global__ void k_geometry3d(int nc, const double4_32a* __restrict__ xyz, const int4* __restrict__ tet,
                             double* volume, double* invJ) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int4 t = tet[c];
    const double4_32a p0 = xyz[t.x], p1 = xyz[t.y], p2 = xyz[t.z], p3 = xyz[t.w];
    const double a0 = p0.x - p3.x, a1 = p0.y - p3.y, a2 = p0.z - p3.z;
    const double b0 = p1.x - p3.x, b1 = p1.y - p3.y, b2 = p1.z - p3.z;
    const double c0 = p2.x - p3.x, c1 = p2.y - p3.y, c2 = p2.z - p3.z;
    // cofactors of the first row
    const double m00 = b1 * c2 - b2 * c1, m01 = b2 * c0 - b0 * c2, m02 = b0 * c1 - b1 * c0;
    const double det = a0 * m00 + a1 * m01 + a2 * m02;
    volume[c] = fabs(det) * (1.0 / 6.0);
    double* J = invJ + 9 * (size_t)c;
    if (fabs(det) < kDoubleMin) {
        for (int k = 0; k < 9; ++k) J[k] = 0.0;
        return;
    }
    const double r = 1.0 / det;
    J[0] = r * m00;
    J[1] = r * (a2 * c1 - a1 * c2);
    J[2] = r * (a1 * b2 - a2 * b1);
    J[3] = r * m01;
    J[4] = r * (a0 * c2 - a2 * c0);
    J[5] = r * (a2 * b0 - a0 * b2);
    J[6] = r * m02;
    J[7] = r * (a1 * c0 - a0 * c1);
    J[8] = r * (a0 * b1 - a1 * b0);
}

__global__ void k_inc_count3(int nc, const int4* __restrict__ tet, int* cnt) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int4 t = tet[c];
    atomicAdd(&cnt[t.x], 1);
    atomicAdd(&cnt[t.y], 1);
    atomicAdd(&cnt[t.z], 1);
    atomicAdd(&cnt[t.w], 1);
}

__global__ void k_inc_fill3(int nc, const int4* __restrict__ tet, const int* __restrict__ off, int* cursor,
                            int* inc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int4 t = tet[c];
    const int v[4] = { t.x, t.y, t.z, t.w };
#pragma unroll
    for (int k = 0; k < 4; ++k) inc[off[v[k]] + atomicAdd(&cursor[v[k]], 1)] = (c << 2) | k;
}

// ascending cell order per node (the atomics above fill in arbitrary order)
__global__ void k_inc_sort3(int nv, const int* __restrict__ off, int* inc, int* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int s = off[i], e = off[i + 1];
    if (e - s > kMaxNodeDegree3) atomicExch(err, (int)DEV_BAD_INPUT);
    for (int a = s + 1; a < e; ++a) {
        const int x = inc[a];
        int b = a - 1;
        while (b >= s && inc[b] > x) { inc[b + 1] = inc[b]; --b; }
        inc[b + 1] = x;
    }
}

// CSR rows: {i} U vertices of the incident cells, ascending (sparse_matrix.cu:56-97)
template <bool FILL>
__global__ void k_rows3(int nv, const int* __restrict__ off, const int* __restrict__ inc, const int4* __restrict__ tet,
                        int* rowlen, const int* __restrict__ rowptr, int* col) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    int buf[1 + 4 * kMaxNodeDegree3];
    int m = 0;
    buf[m++] = i;
    const int s = off[i], e = min(off[i + 1], s + kMaxNodeDegree3);
    for (int q = s; q < e; ++q) {
        const int4 t = tet[inc[q] >> 2];
        buf[m++] = t.x;
        buf[m++] = t.y;
        buf[m++] = t.z;
        buf[m++] = t.w;
    }
    const int u = sort_unique(buf, m);
    if (!FILL) {
        rowlen[i] = u;
    } else {
        const int o = rowptr[i];
        for (int k = 0; k < u; ++k) col[o + k] = buf[k];
    }
}

__global__ void k_diag_pos3(int nv, const int* __restrict__ rowptr, const int* __restrict__ col,
                            const int* __restrict__ off, const int* __restrict__ inc, const int4* __restrict__ tet,
                            int* diag, int* inc_pos, int* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int rs = rowptr[i], re = rowptr[i + 1];
    if (re - rs > kMaxRow3) atomicExch(err, (int)DEV_BAD_INPUT);
    auto find = [&](int target) {
        int lo = rs, hi = re - 1;
        while (lo <= hi) {
            const int m = (lo + hi) >> 1;
            const int cm = col[m];
            if (cm == target) return m - rs;
            if (cm < target) lo = m + 1; else hi = m - 1;
        }
        return 255;
    };
    const int d = find(i);
    diag[i] = rs + (d < kMaxRow3 ? d : 0);
    if (d >= kMaxRow3) atomicExch(err, (int)DEV_BAD_INPUT);
    for (int q = off[i]; q < off[i + 1]; ++q) {
        const int4 t = tet[inc[q] >> 2];
        const int a = find(t.x), b = find(t.y), c = find(t.z), w = find(t.w);
        if (a >= kMaxRow3 || b >= kMaxRow3 || c >= kMaxRow3 || w >= kMaxRow3) atomicExch(err, (int)DEV_BAD_INPUT);
        inc_pos[q] = (a & 255) | ((b & 255) << 8) | ((c & 255) << 16) | ((w & 255) << 24);
    }
}

// Cells sharing exactly three vertices (a face) with cell c, ascending: the lists of
// Mesh3D::fillCellNeighborIndices (mesh_3d.cu:37-82), from the incidence of c's vertices:
// a cell that occurs in three of the four vertex lists shares that face.
template <bool FILL>
__global__ void k_neighbors3(int nc, const int4* __restrict__ tet, const int* __restrict__ off,
                             const int* __restrict__ inc, int* cnt, const int* __restrict__ nb_off, int* nb_idx) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int buf[4 * kMaxNodeDegree3];
    int m = 0;
    const int4 t = tet[c];
    const int v[4] = { t.x, t.y, t.z, t.w };
    for (int k = 0; k < 4; ++k) {
        const int s = off[v[k]], e = min(off[v[k] + 1], s + kMaxNodeDegree3);
        for (int q = s; q < e; ++q) {
            const int cc = inc[q] >> 2;
            if (cc != c) buf[m++] = cc;
        }
    }
    // sort with repeats kept, then keep the runs of length 3
    for (int a = 1; a < m; ++a) {
        const int x = buf[a];
        int b = a - 1;
        while (b >= 0 && buf[b] > x) { buf[b + 1] = buf[b]; --b; }
        buf[b + 1] = x;
    }
    int u = 0, o = FILL ? nb_off[c] : 0;
    for (int q = 0; q < m;) {
        int r = q + 1;
        while (r < m && buf[r] == buf[q]) ++r;
        if (r - q == 3) {
            if (FILL) nb_idx[o + u] = buf[q];
            ++u;
        }
        q = r;
    }
    if (!FILL) cnt[c] = u;
}

// kIntegrateOverCell of cases/Poisson3D/main.cu:26-67, row-centric.  With the gradients
// G_j = invJ * grad N_j (shapeFuncGrad3D: e_0, e_1, e_2, (-1,-1,-1)), the cell's entry
// (k, j) is sum_q lambda (G_k . G_j) w_q and its rhs entry sum_q f(x_q) L_k(q) w_q, both
// times the volume, summed per quadrature point in the reference's order.
__global__ void k_poisson3d(int nv, const int* __restrict__ rowptr, const int* __restrict__ off,
                            const int* __restrict__ inc, const int* __restrict__ inc_pos,
                            const int4* __restrict__ tet, const double4_32a* __restrict__ xyz,
                            const double* __restrict__ volume, const double* __restrict__ invJ, Quad3 Q,
                            double lambda, int rhs_kind, double* val, double* rhs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int rs = rowptr[i], re = rowptr[i + 1];
    for (int p = rs; p < re; ++p) val[p] = 0.0;
    double bi = 0.0;
    for (int q = off[i]; q < off[i + 1]; ++q) {
        const int c = inc[q] >> 2, k = inc[q] & 3;
        const int pos = inc_pos[q];
        const double* J = invJ + 9 * (size_t)c;
        double G[4][3];
        for (int r = 0; r < 3; ++r) {
            G[0][r] = J[3 * r];
            G[1][r] = J[3 * r + 1];
            G[2][r] = J[3 * r + 2];
            G[3][r] = -((G[0][r] + G[1][r]) + G[2][r]);
        }
        const double vol = volume[c];
        for (int j = 0; j < 4; ++j) {
            const double d = G[k][0] * G[j][0] + G[k][1] * G[j][1] + G[k][2] * G[j][2];
            double s = 0.0;
            for (int g = 0; g < kQ3; ++g) s += lambda * d * Q.w[g];
            val[rs + ((pos >> (8 * j)) & 255)] += s * vol;
        }
        const int4 t = tet[c];
        const double4_32a P[4] = { xyz[t.x], xyz[t.y], xyz[t.z], xyz[t.w] };
        double f = 0.0;
        for (int g = 0; g < kQ3; ++g) {
            const double* L = Q.L[g];
            const double x = L[0] * P[0].x + L[1] * P[1].x + L[2] * P[2].x + L[3] * P[3].x;
            const double y = L[0] * P[0].y + L[1] * P[1].y + L[2] * P[2].y + L[3] * P[3].y;
            const double z = L[0] * P[0].z + L[1] * P[1].z + L[2] * P[2].z + L[3] * P[3].z;
            double fx;
            if (rhs_kind == PF2_RHS3D_GAUSSIAN) {
                fx = exp(-(x * x + 10 * y * y + z * z));
            } else {
                const double pi = 3.14159265358979323846;
                fx = 3.0 * pi * pi * sin(pi * x) * sin(pi * y) * sin(pi * z);
            }
            f += fx * L[k] * Q.w[g];
        }
        bi += f * vol;
    }
    rhs[i] = bi;
}

static pf2_status read_err3(const int* d_err, cudaStream_t st, int* h) {
    PF2_CUDA(cudaMemcpyAsync(h, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaStreamSynchronize(st));
    return PF2_OK;
}

static pf2_status build_mesh3d(pf2_mesh3d* M, int nv, const double* xyz, int nc, const int* tet, int fill_nb,
                               cudaStream_t st) {
    PF2_REQUIRE(nv > 0 && nc > 0, PF2_BAD_INPUT, "mesh needs nodes and cells (nv=%d, nc=%d)", nv, nc);
    PF2_REQUIRE(nc < (1 << 29) && nv < (1 << 29), PF2_BAD_INPUT, "mesh too large (nv=%d, nc=%d)", nv, nc);
    M->nv = nv;
    M->nc = nc;
    M->h_xyz.assign(xyz, xyz + 3 * (size_t)nv);
    M->h_tet.assign(tet, tet + 4 * (size_t)nc);
    std::vector<double4_32a> pts(nv);
    for (int i = 0; i < nv; ++i) pts[i] = make_double4_32a(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0);
    DevBuf<int> raw, err;
    PF2_TRY(M->xyz.alloc(nv));
    PF2_TRY(M->tet.alloc(nc));
    PF2_TRY(M->volume.alloc(nc));
    PF2_TRY(M->invJ.alloc(9 * (size_t)nc));
    PF2_TRY(raw.alloc(4 * (size_t)nc));
    PF2_TRY(err.alloc(1));
    PF2_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    PF2_CUDA(cudaMemcpyAsync(M->xyz.p, pts.data(), sizeof(double4_32a) * nv, cudaMemcpyHostToDevice, st));
    PF2_CUDA(cudaMemcpyAsync(raw.p, tet, sizeof(int) * 4 * (size_t)nc, cudaMemcpyHostToDevice, st));
    const unsigned bc = blocks_for(nc), bv = blocks_for(nv);
    k_tet4<<<bc, kThreads, 0, st>>>(nc, raw.p, M->tet.p, nv, err.p);
    PF2_LAUNCH_CHECK();
    int h_err = 0;
    PF2_TRY(read_err3(err.p, st, &h_err));
    PF2_REQUIRE(h_err == 0, PF2_BAD_INPUT, "tetrahedron vertex index out of range or repeated");
    k_geometry3d<<<bc, kThreads, 0, st>>>(nc, M->xyz.p, M->tet.p, M->volume.p, M->invJ.p);
    PF2_LAUNCH_CHECK();
    // node incidence
    DevBuf<int> cnt, scratch;
    PF2_TRY(cnt.alloc((size_t)std::max(nv, nc) + 1));
    PF2_TRY(scratch.alloc(scan_scratch_ints(std::max(nv, nc) + 1)));
    PF2_TRY(M->inc_off.alloc(nv + 1));
    PF2_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * nv, st));
    k_inc_count3<<<bc, kThreads, 0, st>>>(nc, M->tet.p, cnt.p);
    PF2_LAUNCH_CHECK();
    PF2_TRY(exclusive_scan(cnt.p, M->inc_off.p, nv, scratch.p, st));
    PF2_TRY(M->inc.alloc(4 * (size_t)nc));
    PF2_TRY(M->inc_pos.alloc(4 * (size_t)nc));
    PF2_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * nv, st));
    k_inc_fill3<<<bc, kThreads, 0, st>>>(nc, M->tet.p, M->inc_off.p, cnt.p, M->inc.p);
    PF2_LAUNCH_CHECK();
    k_inc_sort3<<<bv, kThreads, 0, st>>>(nv, M->inc_off.p, M->inc.p, err.p);
    PF2_LAUNCH_CHECK();
    PF2_TRY(read_err3(err.p, st, &h_err));
    PF2_REQUIRE(h_err == 0, PF2_BAD_INPUT, "a node touches more than %d cells", kMaxNodeDegree3);
    // CSR pattern of the node graph
    pf2_mesh& G = M->graph;
    G.nv = nv;
    G.nc = 0;
    PF2_TRY(G.rowptr.alloc(nv + 1));
    k_rows3<false><<<bv, kThreads, 0, st>>>(nv, M->inc_off.p, M->inc.p, M->tet.p, cnt.p, nullptr, nullptr);
    PF2_LAUNCH_CHECK();
    PF2_TRY(exclusive_scan(cnt.p, G.rowptr.p, nv, scratch.p, st));
    PF2_CUDA(cudaMemcpyAsync(&G.nnz, G.rowptr.p + nv, sizeof(int), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaStreamSynchronize(st));
    PF2_TRY(G.col.alloc(G.nnz));
    PF2_TRY(G.diag.alloc(nv));
    k_rows3<true><<<bv, kThreads, 0, st>>>(nv, M->inc_off.p, M->inc.p, M->tet.p, nullptr, G.rowptr.p, G.col.p);
    PF2_LAUNCH_CHECK();
    k_diag_pos3<<<bv, kThreads, 0, st>>>(nv, G.rowptr.p, G.col.p, M->inc_off.p, M->inc.p, M->tet.p, G.diag.p,
                                          M->inc_pos.p, err.p);
    PF2_LAUNCH_CHECK();
    PF2_TRY(read_err3(err.p, st, &h_err));
    PF2_REQUIRE(h_err == 0, PF2_BAD_INPUT, "a matrix row has more than %d entries", kMaxRow3);
    // face-sharing neighbour lists
    PF2_TRY(M->nb_off.alloc(nc + 1));
    if (fill_nb) {
        k_neighbors3<false><<<bc, kThreads, 0, st>>>(nc, M->tet.p, M->inc_off.p, M->inc.p, cnt.p, nullptr, nullptr);
        PF2_LAUNCH_CHECK();
        PF2_TRY(exclusive_scan(cnt.p, M->nb_off.p, nc, scratch.p, st));
        PF2_CUDA(cudaMemcpyAsync(&M->nnb, M->nb_off.p + nc, sizeof(int), cudaMemcpyDeviceToHost, st));
        PF2_CUDA(cudaStreamSynchronize(st));
        PF2_TRY(M->nb_idx.alloc(M->nnb));
        k_neighbors3<true><<<bc, kThreads, 0, st>>>(nc, M->tet.p, M->inc_off.p, M->inc.p, nullptr, M->nb_off.p,
                                                     M->nb_idx.p);
        PF2_LAUNCH_CHECK();
    } else {
        PF2_CUDA(cudaMemsetAsync(M->nb_off.p, 0, sizeof(int) * (nc + 1), st));
        M->nnb = 0;
        PF2_TRY(M->nb_idx.alloc(1));
    }
    PF2_CUDA(cudaStreamSynchronize(st));
    return PF2_OK;
}

// Mesh3D::loadMeshFromFile (mesh_3d.cu:84-147).  Tokens are read until the end of the
// file; entities other than tetrahedra (type 304) are skipped by their vertex count
// (type % 100).
static pf2_status read_dat3(const char* path, double scale, std::vector<double>& xyz, std::vector<int>& tet) {
    std::ifstream f(path);
    PF2_REQUIRE(f.is_open(), PF2_IO_ERROR, "cannot open mesh file '%s'", path);
    long long nv = -1, ne = -1;
    f >> nv >> ne;
    PF2_REQUIRE(f && nv > 0 && ne >= 0, PF2_IO_ERROR, "bad DAT header in '%s'", path);
    xyz.resize(3 * (size_t)nv);
    for (long long i = 0; i < nv; ++i) {
        long long id;
        double x, y, z;
        f >> id >> x >> y >> z;
        PF2_REQUIRE(f, PF2_IO_ERROR, "truncated vertex list in '%s' at vertex %lld", path, i + 1);
        xyz[3 * i] = scale * x;
        xyz[3 * i + 1] = scale * y;
        xyz[3 * i + 2] = scale * z;
    }
    tet.clear();
    long long id, type;
    while (f >> id >> type) {
        const int nvert = (int)(type % 100);
        PF2_REQUIRE(nvert >= 1 && nvert <= 8, PF2_IO_ERROR, "unknown entity type %lld in '%s'", type, path);
        long long v[8];
        for (int k = 0; k < nvert; ++k) f >> v[k];
        PF2_REQUIRE(f, PF2_IO_ERROR, "truncated entity %lld in '%s'", id, path);
        if (type == 304)
            for (int k = 0; k < 4; ++k) tet.push_back((int)(v[k] - 1));
    }
    PF2_REQUIRE(!tet.empty(), PF2_IO_ERROR, "no tetrahedra in '%s'", path);
    return PF2_OK;
}

}  // namespace pf2

using namespace pf2;

extern "C" {

pf2_status pf2_mesh3d_create(int nv, const double* xyz, int nc, const int* tet, int fill_neighbors, void* stream,
                             pf2_mesh3d** out) {
    PF2_REQUIRE(out && xyz && tet, PF2_BAD_INPUT, "pf2_mesh3d_create: null argument");
    *out = nullptr;
    pf2_mesh3d* M = new pf2_mesh3d();
    const pf2_status s = build_mesh3d(M, nv, xyz, nc, tet, fill_neighbors, as_stream(stream));
    if (s != PF2_OK) {
        delete M;
        return s;
    }
    *out = M;
    return PF2_OK;
}

pf2_status pf2_mesh3d_load_dat(const char* path, int fill_neighbors, double scale, void* stream, pf2_mesh3d** out) {
    PF2_REQUIRE(path && out, PF2_BAD_INPUT, "pf2_mesh3d_load_dat: null argument");
    std::vector<double> xyz;
    std::vector<int> tet;
    PF2_TRY(read_dat3(path, scale, xyz, tet));
    for (int v : tet)
        PF2_REQUIRE(v >= 0 && (size_t)v < xyz.size() / 3, PF2_IO_ERROR, "vertex id out of range in '%s'", path);
    return pf2_mesh3d_create((int)(xyz.size() / 3), xyz.data(), (int)(tet.size() / 4), tet.data(), fill_neighbors,
                             stream, out);
}

pf2_status pf2_mesh3d_destroy(pf2_mesh3d* mesh) {
    delete mesh;
    return PF2_OK;
}

pf2_status pf2_mesh3d_sizes(const pf2_mesh3d* m, int* nv, int* nc, int* nnb) {
    PF2_REQUIRE(m, PF2_BAD_INPUT, "null mesh");
    if (nv) *nv = m->nv;
    if (nc) *nc = m->nc;
    if (nnb) *nnb = m->nnb;
    return PF2_OK;
}

pf2_status pf2_mesh3d_view_get(const pf2_mesh3d* m, pf2_mesh3d_view* v) {
    PF2_REQUIRE(m && v, PF2_BAD_INPUT, "null argument");
    v->nv = m->nv;
    v->nc = m->nc;
    v->n_neighbor_entries = m->nnb;
    v->xyz4 = reinterpret_cast<const double*>(m->xyz.p);
    v->tet = reinterpret_cast<const int*>(m->tet.p);
    v->volume = m->volume.p;
    v->inv_jacobi = m->invJ.p;
    v->neighbor_offsets = m->nb_off.p;
    v->neighbor_indices = m->nb_idx.p;
    return PF2_OK;
}

pf2_status pf2_mesh3d_download(const pf2_mesh3d* m, int field, void* dst) {
    PF2_REQUIRE(m && dst, PF2_BAD_INPUT, "null argument");
    PF2_CUDA(cudaDeviceSynchronize());
    switch (field) {
    case PF2_MESH3D_XYZ:
        memcpy(dst, m->h_xyz.data(), sizeof(double) * m->h_xyz.size());
        return PF2_OK;
    case PF2_MESH3D_TET:
        memcpy(dst, m->h_tet.data(), sizeof(int) * m->h_tet.size());
        return PF2_OK;
    case PF2_MESH3D_VOLUME:
        PF2_CUDA(cudaMemcpy(dst, m->volume.p, sizeof(double) * m->nc, cudaMemcpyDeviceToHost));
        return PF2_OK;
    case PF2_MESH3D_INV_JACOBI:
        PF2_CUDA(cudaMemcpy(dst, m->invJ.p, sizeof(double) * 9 * (size_t)m->nc, cudaMemcpyDeviceToHost));
        return PF2_OK;
    case PF2_MESH3D_NEIGHBOR_OFFSETS:
        PF2_CUDA(cudaMemcpy(dst, m->nb_off.p, sizeof(int) * (m->nc + 1), cudaMemcpyDeviceToHost));
        return PF2_OK;
    case PF2_MESH3D_NEIGHBOR_INDICES:
        if (m->nnb) PF2_CUDA(cudaMemcpy(dst, m->nb_idx.p, sizeof(int) * m->nnb, cudaMemcpyDeviceToHost));
        return PF2_OK;
    default:
        break;
    }
    PF2_REQUIRE(false, PF2_BAD_INPUT, "unknown 3D mesh field %d", field);
    return PF2_OK;
}

pf2_status pf2_csr_create_3d(const pf2_mesh3d* m, pf2_csr** out) {
    PF2_REQUIRE(m && out, PF2_BAD_INPUT, "null argument");
    return pf2_csr_create(&m->graph, out);
}

pf2_status pf2_assemble_poisson_3d(const pf2_mesh3d* m, pf2_csr* A, double* rhs, int rhs_kind, double lambda,
                                   const pf2_bc* bc, void* stream) {
    PF2_REQUIRE(m && A && rhs, PF2_BAD_INPUT, "null argument");
    PF2_REQUIRE(A->mesh == &m->graph, PF2_BAD_INPUT, "matrix was not created for this 3D mesh");
    PF2_REQUIRE(rhs_kind == PF2_RHS3D_GAUSSIAN || rhs_kind == PF2_RHS3D_SINSINSIN, PF2_BAD_INPUT,
                "unknown rhs kind %d", rhs_kind);
    cudaStream_t st = as_stream(stream);
    k_poisson3d<<<blocks_for(m->nv), kThreads, 0, st>>>(m->nv, m->graph.rowptr.p, m->inc_off.p, m->inc.p,
                                                         m->inc_pos.p, m->tet.p, m->xyz.p, m->volume.p, m->invJ.p,
                                                         quad3(), lambda, rhs_kind, A->val.p, rhs);
    PF2_LAUNCH_CHECK();
    if (bc) PF2_TRY(pf2_bc_apply(bc, A, rhs, stream));
    return PF2_OK;
}

}  // extern "C"
