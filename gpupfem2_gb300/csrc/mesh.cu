// mesh.cu - Mesh2D on the device: geometry, node incidence, CSR pattern, vertex-sharing
// neighbour lists and edge boundary ids, all built by O(N) kernels.
//
// Reference: src/mesh_2d.cu (geometry :10-34, DAT reader :36-96, all-pairs neighbour
// search :107-139) and src/linear_algebra/sparse_matrix.cu:8-54 (CSR pattern).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>

#include "common.cuh"
#include "device.cuh"

namespace pf2 {

// kCalculateCellArea / kCalculateInvJacobi (mesh_2d.cu:10-34) with
// Matrix2x2::inverse (cuda_math.cuh:124-141).
__global__ void k_geometry(int nc, const double2* __restrict__ xy, const int4* __restrict__ tri, double* area,
                           double4_32a* invJ, double2* v3, float4* invJf, float2* v3f) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int4 t = tri[c];
    const double2 A = xy[t.x], B = xy[t.y], D = xy[t.z];
    const double v12x = __dsub_rn(B.x, A.x), v12y = __dsub_rn(B.y, A.y);
    const double v13x = __dsub_rn(D.x, A.x), v13y = __dsub_rn(D.y, A.y);
    area[c] = fabs(__fma_rn(v12x, v13y, -__dmul_rn(v12y, v13x))) * 0.5;
    const double d0 = __dsub_rn(A.x, D.x), d1 = __dsub_rn(A.y, D.y);
    const double d2 = __dsub_rn(B.x, D.x), d3 = __dsub_rn(B.y, D.y);
    const double det = __fma_rn(d0, d3, -__dmul_rn(d1, d2));
    const double inv = __ddiv_rn(1.0, det);
    const double4_32a J = make_double4_32a(__dmul_rn(d3, inv), __dmul_rn(-d1, inv), __dmul_rn(-d2, inv),
                                           __dmul_rn(d0, inv));
    invJ[c] = J;
    v3[c] = D;
    invJf[c] = make_float4((float)J.x, (float)J.y, (float)J.z, (float)J.w);
    v3f[c] = make_float2((float)D.x, (float)D.y);
}

__global__ void k_tri4(int nc, const int* __restrict__ tri, int4* tri4, int nv, int* err) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int a = tri[3 * c], b = tri[3 * c + 1], d = tri[3 * c + 2];
    if (a < 0 || a >= nv || b < 0 || b >= nv || d < 0 || d >= nv || a == b || b == d || a == d)
        atomicExch(err, (int)DEV_BAD_INPUT);
    tri4[c] = make_int4(a, b, d, 0);
}

__global__ void k_inc_count(int nc, const int4* __restrict__ tri, int nv, int* cnt) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int4 t = tri[c];
    if (t.x >= 0 && t.x < nv) atomicAdd(&cnt[t.x], 1);
    if (t.y >= 0 && t.y < nv) atomicAdd(&cnt[t.y], 1);
    if (t.z >= 0 && t.z < nv) atomicAdd(&cnt[t.z], 1);
}

__global__ void k_inc_fill(int nc, const int4* __restrict__ tri, const int* __restrict__ off, int* cursor, int* inc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int4 t = tri[c];
    const int v[3] = { t.x, t.y, t.z };
#pragma unroll
    for (int k = 0; k < 3; ++k) inc[off[v[k]] + atomicAdd(&cursor[v[k]], 1)] = (c << 2) | k;
}

// ascending cell order per node (the atomics above fill in arbitrary order)
__global__ void k_inc_sort(int nv, const int* __restrict__ off, int* inc, int* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int s = off[i], e = off[i + 1];
    if (e - s > kMaxNodeDegree) atomicExch(err, (int)DEV_BAD_INPUT);
    for (int a = s + 1; a < e; ++a) {
        const int x = inc[a];
        int b = a - 1;
        while (b >= s && inc[b] > x) { inc[b + 1] = inc[b]; --b; }
        inc[b + 1] = x;
    }
}


// CSR rows: {i} U vertices of incident cells, sorted (sparse_matrix.cu:14-45)
template <bool FILL>
__global__ void k_rows(int nv, const int* __restrict__ off, const int* __restrict__ inc, const int4* __restrict__ tri,
                       int* rowlen, const int* __restrict__ rowptr, int* col) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    int buf[1 + 3 * kMaxNodeDegree];
    int m = 0;
    buf[m++] = i;
    const int s = off[i], e = min(off[i + 1], s + kMaxNodeDegree);
    for (int q = s; q < e; ++q) {
        const int4 t = tri[inc[q] >> 2];
        buf[m++] = t.x;
        buf[m++] = t.y;
        buf[m++] = t.z;
    }
    const int u = sort_unique(buf, m);
    if (!FILL) {
        rowlen[i] = u;
    } else {
        const int o = rowptr[i];
        for (int k = 0; k < u; ++k) col[o + k] = buf[k];
    }
}

__global__ void k_diag_and_pos(int nv, const int* __restrict__ rowptr, const int* __restrict__ col,
                               const int* __restrict__ off, const int* __restrict__ inc, const int4* __restrict__ tri,
                               int* diag, int* inc_pos, int* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int rs = rowptr[i], re = rowptr[i + 1];
    if (re - rs > kMaxRow) atomicExch(err, (int)DEV_BAD_INPUT);
    auto find = [&](int target) {
        int lo = rs, hi = re - 1;
        while (lo <= hi) {
            const int m = (lo + hi) >> 1;
            const int cm = col[m];
            if (cm == target) return m - rs;
            if (cm < target) lo = m + 1; else hi = m - 1;
        }
        return 1023;
    };
    const int d = find(i);
    diag[i] = rs + (d < kMaxRow ? d : 0);
    if (d >= kMaxRow) atomicExch(err, (int)DEV_BAD_INPUT);
    for (int q = off[i]; q < off[i + 1]; ++q) {
        const int4 t = tri[inc[q] >> 2];
        const int a = find(t.x), b = find(t.y), c = find(t.z);
        // the assembly kernels index a per-thread row buffer with these positions
        if (a >= kMaxRow || b >= kMaxRow || c >= kMaxRow) atomicExch(err, (int)DEV_BAD_INPUT);
        inc_pos[q] = (a & 1023) | ((b & 1023) << 10) | ((c & 1023) << 20);
    }
}

// Cells sharing at least one vertex, ascending, without the cell itself: the lists of
// Mesh2D::fillCellNeighborIndices (mesh_2d.cu:107-139), from the node incidence.
template <bool FILL>
__global__ void k_neighbors(int nc, const int4* __restrict__ tri, const int* __restrict__ off,
                            const int* __restrict__ inc, int* cnt, const int* __restrict__ nb_off, int* nb_idx) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int buf[3 * kMaxNodeDegree];
    int m = 0;
    const int4 t = tri[c];
    const int v[3] = { t.x, t.y, t.z };
    for (int k = 0; k < 3; ++k) {
        const int s = off[v[k]], e = min(off[v[k] + 1], s + kMaxNodeDegree);
        for (int q = s; q < e; ++q) {
            const int cc = inc[q] >> 2;
            if (cc != c) buf[m++] = cc;
        }
    }
    const int u = sort_unique(buf, m);
    if (!FILL) {
        cnt[c] = u;
    } else {
        const int o = nb_off[c];
        for (int k = 0; k < u; ++k) nb_idx[o + k] = buf[k];
    }
}

// kSetEdgeBoundaryIDs (cases/Cylinder2D/main.cu:35-70)
__global__ void k_channel_ids(int nc, const double2* __restrict__ xy, const int4* __restrict__ tri, double lx,
                              double ly, int has_cyl, double cx, double cy, double r, int* ids) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int4 t = tri[c];
    const int v[3] = { t.x, t.y, t.z };
    for (int i = 0; i < 3; ++i) {
        const double2 s = xy[v[i]], e = xy[v[(i + 1) % 3]];
        const double mx = __dmul_rn(__dadd_rn(s.x, e.x), 0.5);
        const double my = __dmul_rn(__dadd_rn(s.y, e.y), 0.5);
        int id = -1;
        if (fabs(mx) < kDoubleMin) id = 0;
        else if (fabs(mx - lx) < kDoubleMin) id = 1;
        else if (fabs(my) < kDoubleMin || fabs(my - ly) < kDoubleMin) id = 2;
        else if (has_cyl) {
            const double dx = mx - cx, dy = my - cy;
            if (fabs(sqrt(dx * dx + dy * dy) - r) < 0.001) id = 3;
        }
        ids[3 * c + i] = id;
    }
}

static pf2_status read_err(const int* d_err, cudaStream_t st, int* h) {
    PF2_CUDA(cudaMemcpyAsync(h, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaStreamSynchronize(st));
    return PF2_OK;
}

static pf2_status build_mesh(pf2_mesh* M, int nv, const double* xy, int nc, const int* tri, int fill_nb,
                             cudaStream_t st) {
    PF2_REQUIRE(nv > 0 && nc > 0, PF2_BAD_INPUT, "mesh needs nodes and cells (nv=%d, nc=%d)", nv, nc);
    PF2_REQUIRE(nc <= kMaxCells / 4 && nv < (1 << 29), PF2_BAD_INPUT, "mesh too large (nv=%d, nc=%d)", nv, nc);
    M->nv = nv;
    M->nc = nc;
    M->h_xy.assign(xy, xy + 2 * (size_t)nv);
    M->h_tri.assign(tri, tri + 3 * (size_t)nc);
    PF2_TRY(M->xy.alloc(nv));
    PF2_TRY(M->tri.alloc(3 * (size_t)nc));
    PF2_TRY(M->tri4.alloc(nc));
    PF2_TRY(M->area.alloc(nc));
    PF2_TRY(M->invJ.alloc(nc));
    PF2_TRY(M->v3.alloc(nc));
    PF2_TRY(M->invJf.alloc(nc));
    PF2_TRY(M->v3f.alloc(nc));
    PF2_TRY(M->edge_ids.alloc(3 * (size_t)nc));
    DevBuf<int> err;
    PF2_TRY(err.alloc(1));
    PF2_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    PF2_CUDA(cudaMemcpyAsync(M->xy.p, xy, sizeof(double2) * nv, cudaMemcpyHostToDevice, st));
    PF2_CUDA(cudaMemcpyAsync(M->tri.p, tri, sizeof(int) * 3 * (size_t)nc, cudaMemcpyHostToDevice, st));
    PF2_CUDA(cudaMemsetAsync(M->edge_ids.p, 0xff, sizeof(int) * 3 * (size_t)nc, st));
    const unsigned bc = blocks_for(nc), bv = blocks_for(nv);
    k_tri4<<<bc, kThreads, 0, st>>>(nc, M->tri.p, M->tri4.p, nv, err.p);
    PF2_LAUNCH_CHECK();
    int h_err = 0;
    PF2_TRY(read_err(err.p, st, &h_err));
    PF2_REQUIRE(h_err == 0, PF2_BAD_INPUT, "triangle vertex index out of range or repeated");
    k_geometry<<<bc, kThreads, 0, st>>>(nc, M->xy.p, M->tri4.p, M->area.p, M->invJ.p, M->v3.p, M->invJf.p,
                                        M->v3f.p);
    PF2_LAUNCH_CHECK();
    // node incidence
    DevBuf<int> cnt, scratch;
    PF2_TRY(cnt.alloc((size_t)std::max(nv, nc) + 1));
    PF2_TRY(scratch.alloc(scan_scratch_ints(std::max(nv, nc) + 1)));
    PF2_TRY(M->inc_off.alloc(nv + 1));
    PF2_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * nv, st));
    k_inc_count<<<bc, kThreads, 0, st>>>(nc, M->tri4.p, nv, cnt.p);
    PF2_LAUNCH_CHECK();
    PF2_TRY(exclusive_scan(cnt.p, M->inc_off.p, nv, scratch.p, st));
    M->ninc = 3 * nc;
    PF2_TRY(M->inc.alloc(M->ninc));
    PF2_TRY(M->inc_pos.alloc(M->ninc));
    PF2_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * nv, st));
    k_inc_fill<<<bc, kThreads, 0, st>>>(nc, M->tri4.p, M->inc_off.p, cnt.p, M->inc.p);
    PF2_LAUNCH_CHECK();
    k_inc_sort<<<bv, kThreads, 0, st>>>(nv, M->inc_off.p, M->inc.p, err.p);
    PF2_LAUNCH_CHECK();
    PF2_TRY(read_err(err.p, st, &h_err));
    PF2_REQUIRE(h_err == 0, PF2_BAD_INPUT, "a node touches more than %d cells", kMaxNodeDegree);
    // CSR pattern
    PF2_TRY(M->rowptr.alloc(nv + 1));
    k_rows<false><<<bv, kThreads, 0, st>>>(nv, M->inc_off.p, M->inc.p, M->tri4.p, cnt.p, nullptr, nullptr);
    PF2_LAUNCH_CHECK();
    PF2_TRY(exclusive_scan(cnt.p, M->rowptr.p, nv, scratch.p, st));
    PF2_CUDA(cudaMemcpyAsync(&M->nnz, M->rowptr.p + nv, sizeof(int), cudaMemcpyDeviceToHost, st));
    PF2_CUDA(cudaStreamSynchronize(st));
    PF2_TRY(M->col.alloc(M->nnz));
    PF2_TRY(M->diag.alloc(nv));
    k_rows<true><<<bv, kThreads, 0, st>>>(nv, M->inc_off.p, M->inc.p, M->tri4.p, nullptr, M->rowptr.p, M->col.p);
    PF2_LAUNCH_CHECK();
    k_diag_and_pos<<<bv, kThreads, 0, st>>>(nv, M->rowptr.p, M->col.p, M->inc_off.p, M->inc.p, M->tri4.p,
                                            M->diag.p, M->inc_pos.p, err.p);
    PF2_LAUNCH_CHECK();
    PF2_TRY(read_err(err.p, st, &h_err));
    PF2_REQUIRE(h_err == 0, PF2_BAD_INPUT, "a matrix row has more than %d entries", kMaxRow);
    // neighbour lists
    PF2_TRY(M->nb_off.alloc(nc + 1));
    if (fill_nb) {
        k_neighbors<false><<<bc, kThreads, 0, st>>>(nc, M->tri4.p, M->inc_off.p, M->inc.p, cnt.p, nullptr, nullptr);
        PF2_LAUNCH_CHECK();
        PF2_TRY(exclusive_scan(cnt.p, M->nb_off.p, nc, scratch.p, st));
        PF2_CUDA(cudaMemcpyAsync(&M->nnb, M->nb_off.p + nc, sizeof(int), cudaMemcpyDeviceToHost, st));
        PF2_CUDA(cudaStreamSynchronize(st));
        PF2_TRY(M->nb_idx.alloc(M->nnb));
        k_neighbors<true><<<bc, kThreads, 0, st>>>(nc, M->tri4.p, M->inc_off.p, M->inc.p, nullptr, M->nb_off.p,
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

// Mesh2D::loadMeshFromFile (mesh_2d.cu:36-96).  Tokens are read until the end of the
// file, so a trailing newline adds nothing (the reference's eof loop appends a
// spurious triangle in that case).
static pf2_status read_dat(const char* path, double scale, std::vector<double>& xy, std::vector<int>& tri) {
    std::ifstream f(path);
    PF2_REQUIRE(f.is_open(), PF2_IO_ERROR, "cannot open mesh file '%s'", path);
    long long nv = -1, ne = -1;
    f >> nv >> ne;
    PF2_REQUIRE(f && nv > 0 && ne >= 0, PF2_IO_ERROR, "bad DAT header in '%s'", path);
    xy.resize(2 * (size_t)nv);
    for (long long i = 0; i < nv; ++i) {
        long long id;
        double x, y, z;
        f >> id >> x >> y >> z;
        PF2_REQUIRE(f, PF2_IO_ERROR, "truncated vertex list in '%s' at vertex %lld", path, i + 1);
        xy[2 * i] = scale * x;
        xy[2 * i + 1] = scale * y;
    }
    tri.clear();
    long long id, type;
    while (f >> id >> type) {
        const int nvert = (int)(type % 100);
        PF2_REQUIRE(nvert >= 1 && nvert <= 8, PF2_IO_ERROR, "unknown entity type %lld in '%s'", type, path);
        long long v[8];
        for (int k = 0; k < nvert; ++k) f >> v[k];
        PF2_REQUIRE(f, PF2_IO_ERROR, "truncated entity %lld in '%s'", id, path);
        if (type == 203)
            for (int k = 0; k < 3; ++k) tri.push_back((int)(v[k] - 1));
    }
    PF2_REQUIRE(!tri.empty(), PF2_IO_ERROR, "no triangles in '%s'", path);
    return PF2_OK;
}

}  // namespace pf2

using namespace pf2;

extern "C" {

pf2_status pf2_mesh_create(int nv, const double* xy, int nc, const int* tri, int fill_neighbors, void* stream,
                           pf2_mesh** out) {
    PF2_REQUIRE(out && xy && tri, PF2_BAD_INPUT, "pf2_mesh_create: null argument");
    *out = nullptr;
    pf2_mesh* M = new pf2_mesh();
    const pf2_status s = build_mesh(M, nv, xy, nc, tri, fill_neighbors, as_stream(stream));
    if (s != PF2_OK) { delete M; return s; }
    *out = M;
    return PF2_OK;
}

pf2_status pf2_mesh_load_dat(const char* path, int fill_neighbors, double scale, void* stream, pf2_mesh** out) {
    PF2_REQUIRE(path && out, PF2_BAD_INPUT, "pf2_mesh_load_dat: null argument");
    std::vector<double> xy;
    std::vector<int> tri;
    PF2_TRY(read_dat(path, scale, xy, tri));
    for (int v : tri)
        PF2_REQUIRE(v >= 0 && (size_t)v < xy.size() / 2, PF2_IO_ERROR, "vertex id out of range in '%s'", path);
    return pf2_mesh_create((int)(xy.size() / 2), xy.data(), (int)(tri.size() / 3), tri.data(), fill_neighbors,
                           stream, out);
}

pf2_status pf2_mesh_destroy(pf2_mesh* mesh) {
    delete mesh;
    return PF2_OK;
}

pf2_status pf2_mesh_sizes(const pf2_mesh* m, int* nv, int* nc, int* nnb) {
    PF2_REQUIRE(m, PF2_BAD_INPUT, "null mesh");
    if (nv) *nv = m->nv;
    if (nc) *nc = m->nc;
    if (nnb) *nnb = m->nnb;
    return PF2_OK;
}

pf2_status pf2_mesh_view_get(const pf2_mesh* m, pf2_mesh_view* v) {
    PF2_REQUIRE(m && v, PF2_BAD_INPUT, "null argument");
    v->nv = m->nv;
    v->nc = m->nc;
    v->n_neighbor_entries = m->nnb;
    v->xy = reinterpret_cast<const double*>(m->xy.p);
    v->tri = m->tri.p;
    v->area = m->area.p;
    v->inv_jacobi = reinterpret_cast<const double*>(m->invJ.p);
    v->neighbor_offsets = m->nb_off.p;
    v->neighbor_indices = m->nb_idx.p;
    v->edge_boundary_ids = m->edge_ids.p;
    return PF2_OK;
}

pf2_status pf2_mesh_download(const pf2_mesh* m, int field, void* dst) {
    PF2_REQUIRE(m && dst, PF2_BAD_INPUT, "null argument");
    const void* src = nullptr;
    size_t bytes = 0;
    switch (field) {
        case PF2_MESH_XY: src = m->xy.p; bytes = sizeof(double2) * m->nv; break;
        case PF2_MESH_TRI: src = m->tri.p; bytes = sizeof(int) * 3 * (size_t)m->nc; break;
        case PF2_MESH_AREA: src = m->area.p; bytes = sizeof(double) * m->nc; break;
        case PF2_MESH_INV_JACOBI: src = m->invJ.p; bytes = sizeof(double4_32a) * m->nc; break;
        case PF2_MESH_NEIGHBOR_OFFSETS: src = m->nb_off.p; bytes = sizeof(int) * (m->nc + 1); break;
        case PF2_MESH_NEIGHBOR_INDICES: src = m->nb_idx.p; bytes = sizeof(int) * m->nnb; break;
        case PF2_MESH_EDGE_IDS: src = m->edge_ids.p; bytes = sizeof(int) * 3 * (size_t)m->nc; break;
        default: PF2_REQUIRE(false, PF2_BAD_INPUT, "unknown mesh field %d", field);
    }
    PF2_CUDA(cudaDeviceSynchronize());
    if (bytes) PF2_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return PF2_OK;
}

pf2_status pf2_mesh_set_channel_boundary_ids(pf2_mesh* m, double lx, double ly, int has_cyl, double cx, double cy,
                                             double r, void* stream) {
    PF2_REQUIRE(m, PF2_BAD_INPUT, "null mesh");
    k_channel_ids<<<blocks_for(m->nc), kThreads, 0, as_stream(stream)>>>(m->nc, m->xy.p, m->tri4.p, lx, ly, has_cyl,
                                                                          cx, cy, r, m->edge_ids.p);
    PF2_LAUNCH_CHECK();
    return PF2_OK;
}

pf2_status pf2_mesh_set_edge_boundary_ids(pf2_mesh* m, const int* ids) {
    PF2_REQUIRE(m && ids, PF2_BAD_INPUT, "null argument");
    PF2_CUDA(cudaMemcpy(m->edge_ids.p, ids, sizeof(int) * 3 * (size_t)m->nc, cudaMemcpyHostToDevice));
    return PF2_OK;
}

}  // extern "C"
