// common.cuh - shared internals of the PFEM-2 engine: error handling, device buffers,
// the object layouts behind the C ABI, and small device helpers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "../../include/pf2.h"

namespace pf2 {

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
pf2_status cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define PF2_CUDA(call)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) return ::pf2::cuda_fail(e_, #call, __FILE__, __LINE__);   \
    } while (0)

#define PF2_REQUIRE(cond, status, ...)                                                   \
    do {                                                                                 \
        if (!(cond)) {                                                                   \
            ::pf2::set_error(__VA_ARGS__);                                               \
            return status;                                                               \
        }                                                                                \
    } while (0)

#define PF2_TRY(expr)                                                                    \
    do {                                                                                 \
        pf2_status s_ = (expr);                                                          \
        if (s_ != PF2_OK) return s_;                                                     \
    } while (0)

// Every kernel launch of the engine goes through one of these two macros, which also
// count the launches (pf2_kernel_launches).
void count_launch();
#define PF2_LAUNCH_CHECK()                                                               \
    do {                                                                                 \
        ::pf2::count_launch();                                                           \
        PF2_CUDA(cudaGetLastError());                                                    \
    } while (0)
#define PF2_COOP_LAUNCH(fn, grid, block, args, smem, st)                                 \
    do {                                                                                 \
        ::pf2::count_launch();                                                           \
        PF2_CUDA(cudaLaunchCooperativeKernel((fn), (grid), (block), (args), (smem), (st))); \
    } while (0)

// ------------------------------------------------------ device buffers
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    pf2_status alloc(size_t count) {
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) { p = nullptr; return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__); }
        n = count;
        return PF2_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
};

template <class T>
struct PinnedBuf {
    T* p = nullptr;
    size_t n = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() { if (p) cudaFreeHost(p); }
    pf2_status alloc(size_t count) {
        if (p) cudaFreeHost(p);
        cudaError_t e = cudaMallocHost(&p, (count ? count : 1) * sizeof(T));
        if (e != cudaSuccess) { p = nullptr; return cuda_fail(e, "cudaMallocHost", __FILE__, __LINE__); }
        n = count;
        return PF2_OK;
    }
};

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

constexpr int kThreads = 256;
inline unsigned blocks_for(long long n, int threads = kThreads) {
    return (unsigned)((n + threads - 1) / threads);
}
int num_sms();

// Device-side status word values (written by kernels, read by the host).
enum DevStatus : int {
    DEV_OK = 0,
    DEV_NOT_CONVERGED = 1,
    DEV_BAD_INPUT = 2,
    DEV_OVERFLOW = 3,
    DEV_TIMEOUT = 5,
};

// Limits of the local (per-thread) arrays of the setup and assembly kernels.
constexpr int kMaxNodeDegree = 32;   // cells around one node
constexpr int kMaxRow = 32;          // CSR entries of one row
constexpr int kMaxLevel = 4;         // cellDivisionLevel (src/common/constants.h:15)
constexpr int kMaxPerCell = kMaxLevel * kMaxLevel;
constexpr double kDoubleMin = 2e-6;  // CONSTANTS::DOUBLE_MIN (src/common/constants.h:5)

// Cell word of a particle: bits 0..25 the cell, bits 26..30 = 1 + sub-cell index for a
// particle that still sits at a sub-cell centroid (seeded or reseeded and not yet
// located), whose third barycentric coordinate is the centroid's stored one rather
// than 1 - l0 - l1.
constexpr int kCellBits = 26;  // cell index bits; bits 26..30 hold 1 + sub-cell, the sign bit stays clear
constexpr int kCellMask = (1 << kCellBits) - 1;
constexpr int kMaxCells = kCellMask;

// ------------------------------------------------------------- scan
// Exclusive prefix sum of n int32 values produced by a functor (out has n+1 entries,
// out[n] = total).  Scratch size from scan_scratch_ints().
size_t scan_scratch_ints(long long n);
pf2_status exclusive_scan(const int* in, int* out, long long n, int* scratch, cudaStream_t st);

}  // namespace pf2

// ---------------------------------------------------------------- objects
struct pf2_mesh {
    int nv = 0, nc = 0, nnb = 0, nnz = 0, ninc = 0;
    int max_row = 0, max_degree = 0;
    pf2::DevBuf<double2> xy;
    pf2::DevBuf<int> tri;          // int[3*nc]
    pf2::DevBuf<int4> tri4;        // (a, b, c, 0)
    pf2::DevBuf<double> area;
    pf2::DevBuf<double4_32a> invJ;     // row-major {(0,0),(0,1),(1,0),(1,1)}
    pf2::DevBuf<double2> v3;       // third vertex of each cell
    pf2::DevBuf<float4> invJf;     // FP32 copies of invJ and v3 (cell-location pre-filter only)
    pf2::DevBuf<float2> v3f;
    pf2::DevBuf<int> nb_off, nb_idx;
    pf2::DevBuf<int> edge_ids;     // int[3*nc]
    // node -> incident cells (ascending), packed (cell << 2 | local vertex)
    pf2::DevBuf<int> inc_off, inc;
    // CSR pattern shared by every matrix of this mesh
    pf2::DevBuf<int> rowptr, col, diag;
    // positions in row i of the three vertices of each incident cell, 3 x 10 bits
    pf2::DevBuf<int> inc_pos;
    std::vector<double> h_xy;
    std::vector<int> h_tri;
};

// Mesh3D: linear tetrahedra.  The node graph's CSR pattern sits in `graph`, a pf2_mesh
// with no cells of its own, so that matrices, boundary sets and solvers of 3D meshes use
// the same objects as 2D ones.
struct pf2_mesh3d {
    int nv = 0, nc = 0, nnb = 0;
    pf2::DevBuf<double4_32a> xyz;  // (x, y, z, 0)
    pf2::DevBuf<int4> tet;
    pf2::DevBuf<double> volume;
    pf2::DevBuf<double> invJ;      // 9 per cell, row-major
    pf2::DevBuf<int> nb_off, nb_idx;
    // node -> incident cells (ascending), packed (cell << 2 | local vertex), and the
    // positions in row i of the cell's four vertices, 4 x 8 bits
    pf2::DevBuf<int> inc_off, inc, inc_pos;
    pf2_mesh graph;
    std::vector<double> h_xyz;
    std::vector<int> h_tet;
};

struct pf2_csr {
    const pf2_mesh* mesh = nullptr;
    int n = 0, nnz = 0;
    pf2::DevBuf<double> val;
};

struct pf2_bc {
    int n_nodes = 0, n_bc = 0;
    pf2::DevBuf<int> node;        // boundary node of each entry
    pf2::DevBuf<double> value;    // boundary value
    pf2::DevBuf<int> node_to_bc;  // -1 or entry index, per node
    std::vector<int> h_node;
};
