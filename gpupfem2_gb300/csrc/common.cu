// common.cu - error reporting, the device scan, and status strings.
#include <atomic>
#include <cstdarg>
#include <cstring>

#include "common.cuh"
#include "device.cuh"

namespace pf2 {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

pf2_status cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    const char* f = strrchr(file, '/');
    set_error("%s failed: %s (%s:%d)", what, cudaGetErrorString(e), f ? f + 1 : file, line);
    return PF2_CUDA_ERROR;
}

static std::atomic<unsigned long long> g_launches{ 0 };
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int num_sms() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

// ------------------------------------------------------------------ scan
// Three-pass exclusive scan: per-block sums (2048 items per block), a scan of the block
// sums (recursively), then a block-local scan plus the block offset.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan_int(int v, int* sh, int& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = lane < (kScanThreads / 32) ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < (kScanThreads / 32)) sh[lane] = s;
    }
    __syncthreads();
    const int before = (w > 0 ? sh[w - 1] : 0) + x - v;
    total = sh[kScanThreads / 32 - 1];
    __syncthreads();
    return before;
}

__global__ void k_scan_reduce(const int* __restrict__ in, long long n, int* __restrict__ bsum) {
    __shared__ int sh[32];
    const long long base = (long long)blockIdx.x * kScanTile;
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const long long i = base + (long long)threadIdx.x * kScanItems + k;
        if (i < n) s += in[i];
    }
    int total;
    block_exclusive_scan_int(s, sh, total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void k_scan_apply(const int* __restrict__ in, long long n, const int* __restrict__ boff,
                             int* __restrict__ out, int write_total) {
    __shared__ int sh[32];
    const long long base = (long long)blockIdx.x * kScanTile;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const long long i = base + (long long)threadIdx.x * kScanItems + k;
        v[k] = (i < n) ? in[i] : 0;
        s += v[k];
    }
    int total;
    int run = block_exclusive_scan_int(s, sh, total) + (boff ? boff[blockIdx.x] : 0);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const long long i = base + (long long)threadIdx.x * kScanItems + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (write_total && threadIdx.x == kScanThreads - 1 && base + kScanTile >= n) out[n] = run;
}

size_t scan_scratch_ints(long long n) {
    size_t total = 0;
    long long m = n;
    while (m > kScanTile) {
        const long long nb = (m + kScanTile - 1) / kScanTile;
        total += (size_t)nb + 1;
        m = nb;
    }
    return total + 1;
}

static pf2_status scan_level(const int* in, int* out, long long n, int* scratch, cudaStream_t st) {
    const long long nb = (n + kScanTile - 1) / kScanTile;
    if (nb <= 1) {
        k_scan_apply<<<1, kScanThreads, 0, st>>>(in, n, nullptr, out, 1);
        PF2_LAUNCH_CHECK();
        return PF2_OK;
    }
    int* bsum = scratch;         // nb + 1 entries (exclusive scan of the sums)
    int* rest = scratch + nb + 1;
    k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, bsum);
    PF2_LAUNCH_CHECK();
    PF2_TRY(scan_level(bsum, bsum, nb, rest, st));
    k_scan_apply<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, bsum, out, 0);
    PF2_LAUNCH_CHECK();
    // out[n] = total: the exclusive scan of block sums has it at bsum[nb]
    PF2_CUDA(cudaMemcpyAsync(out + n, bsum + nb, sizeof(int), cudaMemcpyDeviceToDevice, st));
    return PF2_OK;
}

pf2_status exclusive_scan(const int* in, int* out, long long n, int* scratch, cudaStream_t st) {
    if (n <= 0) {
        PF2_CUDA(cudaMemsetAsync(out, 0, sizeof(int), st));
        return PF2_OK;
    }
    return scan_level(in, out, n, scratch, st);
}

}  // namespace pf2

extern "C" {

const char* pf2_last_error(void) { return pf2::g_err; }

const char* pf2_status_string(pf2_status s) {
    switch (s) {
        case PF2_OK: return "ok";
        case PF2_NOT_CONVERGED: return "solver did not converge";
        case PF2_BAD_INPUT: return "bad input";
        case PF2_OVERFLOW: return "capacity overflow";
        case PF2_CUDA_ERROR: return "CUDA error";
        case PF2_TIMEOUT: return "device wait timed out";
        case PF2_IO_ERROR: return "I/O error";
    }
    return "unknown status";
}

int pf2_abi_version(void) { return PF2_ABI_VERSION; }

unsigned long long pf2_kernel_launches(void) { return pf2::g_launches.load(); }

}  // extern "C"
