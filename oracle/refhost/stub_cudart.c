/*
 * stub_cudart.c - host-memory stand-in for the few CUDA runtime entry points that the
 * reference's host-side setup code calls (TEST INFRASTRUCTURE ONLY).
 *
 * Linked instead of libcudart into oracle/_ref/ref_host_dump, it lets the reference's
 * own DAT reader, CSR pattern builder, neighbour-list builder and particle-handler
 * constructor run on a CPU: "device" allocations are host allocations, copies are
 * memcpy, symbol copies write the host shadow of the __constant__ variable, and kernel
 * launches do nothing (no kernel result is read from this program).
 */
#include <stdlib.h>
#include <string.h>

static char stub_handle[64];

void** __cudaRegisterFatBinary(void* fat) { (void)fat; return (void**)stub_handle; }
void __cudaRegisterFatBinaryEnd(void** h) { (void)h; }
void __cudaUnregisterFatBinary(void** h) { (void)h; }
void __cudaRegisterFunction() {}
void __cudaRegisterVar() {}
char __cudaInitModule(void** h) { (void)h; return 1; }
unsigned __cudaPushCallConfiguration() { return 0; }
int __cudaPopCallConfiguration() { return 1; /* non-zero: the launch stub returns */ }
int __cudaGetKernel(void** k, const void* f) { *k = (void*)f; return 0; }
int __cudaLaunchKernel() { return 0; }
int cudaLaunchKernel() { return 0; }

int cudaMalloc(void** p, size_t n) { *p = calloc(n ? n : 1, 1); return *p ? 0 : 2; }
int cudaMallocHost(void** p, size_t n) { return cudaMalloc(p, n); }
int cudaFree(void* p) { free(p); return 0; }
int cudaFreeHost(void* p) { free(p); return 0; }
int cudaMemcpy(void* d, const void* s, size_t n, int kind) { (void)kind; memmove(d, s, n); return 0; }
int cudaMemcpyAsync(void* d, const void* s, size_t n, int kind, void* st) { (void)kind; (void)st; memmove(d, s, n); return 0; }
int cudaMemsetAsync(void* p, int v, size_t n, void* st) { (void)st; memset(p, v, n); return 0; }
int cudaMemset(void* p, int v, size_t n) { memset(p, v, n); return 0; }
int cudaMemcpyToSymbolAsync(const void* sym, const void* s, size_t n, size_t off, int kind, void* st)
{ (void)kind; (void)st; memcpy((char*)sym + off, s, n); return 0; }
int cudaMemcpyToSymbol(const void* sym, const void* s, size_t n, size_t off, int kind)
{ (void)kind; memcpy((char*)sym + off, s, n); return 0; }
int cudaMemcpyFromSymbol(void* d, const void* sym, size_t n, size_t off, int kind)
{ (void)kind; memcpy(d, (const char*)sym + off, n); return 0; }
int cudaDeviceSynchronize(void) { return 0; }
int cudaGetLastError(void) { return 0; }
const char* cudaGetErrorName(int e) { (void)e; return "stub"; }
const char* cudaGetErrorString(int e) { (void)e; return "stub"; }

/* Referenced by the CUB scan in Mesh3D::fillCellNeighborIndices (mesh_3d.cu:198-227),
 * which the 3D dump never calls (neighbour lists off): each reports an error. */
int cudaGetDevice(int* d) { (void)d; return 1; }
int cudaSetDevice(int d) { (void)d; return 1; }
int cudaGetDeviceCount(int* n) { if (n) *n = 0; return 1; }
int cudaDeviceGetAttribute(int* v, int attr, int dev) { (void)v; (void)attr; (void)dev; return 1; }
int cudaFuncGetAttributes(void* a, const void* f) { (void)a; (void)f; return 1; }
int cudaOccupancyMaxActiveBlocksPerMultiprocessorWithFlags(int* n, const void* f, int b, size_t s, unsigned fl)
{ (void)n; (void)f; (void)b; (void)s; (void)fl; return 1; }
int cudaPeekAtLastError(void) { return 0; }
