// ocsl_dot_noalloc: the dot product of ocsl_dot_device without any device
// allocation, for callers that cannot call cudaMalloc -- host programs
// whose device memory is entirely reserved up front by another allocator (a
// framework's caching pool, a fixed embedded budget), where a cudaMalloc
// would fail, and hosts whose plugins may not allocate or free device memory
// while they run, because cudaMalloc and cudaFree can synchronise the device
// and stall the host's other streams.  No context is needed either.
//
// The per-tile partial sums and the completion counter live in one
// file-scope __device__ array of fixed size, so every GPU that loads this
// library holds kNoAllocScratchBytes (32,832 bytes) until the process exits.
// Host code cannot use the array's name as a device address: it is resolved
// with cudaGetSymbolAddress once per device, with that device current, the
// first time ocsl_dot_noalloc runs on that device.
//
// The arithmetic is the library's fixed tile order (2048-element tiles, lane
// fma chains from 0, xor butterfly per warp, warp sums in order, then the
// same over the tile sums), so the result equals ocsl_dot_device bit for bit.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/ocsl.h"

namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 8;
constexpr int kTile = kThreads * kPerThread;          // 2048 elements
constexpr int kMaxTiles = 4096;                        // n <= 8,388,608
constexpr size_t kMaxN = (size_t)kMaxTiles * kTile;
constexpr int kScratchDoubles = kMaxTiles + 8;         // partials + counter slot
constexpr int kMaxDevices = 64;

// The scratch: kMaxTiles tile partials, then (in slot kMaxTiles) the 32-bit
// counter of finished CTAs.  Shared by every call on the device.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;
thread_local std::string g_noalloc_error;

__device__ __forceinline__ double warp_butterfly(double v)
{
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

__device__ __forceinline__ double cta_sum(double v, double* s_red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double w = warp_butterfly(v);
    if (lane == 0) s_red[warp] = w;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0) {
        s = s_red[0];
        for (int k = 1; k < kThreads / 32; ++k) s = s + s_red[k];
    }
    __syncthreads();
    return s;
}

__global__ void __launch_bounds__(kThreads)
dot_noalloc_kernel(int n, const double* __restrict__ x, const double* __restrict__ y,
                   double* scratch, double* result)
{
    __shared__ double s_red[kThreads / 32];
    __shared__ int s_last;
    const int tile = blockIdx.x;
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < kPerThread; ++j) {
        const int e = tile * kTile + j * kThreads + (int)threadIdx.x;
        if (e < n) acc = fma(x[e], y[e], acc);
    }
    const double s = cta_sum(acc, s_red);
    unsigned* counter = reinterpret_cast<unsigned*>(scratch + kMaxTiles);
    if (threadIdx.x == 0) {
        scratch[tile] = s;
        __threadfence();
        s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double a = 0.0;
    for (int t = threadIdx.x; t < (int)gridDim.x; t += kThreads) a = a + __ldcg(scratch + t);
    const double total = cta_sum(a, s_red);
    if (threadIdx.x == 0) {
        *result = total;
        *counter = 0u;
    }
}

bool aligned8(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 7u) == 0; }

// Address of the scratch array on the current device; resolved once per device.
int scratch_for_current_device(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        g_noalloc_error = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
        return e == cudaErrorNoDevice ? OCSL_NO_DEVICE : OCSL_CUDA_ERROR;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        g_noalloc_error = "device index beyond the no-alloc table";
        return OCSL_BAD_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            g_noalloc_error = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return OCSL_CUDA_ERROR;
        }
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return OCSL_OK;
}

}  // namespace

extern "C" {

int ocsl_dot_noalloc(size_t n, const double* d_x, const double* d_y, double* d_result,
                     void* stream)
{
    if (!d_result || (n > 0 && (!d_x || !d_y))) {
        g_noalloc_error = "null pointer";
        return OCSL_BAD_ARGUMENT;
    }
    // the kernel loads and stores whole doubles: a pointer off an 8-byte
    // boundary would fault in the caller's context, so it is refused here
    if (!aligned8(d_result) || (n > 0 && (!aligned8(d_x) || !aligned8(d_y)))) {
        g_noalloc_error = "pointer not aligned to 8 bytes";
        return OCSL_BAD_ARGUMENT;
    }
    if (n > kMaxN) {
        g_noalloc_error = "n = " + std::to_string(n) + " exceeds the no-alloc limit of " +
                          std::to_string(kMaxN) + " elements";
        return OCSL_BAD_ARGUMENT;
    }
    double* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != OCSL_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (n == 0) {
        e = cudaMemsetAsync(d_result, 0, sizeof(double), st);
    } else {
        // the counter must start at 0 (the last CTA also resets it)
        e = cudaMemsetAsync(scratch + kMaxTiles, 0, sizeof(unsigned), st);
        if (e == cudaSuccess) {
            const int tiles = (int)((n + kTile - 1) / kTile);
            dot_noalloc_kernel<<<tiles, kThreads, 0, st>>>((int)n, d_x, d_y, scratch, d_result);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        g_noalloc_error = std::string("launch: ") + cudaGetErrorString(e);
        return OCSL_CUDA_ERROR;
    }
    return OCSL_OK;
}

const char* ocsl_noalloc_last_error(void) { return g_noalloc_error.c_str(); }

}  // extern "C"
