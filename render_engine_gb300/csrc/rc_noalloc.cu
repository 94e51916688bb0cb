// Error sums of a radiance cache with no device allocation (rc_error_sums_noalloc).
//
// Some callers cannot allocate device memory themselves: a renderer whose per-frame path
// runs under a fixed budget set aside at start-up (cudaMalloc and cudaFree synchronise the
// device and can fail in the middle of a frame), or a host process whose own memory manager
// owns all device memory and hands this library only buffers it already holds.  For them
// this entry point computes the same FP64 sums as the error path of rc_frame -- sum of
// squared errors of the cache estimate against the reference, sum of the reference, count
// of valid points -- from buffers the caller passes, and keeps its scratch space (per-block
// partial sums and a completion counter) in a fixed array declared in this file, which every
// GPU that loads the library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/rc_api.h"
#include "rc_internal.h"

namespace {

constexpr int NA_BLOCK = rc::BLOCK;
constexpr int NA_MAX_BLOCKS = RC_NOALLOC_MAX_POINTS / NA_BLOCK;   // 16384 blocks of 256 points
constexpr int NA_PARTS = 3 * NA_MAX_BLOCKS;                        // three sums per block

// Scratch: NA_PARTS doubles of block partials, then the completion counter (as 8 bytes).
// 393,224 bytes per device.
static __device__ __align__(256) double g_noalloc_scratch[NA_PARTS + 1];

std::mutex g_setup_mutex;
double* g_scratch_addr[64] = {nullptr};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// One thread per point; block sums in warp order, the grid's last block adds the block sums
// in a fixed order and writes out3.  est = sum over the lit lights of the cache (the
// reference's est_of, poc_gpu.cu:427-431); error terms as k_error (poc_gpu.cu:683-696).
__global__ void __launch_bounds__(NA_BLOCK) k_error_noalloc(const float* __restrict__ lc, int stride, int nl, int dormant,
                                                            const float* __restrict__ ref, const uint8_t* __restrict__ valid,
                                                            int np, double* __restrict__ out3, double* scratch) {
    __shared__ double sh[3][NA_BLOCK / 32];
    __shared__ bool last;
    unsigned* ticket = reinterpret_cast<unsigned*>(scratch + NA_PARTS);
    const int i = blockIdx.x * NA_BLOCK + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    if (i < np && valid[i]) {
        float e = 0.f;
        for (int l = 0; l < nl; ++l)
            if (!((dormant >> l) & 1)) e += lc[(size_t)stride * i + l];
        e = e - ref[i];
        v[0] = double(e) * e;
        v[1] = ref[i];
        v[2] = 1.0;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double r = warp_sum(v[k]);
        if (lane == 0) sh[k][w] = r;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double s = sh[k][0];
            for (int j = 1; j < NA_BLOCK / 32; ++j) s = s + sh[k][j];
            scratch[3 * blockIdx.x + k] = s;
        }
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // slot t sums partials t, t+256, ... in order; then each group of 32 slots goes through the
    // butterfly and the 8 group sums are added in order
    const int G = gridDim.x;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double x = 0.0;
        if ((int)threadIdx.x < G) x = __ldcg(scratch + 3 * threadIdx.x + k);
        for (int b = threadIdx.x + NA_BLOCK; b < G; b += NA_BLOCK) x = x + __ldcg(scratch + 3 * b + k);
        x = warp_sum(x);
        if (lane == 0) sh[k][w] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double s = sh[k][0];
            for (int j = 1; j < NA_BLOCK / 32; ++j) s = s + sh[k][j];
            out3[k] = s;
        }
        *ticket = 0u;
    }
}

// Address of this file's scratch array on the current device, looked up once per device and kept
// for the life of the process (a cudaDeviceReset unloads the array and leaves the kept address
// stale: the entry point is not for use on a device after a reset).
cudaError_t scratch_for_current_device(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        double* p = nullptr;
        e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" rc_status rc_error_sums_noalloc(const float* lc, int lc_stride, int nl, int dormant, const float* ref,
                                           const uint8_t* valid, int np, double* out3, void* stream) {
    if (!lc || !ref || !valid || !out3 || nl <= 0 || nl > 32 || lc_stride < nl || np <= 0) return RC_ERR_ARG;
    if (np > RC_NOALLOC_MAX_POINTS) return RC_ERR_ARG;   // beyond the fixed scratch array
    double* scratch = nullptr;
    if (scratch_for_current_device(&scratch) != cudaSuccess) return RC_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    // the completion counter must start at zero (a call that was cut short can leave it set)
    if (cudaMemsetAsync(scratch + NA_PARTS, 0, sizeof(double), st) != cudaSuccess) return RC_ERR_CUDA;
    const int grid = (np + NA_BLOCK - 1) / NA_BLOCK;
    k_error_noalloc<<<grid, NA_BLOCK, 0, st>>>(lc, lc_stride, nl, dormant, ref, valid, np, out3, scratch);
    return cudaGetLastError() == cudaSuccess ? RC_OK : RC_ERR_CUDA;
}
