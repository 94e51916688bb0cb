// Learned radiance cache on the fifth-generation tensor cores (include/rc_mlp.h).
//
// Every layer product runs as tcgen05.mma: bf16 operands staged in shared memory in the
// canonical no-swizzle K-major layout (rc_umma.cuh), FP32 accumulators in tensor memory read
// back with tcgen05.ld, one elected thread issuing the MMAs and an mbarrier signalled by
// tcgen05.commit.  Every wait is bounded; a wait that gives up sets the error flag, and the
// kernel still releases its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/rc_mlp.h"
#include "rc_umma.cuh"

namespace {

using namespace rc::umma;

constexpr uint32_t WAIT_LIMIT = 1u << 24;
constexpr int TILE_M = 128;

// ---------------------------------------------------------------- one tile product
// D[128 x N] = A[128 x K] B[N x K]^T, bf16 in, FP32 out; 128 threads (one warpgroup).
__global__ void __launch_bounds__(128) k_tile_product(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                      float* __restrict__ D, int K, int N, unsigned* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_base;
    uint8_t* sa = smem;
    uint8_t* sb = smem + (size_t)TILE_M * K * 2;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // stage A and B in the K-major core-matrix layout
    for (int idx = tid; idx < TILE_M * K; idx += 128) {
        const int r = idx / K, k = idx % K;
        *reinterpret_cast<uint16_t*>(sa + kmajor_offset(r, k, K)) = A[idx];
    }
    for (int idx = tid; idx < N * K; idx += 128) {
        const int r = idx / K, k = idx % K;
        *reinterpret_cast<uint16_t*>(sb + kmajor_offset(r, k, K)) = B[idx];
    }
    fence_proxy_async();
    if (tid == 0) mbar_init(&mbar, 1);
    const uint32_t ncols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
    if (warp == 0) tmem_alloc(&tmem_base, ncols);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = tmem_base;
    if (tid == 0) {
        const uint32_t idesc = idesc_bf16_f32(TILE_M, N);
        const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
        for (int kk = 0; kk < K / 16; ++kk)
            mma_bf16(tmem, smem_desc(a0 + 256u * kk, 128u, 16u * K), smem_desc(b0 + 256u * kk, 128u, 16u * K), idesc, kk > 0);
        mma_commit(&mbar);
    }
    const bool ok = mbar_wait(&mbar, 0, WAIT_LIMIT);
    if (!ok && lane == 0) atomicOr(err, 1u);
    fence_after_sync();
    if (ok) {
        const int row = warp * 32 + lane;
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
            tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 16; ++i) D[(size_t)row * N + c + i] = v[i];
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
}

}  // namespace

extern "C" rc_status rc_mlp_tile_product(const uint16_t* d_a, const uint16_t* d_b, float* d_d, int K, int N, unsigned* d_err,
                                         void* stream) {
    if (!d_a || !d_b || !d_d || !d_err || K < 16 || K > 256 || K % 16 || N < 16 || N > 256 || N % 16) return RC_ERR_ARG;
    const size_t smem = (size_t)(TILE_M + N) * K * 2;
    if (smem > 200 * 1024) return RC_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (smem > 48 * 1024 && cudaFuncSetAttribute(k_tile_product, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return RC_ERR_CUDA;
    k_tile_product<<<1, 128, smem, st>>>(d_a, d_b, d_d, K, N, d_err);
    return cudaGetLastError() == cudaSuccess ? RC_OK : RC_ERR_CUDA;
}
