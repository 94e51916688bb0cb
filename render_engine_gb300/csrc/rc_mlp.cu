// Learned radiance cache on the fifth-generation tensor cores (include/rc_mlp.h).
//
// Every layer product runs as tcgen05.mma: bf16 operands staged in shared memory in the
// canonical no-swizzle K-major layout (rc_umma.cuh), FP32 accumulators in tensor memory read
// back with tcgen05.ld, one elected thread issuing the MMAs and an mbarrier signalled by
// tcgen05.commit.  Every wait is bounded; a wait that gives up sets the error flag, and the
// kernel still releases its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

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

// The bounded wait on its own: an mbarrier of one expected arrival, which one thread provides
// or nobody does; one thread polls it at most `polls` times.
__global__ void k_wait_check(uint32_t polls, int arrive, unsigned* __restrict__ err) {
    __shared__ uint64_t mbar;
    if (threadIdx.x == 0) mbar_init(&mbar, 1);
    __syncwarp();
    if (arrive && threadIdx.x == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&mbar)) : "memory");
    __syncwarp();
    if (threadIdx.x == 0 && !mbar_wait(&mbar, 0, polls)) atomicOr(err, 1u);
}

// ---------------------------------------------------------------- the network
// 168 input features (padded to 176) -> 64 -> 64 -> 64 -> 64 -> 16 outputs (the first n_out
// used), ReLU between layers, no biases.  Weights live as FP32 masters with their Adam
// moments, and as bf16 tiles in the K-major core-matrix layout the MMAs read: W_l (rows =
// outputs, K = inputs) for the forward products and W_l^T (rows = inputs, K = outputs) for
// the gradients that flow back.
constexpr int K0 = 176, HID = 64, OUTP = 16, NLAYER = 5;
__host__ __device__ constexpr int in_dim(int l) { return l == 0 ? K0 : HID; }
__host__ __device__ constexpr int out_dim(int l) { return l == NLAYER - 1 ? OUTP : HID; }
__host__ __device__ constexpr int master_off(int l) { return l == 0 ? 0 : HID * K0 + (l - 1) * HID * HID; }
constexpr int NWEIGHT = HID * K0 + 3 * HID * HID + OUTP * HID;   // 24,576
// bf16 tile byte offsets: forward tiles, then the transposed ones of layers 1..4
__host__ __device__ constexpr int wf_off(int l) { return 2 * master_off(l); }
constexpr int WF_BYTES = 2 * NWEIGHT;                                 // 49,152
__host__ __device__ constexpr int wb_off(int l) { return WF_BYTES + 2 * (master_off(l) - master_off(1)); }
constexpr int WB_BYTES = 2 * (3 * HID * HID + OUTP * HID);            // 26,624
// activation tiles of one 128-sample tile kept for the backward pass (training)
constexpr int ACT_X0T = 0;                                            // X0^T: 176 x 128
__host__ __device__ constexpr int act_ht(int l) { return K0 * 128 * 2 + (l - 1) * HID * 128 * 2; }   // H_l^T, l = 1..4
constexpr int ACT_DY = K0 * 128 * 2 + 4 * HID * 128 * 2;              // dY: 128 x 16 (K-major)
constexpr int ACT_DYT = ACT_DY + 128 * OUTP * 2;                      // dY^T: 16 x 128
constexpr int ACT_BYTES = ACT_DYT + OUTP * 128 * 2;                   // 122,880 per tile

struct MlpArgs {
    const uint8_t* wbf;        // bf16 tiles (forward, then transposed)
    const float4* P;           // point position (xyz)
    const float4* N;           // point normal (xyz)
    const float4* aux;         // albedo, direct light of lights 0..2
    const float* target;       // training targets, tstride floats per sample
    int tstride;
    const int* idx;            // sample -> point (null: identity)
    int n;                     // samples (a multiple of 128 when training)
    float* out;                // inference output, ostride floats per sample
    int ostride;
    int n_out;
    float lo[3], inv_ext[3];   // encoding box
    uint8_t* act;              // training: activation tiles, ACT_BYTES per tile
    float* dwpart;             // training: weight gradients of each backward CTA, NWEIGHT per CTA
    float* loss;               // training: sum of the relative L2 loss (for reporting)
    float loss_scale;          // 1 / (samples x n_out)
    const float* scale;        // training: the loss scale of this step (device, MlpState::SCALE)
    unsigned* err;
};

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ float bf16_at(const uint8_t* base, uint32_t off) {
    return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(base + off));
}
__device__ __forceinline__ void st_bf16(uint8_t* base, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}

// The 168 input features of one point (the rest of the 176 are zero): frequency encodings of
// the position in the box (12 octaves) and of the normal (4 octaves), one-blob encodings of
// both (16 and 4 bins per axis), the raw position, normal, direct light of three lights,
// albedo and a constant.  Produced eight at a time (one 16-byte group of the K-major tile);
// emit(group, f) stores them.  Two threads share a point: half 0 produces groups 0..8 (the
// position octaves), half 1 groups 9..21 (about the same work).
template <class Emit>
__device__ __forceinline__ void encode(const MlpArgs& a, int pt, int half, Emit&& emit) {
    const float4 P = a.P[pt], Nn = a.N[pt];
    const float p[3] = {fminf(fmaxf((P.x - a.lo[0]) * a.inv_ext[0], 0.f), 1.f), fminf(fmaxf((P.y - a.lo[1]) * a.inv_ext[1], 0.f), 1.f),
                        fminf(fmaxf((P.z - a.lo[2]) * a.inv_ext[2], 0.f), 1.f)};
    const float nv[3] = {Nn.x, Nn.y, Nn.z};
    float f[8];
    // Four octaves per group: sincosf at the first, then the double-angle identities
    // sin 2w = 2 sin w cos w, cos 2w = (cos w - sin w)(cos w + sin w).  Three doublings grow the
    // error of the exact pair by at most about 8x (a few 1e-7), far below the bf16 rounding of
    // the features.
    auto octaves = [&](float w) {
        sincosf(w, &f[0], &f[1]);
#pragma unroll
        for (int j = 1; j < 4; ++j) {
            const float s = f[2 * j - 2], c = f[2 * j - 1];
            f[2 * j] = 2.f * s * c;
            f[2 * j + 1] = (c - s) * (c + s);
        }
    };
    if (half == 0) {
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {   // features 24 ax .. 24 ax + 23: sin / cos of 2^o pi p
            float w = 3.14159265f * p[ax];
#pragma unroll
            for (int g = 0; g < 3; ++g, w *= 16.f) {
                octaves(w);
                emit(ax * 3 + g, f);
            }
        }
        return;
    }
    const float4 X = a.aux[pt];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {   // 72 + 8 ax: sin / cos of 2^o pi n
        octaves(3.14159265f * nv[ax]);
        emit(9 + ax, f);
    }
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {   // 96 + 16 ax: one-blob of p, 16 bins
        const float bp = p[ax] * 16.f;
        for (int g = 0; g < 2; ++g) {
#pragma unroll
            for (int j = 0; j < 8; ++j) f[j] = fmaxf(0.f, 1.f - fabsf(bp - (8 * g + j + 0.5f)));
            emit(12 + 2 * ax + g, f);
        }
    }
    float nb[12];   // 144 + 4 ax: one-blob of n, 4 bins
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        const float bn = (nv[ax] * 0.5f + 0.5f) * 4.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) nb[4 * ax + j] = fmaxf(0.f, 1.f - fabsf(bn - (j + 0.5f)));
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) f[j] = nb[j];
    emit(18, f);
    f[0] = nb[8]; f[1] = nb[9]; f[2] = nb[10]; f[3] = nb[11];
    f[4] = p[0]; f[5] = p[1]; f[6] = p[2]; f[7] = nv[0];          // 156..159
    emit(19, f);
    f[0] = nv[1]; f[1] = nv[2]; f[2] = X.y; f[3] = X.z; f[4] = X.w; f[5] = X.x; f[6] = 1.f; f[7] = 0.f;   // 160..167
    emit(20, f);
#pragma unroll
    for (int j = 0; j < 8; ++j) f[j] = 0.f;
    emit(21, f);
}

// Forward pass over tiles of 128 samples.  A CTA holds the bf16 weights once and runs GROUPS
// tiles at a time, each on its own group of two warpgroups (thread t of a group works on sample
// row t % 128; the two threads of a row split the input features and the columns of each
// accumulator, warp w reading the tensor-memory lanes of its quarter w % 4), with its own
// activation tile, mbarrier, named barrier and 64 tensor-memory columns; the groups overlap
// one tile's products with another's encoding and epilogues.
// TRAIN: also keeps X0^T, H_l^T and dY (with dY^T) of each tile in global memory and adds the
// loss; otherwise writes the n_out outputs.
constexpr int FWD_THREADS = 256;                               // threads of one group
constexpr int INFER_GROUPS = 4;                                // tiles in flight per inference CTA
constexpr size_t GROUP_SMEM_INFER = (size_t)128 * K0 * 2;      // activation tile
constexpr size_t GROUP_SMEM_TRAIN = GROUP_SMEM_INFER + (size_t)K0 * 128 * 2;   // + transposed staging
template <bool TRAIN, int GROUPS>
__global__ void __launch_bounds__(FWD_THREADS * GROUPS) k_mlp_forward(const MlpArgs a) {
    const float sc = TRAIN ? __ldg(a.scale) : 1.f;   // loss scale (a power of two)
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar[GROUPS];
    __shared__ uint32_t tmem_base;
    __shared__ int gflag[GROUPS];
    constexpr uint32_t TCOLS = GROUPS == 1 ? 64u : (GROUPS == 2 ? 128u : 256u);
    uint8_t* sw = smem;                               // forward weight tiles, WF_BYTES
    const int grp = threadIdx.x / FWD_THREADS, tid = threadIdx.x % FWD_THREADS;
    // this group's activation tile: X0 (128 x 176) and then each H_l (128 x 64) in its place,
    // H_{l+1} written once the product that reads H_l has completed
    uint8_t* sx = smem + WF_BYTES + (size_t)grp * (TRAIN ? GROUP_SMEM_TRAIN : GROUP_SMEM_INFER);
    uint8_t* st = sx + 128 * K0 * 2;                  // TRAIN: transposed staging, 176 x 128
    const int warp = tid >> 5, lane = tid & 31;
    const int row = tid & 127, half = tid >> 7, quarter = warp & 3;
    for (int i = threadIdx.x; i < WF_BYTES / 16; i += FWD_THREADS * GROUPS)
        reinterpret_cast<uint4*>(sw)[i] = reinterpret_cast<const uint4*>(a.wbf)[i];
    if (threadIdx.x < GROUPS) mbar_init(&mbar[threadIdx.x], 1);
    if (threadIdx.x < 32) tmem_alloc(&tmem_base, TCOLS);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = tmem_base + 64u * (uint32_t)grp;
    // the group's barrier (named barrier 1 + group; barrier 0 is the whole CTA's)
    auto gsync = [&]() { asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(FWD_THREADS) : "memory"); };
    uint32_t phase = 0;
    bool ok = true;
    const int ntiles = (a.n + 127) / 128;
    for (int tile = blockIdx.x * GROUPS + grp; tile < ntiles && ok; tile += gridDim.x * GROUPS) {
        const int s = tile * 128 + row;
        const bool live = s < a.n;
        const int pt = live ? (a.idx ? a.idx[s] : s) : 0;
        encode(a, pt, half, [&](int k8, const float (&f)[8]) {
            uint4 v;
            v.x = pack_bf16(f[0], f[1]);
            v.y = pack_bf16(f[2], f[3]);
            v.z = pack_bf16(f[4], f[5]);
            v.w = pack_bf16(f[6], f[7]);
            *reinterpret_cast<uint4*>(sx + kmajor_offset(row, 8 * k8, K0)) = v;
            if (TRAIN)
                for (int j = 0; j < 8; ++j) st_bf16(st, kmajor_offset(8 * k8 + j, row, 128), f[j]);
        });
        fence_proxy_async();
        gsync();
        if (TRAIN) {
            uint4* dst = reinterpret_cast<uint4*>(a.act + (size_t)tile * ACT_BYTES + ACT_X0T);
            for (int i = tid; i < K0 * 128 * 2 / 16; i += FWD_THREADS) dst[i] = reinterpret_cast<const uint4*>(st)[i];
            gsync();
        }
        for (int l = 0; l < NLAYER && ok; ++l) {
            const int K = in_dim(l), N = out_dim(l);
            uint8_t* A = sx;
            uint8_t* Hn = sx;
            if (tid == 0) {
                const uint32_t a0 = smem_u32(A), b0 = smem_u32(sw + wf_off(l));
                for (int kk = 0; kk < K / 16; ++kk)
                    mma_bf16(tmem, smem_desc(a0 + 256u * kk, 128u, 16u * K), smem_desc(b0 + 256u * kk, 128u, 16u * K),
                             idesc_bf16_f32(128, N), kk > 0);
                mma_commit(&mbar[grp]);
            }
            // one warp watches the barrier; the others wait at the group barrier without issuing
            // (the fence orders the products before the barrier for every thread of the group)
            if (warp == 0) {
                ok = mbar_wait(&mbar[grp], phase, WAIT_LIMIT);
                fence_before_sync();
                if (lane == 0) gflag[grp] = ok ? 1 : 0;
            }
            phase ^= 1u;
            gsync();
            ok = gflag[grp] != 0;   // the whole group leaves together
            if (!ok) {
                if (tid == 0) atomicOr(a.err, 1u);
                break;
            }
            fence_after_sync();
            // columns of this thread: one half of a hidden layer; all 16 outputs for half 0
            const int c0 = l < NLAYER - 1 ? half * (N / 2) : 0;
            const int c1 = l < NLAYER - 1 ? c0 + N / 2 : (half == 0 ? N : 0);
            for (int c = c0; c < c1; c += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c, v);
                tmem_wait_ld();
                if (l < NLAYER - 1) {
                    uint4 lo4, hi4;
                    lo4.x = pack_bf16(fmaxf(v[0], 0.f), fmaxf(v[1], 0.f));
                    lo4.y = pack_bf16(fmaxf(v[2], 0.f), fmaxf(v[3], 0.f));
                    lo4.z = pack_bf16(fmaxf(v[4], 0.f), fmaxf(v[5], 0.f));
                    lo4.w = pack_bf16(fmaxf(v[6], 0.f), fmaxf(v[7], 0.f));
                    hi4.x = pack_bf16(fmaxf(v[8], 0.f), fmaxf(v[9], 0.f));
                    hi4.y = pack_bf16(fmaxf(v[10], 0.f), fmaxf(v[11], 0.f));
                    hi4.z = pack_bf16(fmaxf(v[12], 0.f), fmaxf(v[13], 0.f));
                    hi4.w = pack_bf16(fmaxf(v[14], 0.f), fmaxf(v[15], 0.f));
                    *reinterpret_cast<uint4*>(Hn + kmajor_offset(row, c, HID)) = lo4;
                    *reinterpret_cast<uint4*>(Hn + kmajor_offset(row, c + 8, HID)) = hi4;
                    if (TRAIN)
                        for (int j = 0; j < 16; ++j) st_bf16(st, kmajor_offset(c + j, row, 128), fmaxf(v[j], 0.f));
                } else if (!TRAIN) {
                    if (live)
                        for (int j = 0; j < a.n_out; ++j) a.out[(size_t)s * a.ostride + j] = v[j];
                } else {
                    // relative L2 loss (y - t)^2 / (sg(y)^2 + 0.01) and its gradient
                    float lsum = 0.f;
                    uint8_t* dy = a.act + (size_t)tile * ACT_BYTES + ACT_DY;
                    uint8_t* dyt = a.act + (size_t)tile * ACT_BYTES + ACT_DYT;
                    for (int j = 0; j < OUTP; ++j) {
                        float g = 0.f;
                        if (live && j < a.n_out) {
                            const float t = a.target[(size_t)pt * a.tstride + j];   // the target of the sample's point
                            const float d = v[j] - t, den = v[j] * v[j] + 0.01f;
                            lsum += d * d / den;
                            g = 2.f * d / den * a.loss_scale * sc;
                        }
                        st_bf16(dy, kmajor_offset(row, j, OUTP), g);
                        st_bf16(dyt, kmajor_offset(j, row, 128), g);
                    }
                    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
                    if (lane == 0 && lsum != 0.f) atomicAdd(a.loss, lsum);
                }
            }
            fence_before_sync();
            fence_proxy_async();
            gsync();
            if (TRAIN && l < NLAYER - 1) {
                uint4* dst = reinterpret_cast<uint4*>(a.act + (size_t)tile * ACT_BYTES + act_ht(l + 1));
                for (int i = tid; i < HID * 128 * 2 / 16; i += FWD_THREADS) dst[i] = reinterpret_cast<const uint4*>(st)[i];
                gsync();
            }
            fence_after_sync();
        }
    }
    fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tmem_dealloc(tmem_base, TCOLS);
}

// 16-byte asynchronous copies global -> shared (no register staging)
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(sdst)), "l"(gsrc) : "memory");
}

// Backward pass (128 threads per CTA, one CTA per SM, tiles blockIdx.x, blockIdx.x + gridDim.x,
// ... in that order): for each tile and l = 4 .. 0, dW_l += dZ_l^T A_l over the tile's samples
// (rows of dZ^T beyond the layer's outputs are zero) and, for l >= 1,
// dZ_{l-1} = (dZ_l W_l) masked by ReLU'(H_l).  The weight gradients of all five layers stay in
// tensor memory across the CTA's tiles (the MMAs accumulate into them; columns bw_dw_col(l),
// 432 in all) and leave once, as the CTA's slot of dwpart; dZ_l W_l goes to columns BW_DA ..
// BW_DA + 63, per tile.  The transposed weights stay in shared memory for the whole kernel;
// each step's activation tile A_l^T is loaded into one of two buffers while the step before
// runs its products and its epilogue (and the next tile's dY, dY^T while its layers 3 .. 0
// run).  The tile order within a CTA and the number of CTAs are fixed, so the sums are
// reproducible.
constexpr uint32_t BW_COLS = 512;
constexpr uint32_t BW_DA = 448;
__host__ __device__ constexpr uint32_t bw_dw_col(int l) { return l == 0 ? 0u : (uint32_t)(K0 + (l - 1) * HID); }
static_assert(bw_dw_col(NLAYER - 1) + HID <= BW_DA && BW_DA + HID <= BW_COLS, "tensor-memory columns of the backward pass");
// shared-memory carve-up (bytes)
constexpr int BS_SAT = K0 * 128 * 2;                 // one A_l^T buffer (the largest, layer 0)
constexpr int BS_SWT = 2 * BS_SAT;                   // W_l^T of layers 1..4 (WB_BYTES)
constexpr int BS_SDZ = BS_SWT + WB_BYTES;            // dZ, 128 x 64 (K-major)
constexpr int BS_SDZT = BS_SDZ + 128 * HID * 2;      // dZ^T, 128 x 128 (rows 64.. zero)
constexpr int BS_SDY = BS_SDZT + 128 * 128 * 2;      // dY, 128 x 16 (K-major)
constexpr int BS_SDYT = BS_SDY + 128 * OUTP * 2;     // dY^T, 128 x 128 (rows 16.. zero)
constexpr int BS_END = BS_SDYT + 128 * 128 * 2;      // 202,752
__global__ void __launch_bounds__(128) k_mlp_backward(const MlpArgs a, int ntiles) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_base;
    uint8_t* sat[2] = {smem, smem + BS_SAT};
    uint8_t* swt = smem + BS_SWT;
    uint8_t* sdz = smem + BS_SDZ;
    uint8_t* sdzt = smem + BS_SDZT;
    uint8_t* sdy = smem + BS_SDY;
    uint8_t* sdyt = smem + BS_SDYT;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < 128 * 128 * 2 / 16; i += 128) {
        reinterpret_cast<uint4*>(sdzt)[i] = make_uint4(0u, 0u, 0u, 0u);
        reinterpret_cast<uint4*>(sdyt)[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncthreads();
    // the transposed weights, once; the first tile's dY, dY^T and A_4^T
    for (int i = tid; i < WB_BYTES / 16; i += 128) cp_async16(reinterpret_cast<uint4*>(swt) + i, reinterpret_cast<const uint4*>(a.wbf + WF_BYTES) + i);
    auto load_dy = [&](int tile) {
        const uint8_t* act = a.act + (size_t)tile * ACT_BYTES;
        for (int i = tid; i < 128 * OUTP * 2 / 16; i += 128) cp_async16(reinterpret_cast<uint4*>(sdy) + i, reinterpret_cast<const uint4*>(act + ACT_DY) + i);
        for (int i = tid; i < OUTP * 128 * 2 / 16; i += 128) cp_async16(reinterpret_cast<uint4*>(sdyt) + i, reinterpret_cast<const uint4*>(act + ACT_DYT) + i);
    };
    auto load_at = [&](int tile, int l, uint8_t* dst) {
        const uint4* src = reinterpret_cast<const uint4*>(a.act + (size_t)tile * ACT_BYTES + (l == 0 ? ACT_X0T : act_ht(l)));
        for (int i = tid; i < in_dim(l) * 128 * 2 / 16; i += 128) cp_async16(reinterpret_cast<uint4*>(dst) + i, src + i);
    };
    load_dy(blockIdx.x);
    load_at(blockIdx.x, NLAYER - 1, sat[0]);
    asm volatile("cp.async.commit_group;" ::: "memory");
    if (tid == 0) mbar_init(&mbar, 1);
    if (warp == 0) tmem_alloc(&tmem_base, BW_COLS);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = tmem_base;
    uint32_t phase = 0;
    int step = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const bool first = tile == (int)blockIdx.x;
        for (int l = NLAYER - 1; l >= 0; --l, ++step) {
            const int Kin = in_dim(l), Nout = out_dim(l);
            uint8_t* cur = sat[step & 1];
            asm volatile("cp.async.wait_group 0;" ::: "memory");
            fence_proxy_async();
            __syncthreads();
            if (tid == 0) {
                const uint32_t zt = smem_u32(l == NLAYER - 1 ? sdyt : sdzt), at = smem_u32(cur);
                for (int kk = 0; kk < 8; ++kk)
                    mma_bf16(tmem + bw_dw_col(l), smem_desc(zt + 256u * kk, 128u, 16u * 128), smem_desc(at + 256u * kk, 128u, 16u * 128),
                             idesc_bf16_f32(128, Kin), (kk > 0 || !first) ? 1u : 0u);
                if (l >= 1) {
                    const uint32_t z = smem_u32(l == NLAYER - 1 ? sdy : sdz), w = smem_u32(swt + (wb_off(l) - WF_BYTES));
                    for (int kk = 0; kk < Nout / 16; ++kk)
                        mma_bf16(tmem + BW_DA, smem_desc(z + 256u * kk, 128u, 16u * Nout), smem_desc(w + 256u * kk, 128u, 16u * Nout),
                                 idesc_bf16_f32(128, HID), kk > 0);
                }
                mma_commit(&mbar);
            }
            // the next step's operands, into the other buffer, while this one runs
            if (l > 0) {
                load_at(tile, l - 1, sat[(step + 1) & 1]);
            } else if (tile + (int)gridDim.x < ntiles) {
                load_dy(tile + gridDim.x);
                load_at(tile + gridDim.x, NLAYER - 1, sat[(step + 1) & 1]);
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
            bool seen = true;
            if (warp == 0) {   // one warp watches the barrier (see k_mlp_forward)
                seen = mbar_wait(&mbar, phase, WAIT_LIMIT);
                fence_before_sync();
            }
            ok = __syncthreads_and(seen);
            phase ^= 1u;
            if (!ok) {
                if (tid == 0) atomicOr(a.err, 1u);
                break;
            }
            fence_after_sync();
            if (l >= 1) {
                // dZ_{l-1} = (dZ_l W_l) * [H_l > 0], row = sample
                const int m = tid;
                for (int c = 0; c < HID; c += 16) {
                    float v[16];
                    tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + BW_DA + (uint32_t)c, v);
                    tmem_wait_ld();
                    for (int j = 0; j < 16; ++j) {
                        const int k = c + j;
                        const float h = bf16_at(cur, kmajor_offset(k, m, 128));
                        v[j] = h > 0.f ? v[j] : 0.f;
                    }
                    for (int j = 0; j < 16; ++j) {
                        st_bf16(sdz, kmajor_offset(m, c + j, HID), v[j]);
                        st_bf16(sdzt, kmajor_offset(c + j, m, 128), v[j]);
                    }
                }
            }
            fence_before_sync();
            fence_proxy_async();
            __syncthreads();
            fence_after_sync();
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    // the CTA's weight gradients: rows = outputs (warps 0 and 1 hold rows 0..63), 16-byte stores
    if (ok && warp < 2) {
        const int row = warp * 32 + lane;
        float* dw = a.dwpart + (size_t)blockIdx.x * NWEIGHT;
        for (int l = 0; l < NLAYER; ++l) {
            const int Kin = in_dim(l), Nout = out_dim(l);
            for (int c = 0; c < Kin; c += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + bw_dw_col(l) + (uint32_t)c, v);
                tmem_wait_ld();
                if (row < Nout) {
                    float4* d4 = reinterpret_cast<float4*>(dw + master_off(l) + row * Kin + c);
                    for (int j = 0; j < 4; ++j) d4[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                }
            }
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, BW_COLS);
}

// Master weights (FP32, [out][in] per layer) -> bf16 tiles: W_l (rows out, K in) and, for
// layers 1..4, W_l^T (rows in, K out).
__global__ void k_mlp_pack(const float* __restrict__ w, uint8_t* __restrict__ wbf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NWEIGHT) return;
    int l = 0;
    while (l + 1 < NLAYER && i >= master_off(l + 1)) ++l;
    const int K = in_dim(l), r = (i - master_off(l)) / K, k = (i - master_off(l)) % K;
    const float v = w[i];
    st_bf16(wbf + wf_off(l), kmajor_offset(r, k, K), v);
    if (l >= 1) st_bf16(wbf + wb_off(l), kmajor_offset(k, r, out_dim(l)), v);
}

// Gradient of each weight = the tile gradients added in a fixed order (reproducible): slice s
// of GSLICES adds tiles s, s + GSLICES, ... in order, then the slices are added in order; then
// one Adam step on the FP32 master weight, and its bf16 copies.
constexpr int GSLICES = 16;
__global__ void k_mlp_gsum(const float* __restrict__ part, int ntiles, float* __restrict__ slices) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
    if (i >= NWEIGHT) return;
    float g = 0.f;
    for (int t = s; t < ntiles; t += GSLICES) g += part[(size_t)t * NWEIGHT + i];
    slices[(size_t)s * NWEIGHT + i] = g;
}
// Loss scaling.  The output gradient is multiplied by a power-of-two scale before it goes
// through the bf16 backward pass and divided out of the summed weight gradient (exact for a power
// of two, barring overflow).  A step whose summed gradient is not finite is skipped and the
// scale halved; after SCALE_RUN finite steps in a row it doubles, up to SCALE_MAX.
// Device state, floats: scale for the next step, steps applied, finite steps in a row, steps
// skipped, Adam's bias corrections c1 and c2 of this step, 1 / the scale of this step.
enum MlpState { ST_SCALE = 0, ST_STEPS, ST_RUN, ST_SKIPPED, ST_C1, ST_C2, ST_INV, ST_COUNT };
constexpr float SCALE_MAX = 65536.f;
constexpr int SCALE_RUN = 1000;
__global__ void k_mlp_gcheck(const float* __restrict__ slices, unsigned* __restrict__ nonfinite) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NWEIGHT) return;
    float g = 0.f;
    for (int s = 0; s < GSLICES; ++s) g += slices[(size_t)s * NWEIGHT + i];
    if (!isfinite(g)) atomicOr(nonfinite, 1u);
}
__global__ void k_mlp_step(float* __restrict__ st, const unsigned* __restrict__ nonfinite, float b1, float b2) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    st[ST_INV] = 1.f / st[ST_SCALE];
    if (*nonfinite) {
        st[ST_SCALE] = fmaxf(st[ST_SCALE] * 0.5f, 1.f);
        st[ST_RUN] = 0.f;
        st[ST_SKIPPED] += 1.f;
        return;
    }
    // Adam's bias corrections 1 / (1 - b^t), in FP32 (a double pow is a long chain of the GPU's
    // slow FP64 operations on one thread: about 9 us per step)
    const float t = st[ST_STEPS] + 1.f;
    st[ST_STEPS] = t;
    st[ST_C1] = 1.f / (1.f - powf(b1, t));
    st[ST_C2] = 1.f / (1.f - powf(b2, t));
    st[ST_RUN] += 1.f;
    if (st[ST_RUN] >= (float)SCALE_RUN) {
        st[ST_SCALE] = fminf(st[ST_SCALE] * 2.f, SCALE_MAX);
        st[ST_RUN] = 0.f;
    }
}
__global__ void k_mlp_adam(const float* __restrict__ slices, float* __restrict__ w, float* __restrict__ m1, float* __restrict__ m2,
                           float* __restrict__ grad, uint8_t* __restrict__ wbf, float lr, float b1, float b2, float eps,
                           const float* __restrict__ st, const unsigned* __restrict__ nonfinite) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NWEIGHT || *nonfinite) return;
    const float c1 = st[ST_C1], c2 = st[ST_C2];
    float g = 0.f;
    for (int s = 0; s < GSLICES; ++s) g += slices[(size_t)s * NWEIGHT + i];
    g *= st[ST_INV];
    grad[i] = g;
    const float m = b1 * m1[i] + (1.f - b1) * g;
    const float v = b2 * m2[i] + (1.f - b2) * g * g;
    m1[i] = m;
    m2[i] = v;
    const float x = w[i] - lr * (m * c1) / (sqrtf(v * c2) + eps);
    w[i] = x;
    int l = 0;
    while (l + 1 < NLAYER && i >= master_off(l + 1)) ++l;
    const int K = in_dim(l), r = (i - master_off(l)) / K, k = (i - master_off(l)) % K;
    st_bf16(wbf + wf_off(l), kmajor_offset(r, k, K), x);
    if (l >= 1) st_bf16(wbf + wb_off(l), kmajor_offset(k, r, out_dim(l)), x);
}

constexpr size_t FWD_SMEM_INFER = (size_t)WF_BYTES + INFER_GROUPS * GROUP_SMEM_INFER;   // 224 KB: one CTA per SM
constexpr int TRAIN_GROUPS = 2;                                  // tiles in flight per training-forward CTA
constexpr size_t FWD_SMEM_TRAIN = (size_t)WF_BYTES + TRAIN_GROUPS * GROUP_SMEM_TRAIN;   // 224 KB
// operands of the backward pass (more than half an SM's shared memory: one CTA per SM, each
// holding all 512 tensor-memory columns)
constexpr size_t BWD_SMEM = (size_t)BS_END;
static_assert(BWD_SMEM > 114 * 1024 && BWD_SMEM <= 227 * 1024, "backward shared memory");
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

extern "C" rc_status rc_mlp_wait_check(uint32_t polls, int arrive, unsigned* d_err, void* stream) {
    if (!d_err || polls < 1 || polls > (1u << 24)) return RC_ERR_ARG;
    k_wait_check<<<1, 32, 0, (cudaStream_t)stream>>>(polls, arrive != 0, d_err);
    return cudaGetLastError() == cudaSuccess ? RC_OK : RC_ERR_CUDA;
}

// ---------------------------------------------------------------- C ABI of the network
struct rc_mlp {
    rc_mlp_config cfg{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    float *w = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr, *part = nullptr, *slices = nullptr, *loss = nullptr;
    float* state = nullptr;     // loss scale and Adam step state (MlpState)
    uint8_t *wbf = nullptr, *act = nullptr;
    unsigned* err = nullptr;
    unsigned* nonfinite = nullptr;
    int cap_tiles = 0, sms = 0;
    long long step = 0;
    std::string msg;
    // A training step's launches (2 memsets, 6 kernels) as CUDA graphs, one per set of arguments
    // that came twice in a row (a caller that trains on the same buffers every frame replays one
    // graph per call; arguments seen once are launched directly)
    struct StepArgs {
        const void *P = nullptr, *N = nullptr, *aux = nullptr, *target = nullptr, *idx = nullptr;
        int tstride = 0, n = 0;
        const float* loss = nullptr;
        bool operator==(const StepArgs& o) const {
            return P == o.P && N == o.N && aux == o.aux && target == o.target && idx == o.idx && tstride == o.tstride && n == o.n &&
                   loss == o.loss;
        }
    };
    struct StepGraph {
        StepArgs args;
        cudaGraphExec_t exec;
    };
    std::vector<StepGraph> graphs;
    StepArgs last;
};

namespace {

rc_status mfail(rc_mlp* m, rc_status s, const char* what) {
    if (m) m->msg = what;
    return s;
}

MlpArgs args_of(const rc_mlp* m) {
    MlpArgs a{};
    a.wbf = m->wbf;
    a.n_out = m->cfg.n_out;
    for (int k = 0; k < 3; ++k) {
        a.lo[k] = m->cfg.box_lo[k];
        a.inv_ext[k] = 1.f / (m->cfg.box_hi[k] - m->cfg.box_lo[k]);
    }
    a.err = m->err;
    return a;
}

// A small counter-based generator for the initial weights (splitmix64).
uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

extern "C" {

rc_status rc_mlp_create(const rc_mlp_config* cfg, rc_mlp** out) {
    if (!cfg || !out) return RC_ERR_ARG;
    *out = nullptr;
    if (cfg->n_out < 1 || cfg->n_out > OUTP || cfg->max_batch < 128 || !(cfg->lr >= 0.f)) return RC_ERR_ARG;
    for (int k = 0; k < 3; ++k)
        if (!(cfg->box_hi[k] > cfg->box_lo[k])) return RC_ERR_ARG;
    rc_mlp* m = new rc_mlp();
    m->cfg = *cfg;
    auto bad = [&](rc_status s) { rc_mlp_destroy(m); return s; };
    if (cudaSetDevice(cfg->device) != cudaSuccess) return bad(RC_ERR_CUDA);
    if (cfg->stream) m->stream = (cudaStream_t)cfg->stream;
    else {
        if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) return bad(RC_ERR_CUDA);
        m->own_stream = true;
    }
    cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, cfg->device);
    m->cap_tiles = (cfg->max_batch + 127) / 128;
    if (cudaMalloc(&m->w, 4 * NWEIGHT) || cudaMalloc(&m->m1, 4 * NWEIGHT) || cudaMalloc(&m->m2, 4 * NWEIGHT) ||
        cudaMalloc(&m->grad, 4 * NWEIGHT) || cudaMalloc(&m->wbf, WF_BYTES + WB_BYTES) || cudaMalloc(&m->err, 4) ||
        cudaMalloc(&m->loss, 4) || cudaMalloc(&m->part, (size_t)4 * NWEIGHT * std::max(1, std::min(m->cap_tiles, m->sms))) ||
        cudaMalloc(&m->slices, (size_t)4 * NWEIGHT * GSLICES) ||
        cudaMalloc(&m->act, (size_t)ACT_BYTES * m->cap_tiles) || cudaMalloc(&m->state, 4 * ST_COUNT) ||
        cudaMalloc(&m->nonfinite, 4))
        return bad(RC_ERR_NOMEM);
    {
        float st0[ST_COUNT] = {0};
        float sc = cfg->loss_scale > 0.f ? cfg->loss_scale : 1024.f;
        st0[ST_SCALE] = exp2f(floorf(log2f(sc)));   // a power of two
        if (cudaMemcpy(m->state, st0, sizeof st0, cudaMemcpyHostToDevice) != cudaSuccess) return bad(RC_ERR_CUDA);
    }
    // He-uniform initial weights, seeded
    std::vector<float> w(NWEIGHT);
    uint64_t st = 0x5EEDull ^ (uint64_t)cfg->seed * 0x100000001B3ull;
    for (int l = 0; l < NLAYER; ++l) {
        const float lim = sqrtf(6.f / (float)(l == 0 ? 168 : HID));
        for (int i = master_off(l); i < master_off(l) + out_dim(l) * in_dim(l); ++i) {
            const double u = (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
            w[i] = (float)((2.0 * u - 1.0) * lim);
        }
        if (l == NLAYER - 1)   // unused outputs start (and stay, their gradient is zero) at zero
            for (int r = cfg->n_out; r < OUTP; ++r)
                for (int k = 0; k < HID; ++k) w[master_off(l) + r * HID + k] = 0.f;
    }
    rc_status s = rc_mlp_weights(m, w.data(), w.size(), 1);
    if (s != RC_OK) return bad(s);
    if (cudaMemsetAsync(m->m1, 0, 4 * NWEIGHT, m->stream) || cudaMemsetAsync(m->m2, 0, 4 * NWEIGHT, m->stream) ||
        cudaMemsetAsync(m->err, 0, 4, m->stream) || cudaStreamSynchronize(m->stream))
        return bad(RC_ERR_CUDA);
    if (cudaFuncSetAttribute(k_mlp_forward<true, TRAIN_GROUPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FWD_SMEM_TRAIN) ||
        cudaFuncSetAttribute(k_mlp_forward<false, INFER_GROUPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FWD_SMEM_INFER) ||
        cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BWD_SMEM))
        return bad(RC_ERR_CUDA);
    *out = m;
    return RC_OK;
}

void rc_mlp_destroy(rc_mlp* m) {
    if (!m) return;
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->w); cudaFree(m->m1); cudaFree(m->m2); cudaFree(m->grad); cudaFree(m->part); cudaFree(m->slices);
    cudaFree(m->loss); cudaFree(m->wbf); cudaFree(m->act); cudaFree(m->err); cudaFree(m->state); cudaFree(m->nonfinite);
    for (auto& g : m->graphs) cudaGraphExecDestroy(g.exec);
    if (m->own_stream && m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

const char* rc_mlp_last_error(const rc_mlp* m) { return m ? m->msg.c_str() : "no network"; }

rc_status rc_mlp_weights(rc_mlp* m, float* host, size_t n, int to_device) {
    if (!m || !host || n != (size_t)NWEIGHT) return mfail(m, RC_ERR_ARG, "weights: 24576 floats");
    if (to_device) {
        if (cudaMemcpyAsync(m->w, host, 4 * NWEIGHT, cudaMemcpyHostToDevice, m->stream) != cudaSuccess) return mfail(m, RC_ERR_CUDA, "copy");
        if (cudaMemsetAsync(m->wbf, 0, WF_BYTES + WB_BYTES, m->stream) != cudaSuccess) return mfail(m, RC_ERR_CUDA, "clear");
        k_mlp_pack<<<(NWEIGHT + 255) / 256, 256, 0, m->stream>>>(m->w, m->wbf);
        if (cudaGetLastError() != cudaSuccess) return mfail(m, RC_ERR_CUDA, "pack");
    } else if (cudaMemcpyAsync(host, m->w, 4 * NWEIGHT, cudaMemcpyDeviceToHost, m->stream) != cudaSuccess) {
        return mfail(m, RC_ERR_CUDA, "copy");
    }
    return cudaStreamSynchronize(m->stream) == cudaSuccess ? RC_OK : mfail(m, RC_ERR_CUDA, "sync");
}

rc_status rc_mlp_gradients(rc_mlp* m, float* host, size_t n) {
    if (!m || !host || n != (size_t)NWEIGHT) return mfail(m, RC_ERR_ARG, "gradients: 24576 floats");
    if (cudaMemcpyAsync(host, m->grad, 4 * NWEIGHT, cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess)
        return mfail(m, RC_ERR_CUDA, "copy");
    return RC_OK;
}

namespace {
// The launches of one training step on the network's stream.
cudaError_t issue_train(rc_mlp* m, const MlpArgs& a, int ntiles, bool own_loss) {
    cudaError_t e;
    if (own_loss && (e = cudaMemsetAsync(m->loss, 0, 4, m->stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(m->nonfinite, 0, 4, m->stream)) != cudaSuccess) return e;
    k_mlp_forward<true, TRAIN_GROUPS><<<std::min((ntiles + TRAIN_GROUPS - 1) / TRAIN_GROUPS, m->sms), FWD_THREADS * TRAIN_GROUPS,
                                        FWD_SMEM_TRAIN, m->stream>>>(a);
    const int bwd_ctas = std::min(ntiles, m->sms);
    k_mlp_backward<<<bwd_ctas, 128, BWD_SMEM, m->stream>>>(a, ntiles);
    const float b1 = 0.9f, b2 = 0.99f;
    k_mlp_gsum<<<dim3((NWEIGHT + 255) / 256, GSLICES), 256, 0, m->stream>>>(m->part, bwd_ctas, m->slices);
    k_mlp_gcheck<<<(NWEIGHT + 255) / 256, 256, 0, m->stream>>>(m->slices, m->nonfinite);
    k_mlp_step<<<1, 32, 0, m->stream>>>(m->state, m->nonfinite, b1, b2);
    k_mlp_adam<<<(NWEIGHT + 255) / 256, 256, 0, m->stream>>>(m->slices, m->w, m->m1, m->m2, m->grad, m->wbf, m->cfg.lr, b1, b2,
                                                              1e-8f, m->state, m->nonfinite);
    return cudaGetLastError();
}
}  // namespace

rc_status rc_mlp_train(rc_mlp* m, const float* d_pos4, const float* d_nrm4, const float* d_aux4, const float* d_target, int tstride,
                       const int* d_idx, int n, float* d_loss) {
    if (!m || !d_pos4 || !d_nrm4 || !d_aux4 || !d_target || n < 128 || n % 128 || n > 128 * m->cap_tiles || tstride < m->cfg.n_out)
        return mfail(m, RC_ERR_ARG, "train: n a multiple of 128 up to max_batch");
    MlpArgs a = args_of(m);
    a.P = reinterpret_cast<const float4*>(d_pos4);
    a.N = reinterpret_cast<const float4*>(d_nrm4);
    a.aux = reinterpret_cast<const float4*>(d_aux4);
    a.target = d_target;
    a.tstride = tstride;
    a.idx = d_idx;
    a.n = n;
    a.act = m->act;
    a.dwpart = m->part;
    a.loss = d_loss ? d_loss : m->loss;
    a.loss_scale = 1.f / ((float)n * (float)m->cfg.n_out);
    a.scale = m->state + ST_SCALE;
    const int ntiles = n / 128;
    m->step++;
    rc_mlp::StepArgs key;
    key.P = d_pos4; key.N = d_nrm4; key.aux = d_aux4; key.target = d_target; key.idx = d_idx;
    key.tstride = tstride; key.n = n; key.loss = d_loss;
    for (const auto& g : m->graphs)
        if (g.args == key) return cudaGraphLaunch(g.exec, m->stream) == cudaSuccess ? RC_OK : mfail(m, RC_ERR_CUDA, "graph launch");
    // the same arguments twice in a row: capture the step (unless the stream is being captured
    // already or cannot be); otherwise launch it directly
    const bool repeat = key == m->last;
    m->last = key;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (!repeat || m->graphs.size() >= 16 || cudaStreamIsCapturing(m->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone ||
        cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return issue_train(m, a, ntiles, !d_loss) == cudaSuccess ? RC_OK : mfail(m, RC_ERR_CUDA, "launch");
    }
    const cudaError_t le = issue_train(m, a, ntiles, !d_loss);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(m->stream, &graph);
    cudaGraphExec_t exec = nullptr;
    const bool ok = le == cudaSuccess && ce == cudaSuccess && graph && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {   // the step did not run: launch it directly
        cudaGetLastError();
        return issue_train(m, a, ntiles, !d_loss) == cudaSuccess ? RC_OK : mfail(m, RC_ERR_CUDA, "launch");
    }
    m->graphs.push_back({key, exec});
    return cudaGraphLaunch(exec, m->stream) == cudaSuccess ? RC_OK : mfail(m, RC_ERR_CUDA, "graph launch");
}

rc_status rc_mlp_infer(rc_mlp* m, const float* d_pos4, const float* d_nrm4, const float* d_aux4, int n, float* d_out, int ostride) {
    if (!m || !d_pos4 || !d_nrm4 || !d_aux4 || !d_out || n < 1 || ostride < m->cfg.n_out) return mfail(m, RC_ERR_ARG, "infer");
    MlpArgs a = args_of(m);
    a.P = reinterpret_cast<const float4*>(d_pos4);
    a.N = reinterpret_cast<const float4*>(d_nrm4);
    a.aux = reinterpret_cast<const float4*>(d_aux4);
    a.n = n;
    a.out = d_out;
    a.ostride = ostride;
    const int ntiles = (n + 127) / 128;
    k_mlp_forward<false, INFER_GROUPS><<<std::min((ntiles + INFER_GROUPS - 1) / INFER_GROUPS, m->sms), FWD_THREADS * INFER_GROUPS,
                                         FWD_SMEM_INFER, m->stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? RC_OK : mfail(m, RC_ERR_CUDA, "launch");
}

rc_status rc_mlp_loss_scale(rc_mlp* m, float* scale, long long* steps, long long* skipped) {
    if (!m) return RC_ERR_ARG;
    float st[ST_COUNT];
    if (cudaMemcpyAsync(st, m->state, sizeof st, cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess)
        return mfail(m, RC_ERR_CUDA, "copy");
    if (scale) *scale = st[ST_SCALE];
    if (steps) *steps = (long long)st[ST_STEPS];
    if (skipped) *skipped = (long long)st[ST_SKIPPED];
    return RC_OK;
}

rc_status rc_mlp_error_flags(rc_mlp* m, unsigned* flags) {
    if (!m || !flags) return RC_ERR_ARG;
    if (cudaMemcpyAsync(flags, m->err, 4, cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess)
        return mfail(m, RC_ERR_CUDA, "copy");
    return RC_OK;
}

}  // extern "C"
