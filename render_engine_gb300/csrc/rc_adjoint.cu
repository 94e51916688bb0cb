// Adjoint of the radiance-cache transport with respect to the lights' emission.
//
// The cache's fixed point (the quantity the reference's scene preparation converges to,
// prep_mesh.cuh:182-213, and that every frame of poc_gpu.cu:433-530 estimates) is, for a fixed
// set of K rays per point,
//
//     L_l = T (E_l G_l + L_l),   T[i, j] = A_j / K x (rays of point i that reach point j),
//
// with G_l the direct light of light l at unit emission (k_build, poc_gpu.cu:369-391) and E_l
// its emission.  For J = sum_i w_i sum_l L_l[i] the adjoint importance u = w + T^T u gives
//
//     dJ / dE_l = sum_j (T^T u)_j G_l[j] = sum_j (u_j - w_j) G_l[j],
//
// one transposed solve for all lights instead of one forward solve per light.  The rays come
// from Ops<NL>::frozen_hits; this file builds the transposed ray lists (CSR, deterministic
// order), runs the forward and adjoint Jacobi sweeps and reduces the gradient in FP64 with a
// fixed summation order, so a result does not depend on the GPU or on the run.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "rc_adjoint.h"

namespace rc {
namespace adj {

namespace {

constexpr int B = 256;
constexpr int SCAN_ITEMS = 8;                       // per thread
constexpr int SCAN_TILE = B * SCAN_ITEMS;           // 2048 per block

__device__ __forceinline__ unsigned warp_max(unsigned v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// incoming-ray count per point, and the rays that do not count
__global__ void k_count(const int* __restrict__ hits, long long n, int* __restrict__ cnt, unsigned long long* back) {
    unsigned nb = 0;
    for (long long e = blockIdx.x * (long long)B + threadIdx.x; e < n; e += (long long)gridDim.x * B) {
        const int j = hits[e];
        if (j >= 0) atomicAdd(&cnt[j], 1);
        else ++nb;
    }
    for (int o = 16; o > 0; o >>= 1) nb += __shfl_xor_sync(0xffffffffu, nb, o);
    if ((threadIdx.x & 31) == 0 && nb) atomicAdd(back, (unsigned long long)nb);
}

// exclusive scan of one tile of SCAN_TILE ints (in place allowed: a block reads its whole
// tile into registers before writing); the tile's total goes to bsum[blockIdx.x]
__global__ void __launch_bounds__(B) k_scan_tile(const int* in, int* out, int n, int* bsum) {
    __shared__ int wsum[B / 32];
    const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS], t = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        t += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = t;   // inclusive warp scan of the thread totals
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    int wpre = 0, total = 0;
    for (int k = 0; k < B / 32; ++k) {
        if (k < warp) wpre += wsum[k];
        total += wsum[k];
    }
    int run = wpre + x - t;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void k_scan_add(int* out, int n, const int* boff) {
    const long long e = blockIdx.x * (long long)B + threadIdx.x;
    if (e < n) out[e] += boff[e / SCAN_TILE];
}

// every counted ray into its target's segment, in arrival order
__global__ void k_fill(const int* __restrict__ hits, long long n, const int* __restrict__ off, int* __restrict__ fill,
                       int* __restrict__ unordered) {
    for (long long e = blockIdx.x * (long long)B + threadIdx.x; e < n; e += (long long)gridDim.x * B) {
        const int j = hits[e];
        if (j >= 0) unordered[off[j] + atomicAdd(&fill[j], 1)] = (int)e;
    }
}

// the segment of every entry sorted by ray index (rank = entries of the segment with a smaller
// ray index; ray indices are unique), stored as the ray's source point
__global__ void k_rank(const int* __restrict__ off, int Np, const int* __restrict__ unordered, int K, long long cap,
                       int* __restrict__ src, int* maxseg) {
    const long long total = off[Np];
    for (long long q = blockIdx.x * (long long)B + threadIdx.x; q < total && q < cap; q += (long long)gridDim.x * B) {
        int lo = 0, hi = Np;   // largest j with off[j] <= q
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (off[mid] <= q) lo = mid;
            else hi = mid;
        }
        const int a = off[lo], b = off[lo + 1];
        const int e = unordered[q];
        int rank = 0;
        for (int t = a; t < b; ++t) rank += unordered[t] < e;
        src[a + rank] = e / K;
        if (q == a) atomicMax(maxseg, b - a);
    }
}

// per point: direct light summed over the lights (l ascending) and albedo; the first gathered
// values A_j (d_j + L_j) with L = 0.  With `em` (NL emissions, device), the direct light is
// sum_l em_l G_l from the unit-emission build AEu instead of the state's own.
__global__ void k_prep(const float* __restrict__ AE, const float* __restrict__ AEu, const float* __restrict__ em, int aes, int NL,
                       int Np, float2* __restrict__ da, float* __restrict__ g0) {
    const int j = blockIdx.x * B + threadIdx.x;
    if (j >= Np) return;
    const float* ae = AE + (size_t)aes * j;
    float d = 0.f;
    if (em) {
        const float* au = AEu + (size_t)aes * j;
        for (int l = 0; l < NL; ++l) d += em[l] * au[1 + l];
    } else {
        for (int l = 0; l < NL; ++l) d += ae[1 + l];
    }
    da[j] = make_float2(d, ae[0]);
    g0[j] = ae[0] * (d + 0.f);
}

// forward sweep: L_i = (1/K) sum over i's counted rays, in ray order, of g_j = A_j (d_j + L_j)
// from the previous sweep; writes L and the next sweep's g.  Hit lists are read four rays at a
// time when K is a multiple of 4 (rows of 16 K bytes stay 16-byte aligned).
__global__ void __launch_bounds__(B) k_fwd(const int* __restrict__ hits, int K, int Np, const float2* __restrict__ da,
                                           const float* __restrict__ gin, const float* __restrict__ Lprev, float* __restrict__ Lout,
                                           float* __restrict__ gout, unsigned* chg) {
    const int i = blockIdx.x * B + threadIdx.x;
    float v = 0.f, dv = 0.f;
    if (i < Np) {
        float sum = 0.f;
        const int* h = hits + (size_t)i * K;
        if ((K & 3) == 0) {
            const int4* h4 = reinterpret_cast<const int4*>(h);
            for (int r = 0; r < K / 4; ++r) {
                const int4 q = __ldg(h4 + r);
                const float a = q.x >= 0 ? __ldcg(gin + q.x) : 0.f, b = q.y >= 0 ? __ldcg(gin + q.y) : 0.f;
                const float c = q.z >= 0 ? __ldcg(gin + q.z) : 0.f, d = q.w >= 0 ? __ldcg(gin + q.w) : 0.f;
                if (q.x >= 0) sum += a;
                if (q.y >= 0) sum += b;
                if (q.z >= 0) sum += c;
                if (q.w >= 0) sum += d;
            }
        } else {
            for (int r = 0; r < K; ++r) {
                const int j = __ldg(h + r);
                if (j >= 0) sum += __ldcg(gin + j);
            }
        }
        v = sum / (float)K;
        Lout[i] = v;
        const float2 x = da[i];
        gout[i] = x.y * (x.x + v);
        dv = fabsf(v - Lprev[i]);
    }
    if (chg) {   // change of the sweep, and the largest value (non-negative floats order as their bits)
        const unsigned a = warp_max(__float_as_uint(dv)), b = warp_max(__float_as_uint(fabsf(v)));
        if ((threadIdx.x & 31) == 0) {
            atomicMax(&chg[0], a);
            atomicMax(&chg[1], b);
        }
    }
}

// adjoint sweep: uout[j] = w_j + (A_j / K) sum over the rays reaching j, in ray order, of
// uin[source] (four sources fetched at a time)
__global__ void __launch_bounds__(B) k_bwd(const int* __restrict__ off, const int* __restrict__ src, int K, int Np,
                                           const float2* __restrict__ da, const float* __restrict__ w,
                                           const float* __restrict__ uin, float* __restrict__ uout, unsigned* chg) {
    const int j = blockIdx.x * B + threadIdx.x;
    float v = 0.f, dv = 0.f;
    if (j < Np) {
        float sum = 0.f;
        const int a = off[j], b = off[j + 1];
        int q = a;
        for (; q + 4 <= b; q += 4) {
            const int s0 = __ldg(src + q), s1 = __ldg(src + q + 1), s2 = __ldg(src + q + 2), s3 = __ldg(src + q + 3);
            const float x0 = __ldcg(uin + s0), x1 = __ldcg(uin + s1), x2 = __ldcg(uin + s2), x3 = __ldcg(uin + s3);
            sum += x0;
            sum += x1;
            sum += x2;
            sum += x3;
        }
        for (; q < b; ++q) sum += __ldcg(uin + __ldg(src + q));
        v = w[j] + da[j].y * sum / (float)K;
        uout[j] = v;
        dv = fabsf(v - uin[j]);
    }
    if (chg) {
        const unsigned a = warp_max(__float_as_uint(dv)), b = warp_max(__float_as_uint(fabsf(v)));
        if ((threadIdx.x & 31) == 0) {
            atomicMax(&chg[2], a);
            atomicMax(&chg[3], b);
        }
    }
}

// Column c < NL: sum_j (u_j - w_j) G_c[j]; column NL: sum_j w_j L_j.  Block x of column c sums
// a fixed slice of points (thread-strided, then a fixed tree), so the order never changes.
__global__ void __launch_bounds__(B) k_grad_part(const float* __restrict__ AEu, int aes, int NL, int Np, const float* __restrict__ u,
                                                 const float* __restrict__ w, const float* __restrict__ L, double* __restrict__ part) {
    __shared__ double sh[B];
    const int c = blockIdx.y;
    const long long per = ((long long)Np + gridDim.x - 1) / gridDim.x;
    const long long j0 = per * blockIdx.x, j1 = min((long long)Np, j0 + per);
    double s = 0.0;
    for (long long j = j0 + threadIdx.x; j < j1; j += B)
        s += c < NL ? ((double)u[j] - (double)w[j]) * (double)AEu[(size_t)aes * j + 1 + c] : (double)w[j] * (double)L[j];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = B / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(size_t)c * gridDim.x + blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(B) k_grad_final(const double* __restrict__ part, int G, double* __restrict__ out) {
    __shared__ double sh[B];
    const int c = blockIdx.x;
    double s = 0.0;
    for (int k = threadIdx.x; k < G; k += B) s += part[(size_t)c * G + k];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = B / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = sh[0];
}

int blocks_for(long long n) { return (int)((n + B - 1) / B); }
int stride_blocks(long long n) { return (int)(std::min)((n + B - 1) / B, 152LL * 16); }

cudaError_t scan_exclusive(const int* in, int* out, int n, int* scratch, cudaStream_t st) {
    const int nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_tile<<<nb, B, 0, st>>>(in, out, n, scratch);
    if (nb > 1) {
        cudaError_t e = scan_exclusive(scratch, scratch, nb, scratch + nb, st);
        if (e != cudaSuccess) return e;
        k_scan_add<<<blocks_for(n), B, 0, st>>>(out, n, scratch);
    }
    return cudaGetLastError();
}

}  // namespace

size_t scan_scratch_ints(long long n) {
    size_t s = 0;
    while (n > 1) {
        n = (n + SCAN_TILE - 1) / SCAN_TILE;
        s += (size_t)n;
    }
    return s + 1;
}

cudaError_t build_transpose(const Bufs& b, int Np, int K, cudaStream_t st) {
    const long long n = (long long)Np * K;
    cudaError_t e;
    if ((e = cudaMemsetAsync(b.cnt, 0, sizeof(int) * ((size_t)Np + 1), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(b.fill, 0, sizeof(int) * (size_t)Np, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(b.stats, 0, sizeof(Stats), st)) != cudaSuccess) return e;
    k_count<<<stride_blocks(n), B, 0, st>>>(b.hits, n, b.cnt, &b.stats->back);
    if ((e = scan_exclusive(b.cnt, b.off, Np + 1, b.scratch, st)) != cudaSuccess) return e;
    k_fill<<<stride_blocks(n), B, 0, st>>>(b.hits, n, b.off, b.fill, b.unordered);
    k_rank<<<stride_blocks(n), B, 0, st>>>(b.off, Np, b.unordered, K, n, b.src, &b.stats->max_incoming);
    return cudaGetLastError();
}

cudaError_t solve(Bufs* bp, int Np, int K, int NL, int aes, const float* AE, const float* AEu, const float* em, int iters,
                  cudaStream_t st) {
    const Bufs& b = *bp;
    cudaError_t e;
    k_prep<<<blocks_for(Np), B, 0, st>>>(AE, AEu, em, aes, NL, Np, b.da, b.g[0]);
    if ((e = cudaMemsetAsync(b.L[0], 0, sizeof(float) * (size_t)Np, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(b.u[0], b.w, sizeof(float) * (size_t)Np, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
    for (int t = 0; t < iters; ++t) {
        const bool last = t == iters - 1;
        k_fwd<<<blocks_for(Np), B, 0, st>>>(b.hits, K, Np, b.da, b.g[t & 1], b.L[t & 1], b.L[(t + 1) & 1], b.g[(t + 1) & 1],
                                            last ? b.stats->chg : nullptr);
        k_bwd<<<blocks_for(Np), B, 0, st>>>(b.off, b.src, K, Np, b.da, b.w, b.u[t & 1], b.u[(t + 1) & 1], last ? b.stats->chg : nullptr);
    }
    bp->L_final = b.L[iters & 1];
    bp->u_final = b.u[iters & 1];
    k_grad_part<<<dim3(GRAD_BLOCKS, NL + 1), B, 0, st>>>(AEu, aes, NL, Np, bp->u_final, b.w, bp->L_final, b.part);
    k_grad_final<<<NL + 1, B, 0, st>>>(b.part, GRAD_BLOCKS, b.stats->out);
    return cudaGetLastError();
}

}  // namespace adj
}  // namespace rc
