// Kernels of the reference's taa mode that do not depend on the light count
// (poc_gpu.cu:1100-1172): reactive-mask sources (dependency masks, references, per-zone
// statistics) and the per-frame history update fused with its 3x3 neighbourhood statistics
// and the error sums.
#include <cuda_runtime.h>
#include <stdint.h>

#include "rc_taa.h"

namespace rc {
namespace taa {

namespace {

constexpr int B = 256;

int blocks(int n) { return (n + B - 1) / B; }

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Lanes with the same region add their values with one atomic per region and value
// (warp-aggregated; the reference adds per point, in an order the hardware chooses).
template <int NV>
__device__ __forceinline__ void region_add(float* base, int rg, bool on, const float (&v)[NV]) {
    const int lane = threadIdx.x & 31;
    unsigned todo = __ballot_sync(0xffffffffu, on);
    while (todo) {
        const int lead = __ffs(todo) - 1;
        const int r = __shfl_sync(0xffffffffu, rg, lead);
        const unsigned grp = __ballot_sync(0xffffffffu, on && rg == r);
        const bool mine = (grp >> lane) & 1u;
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const float s = warp_sum(mine ? v[q] : 0.f);
            if (lane == lead) atomicAdd(base + (size_t)NV * r + q, s);
        }
        todo &= ~grp;
    }
}

// k_taa_touch (poc_gpu.cu:1136-1145): points whose paths crossed a listed voxel
__global__ void k_touch(const uint32_t* __restrict__ cur, const uint32_t* __restrict__ prev, int Np, const int* __restrict__ V, int nv,
                        int* __restrict__ react, uint8_t* __restrict__ pend, int rf, int to_pending) {
    const int i = blockIdx.x * B + threadIdx.x;
    if (i >= Np) return;
    bool hit = false;
    for (int j = 0; j < nv && !hit; ++j) {
        const int v = V[j];
        const size_t o = (size_t)(v >> 5) * Np + i;
        hit = ((cur[o] | prev[o]) >> (v & 31)) & 1u;
    }
    if (!hit) return;
    if (to_pending) pend[i] = 1;
    else react[i] = rf;
}

// k_taa_oracle (poc_gpu.cu:1146-1150)
__global__ void k_oracle(const float* __restrict__ rold, const float* __restrict__ rnew, int Np, int* __restrict__ react, int rf) {
    const int i = blockIdx.x * B + threadIdx.x;
    if (i >= Np) return;
    if (fabsf(rnew[i] - rold[i]) / (rold[i] + 1e-2f) > 0.10f) react[i] = rf;
}

// k_taa_zone_acc + k_count_zone (poc_gpu.cu:1111-1118, 1129-1134): per region, the sum of
// (sample - history), its square, the history and the count
__global__ void k_zone_acc(const float* __restrict__ x, const float* __restrict__ H, const uint8_t* __restrict__ pend,
                           const int* __restrict__ region, int Np, float* __restrict__ rs, float* __restrict__ cnt, int only_pending) {
    const int i = blockIdx.x * B + threadIdx.x;
    const bool on = i < Np && (!only_pending || pend[i]);
    const int r = on ? region[i] : 0;
    float v[3] = {0.f, 0.f, 0.f};
    if (on) {
        const float d = x[i] - H[i];
        v[0] = d;
        v[1] = d * d;
        v[2] = H[i];
    }
    region_add<3>(rs, r, on, v);
    const float one[1] = {1.f};
    region_add<1>(cnt, r, on, one);
}

// k_taa_zone_decide (poc_gpu.cu:1119-1128)
__global__ void k_zone_decide(const float* __restrict__ rs, const float* __restrict__ cnt, uint8_t* __restrict__ pend,
                              const int* __restrict__ region, int Np, int* __restrict__ react, int only_pending, int rf, int clear_pending) {
    const int i = blockIdx.x * B + threadIdx.x;
    if (i >= Np) return;
    if (only_pending && !pend[i]) return;
    const int r = region[i];
    const float n = cnt[r];
    if (n >= 8.f) {
        const float m = rs[3 * r] / n, se = sqrtf(fmaxf(rs[3 * r + 1] / n - m * m, 0.f) / n), base = rs[3 * r + 2] / n;
        if (fabsf(m) > 2.f * se && fabsf(m) > 0.05f * fmaxf(base, 1e-3f)) react[i] = rf;
    }
    if (clear_pending) pend[i] = 0;
}

// Block partial of one FP64 value per thread, in a fixed order: the warp butterfly, then the
// block's 8 warp sums in warp order by thread 0.
__device__ __forceinline__ void block_partial(double v, double* sh, double* dst) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) sh[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < B / 32; ++w) t += sh[w];
        *dst = t;
    }
}

// Double-float sum (hi + lo, |lo| <= ulp(hi) / 2) of two such pairs: TwoSum of the high parts,
// then the low parts, renormalised; about 48 significant bits, all on the FP32 pipe.  Adds
// and subtractions only (nothing to fuse), and symmetric in a and b, so every lane of an xor
// butterfly ends with the same pair.
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float s = __fadd_rn(a.x, b.x);
    const float bv = __fsub_rn(s, a.x);
    const float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bv)), __fsub_rn(b.x, bv));
    const float lo = __fadd_rn(__fadd_rn(a.y, b.y), err);
    const float hi = __fadd_rn(s, lo);
    return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

// k_taa_stats + k_taa_update + k_taa_err (poc_gpu.cu:1100-1108, 1152-1166) for one point:
// 3x3 mean and deviation of the samples, the clamped and blended history, and this block's
// partial of the squared error of the new history in a fixed order: each e^2 exactly as a
// pair of floats, the warp's sum as a double-float butterfly and the block's 8 warp sums
// added in warp order the same way (the FP64 pipe of this GPU is a small fraction of its
// FP32 rate), one conversion to FP64 per block.  The sums of the
// references and of the valid points, which do not change within a state, come from
// k_ref_sums.  The 3x3
// neighbourhood on the point's quad grid (run_taa_mode's table, poc_gpu.cu:1192-1203) is
// derived from the point's quad: quad[q] = (first point, nu, nv), neighbours in the table's
// order (dv outer, du inner), -1 outside the grid; a point of no quad has no neighbours.
__global__ void __launch_bounds__(B) k_post(const float* __restrict__ x, const int* __restrict__ qid, const int4* __restrict__ quad,
                                            const float* __restrict__ H,
                                            float* __restrict__ H2, float* __restrict__ mu_out, float* __restrict__ sg_out,
                                            int* __restrict__ react, int Np, float alpha, float alpha_r, float gamma,
                                            const float* __restrict__ ref, const uint8_t* __restrict__ valid, double* __restrict__ part) {
    __shared__ float2 sh[B / 32];
    const int i = blockIdx.x * B + threadIdx.x;
    float2 d2 = make_float2(0.f, 0.f);
    if (i < Np) {
        float s1 = 0.f, s2 = 0.f;
        int n = 0;
        const int q = qid[i];
        if (q >= 0) {
            const int4 g = quad[q];   // first point, nu, nv
            const int r = i - g.x, iu = r % g.y, iv = r / g.y;
            // the nine loads are issued together: a neighbour outside the grid reads the point
            // itself and adds an exact +0 (samples are >= 0, so the sums never hold -0), which
            // leaves the sums of the in-grid neighbours in the table's order unchanged
            float v[9];
            bool ok[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const int a = iu + k % 3 - 1, b = iv + k / 3 - 1;
                ok[k] = a >= 0 && a < g.y && b >= 0 && b < g.z;
                v[k] = x[ok[k] ? g.x + b * g.y + a : i];
            }
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const float vv = ok[k] ? v[k] : 0.f;
                s1 += vv;
                s2 += vv * vv;
                n += ok[k] ? 1 : 0;
            }
        }
        const float mu = s1 / n;
        const float sg = sqrtf(fmaxf(s2 / n - mu * mu, 0.f));
        mu_out[i] = mu;
        sg_out[i] = sg;
        float h = H[i];
        if (gamma > 0.f) {
            const float lo = mu - gamma * sg, hi = mu + gamma * sg;
            h = fminf(fmaxf(h, lo), hi);
        }
        float a = alpha, target = x[i];
        const int rc = react[i];
        if (rc > 0) {
            a = alpha_r;
            react[i] = rc - 1;
            target = mu;
        }
        const float hn = h + a * (target - h);
        H2[i] = hn;
        if (ref && valid[i]) {
            const float e = hn - ref[i];
            const float hi = __fmul_rn(e, e);
            d2 = make_float2(hi, __fmaf_rn(e, e, -hi));   // e^2 = hi + lo exactly
        }
    }
    if (!part) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        d2 = df_add(d2, make_float2(__shfl_xor_sync(0xffffffffu, d2.x, o), __shfl_xor_sync(0xffffffffu, d2.y, o)));
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) sh[warp] = d2;
    __syncthreads();
    if (threadIdx.x == 0) {
        float2 t = sh[0];
        for (int w = 1; w < B / 32; ++w) t = df_add(t, sh[w]);
        part[3 * (size_t)blockIdx.x] = (double)t.x + (double)t.y;
    }
}

// The other two error sums of k_post's tree: the references and the count of the valid points.
__global__ void __launch_bounds__(B) k_ref_sums(const float* __restrict__ ref, const uint8_t* __restrict__ valid, int Np,
                                                double* __restrict__ part) {
    __shared__ double sh[2][B / 32];
    const int i = blockIdx.x * B + threadIdx.x;
    const bool on = i < Np && valid[i];
    block_partial(on ? (double)ref[i] : 0.0, sh[0], part + 3 * (size_t)blockIdx.x + 1);
    block_partial(on ? 1.0 : 0.0, sh[1], part + 3 * (size_t)blockIdx.x + 2);
}

// the block partials in block order
__global__ void k_err_final(const double* __restrict__ part, int nblocks, double* __restrict__ out) {
    __shared__ double sh[3][B];
    const int t = threadIdx.x;
    double a = 0.0, b = 0.0, c = 0.0;
    for (int k = t; k < nblocks; k += B) {
        a += part[3 * (size_t)k];
        b += part[3 * (size_t)k + 1];
        c += part[3 * (size_t)k + 2];
    }
    sh[0][t] = a;
    sh[1][t] = b;
    sh[2][t] = c;
    __syncthreads();
    for (int o = B / 2; o > 0; o >>= 1) {
        if (t < o)
            for (int q = 0; q < 3; ++q) sh[q][t] += sh[q][t + o];
        __syncthreads();
    }
    if (t < 3) out[t] = sh[t][0];
}

}  // namespace

int post_blocks(int Np) { return blocks(Np); }

cudaError_t touch(const uint32_t* cur, const uint32_t* prev, int Np, const int* V, int nv, int* react, uint8_t* pend, int rf, int to_pending,
                  cudaStream_t st) {
    k_touch<<<blocks(Np), B, 0, st>>>(cur, prev, Np, V, nv, react, pend, rf, to_pending);
    return cudaGetLastError();
}

cudaError_t oracle(const float* rold, const float* rnew, int Np, int* react, int rf, cudaStream_t st) {
    k_oracle<<<blocks(Np), B, 0, st>>>(rold, rnew, Np, react, rf);
    return cudaGetLastError();
}

cudaError_t zone_acc(const float* x, const float* H, const uint8_t* pend, const int* region, int Np, float* rs, float* cnt, int only_pending,
                     cudaStream_t st) {
    k_zone_acc<<<blocks(Np), B, 0, st>>>(x, H, pend, region, Np, rs, cnt, only_pending);
    return cudaGetLastError();
}

cudaError_t zone_decide(const float* rs, const float* cnt, uint8_t* pend, const int* region, int Np, int* react, int only_pending, int rf,
                        int clear_pending, cudaStream_t st) {
    k_zone_decide<<<blocks(Np), B, 0, st>>>(rs, cnt, pend, region, Np, react, only_pending, rf, clear_pending);
    return cudaGetLastError();
}

cudaError_t post(const float* x, const int* qid, const int4* quad, const float* H, float* H2, float* mu, float* sg, int* react, int Np,
                 float alpha, float alpha_r, float gamma, const float* ref, const uint8_t* valid, double* part, double* out, cudaStream_t st) {
    k_post<<<blocks(Np), B, 0, st>>>(x, qid, quad, H, H2, mu, sg, react, Np, alpha, alpha_r, gamma, ref, valid, part);
    if (part) k_err_final<<<1, B, 0, st>>>(part, blocks(Np), out);
    return cudaGetLastError();
}

cudaError_t ref_sums(const float* ref, const uint8_t* valid, int Np, double* part, double* out, cudaStream_t st) {
    k_ref_sums<<<blocks(Np), B, 0, st>>>(ref, valid, Np, part);
    k_err_final<<<1, B, 0, st>>>(part, blocks(Np), out);
    return cudaGetLastError();
}

}  // namespace taa
}  // namespace rc
