// Kernels of the radiance-cache frame loop for sm_103a.
//
// One thread per cache point, 256 points per block, like the reference's k_trace2 /
// k_update (cuda/poc_gpu.cu:433-602).  What differs is how the work is organised:
//  * a frame without verification, projection or DDGI is ONE kernel: trace + blend +
//    history + Sum 1/(n+1) + error sums, so the per-point rays' result never goes through
//    HBM (the reference writes kk and m, then k_update reads them back);
//  * dynamic triangles are culled by a plane filter over axis-aligned rectangles before the
//    exact Möller-Trumbore test; the exact test runs only on the few rectangles that can
//    hold the closest hit, so hit ids and distances are those of the reference's full scan;
//  * per-point gathers at the hit point are 16-byte vectors (albedo + direct light in one
//    record, the cache padded to 4 lights);
//  * reductions are order-free or fixed-order (Sum 1/(n+1) exactly in 64-bit fixed point,
//    error sums in a fixed tree) and need no block-wide barrier, so runs are reproducible bit
//    for bit and no warp waits for its block's slowest warp;
//  * an event is one kernel applying the reference's per-point event kernels in order.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "../../include/rc_hashgrid.h"
#include "rc_internal.h"

namespace rc {

// ------------------------------------------------------------------ fixed-order reductions
template <typename T>
__device__ __forceinline__ T warp_tree(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
// Fixed-order float sum over the grid without a block-wide barrier.  Level 1, per block of 256
// values: each warp's butterfly sum (lane l += lane l+off, off = 16..1) goes to shared memory
// and the last warp of the block to arrive adds the 8 sums in warp order.  Level 2, done by
// the grid's last such warp over the G block partials: slot t = lane + 32 j sums partials
// t, t+256, ... in order, each group of 32 slots goes through the butterfly and the 8 group
// sums are added in order.  The CPU oracle restates this order exactly.
template <typename T, int NV>
struct WarpTail {
    T sh[NV][BLOCK / 32];
    unsigned arrived;
    int last_block;
};

template <typename T, int NV>
__device__ __forceinline__ bool warp_tail_reduce(const T (&v)[NV], WarpTail<T, NV>& wt, T* part, unsigned* ticket,
                                                 T (&total)[NV]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T r[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) r[k] = warp_tree(v[k]);
    unsigned arrived = 0;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) wt.sh[k][w] = r[k];
        __threadfence_block();
        arrived = atomicAdd(&wt.arrived, 1u);
    }
    arrived = __shfl_sync(0xffffffffu, arrived, 0);
    if (arrived != BLOCK / 32 - 1) return false;
    __threadfence_block();
    unsigned tk = 0;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const volatile T* sv = wt.sh[k];
            T s = sv[0];
#pragma unroll
            for (int j = 1; j < BLOCK / 32; ++j) s = s + sv[j];
            part[(size_t)blockIdx.x * NV + k] = s;
        }
        __threadfence();
        tk = atomicAdd(ticket, 1u);
    }
    tk = __shfl_sync(0xffffffffu, tk, 0);
    if (tk != gridDim.x - 1) return false;
    __threadfence();
    const int G = gridDim.x;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        T acc = T(0);
        for (int j = 0; j < BLOCK / 32; ++j) {
            const int t = lane + 32 * j;
            T x = T(0);
            if (t < G) x = __ldcg(part + (size_t)t * NV + k);
            for (int b = t + BLOCK; b < G; b += BLOCK) x = x + __ldcg(part + (size_t)b * NV + k);
            x = warp_tree(x);
            acc = j == 0 ? x : acc + x;
        }
        total[k] = acc;
    }
    if (lane == 0) *ticket = 0u;
    return lane == 0;
}

// Sum 1/(n+1) over the points, exactly: every term is a float in (0, 1] held as an integer
// number of 2^-40 units (exact for terms >= 2^-16, i.e. histories below 65535 frames), the
// integers are added with 64-bit atomics (order-free, so the sum is reproducible), and the
// total is rounded once to float.  Per block: warp sums into a shared accumulator, the last
// warp to arrive adds it to the global accumulator; the grid's last block converts it.
__device__ __forceinline__ unsigned long long pr_fixed(float pr) { return __float2ull_rn(pr * 1099511627776.0f); }

__device__ __forceinline__ float fixed_to_float(unsigned long long tot) {
    return __ull2float_rn(tot) * (1.0f / 1099511627776.0f);
}

// Order-free integer total over the grid (pending counts, fixed-point sums): warp sums into a
// shared accumulator, the block's last warp adds it to `gacc`, the grid's last block reads and
// clears it.  Returns true in the one thread that holds the total.
struct U64Tail {
    unsigned long long acc;
    unsigned arrived;
};
__device__ __forceinline__ bool u64_tail_reduce(unsigned long long v, U64Tail& t, unsigned long long* gacc, unsigned* ticket,
                                                unsigned long long& total) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    unsigned arrived = 0;
    if (lane == 0) {
        if (v) atomicAdd(&t.acc, v);
        __threadfence_block();
        arrived = atomicAdd(&t.arrived, 1u);
    }
    arrived = __shfl_sync(0xffffffffu, arrived, 0);
    if (arrived != BLOCK / 32 - 1) return false;
    unsigned tk = 0;
    if (lane == 0) {
        __threadfence_block();
        const unsigned long long b = atomicAdd(&t.acc, 0ull);
        if (b) atomicAdd(gacc, b);
        __threadfence();
        tk = atomicAdd(ticket, 1u);
    }
    tk = __shfl_sync(0xffffffffu, tk, 0);
    if (tk != gridDim.x - 1 || lane != 0) return false;
    __threadfence();
    total = atomicExch(gacc, 0ull);
    *ticket = 0u;
    return true;
}

// ------------------------------------------------------------------ per-region sums
// The reference adds per-point statistics into per-region slots with one float atomic per
// point and value (poc_gpu.cu:492-497, 498-512, 517-523).  Neighbouring points mostly share a
// region, so those atomics pile onto a few addresses; here the lanes of a warp that share a
// region first add their values in a butterfly (non-members add 0) and one lane issues the
// atomic.  The sums stay float sums in an unspecified order across warps, as in the
// reference.  Must be called by the whole warp.
__device__ __forceinline__ float warp_bfly(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int NV>
__device__ __forceinline__ void region_add(float* __restrict__ base, int stride, int rg, bool on, const float (&v)[NV]) {
    const int lane = threadIdx.x & 31;
    unsigned todo = __ballot_sync(0xffffffffu, on);
    while (todo) {
        const int lead = __ffs(todo) - 1;
        const int r = __shfl_sync(0xffffffffu, rg, lead);
        const bool mine = on && rg == r;
        const unsigned grp = __ballot_sync(0xffffffffu, mine);
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const float s = warp_bfly(mine ? v[q] : 0.f);
            if (lane == lead) atomicAdd(base + (size_t)stride * r + q, s);
        }
        todo &= ~grp;
    }
}

// Projection normal equations (poc_gpu.cu:498-512): k T_a T_b for a <= b, sum(acc) T_a, k.
__device__ __forceinline__ void proj_region_add(float* __restrict__ neq, int rg, bool on, int K, const float* T, float kf,
                                                float sv) {
    const int lane = threadIdx.x & 31;
    unsigned todo = __ballot_sync(0xffffffffu, on);
    while (todo) {
        const int lead = __ffs(todo) - 1;
        const int r = __shfl_sync(0xffffffffu, rg, lead);
        const bool mine = on && rg == r;
        const unsigned grp = __ballot_sync(0xffffffffu, mine);
        float* qn = neq + (size_t)r * NEQ;
        int ix = 0;
        for (int a = 0; a < K; ++a)
            for (int b = a; b < K; ++b, ++ix) {
                const float s = warp_bfly(mine ? kf * T[a] * T[b] : 0.f);
                if (lane == lead) atomicAdd(qn + ix, s);
            }
        for (int a = 0; a < K; ++a) {
            const float s = warp_bfly(mine ? sv * T[a] : 0.f);
            if (lane == lead) atomicAdd(qn + 21 + a, s);
        }
        const float s = warp_bfly(mine ? kf : 0.f);
        if (lane == lead) atomicAdd(qn + 27, s);
        todo &= ~grp;
    }
}

// ------------------------------------------------------------------ tracing
struct TraceSmem {
    const float4* tri;
    const float4* grp;
    const float4* gpair;   // pass-1 records, 3 float4 per pair of groups
    const int* misc;
};

// Plane filter of two groups of one axis k at once, in paired FP32 arithmetic: the ray's
// crossing of group g's plane (t = (c - o_k) / d_k) is a candidate when it lies ahead of the
// origin and inside the group's outer box, stored as centre and half extent.  The candidate
// bits are shifted in
// (mask = mask << 2 | hit_g << 1 | hit_g+1), so group g ends at bit ng - 1 - g.  The filter
// only has to be conservative (the box margin and the stopping slack of pass 2 are orders of
// magnitude above its rounding), so 1 / d_k is the approximate reciprocal.
//
// The three tests are read off sign bits: 5e-5 - t, |x_a - c_a| - h_a and |x_b - c_b| - h_b are
// all negative exactly when the crossing is a candidate, except on the grown box's boundary
// itself (a zero difference), which lies a full margin away from the group's triangles.
__device__ __forceinline__ float2 abs2(float2 v) { return make_float2(fabsf(v.x), fabsf(v.y)); }

template <typename MaskT>
__device__ __forceinline__ void filter_pair(const float4* __restrict__ gp, int pp, float2 ok, float2 idk, float2 oa, float2 nda,
                                            float2 ob, float2 ndb, MaskT& mask) {
    // records hold -c, -centre_a, -half_a, -centre_b, -half_b; nt = (o_k - c) / d_k = -t
    const float4 P0 = gp[3 * pp], P1 = gp[3 * pp + 1];
    const float2 P2 = *reinterpret_cast<const float2*>(gp + 3 * pp + 2);
    const float2 nt = __fmul2_rn(__fadd2_rn(ok, make_float2(P0.x, P0.y)), idk);
    const float2 ea = __fadd2_rn(__ffma2_rn(nt, nda, oa), make_float2(P0.z, P0.w));
    const float2 eb = __fadd2_rn(__ffma2_rn(nt, ndb, ob), make_float2(P1.z, P1.w));
    const float2 ga = __fadd2_rn(abs2(ea), make_float2(P1.x, P1.y));
    const float2 gb = __fadd2_rn(abs2(eb), P2);
    const float2 gt = __fadd2_rn(nt, make_float2(5e-5f, 5e-5f));
    const unsigned s0 = __float_as_uint(ga.x) & __float_as_uint(gb.x) & __float_as_uint(gt.x);
    const unsigned s1 = __float_as_uint(ga.y) & __float_as_uint(gb.y) & __float_as_uint(gt.y);
    mask = (mask << 2) | (MaskT)((s0 >> 30) & 2u) | (MaskT)(s1 >> 31);
}

// Pass 1 over the groups [a, b) of one axis (a, b even).
template <typename MaskT>
__device__ __forceinline__ void filter_axis(const float4* __restrict__ gp, int a, int b, float ok, float idk, float oa, float da,
                                            float ob, float db, MaskT& mask) {
    const float2 ok2 = make_float2(ok, ok), idk2 = make_float2(idk, idk);
    const float2 oa2 = make_float2(oa, oa), nda2 = make_float2(-da, -da), ob2 = make_float2(ob, ob), ndb2 = make_float2(-db, -db);
#pragma unroll 2
    for (int pp = a >> 1; pp < (b >> 1); ++pp) filter_pair(gp, pp, ok2, idk2, oa2, nda2, ob2, ndb2, mask);
}

template <typename MaskT>
__device__ __forceinline__ void trace_groups(const TraceSmem& sm, const DState& s, f3 o, f3 d, float& tmin, int& q, int& jb) {
    // pass 1: bit ng - 1 - g of mask <=> group g is a candidate
    MaskT mask = 0;
    const float idx = __fdividef(1.f, d.x), idy = __fdividef(1.f, d.y), idz = __fdividef(1.f, d.z);
    filter_axis(sm.gpair, s.gr.g0[0], s.gr.g0[1], o.x, idx, o.y, d.y, o.z, d.z, mask);
    filter_axis(sm.gpair, s.gr.g0[1], s.gr.g0[2], o.y, idy, o.x, d.x, o.z, d.z, mask);
    filter_axis(sm.gpair, s.gr.g0[2], s.gr.g0[3], o.z, idz, o.x, d.x, o.y, d.y, mask);
    // pass 2: candidates nearest first, exact test, stop past the best hit plus the slack
    const int top = s.ng - 1;
    float thr = tmin * 1.0001f + 1e-5f;
    while (mask) {
        float best = __int_as_float(0x7f800000);
        int bb = 0;
        for (MaskT m = mask; m; m &= m - 1) {
            const int b = sizeof(MaskT) == 8 ? __ffsll((long long)m) - 1 : __ffs((int)m) - 1;
            const int g = top - b;
            const float ok = g < s.gr.g0[1] ? o.x : (g < s.gr.g0[2] ? o.y : o.z);
            const float idk = g < s.gr.g0[1] ? idx : (g < s.gr.g0[2] ? idy : idz);
            const float tk = (sm.grp[3 * g].x - ok) * idk;
            if (tk < best) { best = tk; bb = b; }
        }
        if (!(best <= thr)) break;
        mask &= ~((MaskT)1 << bb);
        const int g = top - bb;
        const float4 G1 = sm.grp[3 * g + 1];
        int j = __float_as_int(G1.y), jend = j + __float_as_int(G1.z);
        if (jend - j == 2) {
            // exact test on the triangle whose side of the diagonal holds the crossing (both
            // within eps of the diagonal): the other one cannot hold the hit
            const float4 GL = sm.grp[3 * g + 2];
            const bool ax0 = g < s.gr.g0[1], ax1 = !ax0 && g < s.gr.g0[2];
            const float oa = ax0 ? o.y : o.x, da = ax0 ? d.y : d.x;
            const float ob = ax0 || ax1 ? o.z : o.y, db = ax0 || ax1 ? d.z : d.y;
            const float sd = GL.x * (oa + best * da) + GL.y * (ob + best * db) + GL.z;
            if (sd > GL.w) jend = j + 1;
            else if (sd < -GL.w) j = j + 1;
        }
        for (; j < jend; ++j) mt_tri(sm.tri, j, o, d, tmin, q, jb);
        thr = tmin * 1.0001f + 1e-5f;
    }
}

// Closest dynamic-triangle hit, equal to the reference's in-order scan (poc_gpu.cu:199-220).
// Pass 1 marks the groups whose plane crossing falls in their outer box; pass 2 visits the
// marked groups nearest first, runs the exact Möller-Trumbore on their triangles, and stops
// once the next crossing lies beyond the best exact hit by more than the filter's error.
__device__ __forceinline__ void trace_dyn(const TraceSmem& sm, const DState& s, bool brute, f3 o, f3 d, float& tmin, int& q,
                                          int& jb) {
    tmin = __int_as_float(0x7f800000);
    q = -1;
    jb = 0x7fffffff;
    if (brute || s.ng == 0) {
        for (int j = 0; j < s.nt; ++j) mt_tri(sm.tri, j, o, d, tmin, q, jb);
        return;
    }
    for (int k = 0; k < s.nmisc; ++k) mt_tri(sm.tri, sm.misc[k], o, d, tmin, q, jb);
    if (s.ng <= 32) trace_groups<unsigned>(sm, s, o, d, tmin, q, jb);
    else trace_groups<unsigned long long>(sm, s, o, d, tmin, q, jb);
}

// poc_gpu.cu:288-295.  fs scales the exit distance: 1 reproduces the reference exactly (a
// product by 1 is exact); the watertight mode passes 1 + 4 ulp, which covers the rounding of
// the slab distances (Ize, "Robust BVH Ray Traversal", JCGT 2(2), 2013: 1 + 2 gamma_3), so a
// ray through a box's edge or corner is not culled by every box that touches it.
__device__ __forceinline__ float aabb_enter(float4 a, float4 b, f3 o, f3 inv, float tmax, float fs = 1.f) {
    float tx1 = (a.x - o.x) * inv.x, tx2 = (b.x - o.x) * inv.x;
    float ty1 = (a.y - o.y) * inv.y, ty2 = (b.y - o.y) * inv.y;
    float tz1 = (a.z - o.z) * inv.z, tz2 = (b.z - o.z) * inv.z;
    float tn = fmaxf(fmaxf(fminf(tx1, tx2), fminf(ty1, ty2)), fmaxf(fminf(tz1, tz2), 0.f));
    float tf = fminf(fminf(fmaxf(tx1, tx2), fmaxf(ty1, ty2)), fminf(fmaxf(tz1, tz2), tmax));
    return tn <= tf * fs ? tn : 1e30f;
}
// ------------------------------------------------------------------ watertight test
// Watertight ray/triangle test (Woop, Benthin and Wald, "Watertight Ray/Triangle
// Intersection", JCGT 2(1), 2013), the RC_FLAG_WATERTIGHT alternative to the reference's
// Moller-Trumbore for the static mesh.  The ray frame is permuted so that the ray's largest
// direction component becomes z and sheared so that the ray runs along +z from the origin;
// the triangle's three 2-D edge functions U, V, W are then evaluated with every product and
// difference rounded on its own, so the triangle on the other side of a shared edge gets the
// same value negated, and all three are recomputed in FP64 (exact products, one rounding) when
// one of them is exactly zero.  A hit needs U, V, W of one sign (either side faces the ray).
// The vertices are those of the stored triangle: v0, v0 + e1, v0 + e2.
struct WtRay {
    int kx, ky, kz;
    float sx, sy, sz;
};
__device__ __forceinline__ float sel3(f3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
__device__ __forceinline__ WtRay wt_ray(f3 d) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    WtRay r;
    r.kz = ax >= ay ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
    r.kx = r.kz == 2 ? 0 : r.kz + 1;
    r.ky = r.kx == 2 ? 0 : r.kx + 1;
    const float dz = sel3(d, r.kz);
    if (dz < 0.f) { const int x = r.kx; r.kx = r.ky; r.ky = x; }   // keep the winding
    r.sx = __fdiv_rn(sel3(d, r.kx), dz);
    r.sy = __fdiv_rn(sel3(d, r.ky), dz);
    r.sz = __fdiv_rn(1.f, dz);
    return r;
}
__device__ __forceinline__ f3 sub_rn(f3 a, f3 b) { return mk(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ f3 add_rn(f3 a, f3 b) { return mk(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
__device__ __forceinline__ float edge64(float ax, float by, float ay, float bx) {
    return (float)__dsub_rn(__dmul_rn((double)ax, (double)by), __dmul_rn((double)ay, (double)bx));
}
// Hit distance in units of d, or +inf when the ray misses the triangle.
__device__ __forceinline__ float wt_tri(const WtRay& r, f3 o, f3 v0, f3 e1, f3 e2) {
    const f3 A = sub_rn(v0, o), B = sub_rn(add_rn(v0, e1), o), C = sub_rn(add_rn(v0, e2), o);
    const float az = sel3(A, r.kz), bz = sel3(B, r.kz), cz = sel3(C, r.kz);
    const float Ax = __fsub_rn(sel3(A, r.kx), __fmul_rn(r.sx, az)), Ay = __fsub_rn(sel3(A, r.ky), __fmul_rn(r.sy, az));
    const float Bx = __fsub_rn(sel3(B, r.kx), __fmul_rn(r.sx, bz)), By = __fsub_rn(sel3(B, r.ky), __fmul_rn(r.sy, bz));
    const float Cx = __fsub_rn(sel3(C, r.kx), __fmul_rn(r.sx, cz)), Cy = __fsub_rn(sel3(C, r.ky), __fmul_rn(r.sy, cz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.f || V == 0.f || W == 0.f) {
        U = edge64(Cx, By, Cy, Bx);
        V = edge64(Ax, Cy, Ay, Cx);
        W = edge64(Bx, Ay, By, Ax);
    }
    const float inf = __int_as_float(0x7f800000);
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return inf;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.f) return inf;
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, __fmul_rn(r.sz, az)), __fmul_rn(V, __fmul_rn(r.sz, bz))),
                              __fmul_rn(W, __fmul_rn(r.sz, cz)));
    return __fdiv_rn(T, det);
}
// Static-mesh traversal, the reference's stack algorithm (poc_gpu.cu:297-338), with a visit
// guard against malformed node links.  Nodes are visited in the reference's order (nearest
// child first, far child pushed, same pruning against the running tmin).  A node's link word
// (first child or first triangle, in a.w) and triangle count (b.w) arrive with its bounds
// when its parent tests it, so the stack keeps that pair instead of the node index: a visit
// then waits on one load (the children's bounds) instead of two in a row (the node, then
// its children).
// WT selects the watertight mode: its triangle test and a slab exit scaled by 1 + 4 ulp.
template <bool WT>
__device__ __forceinline__ void trace_bvh_t(const float4* __restrict__ BN, const float4* __restrict__ ST4, int max_visits, f3 o,
                                            f3 d, float& tmin, int& q, unsigned* flags) {
    f3 inv = mk(fabsf(d.x) > 1e-12f ? 1.f / d.x : copysignf(1e30f, d.x),
                fabsf(d.y) > 1e-12f ? 1.f / d.y : copysignf(1e30f, d.y),
                fabsf(d.z) > 1e-12f ? 1.f / d.z : copysignf(1e30f, d.z));
    int2 stack[64];
    int sp = 0, visits = 0;
    int lf = __float_as_int(__ldg(&BN[0].w)), cnt = __float_as_int(__ldg(&BN[1].w));
    const float fs = WT ? __int_as_float(0x3f800004) : 1.f;
    WtRay wr{};
    if constexpr (WT) wr = wt_ray(d);    // the ray's frame, once per ray (the direction never changes)
    while (true) {
        if (++visits > max_visits) { atomicOr(flags, (unsigned)FLAG_BVH_VISITS); break; }
        if (WT && cnt > 0) {
            for (int j = lf; j < lf + cnt; ++j) {
                const float4 x = __ldg(ST4 + 3 * (size_t)j), y = __ldg(ST4 + 3 * (size_t)j + 1), z = __ldg(ST4 + 3 * (size_t)j + 2);
                const float t = wt_tri(wr, o, mk(x.x, x.y, x.z), mk(x.w, y.x, y.y), mk(y.z, y.w, z.x));
                if (t > 1e-4f && t < tmin) { tmin = t; q = -2 - j; }
            }
        } else if (cnt > 0) {
            for (int j = lf; j < lf + cnt; ++j) {
                const float4 x = __ldg(ST4 + 3 * (size_t)j), y = __ldg(ST4 + 3 * (size_t)j + 1), z = __ldg(ST4 + 3 * (size_t)j + 2);
                f3 v0 = mk(x.x, x.y, x.z);
                f3 e1 = mk(x.w, y.x, y.y);
                f3 e2 = mk(y.z, y.w, z.x);
                f3 p = cross(d, e2);
                float det = dot(e1, p);
                if (fabsf(det) <= 1e-12f) continue;
                float iv = 1.f / det;
                f3 tv = o - v0;
                float u = dot(tv, p) * iv;
                if (u < 0.f || u > 1.f) continue;
                f3 qv = cross(tv, e1);
                float v = dot(d, qv) * iv;
                if (v < 0.f || u + v > 1.f) continue;
                float t = dot(e2, qv) * iv;
                if (t > 1e-4f && t < tmin) { tmin = t; q = -2 - j; }
            }
        } else {
            float4 la = __ldg(BN + 2 * lf), lb = __ldg(BN + 2 * lf + 1);
            float4 ra = __ldg(BN + 2 * lf + 2), rb = __ldg(BN + 2 * lf + 3);
            float tl = aabb_enter(la, lb, o, inv, tmin, fs), tr = aabb_enter(ra, rb, o, inv, tmin, fs);
            int2 first = make_int2(__float_as_int(la.w), __float_as_int(lb.w));
            int2 second = make_int2(__float_as_int(ra.w), __float_as_int(rb.w));
            if (tr < tl) { float x = tl; tl = tr; tr = x; int2 y = first; first = second; second = y; }
            if (tl < 1e30f) {
                if (tr < 1e30f && sp < 64) stack[sp++] = second;
                lf = first.x;
                cnt = first.y;
                continue;
            }
        }
        if (sp == 0) break;
        const int2 e = stack[--sp];
        lf = e.x;
        cnt = e.y;
    }
}
// The two modes are separate instantiations chosen once per ray, so the default one runs the
// reference's traversal with no per-node branch or exit factor.
static __device__ __forceinline__ float2 trace_bvh_wt(const float4* BN, const float4* ST4, int max_visits, f3 o, f3 d, float tmin,
                                                   int q, unsigned* flags) {
    trace_bvh_t<true>(BN, ST4, max_visits, o, d, tmin, q, flags);
    return make_float2(tmin, __int_as_float(q));
}
__device__ __forceinline__ void trace_bvh(const DStatic& g, f3 o, f3 d, float& tmin, int& q, unsigned* flags) {
    if (g.watertight) {
        const float2 r = trace_bvh_wt(g.BN, g.ST4, g.max_visits, o, d, tmin, q, flags);
        tmin = r.x;
        q = __float_as_int(r.y);
    } else {
        trace_bvh_t<false>(g.BN, g.ST4, g.max_visits, o, d, tmin, q, flags);
    }
}

// poc_gpu.cu:239-246
__device__ __forceinline__ int point_index(const DState& s, f3 H, int q) {
    const float* Q = s.Q + 12 * q;
    f3 o = mk(__ldg(Q), __ldg(Q + 1), __ldg(Q + 2)), u = mk(__ldg(Q + 3), __ldg(Q + 4), __ldg(Q + 5));
    f3 v = mk(__ldg(Q + 6), __ldg(Q + 7), __ldg(Q + 8));
    f3 dd = H - o;
    float a = dot(dd, u) / dot(u, u), b = dot(dd, v) / dot(v, v);
    int nu = __ldg(s.dims + 2 * q), nv = __ldg(s.dims + 2 * q + 1);
    int iu = min(max(int(a * nu), 0), nu - 1), iv = min(max(int(b * nv), 0), nv - 1);
    return __ldg(s.off + q) + iv * nu + iu;
}
// poc_gpu.cu:263-287
__device__ __forceinline__ int hash_find(const DStatic& g, unsigned long long key) {
    unsigned h = (unsigned)mix64(key) & g.hmask;
    for (int probe = 0; probe < 64; ++probe) {
        unsigned long long k = __ldg(g.HK + h);
        if (k == key) return __ldg(g.HV + h);
        if (k == 0ull) return -1;
        h = (h + 1) & g.hmask;
    }
    return -1;
}
static __device__ int hash_point(const DStatic& g, const Grid& grid, f3 H, f3 n) {
    int b = normal_bucket(n.x, n.y, n.z);
    float ih = 1.f / g.hcell;
    int cx = (int)floorf((H.x - grid.lo[0]) * ih), cy = (int)floorf((H.y - grid.lo[1]) * ih), cz = (int)floorf((H.z - grid.lo[2]) * ih);
    int p = hash_find(g, cell_key(cx, cy, cz, b));
    if (p >= 0) return p;
    for (int dd = 0; dd < 27; ++dd) {
        int dz = dd / 9 - 1, dy = (dd / 3) % 3 - 1, dx = dd % 3 - 1;
        if (dx == 0 && dy == 0 && dz == 0) continue;
        p = hash_find(g, cell_key(cx + dx, cy + dy, cz + dz, b));
        if (p >= 0) return p;
    }
    return -1;
}

struct Hit {
    float t;
    int q;
    int pi;
    bool back;
    f3 H;
};

// The cache point a traced ray reached (poc_gpu.cu:345-358, 466-469): with h.t and h.q set,
// fills the hit point, the point index and whether the hit counts.
__device__ __forceinline__ void resolve_hit(const DState& s, const DStatic& g, const Grid& grid, f3 O, f3 D, int i, Hit& h) {
    const bool hit = h.q != -1;
    h.H = hit ? O + D * h.t : O;
    if (!hit) { h.pi = i; h.back = true; return; }
    if (h.q >= 0) {
        h.pi = point_index(s, h.H, h.q);
        const float* Q = s.Q + 12 * h.q;
        h.back = dot(mk(__ldg(Q + 9), __ldg(Q + 10), __ldg(Q + 11)), D) > 0.f;
        return;
    }
    float4 n4 = __ldg(g.STN + (-2 - h.q));
    f3 n = mk(n4.x, n4.y, n4.z);
    if (dot(n, D) > 0.f) {
        if (!(__float_as_int(n4.w) & 1)) { h.pi = i; h.back = true; return; }
        n = n * -1.f;
    }
    h.pi = hash_point(g, grid, h.H, n);
    h.back = false;
    if (h.pi < 0) { h.pi = i; h.back = true; }
}

// Trace one ray and resolve its cache point (poc_gpu.cu:340-358, 466-469).
__device__ __forceinline__ Hit trace_resolve(const TraceSmem& sm, const DState& s, const DStatic& g, const Grid& grid,
                                             const FrameParams& p, const DevCache& c, f3 O, f3 D, int i) {
    Hit h;
    int jb;
    trace_dyn(sm, s, p.brute != 0, O, D, h.t, h.q, jb);
    if (p.check) {
        float tb; int qb, jbb;
        trace_dyn(sm, s, true, O, D, tb, qb, jbb);
        atomicAdd(c.check + 1, 1ull);
        if (qb != h.q || __float_as_int(tb) != __float_as_int(h.t)) atomicAdd(c.check, 1ull);
    }
    if (g.has_bvh) trace_bvh(g, O, D, h.t, h.q, c.flags);
    resolve_hit(s, g, grid, O, D, i, h);
    return h;
}

__device__ __forceinline__ void stage_smem(float4* sm, const DState& s) {
    float4* st = sm;
    float4* sg = sm + 3 * s.nt;
    const int ngf = grp_float4s(s.ng);
    int* smi = (int*)(sg + ngf);
    for (int j = threadIdx.x; j < 3 * s.nt; j += blockDim.x) st[j] = s.tri[j];
    for (int j = threadIdx.x; j < ngf; j += blockDim.x) sg[j] = s.grp[j];
    for (int j = threadIdx.x; j < s.nmisc; j += blockDim.x) smi[j] = s.misc[j];
}
__device__ __forceinline__ TraceSmem smem_view(float4* sm, const DState& s) {
    TraceSmem t;
    t.tri = sm;
    t.grp = sm + 3 * s.nt;
    t.gpair = t.grp + 3 * s.ng;
    t.misc = (const int*)(t.grp + grp_float4s(s.ng));
    return t;
}

template <int N>
__device__ __forceinline__ float comp(const float4 (&v)[N], int k) {
    const float4 x = v[k >> 2];
    const int r = k & 3;
    return r == 0 ? x.x : (r == 1 ? x.y : (r == 2 ? x.z : x.w));
}

// Ray count of a point this frame (poc_gpu.cu:442-454).
__device__ __forceinline__ int ray_count(const FrameParams& p, const DevCache& c, float n_i, bool pend, float sumpr_cur,
                                         int npend_cur, uint32_t& rs) {
    if (p.mode == 0) {
        float kb = floorf(p.budget);
        return int(kb) + (rnd(rs) < p.budget - kb ? 1 : 0);
    }
    float pr = 1.f / (n_i + 1.f);
    float rrest = float(p.Np - npend_cur);
    float e = rrest * (p.half_inv_np + 0.5f * pr / sumpr_cur) * p.rays;
    float eb = floorf(e);
    return (pend ? 1 : 0) + int(eb) + (rnd(rs) < e - eb ? 1 : 0);
}

// ------------------------------------------------------------------ state build
// poc_gpu.cu:369-391: per point and light, a shadow ray gives the direct light; 20 samples
// along each shadow segment give the static voxel mask (skipped when SV is null: the direct
// light alone).
template <int NL, int NW>
__global__ void __launch_bounds__(BLOCK) k_build(const DState s, const DStatic g, const Grid grid, const float* __restrict__ L,
                                                 const float* __restrict__ inten, float4* __restrict__ AE,
                                                 uint32_t* __restrict__ SV, int Np, unsigned* flags) {
    extern __shared__ float4 sm[];
    stage_smem(sm, s);
    __syncthreads();
    const TraceSmem tsm = smem_view(sm, s);
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    if (i >= Np) return;
    constexpr int AES = aes_of(NL);
    const float4 P4 = s.P4[i], N4 = s.N4[i];
    const f3 P = xyz(P4), N = xyz(N4), O = P + N * 1e-3f;
    uint32_t m[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w) m[w] = 0u;
    float rec[AES];
#pragma unroll
    for (int k = 0; k < AES; ++k) rec[k] = 0.f;
    rec[0] = g.A[i];
#pragma unroll
    for (int l = 0; l < NL; ++l) {
        f3 d = mk(L[3 * l], L[3 * l + 1], L[3 * l + 2]) - P;
        float r = sqrtf(dot(d, d));
        f3 D = d * (1.f / r);
        float cc = dot(N, D), t;
        int q, jb;
        trace_dyn(tsm, s, false, O, D, t, q, jb);
        if (g.has_bvh) trace_bvh(g, O, D, t, q, flags);
        bool vis = t >= r - 1e-3f;
        float rr = fmaxf(r, 0.05f);
        rec[1 + l] = inten[l] * fmaxf(cc, 0.f) / (rr * rr) * (vis ? 1.f : 0.f);
        if (SV != nullptr) {
            f3 a = O, b = O + D * fminf(t, r);
            for (int k = 0; k < 20; ++k) set_bit<NW>(m, vox_of(grid, a + (b - a) * (k / 19.f)));
        }
    }
#pragma unroll
    for (int k = 0; k < AES / 4; ++k) AE[(size_t)i * (AES / 4) + k] = make_float4(rec[4 * k], rec[4 * k + 1], rec[4 * k + 2], rec[4 * k + 3]);
    if (SV != nullptr) {
#pragma unroll
        for (int w = 0; w < NW; ++w) SV[(size_t)NW * i + w] = m[w];
    }
}

// ------------------------------------------------------------------ frame kernel
// FUSED: trace + update + reductions (frames without verification, projection or DDGI).
// !FUSED: trace only, writing kk / m and the region statistics (poc_gpu.cu:492-529).
//
// Persistent: the grid is as many blocks as fit on the GPU at once, and each block walks the
// 256-point tiles blockIdx.x, blockIdx.x + gridDim.x, ...  The dynamic triangles are staged
// into shared memory once per block instead of once per tile, and the frame's totals leave
// the block once.  Error sums keep the fixed tree of one partial per tile: the tile's warp
// sums are added in warp order into part[tile], and the last block to finish adds the tile
// partials in the order of final_tree.
#ifndef RC_FRAME_MINB
#define RC_FRAME_MINB 4
#endif

// Level 2 of the fixed-order error sums over G tile partials, run by one whole warp: slot
// t = lane + 32 j sums partials t, t+256, ... in order, each group of 32 slots goes through
// the butterfly and the 8 group sums are added in order (the same tree as warp_tail_reduce).
template <int NV>
__device__ __forceinline__ void final_tree(const double* part, int G, double (&total)[NV]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double acc = 0.0;
        for (int j = 0; j < BLOCK / 32; ++j) {
            const int t = lane + 32 * j;
            double x = 0.0;
            if (t < G) x = __ldcg(part + (size_t)t * NV + k);
            for (int b = t + BLOCK; b < G; b += BLOCK) x = x + __ldcg(part + (size_t)b * NV + k);
            x = warp_tree(x);
            acc = j == 0 ? x : acc + x;
        }
        total[k] = acc;
    }
}

template <int NL, int NW, bool DEPS, bool FUSED>
__global__ void __launch_bounds__(BLOCK, RC_FRAME_MINB) k_frame(const DState s, const DStatic g, const Grid grid, const DevCache c,
                                                 const FrameParams p) {
    extern __shared__ float4 sm[];
    __shared__ U64Tail prt;
    __shared__ double esh[2][3][BLOCK / 32];
    constexpr int LCS = lcs_of(NL), AES = aes_of(NL);
    stage_smem(sm, s);
    if (threadIdx.x == 0) { prt.acc = 0ull; prt.arrived = 0u; }
    __syncthreads();
    const TraceSmem tsm = smem_view(sm, s);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int ntiles = (p.Np + BLOCK - 1) / BLOCK;
    unsigned long long pr_sum = 0ull;   // this thread's Sum 1/(n+1) terms, in 2^-40 units
    unsigned ray_sum = 0u;
    int par = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, par ^= 1) {
    const int i = tile * BLOCK + threadIdx.x;
    float pr_out = 0.f;
    double e_d2 = 0.0, e_rs = 0.0, e_cn = 0.0;
    int k_rays = 0;
    // split path: per-region statistics, added by whole warps after the point's work
    int rg = 0;
    bool on_r = false, on_p = false, on_d = false;
    float vr[4] = {0.f, 0.f, 0.f, 0.f}, vd[3] = {0.f, 0.f, 0.f};
    float T[KSNAP], sv_p = 0.f;
#pragma unroll
    for (int a = 0; a < KSNAP; ++a) T[a] = 0.f;
    if (i < p.Np) {
            uint32_t rs = hash32(p.seed * 0x9E3779B9u ^ hash32(p.frame * 0x85EBCA6Bu ^ hash32(i + 1)));
            const bool pend = !FUSED && p.pend_left > 0 && c.pending[i];
            const float n_i = c.n[i];
            const int k = ray_count(p, c, n_i, pend, c.sumpr[p.sum_in], c.npend[0], rs);
            k_rays = k;
            const f3 P = xyz(s.P4[i]), N = xyz(s.N4[i]), O = P + N * 1e-3f;
            float acc[NL];
#pragma unroll
            for (int l = 0; l < NL; ++l) acc[l] = 0.f;
            uint32_t m[NW];
#pragma unroll
            for (int w = 0; w < NW; ++w) m[w] = 0u;
            const float c0 = pend ? c.c0[i] : 0.f;
            float sd = 0.f, sq = 0.f;
            // the point's own cache and age, read before tracing so the loads overlap the trace
            float4 own[LCS / 4];
            float age_i = 0.f;
            if (FUSED) {
                const float4* lcp = reinterpret_cast<const float4*>(c.Lc) + (size_t)i * (LCS / 4);
#pragma unroll
                for (int k4 = 0; k4 < LCS / 4; ++k4) own[k4] = __ldcg(lcp + k4);
                if (p.ramp) age_i = c.age[i];
            }
            for (int r = 0; r < k; ++r) {
                const float u1 = rnd(rs);
                const float u2 = rnd(rs);
                Hit h;
                if (p.pre_hit != nullptr && r < p.pre_k) {
                    // traced ahead by k_pretrace: hit point, and the cache point (-1 = none: own)
                    const float4 x = __ldcg(p.pre_hit + (size_t)i * p.pre_k + r);
                    const int code = __float_as_int(x.w);
                    h.H = mk(x.x, x.y, x.z);
                    h.back = code < 0;
                    h.pi = code < 0 ? i : code;
                } else {
                    const f3 D = cosine_dir(N, u1, u2);
                    h = trace_resolve(tsm, s, g, grid, p, c, O, D, i);
                }
                float val = 0.f;
                if (!h.back) {
                    float4 ae[AES / 4], lc[LCS / 4];
                    const float4* aep = s.AE + (size_t)h.pi * (AES / 4);
                    const float4* lcp = reinterpret_cast<const float4*>(c.Lc) + (size_t)h.pi * (LCS / 4);
#pragma unroll
                    for (int k4 = 0; k4 < AES / 4; ++k4) ae[k4] = __ldg(aep + k4);
#pragma unroll
                    for (int k4 = 0; k4 < LCS / 4; ++k4) lc[k4] = __ldcg(lcp + k4);
                    const float A = ae[0].x;
#pragma unroll
                    for (int l = 0; l < NL; ++l) {
                        const float lcv = ((p.dormant >> l) & 1) ? 0.f : comp(lc, l);
                        const float v = A * (comp(ae, l + 1) + lcv);
                        acc[l] += v;
                        val += v;
                    }
                }
                if (DEPS) {
                    const int src = h.back ? i : h.pi;
                    const uint4* sv = reinterpret_cast<const uint4*>(s.SV + (size_t)NW * src);
#pragma unroll
                    for (int w = 0; w < NW / 4; ++w) {
                        const uint4 x = __ldg(sv + w);
                        m[4 * w] |= x.x; m[4 * w + 1] |= x.y; m[4 * w + 2] |= x.z; m[4 * w + 3] |= x.w;
                    }
                    dda_walk<NW>(grid, O, h.H, m);
                }
                if (pend) { float dv = val - c0; sd += dv; sq += dv * dv; }
            }
            const float ik = k > 0 ? 1.f / k : 0.f;
            if (!FUSED) {
                rg = g.region[i];
                if (pend && k > 0) {
                    on_r = true;
                    vr[0] = sd; vr[1] = sq; vr[2] = c0 * k; vr[3] = float(k);
                }
                if (p.proj_left > 0 && k > 0) {
                    on_p = true;
                    for (int a = 0; a < p.projK; ++a) {
                        const float* sp = c.snap + ((size_t)p.slot[a] * p.Np + i) * LCS;
                        float t = 0.f;
#pragma unroll
                        for (int l = 0; l < NL; ++l) if (!((p.dormant >> l) & 1)) t += sp[l];
                        T[a] = t;
                    }
#pragma unroll
                    for (int l = 0; l < NL; ++l) sv_p += acc[l];
                }
                c.kk[i] = k;
                float mo[LCS];
#pragma unroll
                for (int l = 0; l < LCS; ++l) mo[l] = l < NL ? acc[l] * ik : 0.f;
                float4* mp = reinterpret_cast<float4*>(c.m) + (size_t)i * (LCS / 4);
#pragma unroll
                for (int k4 = 0; k4 < LCS / 4; ++k4) mp[k4] = make_float4(mo[4 * k4], mo[4 * k4 + 1], mo[4 * k4 + 2], mo[4 * k4 + 3]);
                if (p.ddgi && k > 0) {
                    float sa = 0.f;
#pragma unroll
                    for (int l = 0; l < NL; ++l) sa += acc[l];
                    float est = 0.f;
#pragma unroll
                    for (int l = 0; l < NL; ++l) if (!((p.dormant >> l) & 1)) est += c.Lc[(size_t)LCS * i + l];
                    on_d = true;
                    vd[0] = sa * ik; vd[1] = est; vd[2] = 1.f;
                }
            } else {
                // k_update (poc_gpu.cu:562-602) on the point's own history.
                const float4 (&lc)[LCS / 4] = own;
                float nn = n_i + k;
                float nmx = p.nmax;
                if (p.ramp) {
                    const float a = age_i;
                    nmx = fminf(p.nmax, (4.f + 0.5f * a) * p.rays);
                    c.age[i] = fminf(a + 1.f, 1e4f);
                }
                const float alpha = k > 0 ? fminf(k / fminf(fmaxf(nn, 1.f), nmx), 1.f) : 0.f;
                const float alpha_r = (k > 0 && p.resp_mask) ? fminf(k / fminf(fmaxf(nn, 1.f), p.nmax_resp), 1.f) : 0.f;
                float out[LCS];
                float est = 0.f;
#pragma unroll
                for (int l = 0; l < LCS; ++l) {
                    if (l < NL) {
                        const float a = comp(lc, l);
                        float al = ((p.resp_mask >> l) & 1) ? alpha_r : alpha;
                        if ((p.dormant >> l) & 1) al = 0.f;
                        // the reference stores m = acc * ik (one rounding) before k_update reads it;
                        // __fmul_rn keeps that rounding (no fused multiply-add into the blend)
                        out[l] = a + al * (__fmul_rn(acc[l], ik) - a);
                        if (!((p.dormant >> l) & 1)) est += out[l];
                    } else {
                        out[l] = 0.f;
                    }
                }
                float4* op = reinterpret_cast<float4*>(c.Lc2) + (size_t)i * (LCS / 4);
#pragma unroll
                for (int k4 = 0; k4 < LCS / 4; ++k4) op[k4] = make_float4(out[4 * k4], out[4 * k4 + 1], out[4 * k4 + 2], out[4 * k4 + 3]);
                const float nf = fminf(nn, nmx);
                c.n[i] = nf;
                pr_out = 1.f / (nf + 1.f);
                if (p.want_err && s.valid[i]) {
                    const float e = est - s.ref[i];
                    e_d2 = double(e) * e;
                    e_rs = s.ref[i];
                    e_cn = 1.0;
                }
            }
            if (p.mask_op == MASK_OR) {
                if (DEPS && k > 0) {
#pragma unroll
                    for (int w = 0; w < NW; ++w) {
                        const uint32_t old = c.cur[(size_t)w * p.Np + i];
                        if ((old | m[w]) != old) c.cur[(size_t)w * p.Np + i] = old | m[w];
                    }
                }
            } else if (p.mask_op == MASK_FRESH || p.mask_op == MASK_ZERO) {
#pragma unroll
                for (int w = 0; w < NW; ++w) c.cur[(size_t)w * p.Np + i] = (DEPS && p.mask_op == MASK_FRESH && k > 0) ? m[w] : 0u;
            }
    }
    ray_sum += (unsigned)k_rays;
    if (FUSED) pr_sum += pr_fixed(pr_out);
    if (!FUSED) {
        region_add<4>(c.rstat, 4, rg, on_r, vr);
        if (p.proj_left > 0) proj_region_add(c.neq, rg, on_p, p.projK, T, float(k_rays), sv_p);
        if (p.ddgi) region_add<3>(c.dstat, 3, rg, on_d, vd);
    }
    if (FUSED && p.want_err) {
        // this tile's error partial: warp sums, then the 8 warp sums in warp order
        const double ev[3] = {e_d2, e_rs, e_cn};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double r = warp_tree(ev[k]);
            if (lane == 0) esh[par][k][wid] = r;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                double t = esh[par][k][0];
#pragma unroll
                for (int j = 1; j < BLOCK / 32; ++j) t = t + esh[par][k][j];
                c.partd[(size_t)tile * 3 + k] = t;
            }
        }
    }
    }
    {
        // ray count of the frame: warp sum, one 64-bit atomic per warp
        const unsigned wk = __reduce_add_sync(0xffffffffu, ray_sum);
        if (lane == 0 && wk) atomicAdd(c.rays, (unsigned long long)wk);
    }
    if (FUSED) {
        unsigned long long tot;
        if (u64_tail_reduce(pr_sum, prt, c.pracc, c.ticket, tot)) c.sumpr[p.sum_out] = fixed_to_float(tot);
        if (p.want_err && wid == 0) {
            unsigned tk = 0;
            if (lane == 0) {
                __threadfence();
                tk = atomicAdd(c.ticket + 1, 1u);
            }
            tk = __shfl_sync(0xffffffffu, tk, 0);
            if (tk == gridDim.x - 1) {
                __threadfence();
                double tot3[3];
                final_tree<3>(c.partd, ntiles, tot3);
                if (lane == 0) {
                    c.err[3 * p.err_frame] = tot3[0];
                    c.err[3 * p.err_frame + 1] = tot3[1];
                    c.err[3 * p.err_frame + 2] = tot3[2];
                    c.ticket[1] = 0u;
                }
            }
        }
    }
}

// ------------------------------------------------------------------ traced ahead
// Scenes with a static mesh spend nearly all of a frame in the tree traversal, which is
// latency bound; it runs here as its own kernel with fewer registers per thread than the frame
// kernel, so more warps hide the latency.  The rays are the frame kernel's (same seed, ray
// count and directions); the first pre_k of each point are traced, and their hit points and
// cache points written for the frame kernel to read.  The grid is persistent: each warp takes
// 32 consecutive points at a time from a counter (c.rayctr[1], zeroed before the launch), so a
// warp whose rays were short takes more points instead of leaving its block's slot idle until
// the block's slowest warp ends (1.8 % per frame on a 199 k-triangle street).  Which warp
// traces a point does not change its rays or its hits.
#ifndef RC_PRETRACE_MINB
#define RC_PRETRACE_MINB 5
#endif
template <int NL>
__global__ void __launch_bounds__(BLOCK, RC_PRETRACE_MINB) k_pretrace(const DState s, const DStatic g, const Grid grid,
                                                                      const DevCache c, const FrameParams p, float4* __restrict__ out) {
    extern __shared__ float4 sm[];
    stage_smem(sm, s);
    __syncthreads();
    const TraceSmem tsm = smem_view(sm, s);
    const int lane = threadIdx.x & 31;
    while (true) {
        int base = 0;
        if (lane == 0) base = (int)atomicAdd(c.rayctr + 1, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= p.Np) break;
        const int i = base + lane;
        if (i >= p.Np) continue;
        uint32_t rs = hash32(p.seed * 0x9E3779B9u ^ hash32(p.frame * 0x85EBCA6Bu ^ hash32(i + 1)));
        const bool pend = p.pend_left > 0 && c.pending[i];
        const int k = min(ray_count(p, c, c.n[i], pend, c.sumpr[p.sum_in], c.npend[0], rs), p.pre_k);
        const f3 P = xyz(s.P4[i]), N = xyz(s.N4[i]), O = P + N * 1e-3f;
        for (int r = 0; r < k; ++r) {
            const float u1 = rnd(rs);
            const float u2 = rnd(rs);
            const f3 D = cosine_dir(N, u1, u2);
            const Hit h = trace_resolve(tsm, s, g, grid, p, c, O, D, i);
            out[(size_t)i * p.pre_k + r] = make_float4(h.H.x, h.H.y, h.H.z, __int_as_float(h.back ? -1 : h.pi));
        }
    }
}

// ------------------------------------------------------------------ ray-queue traversal
// An alternative to k_pretrace for the traced-ahead rays of static-mesh scenes
// (RC_FLAG_RAY_QUEUE):
//   k_ray_queue    writes every ray (origin + output slot, direction + point) into a compacted
//                  queue in point order: per warp a scan of the lanes' ray counts and one
//                  atomicAdd on the queue's tail;
//   k_trace_queue  persistent warps: a warp takes chunks of WQ_CHUNK consecutive rays with one
//                  atomicAdd each and refills its idle lanes from its chunk once at least
//                  WQ_REFILL of them are idle (warp ballot, rank by popcount); each lane walks
//                  its ray in the traversal's visit order (inner nodes until a leaf, then the
//                  leaf: Aila and Laine's while-while), the top WQ_STACK entries of its stack in
//                  shared memory and deeper ones in local memory (64 in all, as the reference),
//                  and writes the resolved hit where k_pretrace would.
// Same rays, same per-ray visit order and pruning: the hits equal k_pretrace's bit for bit.
// Measured slower than k_pretrace at about half a million rays per frame (a resident warp gets
// only a few rays per lane per frame, so the refills do not pay for their own cost), hence not
// the default.
constexpr int WQ_BLOCK = 128;
constexpr int WQ_STACK = 16;
constexpr int WQ_REFILL = 16;
constexpr int WQ_CHUNK = 32;
constexpr int WQ_MAXSTACK = 64;

template <int NL>
__global__ void __launch_bounds__(BLOCK) k_ray_queue(const DState s, const DevCache c, const FrameParams p) {
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int k = 0;
    f3 O = mk(0.f, 0.f, 0.f), N = mk(0.f, 0.f, 1.f);
    uint32_t rs = 0;
    if (i < p.Np) {
        rs = hash32(p.seed * 0x9E3779B9u ^ hash32(p.frame * 0x85EBCA6Bu ^ hash32(i + 1)));
        const bool pend = p.pend_left > 0 && c.pending[i];
        k = min(ray_count(p, c, c.n[i], pend, c.sumpr[p.sum_in], c.npend[0], rs), p.pre_k);
        const f3 P = xyz(s.P4[i]);
        N = xyz(s.N4[i]);
        O = P + N * 1e-3f;
    }
    int x = k;   // warp inclusive scan of the ray counts
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    const int total = __shfl_sync(0xffffffffu, x, 31);
    unsigned base = 0;
    if (lane == 31 && total) base = atomicAdd(c.rayctr, (unsigned)total);
    unsigned at = __shfl_sync(0xffffffffu, base, 31) + (unsigned)(x - k);
    const unsigned cap = (unsigned)(p.Np * p.pre_k);
    for (int r = 0; r < k; ++r, ++at) {
        const float u1 = rnd(rs);
        const float u2 = rnd(rs);
        const f3 D = cosine_dir(N, u1, u2);
        if (at < cap) {
            c.rayq[2 * (size_t)at] = make_float4(O.x, O.y, O.z, __int_as_float(i * p.pre_k + r));
            c.rayq[2 * (size_t)at + 1] = make_float4(D.x, D.y, D.z, __int_as_float(i));
        }
    }
}

template <bool WT>
__global__ void __launch_bounds__(WQ_BLOCK) k_trace_queue(const DState s, const DStatic g, const Grid grid, const DevCache c,
                                                          const FrameParams p, float4* __restrict__ out) {
    extern __shared__ float4 sm[];
    stage_smem(sm, s);
    __syncthreads();
    const TraceSmem tsm = smem_view(sm, s);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int dyn4 = (int)((frame_smem_bytes(s) + 15) / 16);
    int2* sstk = reinterpret_cast<int2*>(sm + dyn4) + warp * (WQ_STACK * 32) + lane;   // entry e at sstk[32 e]
    int2 deep[WQ_MAXSTACK - WQ_STACK];
    const unsigned nrays = min(__ldcg(c.rayctr), (unsigned)(p.Np * p.pre_k));
    const unsigned lt = (1u << lane) - 1u;
    const float fs = WT ? __int_as_float(0x3f800004) : 1.f;
    bool active = false, drained = false;
    unsigned cbase = 0, cend = 0;   // the warp's current chunk of the queue
    f3 O = mk(0.f, 0.f, 0.f), D = mk(0.f, 0.f, 1.f), inv = mk(0.f, 0.f, 0.f);
    float tmin = 0.f;
    int q = -1, lf = 0, cnt = 0, sp = 0, visits = 0, slot = 0, pt = 0;
    WtRay wr{};
    while (true) {
        const unsigned idle = __ballot_sync(0xffffffffu, !active);
        if (!drained && __popc(idle) >= WQ_REFILL) {
            const int nidle = __popc(idle);
            if (cbase >= cend) {   // the warp's chunk is used up: one atomicAdd for the next
                unsigned base = 0;
                if (lane == 0) base = atomicAdd(c.rayctr + 1, (unsigned)WQ_CHUNK);
                base = __shfl_sync(0xffffffffu, base, 0);
                if (base >= nrays) drained = true;
                else { cbase = base; cend = min(base + WQ_CHUNK, nrays); }
            }
            const unsigned avail = cend - cbase;
            const unsigned take = min((unsigned)nidle, avail);
            const unsigned base = cbase;
            cbase += take;
            if (!active) {
                const unsigned rank = (unsigned)__popc(idle & lt);
                const unsigned r = base + rank;
                if (rank < take) {
                    const float4 a = __ldcs(c.rayq + 2 * (size_t)r), b = __ldcs(c.rayq + 2 * (size_t)r + 1);
                    O = mk(a.x, a.y, a.z);
                    slot = __float_as_int(a.w);
                    D = mk(b.x, b.y, b.z);
                    pt = __float_as_int(b.w);
                    int jb;
                    trace_dyn(tsm, s, p.brute != 0, O, D, tmin, q, jb);
                    if (p.check) {
                        float tb;
                        int qb, jbb;
                        trace_dyn(tsm, s, true, O, D, tb, qb, jbb);
                        atomicAdd(c.check + 1, 1ull);
                        if (qb != q || __float_as_int(tb) != __float_as_int(tmin)) atomicAdd(c.check, 1ull);
                    }
                    inv = mk(fabsf(D.x) > 1e-12f ? 1.f / D.x : copysignf(1e30f, D.x),
                             fabsf(D.y) > 1e-12f ? 1.f / D.y : copysignf(1e30f, D.y),
                             fabsf(D.z) > 1e-12f ? 1.f / D.z : copysignf(1e30f, D.z));
                    if constexpr (WT) wr = wt_ray(D);
                    lf = __float_as_int(__ldg(&g.BN[0].w));
                    cnt = __float_as_int(__ldg(&g.BN[1].w));
                    sp = 0;
                    visits = 0;
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (drained) break;
            continue;
        }
        bool done = false;
        if (active) {
            // inner nodes until a leaf (its visit counted) or the end of the walk
            while (true) {
                if (++visits > g.max_visits) { atomicOr(c.flags, (unsigned)FLAG_BVH_VISITS); done = true; break; }
                if (cnt > 0) break;
                const float4 la = __ldg(g.BN + 2 * lf), lb = __ldg(g.BN + 2 * lf + 1);
                const float4 ra = __ldg(g.BN + 2 * lf + 2), rb = __ldg(g.BN + 2 * lf + 3);
                float tl = aabb_enter(la, lb, O, inv, tmin, fs), tr = aabb_enter(ra, rb, O, inv, tmin, fs);
                int2 first = make_int2(__float_as_int(la.w), __float_as_int(lb.w));
                int2 second = make_int2(__float_as_int(ra.w), __float_as_int(rb.w));
                if (tr < tl) { const float x = tl; tl = tr; tr = x; const int2 y = first; first = second; second = y; }
                if (tl < 1e30f) {
                    if (tr < 1e30f && sp < WQ_MAXSTACK) {
                        if (sp < WQ_STACK) sstk[32 * sp] = second;
                        else deep[sp - WQ_STACK] = second;
                        ++sp;
                    }
                    lf = first.x;
                    cnt = first.y;
                    continue;
                }
                if (sp == 0) { done = true; break; }
                --sp;
                const int2 e = sp < WQ_STACK ? sstk[32 * sp] : deep[sp - WQ_STACK];
                lf = e.x;
                cnt = e.y;
            }
            if (!done) {
                // the leaf
                if constexpr (WT) {
                    for (int j = lf; j < lf + cnt; ++j) {
                        const float4 x = __ldg(g.ST4 + 3 * (size_t)j), y = __ldg(g.ST4 + 3 * (size_t)j + 1), z = __ldg(g.ST4 + 3 * (size_t)j + 2);
                        const float t = wt_tri(wr, O, mk(x.x, x.y, x.z), mk(x.w, y.x, y.y), mk(y.z, y.w, z.x));
                        if (t > 1e-4f && t < tmin) { tmin = t; q = -2 - j; }
                    }
                } else {
                    for (int j = lf; j < lf + cnt; ++j) {
                        const float4 x = __ldg(g.ST4 + 3 * (size_t)j), y = __ldg(g.ST4 + 3 * (size_t)j + 1), z = __ldg(g.ST4 + 3 * (size_t)j + 2);
                        const f3 v0 = mk(x.x, x.y, x.z), e1 = mk(x.w, y.x, y.y), e2 = mk(y.z, y.w, z.x);
                        const f3 pv = cross(D, e2);
                        const float det = dot(e1, pv);
                        if (fabsf(det) <= 1e-12f) continue;
                        const float iv = 1.f / det;
                        const f3 tv = O - v0;
                        const float u = dot(tv, pv) * iv;
                        if (u < 0.f || u > 1.f) continue;
                        const f3 qv = cross(tv, e1);
                        const float v = dot(D, qv) * iv;
                        if (v < 0.f || u + v > 1.f) continue;
                        const float t = dot(e2, qv) * iv;
                        if (t > 1e-4f && t < tmin) { tmin = t; q = -2 - j; }
                    }
                }
                if (sp == 0) done = true;
                else {
                    --sp;
                    const int2 e = sp < WQ_STACK ? sstk[32 * sp] : deep[sp - WQ_STACK];
                    lf = e.x;
                    cnt = e.y;
                }
            }
        }
        if (done) {
            if ((unsigned)slot < (unsigned)(p.Np * p.pre_k) && (unsigned)pt < (unsigned)p.Np) {
                Hit h;
                h.t = tmin;
                h.q = q;
                resolve_hit(s, g, grid, O, D, pt, h);
                out[slot] = make_float4(h.H.x, h.H.y, h.H.z, __int_as_float(h.back ? -1 : h.pi));
            } else {
                atomicOr(c.flags, (unsigned)FLAG_BAD_INDEX);   // a malformed queue record: skipped
            }
            active = false;
        }
    }
}

static size_t trace_queue_smem(const DState& s) {
    return ((frame_smem_bytes(s) + 15) / 16) * 16 + (size_t)(WQ_BLOCK / 32) * WQ_STACK * 32 * sizeof(int2);
}

// ------------------------------------------------------------------ split update
// k_decide + k_update (poc_gpu.cu:532-602) for one point, then Sum 1/(n+1), the error sums
// and the pending count, reduced by the last block.
template <int NL>
__global__ void __launch_bounds__(BLOCK) k_update(const DState s, const DStatic g, const DevCache c, const FrameParams p) {
    __shared__ U64Tail prt, npt;
    __shared__ WarpTail<double, 3> taild;
    constexpr int LCS = lcs_of(NL);
    if (threadIdx.x == 0) { prt.acc = 0ull; prt.arrived = 0u; npt.acc = 0ull; npt.arrived = 0u; taild.arrived = 0u; }
    __syncthreads();
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    float pr_out = 0.f;
    double e_d2 = 0.0, e_rs = 0.0, e_cn = 0.0;
    int cnt = 0;
    if (i < p.Np) {
        const int rg = g.region[i];
        if (p.decide && c.pending[i]) {
            const float* r4 = c.rstat + 4 * rg;
            const float cn = r4[3];
            bool done = false;
            if (cn >= 8.f) {
                float mean = r4[0] / cn;
                float se = sqrtf(fmaxf(r4[1] / cn - mean * mean, 0.f) / cn);
                float base = r4[2] / cn;
                float rel = mean / base;
                if (fabsf(mean) > 2.f * se && fabsf(rel) > 0.03f) {
                    float tgt = fminf(fmaxf(0.5f / fabsf(rel), 1.f) * p.rays, p.nmax);
                    c.n[i] = fminf(c.n[i], tgt);
                    c.pending[i] = 0;
                    done = true;
                }
            }
            if (!done) {
                if (p.pend_left <= 1) c.pending[i] = 0;
                else cnt = 1;
            }
        }
        const int k = c.kk[i];
        float n = c.n[i], nn = n + k;
        float nmx = p.nmax;
        if (p.ramp) {
            float a = c.age[i];
            nmx = fminf(p.nmax, (4.f + 0.5f * a) * p.rays);
            c.age[i] = fminf(a + 1.f, 1e4f);
        }
        const float alpha = k > 0 ? fminf(k / fminf(fmaxf(nn, 1.f), nmx), 1.f) : 0.f;
        const float* lci = c.Lc + (size_t)LCS * i;
        const float* mi = c.m + (size_t)LCS * i;
        float* lo = c.Lc2 + (size_t)LCS * i;
        float est = 0.f;
        if (p.ddgi) {
            const float* d3 = c.dstat + 3 * rg;
            float scale = 1.f, h = p.ddgi_h;
            if (d3[2] > 0.f) {
                float mn = d3[0] / d3[2], mc = d3[1] / d3[2];
                float rel = fabsf(mn - mc) / fmaxf(mc, 1e-3f);
                if (rel > p.ddgi_thr) h = fmaxf(0.f, h - 0.75f);
                if (p.ddgi_clamp && rel > 0.10f) scale = 0.25f;
            }
            const float w = k > 0 ? (1.f - h) * scale : 0.f;
#pragma unroll
            for (int l = 0; l < NL; ++l) {
                const float a = lci[l];
                lo[l] = ((p.dormant >> l) & 1) ? a : a + w * (mi[l] - a);
                if (!((p.dormant >> l) & 1)) est += lo[l];
            }
        } else {
            const float alpha_r = k > 0 ? fminf(k / fminf(fmaxf(nn, 1.f), p.nmax_resp), 1.f) : 0.f;
#pragma unroll
            for (int l = 0; l < NL; ++l) {
                const float a = lci[l];
                float al = ((p.resp_mask >> l) & 1) ? alpha_r : alpha;
                if ((p.dormant >> l) & 1) al = 0.f;
                lo[l] = a + al * (mi[l] - a);
                if (!((p.dormant >> l) & 1)) est += lo[l];
            }
        }
#pragma unroll
        for (int l = NL; l < LCS; ++l) lo[l] = 0.f;
        n = fminf(nn, nmx);
        c.n[i] = n;
        pr_out = 1.f / (n + 1.f);
        if (p.want_err && s.valid[i]) {
            const float e = est - s.ref[i];
            e_d2 = double(e) * e;
            e_rs = s.ref[i];
            e_cn = 1.0;
        }
    }
    unsigned long long tot;
    if (u64_tail_reduce(pr_fixed(pr_out), prt, c.pracc, c.ticket, tot)) c.sumpr[p.sum_out] = fixed_to_float(tot);
    if (p.want_err) {
        const double vd[3] = {e_d2, e_rs, e_cn};
        double totd[3];
        if (warp_tail_reduce<double, 3>(vd, taild, c.partd, c.ticket + 1, totd)) {
            c.err[3 * p.err_frame] = totd[0];
            c.err[3 * p.err_frame + 1] = totd[1];
            c.err[3 * p.err_frame + 2] = totd[2];
        }
    }
    if (p.decide && u64_tail_reduce((unsigned long long)cnt, npt, c.npacc, c.ticket + 2, tot)) {
        c.npend[0] = (int)tot;
        c.npend[1] = (int)tot;
    }
}

// ------------------------------------------------------------------ events
template <int NL>
__device__ __forceinline__ float est_point(const float* lc, int dormant) {
    float e = 0.f;
#pragma unroll
    for (int l = 0; l < NL; ++l) if (!((dormant >> l) & 1)) e += lc[l];
    return e;
}

// The per-point kernels of one event (poc_gpu.cu:612-681), applied in launch order to each
// point; then the pending count and, in adaptive mode, Sum 1/(n+1) (poc_gpu.cu:938-941).
template <int NL>
__global__ void __launch_bounds__(BLOCK) k_event(const __grid_constant__ EvProgram ev, const DevCache c) {
    __shared__ U64Tail prt, npt;
    constexpr int LCS = lcs_of(NL);
    if (threadIdx.x == 0) { prt.acc = 0ull; prt.arrived = 0u; npt.acc = 0ull; npt.arrived = 0u; }
    __syncthreads();
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    const int Np = ev.Np;
    if (ev.zero_rstat)
        for (int x = i; x < 4 * ev.NR; x += gridDim.x * BLOCK) c.rstat[x] = 0.f;
    if (ev.zero_neq)
        for (int x = i; x < NEQ * ev.NR; x += gridDim.x * BLOCK) c.neq[x] = 0.f;
    int cnt = 0;
    float pr = 0.f;
    if (i < Np) {
        float* lc = c.Lc + (size_t)LCS * i;
        for (int o = 0; o < ev.nops; ++o) {
            const EvOp& op = ev.ops[o];
            switch (op.kind) {
                case EV_SNAP_SAVE: {
                    float* sp = c.snap + ((size_t)op.a * Np + i) * LCS;
#pragma unroll
                    for (int l = 0; l < LCS; ++l) sp[l] = lc[l];
                } break;
                case EV_SNAP_RESTORE: {
                    const float* sp = c.snap + ((size_t)op.a * Np + i) * LCS;
#pragma unroll
                    for (int l = 0; l < LCS; ++l) lc[l] = sp[l];
                } break;
                case EV_ORACLE: {
                    float rel = fabsf(op.r1[i] - op.r0[i]) / (op.r0[i] + 1e-2f);
                    c.n[i] *= 1.f - fminf(fmaxf(4.f * rel, 0.f), 1.f);
                } break;
                case EV_RESCALE:
                    lc[op.a] *= op.x;
                    break;
                case EV_WAKE:
                    if ((c.stale[i] >> op.a) & 1u) {
                        if (op.b) {
                            c.pending[i] = 1;
                            c.c0[i] = est_point<NL>(lc, op.dormant);
                            if (op.count) cnt++;
                        } else {
                            lc[op.a] = 0.f;
                            c.n[i] = 0.f;
                            c.age[i] = 0.f;
                        }
                        c.stale[i] &= ~(1u << op.a);
                    }
                    break;
                case EV_TOUCHED: {
                    bool t = false;
                    for (int j = 0; j < op.b && !t; ++j) {
                        const int v = op.list[j];
                        const size_t oo = (size_t)(v >> 5) * Np + i;
                        t = ((c.cur[oo] | c.prev[oo]) >> (v & 31)) & 1u;
                    }
                    if (t) {
                        if (op.a == 0) { c.n[i] = 0.f; c.age[i] = 0.f; }
                        else if (op.a == 1) {
                            c.pending[i] = 1;
                            c.c0[i] = est_point<NL>(lc, op.dormant);
                            if (op.count) cnt++;
                        }
                        if (op.a >= 1 && op.dormant) c.stale[i] |= (uint32_t)op.dormant;
                    }
                } break;
                case EV_RESTORED:
                    c.n[i] = ev.nmax;
                    c.age[i] = 1e4f;
                    c.pending[i] = 0;
                    if (op.a) {
                        c.pending[i] = 1;
                        c.c0[i] = est_point<NL>(lc, op.dormant);
                        if (op.count) cnt++;
                    }
                    break;
            }
        }
        pr = 1.f / (c.n[i] + 1.f);
    }
    if (!ev.want_sumpr && ev.npend_mode != 1) {
        if (ev.npend_mode == 2 && blockIdx.x == 0 && threadIdx.x == 0) { c.npend[0] = 0; c.npend[1] = 0; }
        return;
    }
    unsigned long long tot;
    if (ev.want_sumpr && u64_tail_reduce(pr_fixed(pr), prt, c.pracc, c.ticket, tot)) c.sumpr[ev.sum_slot] = fixed_to_float(tot);
    if (ev.npend_mode == 1 && u64_tail_reduce((unsigned long long)cnt, npt, c.npacc, c.ticket + 2, tot)) {
        c.npend[0] = (int)tot;
        c.npend[1] = (int)tot;
    }
    if (ev.npend_mode == 2 && blockIdx.x == 0 && threadIdx.x == 0) { c.npend[0] = 0; c.npend[1] = 0; }
}

// poc_gpu.cu:620-635 + the pending-count reset / publish around it (poc_gpu.cu:990-993).
template <int NL>
__global__ void __launch_bounds__(BLOCK) k_proj_apply(const DevCache c, const DStatic g, const FrameParams p) {
    __shared__ U64Tail npt;
    constexpr int LCS = lcs_of(NL);
    if (threadIdx.x == 0) { npt.acc = 0ull; npt.arrived = 0u; }
    __syncthreads();
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    for (int x = i; x < 4 * p.NR; x += gridDim.x * BLOCK) c.rstat[x] = 0.f;
    int cnt = 0;
    if (i < p.Np && !(c.n[i] >= 16.f)) {
        const float* cf = c.coef + (size_t)g.region[i] * KSNAP;
        if (!isnan(cf[0])) {
            float* lc = c.Lc + (size_t)LCS * i;
            for (int l = 0; l < NL; ++l) {
                if ((p.dormant >> l) & 1) continue;
                float v = 0.f;
                for (int a = 0; a < p.projK; ++a) v += cf[a] * c.snap[((size_t)p.slot[a] * p.Np + i) * LCS + l];
                lc[l] = fmaxf(v, 0.f);
            }
            c.n[i] = 8.f * p.rays;
            c.age[i] = 8.f;
            c.pending[i] = 1;
            c.c0[i] = est_point<NL>(lc, p.dormant);
            cnt = 1;
        }
    }
    unsigned long long tot;
    if (u64_tail_reduce((unsigned long long)cnt, npt, c.npacc, c.ticket + 2, tot)) {
        c.npend[0] = (int)tot;
        c.npend[1] = (int)tot;
    }
}

// poc_gpu.cu:683-696: FP64 error sums of the current cache over valid points (used on
// frames whose cache changes after the update, i.e. when the projection is applied).
template <int NL>
__global__ void __launch_bounds__(BLOCK) k_error(const DState s, const DevCache c, const FrameParams p) {
    __shared__ WarpTail<double, 3> taild;
    constexpr int LCS = lcs_of(NL);
    if (threadIdx.x == 0) taild.arrived = 0u;
    __syncthreads();
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    double d2 = 0.0, rs = 0.0, cn = 0.0;
    if (i < p.Np && s.valid[i]) {
        const float e = est_point<NL>(c.Lc + (size_t)LCS * i, p.dormant) - s.ref[i];
        d2 = double(e) * e;
        rs = s.ref[i];
        cn = 1.0;
    }
    const double vd[3] = {d2, rs, cn};
    double totd[3];
    if (warp_tail_reduce<double, 3>(vd, taild, c.partd, c.ticket + 1, totd)) {
        c.err[3 * p.err_frame] = totd[0];
        c.err[3 * p.err_frame + 1] = totd[1];
        c.err[3 * p.err_frame + 2] = totd[2];
    }
}

// ------------------------------------------------------------------ image pass
// One primary ray per pixel from a pinhole camera: closest hit with the frame's tracer, the
// hit's cache point, and the light leaving it toward the camera, A * sum over the lit lights
// of (direct + cached indirect) -- the quantity every cache ray gathers (poc_gpu.cu:471-478).
// Pixels whose ray hits nothing, a back face or an absent cell are 0.  16 x 16 pixel tiles.
template <int NL>
__global__ void __launch_bounds__(BLOCK) k_camera(const DState s, const DStatic g, const Grid grid, const DevCache c,
                                                  const FrameParams p, const CameraD cam, float* __restrict__ img) {
    extern __shared__ float4 sm[];
    constexpr int LCS = lcs_of(NL), AES = aes_of(NL);
    stage_smem(sm, s);
    __syncthreads();
    const TraceSmem tsm = smem_view(sm, s);
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= cam.w || y >= cam.h) return;
    const float sx = ((x + 0.5f) / cam.w * 2.f - 1.f) * cam.tx, sy = (1.f - (y + 0.5f) / cam.h * 2.f) * cam.ty;
    f3 D = mk(cam.fwd[0] + cam.right[0] * sx + cam.up[0] * sy, cam.fwd[1] + cam.right[1] * sx + cam.up[1] * sy,
              cam.fwd[2] + cam.right[2] * sx + cam.up[2] * sy);
    D = D * rsqrtf(dot(D, D));
    const f3 O = mk(cam.eye[0], cam.eye[1], cam.eye[2]);
    const Hit h = trace_resolve(tsm, s, g, grid, p, c, O, D, 0);
    float val = 0.f;
    if (h.q != -1 && !h.back) {
        float4 ae[AES / 4], lc[LCS / 4];
        const float4* aep = s.AE + (size_t)h.pi * (AES / 4);
        const float4* lcp = reinterpret_cast<const float4*>(c.Lc) + (size_t)h.pi * (LCS / 4);
#pragma unroll
        for (int k4 = 0; k4 < AES / 4; ++k4) ae[k4] = __ldg(aep + k4);
#pragma unroll
        for (int k4 = 0; k4 < LCS / 4; ++k4) lc[k4] = __ldcg(lcp + k4);
        const float A = ae[0].x;
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            const float lcv = ((p.dormant >> l) & 1) ? 0.f : comp(lc, l);
            val += A * (comp(ae, l + 1) + lcv);
        }
    }
    img[(size_t)y * cam.w + x] = val;
}

// ------------------------------------------------------------------ camera paths
// One path per pixel feeding the hash-grid cache (rc_hg_camera_paths, new: the reference has
// no camera).  Same trace, hit resolution and cosine sampling as the frames; RGB light.
__device__ __forceinline__ float lum(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

// a 64-byte vertex record as four 16-byte stores
__device__ __forceinline__ void store_vertex(rc_hg_vertex* dst, const rc_hg_vertex& v) {
    static_assert(sizeof(rc_hg_vertex) == 64, "vertex record: 64 bytes");
    const float4* src = reinterpret_cast<const float4*>(&v);
    float4* d = reinterpret_cast<float4*>(dst);
#pragma unroll
    for (int k = 0; k < 4; ++k) d[k] = src[k];
}

// closest hit distance along a shadow ray (no cache-point resolution)
__device__ __forceinline__ float shadow_t(const TraceSmem& sm, const DState& s, const DStatic& g, f3 O, f3 D, unsigned* flags) {
    float t;
    int q, jb;
    trace_dyn(sm, s, false, O, D, t, q, jb);
    if (g.has_bvh) trace_bvh(g, O, D, t, q, flags);
    return q == -1 ? INFINITY : t;
}

template <int NL>
__global__ void __launch_bounds__(BLOCK) k_paths(const DState s, const DStatic g, const Grid grid, const DevCache c, const FrameParams p,
                                                 const CameraD cam, const PathD pd, float* __restrict__ pos, float* __restrict__ nrm,
                                                 float* __restrict__ rgb, rc_hg_vertex* __restrict__ vtx, int* __restrict__ plen,
                                                 float* __restrict__ img) {
    extern __shared__ float4 sm[];
    stage_smem(sm, s);
    __syncthreads();
    const TraceSmem tsm = smem_view(sm, s);
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= cam.w || y >= cam.h) return;
    const size_t pix = (size_t)y * cam.w + x, base = pix * pd.slots;
    uint32_t rs = hash32(pd.seed * 0x9E3779B9u ^ hash32(pd.frame * 0x85EBCA6Bu ^ hash32((uint32_t)pix + 1u)));
    const float sx = ((x + 0.5f) / cam.w * 2.f - 1.f) * cam.tx, sy = (1.f - (y + 0.5f) / cam.h * 2.f) * cam.ty;
    f3 D = mk(cam.fwd[0] + cam.right[0] * sx + cam.up[0] * sy, cam.fwd[1] + cam.right[1] * sx + cam.up[1] * sy,
              cam.fwd[2] + cam.right[2] * sx + cam.up[2] * sy);
    D = D * rsqrtf(dot(D, D));
    f3 O = mk(cam.eye[0], cam.eye[1], cam.eye[2]);
    float A[RC_HG_MAX_DEPTH], E[RC_HG_MAX_DEPTH][3];
    int n = 0;
    bool escaped = false;
    for (int k = 0; k < pd.slots; ++k) {
        const Hit h = trace_resolve(tsm, s, g, grid, p, c, O, D, 0);
        rc_hg_vertex vx;
        vx.origin[0] = O.x; vx.origin[1] = O.y; vx.origin[2] = O.z;
        vx.dir[0] = D.x; vx.dir[1] = D.y; vx.dir[2] = D.z;
        vx.to_light[0] = vx.to_light[1] = vx.to_light[2] = 0.f;
        vx.light_dist = 0.f;
        vx.light_index = -1;
        vx.entry = RC_HG_INVALID;
        vx.flags = 0u;
        if (h.q == -1) {   // escaped: the sky
            vx.hit[0] = O.x; vx.hit[1] = O.y; vx.hit[2] = O.z;
            vx.flags = RC_HG_MISS;
            store_vertex(vtx + base + k, vx);
            escaped = true;
            n = k + 1;
            break;
        }
        if (h.back) break;   // back face or no cache point: the path ends
        const f3 H = h.H;
        f3 nn;
        if (h.q >= 0) {
            const float* Q = s.Q + 12 * h.q;
            nn = mk(__ldg(Q + 9), __ldg(Q + 10), __ldg(Q + 11));
        } else {
            const float4 n4 = __ldg(g.STN + (-2 - h.q));
            nn = mk(n4.x, n4.y, n4.z);
            if (dot(nn, D) > 0.f) nn = nn * -1.f;
        }
        const float alb = __ldg(g.A + h.pi);
        const f3 Os = H + nn * 1e-3f;
        // light choice proportional to the unshadowed contribution (never zero for the rectangle)
        float W = 0.f;
        for (int l = 0; l < pd.nl; ++l) {
            const f3 d = mk(pd.lpos[l][0], pd.lpos[l][1], pd.lpos[l][2]) - H;
            const float r = sqrtf(dot(d, d)), rr = fmaxf(r, 0.05f);
            W += pd.lint[l] * lum(pd.lrgb[l][0], pd.lrgb[l][1], pd.lrgb[l][2]) * fmaxf(dot(nn, d) / r, 0.f) / (rr * rr);
        }
        float wa = 0.f, ws = 0.f;
        if (pd.area_on) {
            const f3 C = mk(pd.ac[0] + 0.5f * (pd.au[0] + pd.av[0]), pd.ac[1] + 0.5f * (pd.au[1] + pd.av[1]),
                            pd.ac[2] + 0.5f * (pd.au[2] + pd.av[2]));
            const f3 d = C - H;
            const float r = sqrtf(dot(d, d)), rr = fmaxf(r, 0.05f);
            const f3 w = d * (1.f / r);
            wa = lum(pd.argb[0], pd.argb[1], pd.argb[2]) * pd.aarea * fmaxf(dot(nn, w), 0.1f) *
                 fmaxf(-(pd.an[0] * w.x + pd.an[1] * w.y + pd.an[2] * w.z), 0.1f) / (rr * rr);
        }
        if (pd.sun_on) ws = lum(pd.srgb[0], pd.srgb[1], pd.srgb[2]) * fmaxf(nn.x * pd.sdir[0] + nn.y * pd.sdir[1] + nn.z * pd.sdir[2], 0.f);
        const float Wt = W + wa + ws;
        float e3[3] = {0.f, 0.f, 0.f};
        if (Wt > 0.f) {
            // the sampled light: direction, distance, unshadowed contribution over its probability
            f3 w = mk(0.f, 0.f, 1.f);
            float r = 0.f, c3[3] = {0.f, 0.f, 0.f};
            bool open = true, sun = false;
            int li = -1;
            const float u = rnd(rs) * Wt;
            if (u < W) {   // a point light
                int l = 0;
                float acc = 0.f, wl = 0.f;
                f3 d = mk(0.f, 0.f, 0.f);
                for (l = 0; l < pd.nl; ++l) {
                    d = mk(pd.lpos[l][0], pd.lpos[l][1], pd.lpos[l][2]) - H;
                    r = sqrtf(dot(d, d));
                    const float rr = fmaxf(r, 0.05f);
                    const float cs = fmaxf(dot(nn, d) / r, 0.f);
                    wl = pd.lint[l] * lum(pd.lrgb[l][0], pd.lrgb[l][1], pd.lrgb[l][2]) * cs / (rr * rr);
                    acc += wl;
                    if (u < acc && wl > 0.f) break;
                }
                l = min(l, pd.nl - 1);
                w = d * (1.f / r);
                li = l;
                open = wl > 0.f;
                const float ln = lum(pd.lrgb[l][0], pd.lrgb[l][1], pd.lrgb[l][2]);
                for (int ch = 0; ch < 3; ++ch) c3[ch] = Wt * pd.lrgb[l][ch] / ln;
            } else if (u < W + wa) {   // a point of the rectangle
                const float u1 = rnd(rs);
                const float u2 = rnd(rs);
                const f3 Y = mk(pd.ac[0] + u1 * pd.au[0] + u2 * pd.av[0], pd.ac[1] + u1 * pd.au[1] + u2 * pd.av[1],
                                pd.ac[2] + u1 * pd.au[2] + u2 * pd.av[2]);
                const f3 d = Y - H;
                r = sqrtf(dot(d, d));
                const float rr = fmaxf(r, 0.05f);
                w = d * (1.f / r);
                const float cs = fmaxf(dot(nn, w), 0.f), ca = fmaxf(-(pd.an[0] * w.x + pd.an[1] * w.y + pd.an[2] * w.z), 0.f);
                open = cs > 0.f && ca > 0.f;
                li = pd.nl;
                const float geo = pd.aarea * cs * ca / (rr * rr) * (Wt / wa);
                for (int ch = 0; ch < 3; ++ch) c3[ch] = pd.argb[ch] * geo;
            } else {   // the sun
                w = mk(pd.sdir[0], pd.sdir[1], pd.sdir[2]);
                r = pd.td;
                sun = true;
                li = pd.nl + 1;
                const float ln = lum(pd.srgb[0], pd.srgb[1], pd.srgb[2]);
                for (int ch = 0; ch < 3; ++ch) c3[ch] = Wt * pd.srgb[ch] / ln;
            }
            // one shadow ray for whichever light was chosen
            const float ts = open ? shadow_t(tsm, s, g, Os, w, c.flags) : 0.f;
            const bool vis = open && (sun ? ts == INFINITY : ts >= r - 1e-3f);
            vx.to_light[0] = w.x; vx.to_light[1] = w.y; vx.to_light[2] = w.z;
            vx.light_dist = r;
            vx.light_index = li;
            if (vis) {
                vx.flags |= RC_HG_LIGHT_VISIBLE;
                for (int ch = 0; ch < 3; ++ch) e3[ch] = c3[ch];
            }
        }
        vx.hit[0] = H.x; vx.hit[1] = H.y; vx.hit[2] = H.z;
        store_vertex(vtx + base + k, vx);
        pos[3 * (base + k)] = H.x; pos[3 * (base + k) + 1] = H.y; pos[3 * (base + k) + 2] = H.z;
        nrm[3 * (base + k)] = nn.x; nrm[3 * (base + k) + 1] = nn.y; nrm[3 * (base + k) + 2] = nn.z;
        A[k] = alb;
        E[k][0] = e3[0]; E[k][1] = e3[1]; E[k][2] = e3[2];
        n = k + 1;
        const float u1 = rnd(rs);
        const float u2 = rnd(rs);
        O = Os;
        D = cosine_dir(nn, u1, u2);
    }
    // radiance leaving each vertex toward the previous one, from the last surface vertex back;
    // slots without a surface vertex (the escaping ray, unused slots) get a zero normal: no entry
    const int nsurf = n - (escaped ? 1 : 0);
    for (int k = nsurf; k < pd.slots; ++k) {
        for (int ch = 0; ch < 3; ++ch) {
            rgb[3 * (base + k) + ch] = 0.f;
            nrm[3 * (base + k) + ch] = 0.f;
            pos[3 * (base + k) + ch] = 0.f;
        }
    }
    float L[3] = {0.f, 0.f, 0.f};
    if (escaped) { L[0] = pd.sky[0]; L[1] = pd.sky[1]; L[2] = pd.sky[2]; }
    for (int k = nsurf - 1; k >= 0; --k)
        for (int ch = 0; ch < 3; ++ch) {
            L[ch] = A[k] * (E[k][ch] + L[ch]);
            rgb[3 * (base + k) + ch] = L[ch];
        }
    plen[pix] = n;
    if (img)   // the pixel: the primary vertex's radiance (L after the loop), the sky, or black
        for (int ch = 0; ch < 3; ++ch) img[3 * pix + ch] = nsurf > 0 || escaped ? L[ch] : 0.f;
}

// ------------------------------------------------------------------ probe
struct RayRecD { int point, ray, q, pi, back; float t; float dir[3], hit[3]; };

template <int NL, int NW>
__global__ void __launch_bounds__(BLOCK) k_probe(const DState s, const DStatic g, const Grid grid, const DevCache c,
                                                 const FrameParams p, const int* __restrict__ pts, int npts,
                                                 RayRecD* __restrict__ out, int maxrec, int* __restrict__ nrec) {
    extern __shared__ float4 sm[];
    stage_smem(sm, s);
    __syncthreads();
    const TraceSmem tsm = smem_view(sm, s);
    const int t = blockIdx.x * BLOCK + threadIdx.x;
    if (t >= npts) return;
    const int i = pts[t];
    if (i < 0 || i >= p.Np) return;
    uint32_t rs = hash32(p.seed * 0x9E3779B9u ^ hash32(p.frame * 0x85EBCA6Bu ^ hash32(i + 1)));
    const bool pend = p.pend_left > 0 && c.pending[i];
    const int k = ray_count(p, c, c.n[i], pend, c.sumpr[p.sum_in], c.npend[0], rs);
    const f3 P = xyz(s.P4[i]), N = xyz(s.N4[i]), O = P + N * 1e-3f;
    for (int r = 0; r < k; ++r) {
        const float u1 = rnd(rs);
        const float u2 = rnd(rs);
        const f3 D = cosine_dir(N, u1, u2);
        const Hit h = trace_resolve(tsm, s, g, grid, p, c, O, D, i);
        const int slot = atomicAdd(nrec, 1);
        if (slot < maxrec) {
            RayRecD x;
            x.point = i; x.ray = r; x.q = h.q; x.pi = h.pi; x.back = h.back ? 1 : 0;
            x.t = h.q != -1 ? h.t : __int_as_float(0x7f800000);
            x.dir[0] = D.x; x.dir[1] = D.y; x.dir[2] = D.z;
            x.hit[0] = h.H.x; x.hit[1] = h.H.y; x.hit[2] = h.H.z;
            out[slot] = x;
        }
    }
}

// ------------------------------------------------------------------ converged references
// One stochastic Jacobi iteration of the reference's scene preparation (prep_mesh.cuh:182-213):
// each point averages K rays of albedo x (direct light + the previous iterate) at its hit
// points; the iterate of every light goes to Lout, and is added to acc from the warm-up on.
// close counts the rays that hit within 0.02 (points mostly hemmed in are not valid for the
// error metric).  Buffers are padded like the cache (LCS floats per point).
template <int NL>
__global__ void __launch_bounds__(BLOCK) k_ref(const DState s, const DStatic g, const Grid grid, const DevCache c, const FrameParams p,
                                               const float* __restrict__ Lin, float* __restrict__ Lout, float* __restrict__ acc,
                                               float* __restrict__ closec, uint32_t seed, int K, int accumulate, int count_close) {
    extern __shared__ float4 sm[];
    constexpr int LCS = lcs_of(NL), AES = aes_of(NL);
    stage_smem(sm, s);
    __syncthreads();
    const TraceSmem tsm = smem_view(sm, s);
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    if (i >= p.Np) return;
    uint32_t rs = hash32(seed ^ hash32(i + 1));
    const f3 P = xyz(s.P4[i]), N = xyz(s.N4[i]), O = P + N * 1e-3f;
    float sum[NL];
#pragma unroll
    for (int l = 0; l < NL; ++l) sum[l] = 0.f;
    int close = 0;
    for (int r = 0; r < K; ++r) {
        const float u1 = rnd(rs);
        const float u2 = rnd(rs);
        const f3 D = cosine_dir(N, u1, u2);
        const Hit h = trace_resolve(tsm, s, g, grid, p, c, O, D, i);
        if (h.q != -1 && h.t < 0.02f) close++;
        if (h.back) continue;
        float4 ae[AES / 4], lc[LCS / 4];
        const float4* aep = s.AE + (size_t)h.pi * (AES / 4);
        const float4* lcp = reinterpret_cast<const float4*>(Lin) + (size_t)h.pi * (LCS / 4);
#pragma unroll
        for (int k4 = 0; k4 < AES / 4; ++k4) ae[k4] = __ldg(aep + k4);
#pragma unroll
        for (int k4 = 0; k4 < LCS / 4; ++k4) lc[k4] = __ldcg(lcp + k4);
        const float A = ae[0].x;
#pragma unroll
        for (int l = 0; l < NL; ++l) sum[l] += A * (comp(ae, l + 1) + comp(lc, l));
    }
#pragma unroll
    for (int l = 0; l < NL; ++l) {
        const float v = sum[l] / K;
        Lout[(size_t)LCS * i + l] = v;
        if (accumulate) acc[(size_t)LCS * i + l] += v;
    }
    if (count_close) closec[i] += (float)close;
}

// One sample per point of the reference's taa mode (k_taa_pt, poc_gpu.cu:1062-1098): one cosine
// ray; the radiance at its hit point = A x (direct light summed over lights + the converged
// reference), 0 when the ray does not count; with DEPS the ray's dependency mask (the hit's
// shadow voxels and the ray's own transit voxels) is or-ed into cur.
template <int NL, int NW, bool DEPS>
__global__ void __launch_bounds__(BLOCK) k_taa_pt(const DState s, const DStatic g, const Grid grid, const DevCache c, const FrameParams p,
                                                  float* __restrict__ x, uint32_t* __restrict__ cur, uint32_t seed, uint32_t frame) {
    extern __shared__ float4 sm[];
    stage_smem(sm, s);
    __syncthreads();
    const TraceSmem tsm = smem_view(sm, s);
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    if (i >= p.Np) return;
    constexpr int AES = aes_of(NL);
    uint32_t rs = hash32(seed * 0x9E3779B9u ^ hash32(frame * 0x85EBCA6Bu ^ hash32(i + 7)));
    const f3 P = xyz(s.P4[i]), N = xyz(s.N4[i]), O = P + N * 1e-3f;
    const float u1 = rnd(rs);
    const float u2 = rnd(rs);
    const f3 D = cosine_dir(N, u1, u2);
    const Hit h = trace_resolve(tsm, s, g, grid, p, c, O, D, i);
    float v = 0.f;
    if (!h.back) {
        float4 ae[AES / 4];
        const float4* aep = s.AE + (size_t)h.pi * (AES / 4);
#pragma unroll
        for (int k4 = 0; k4 < AES / 4; ++k4) ae[k4] = __ldg(aep + k4);
        float ed = 0.f;
#pragma unroll
        for (int l = 0; l < NL; ++l) ed += comp(ae, l + 1);
        v = ae[0].x * (ed + s.ref[h.pi]);
    }
    x[i] = v;
    if (DEPS) {
        uint32_t m[NW];
#pragma unroll
        for (int w = 0; w < NW; ++w) m[w] = 0u;
        const uint4* sv = reinterpret_cast<const uint4*>(s.SV + (size_t)NW * (h.back ? i : h.pi));
#pragma unroll
        for (int w = 0; w < NW / 4; ++w) {
            const uint4 a = __ldg(sv + w);
            m[4 * w] |= a.x; m[4 * w + 1] |= a.y; m[4 * w + 2] |= a.z; m[4 * w + 3] |= a.w;
        }
        dda_walk<NW>(grid, O, h.H, m);
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            const uint32_t o = cur[(size_t)w * p.Np + i];
            if ((o | m[w]) != o) cur[(size_t)w * p.Np + i] = o | m[w];
        }
    }
}

// The rays of one k_ref iteration with this seed (prep_mesh.cuh:182-200: same seed, directions
// and hit resolution), kept: hits[i * K + r] = the cache point ray r of point i reaches, or -1
// when the ray does not count (no hit, back face, cell absent).  The frozen ray set defines a
// fixed linear transport for the adjoint.
template <int NL>
__global__ void __launch_bounds__(BLOCK) k_frozen(const DState s, const DStatic g, const Grid grid, const DevCache c, const FrameParams p,
                                                  uint32_t seed, int K, int* __restrict__ hits) {
    extern __shared__ float4 sm[];
    stage_smem(sm, s);
    __syncthreads();
    const TraceSmem tsm = smem_view(sm, s);
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    if (i >= p.Np) return;
    uint32_t rs = hash32(seed ^ hash32(i + 1));
    const f3 P = xyz(s.P4[i]), N = xyz(s.N4[i]), O = P + N * 1e-3f;
    for (int r = 0; r < K; ++r) {
        const float u1 = rnd(rs);
        const float u2 = rnd(rs);
        const f3 D = cosine_dir(N, u1, u2);
        const Hit h = trace_resolve(tsm, s, g, grid, p, c, O, D, i);
        hits[(size_t)i * K + r] = h.back ? -1 : h.pi;
    }
}

// ------------------------------------------------------------------ launch wrappers

static int grid_of(int Np) { return (Np + BLOCK - 1) / BLOCK; }

template <typename K>
static cudaError_t prep_smem(K kern, size_t smem) {
    if (smem > 48 * 1024) return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return cudaSuccess;
}

static cudaError_t resident_grid(const void* kern, size_t smem, int& out, int threads);

template <int NL>
cudaError_t Ops<NL>::pretrace(const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                              float4* out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(c.rayctr, 0, 2 * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if (!p.wavefront || !c.rayq) {   // one thread per point, persistent warps
        const size_t smem = frame_smem_bytes(s);
        if ((e = prep_smem(k_pretrace<NL>, smem)) != cudaSuccess) return e;
        int resident = 0;
        if ((e = resident_grid((const void*)k_pretrace<NL>, smem, resident, BLOCK)) != cudaSuccess) return e;
        k_pretrace<NL><<<std::max(1, std::min(resident, grid_of(p.Np))), BLOCK, smem, st>>>(s, g, grid, c, p, out);
        return cudaGetLastError();
    }
    // ray queue: compacted rays, then the persistent traversal
    k_ray_queue<NL><<<grid_of(p.Np), BLOCK, 0, st>>>(s, c, p);
    const size_t smem = trace_queue_smem(s);
    auto kern = g.watertight ? k_trace_queue<true> : k_trace_queue<false>;
    if ((e = prep_smem(kern, smem)) != cudaSuccess) return e;
    // persistent: as many blocks as are resident
    int resident = 0;
    if ((e = resident_grid((const void*)kern, smem, resident, WQ_BLOCK)) != cudaSuccess) return e;
    const int maxrays = p.Np * p.pre_k;
    const int blocks = std::max(1, std::min(resident, (maxrays + WQ_BLOCK - 1) / WQ_BLOCK));
    kern<<<blocks, WQ_BLOCK, smem, st>>>(s, g, grid, c, p, out);
    return cudaGetLastError();
}

template <int NL>
cudaError_t Ops<NL>::frozen_hits(const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                                 uint32_t seed, int K, int* hits, cudaStream_t st) {
    const size_t smem = frame_smem_bytes(s);
    cudaError_t e = prep_smem(k_frozen<NL>, smem);
    if (e != cudaSuccess) return e;
    k_frozen<NL><<<grid_of(p.Np), BLOCK, smem, st>>>(s, g, grid, c, p, seed, K, hits);
    return cudaGetLastError();
}

template <int NL>
cudaError_t Ops<NL>::ref_iter(const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                              const float* Lin, float* Lout, float* acc, float* closec, uint32_t seed, int K, int accumulate,
                              int count_close, cudaStream_t st) {
    const size_t smem = frame_smem_bytes(s);
    cudaError_t e = prep_smem(k_ref<NL>, smem);
    if (e != cudaSuccess) return e;
    k_ref<NL><<<grid_of(p.Np), BLOCK, smem, st>>>(s, g, grid, c, p, Lin, Lout, acc, closec, seed, K, accumulate, count_close);
    return cudaGetLastError();
}

// Mask widths built for every light count (NW = voxels / 32 of the transit grid).
#define RC_NW_LIST(X) X(4) X(24)

template <int NL>
cudaError_t Ops<NL>::taa_sample(int NW, bool deps, const DState& s, const DStatic& g, const Grid& grid, const DevCache& c,
                                const FrameParams& p, float* x, uint32_t* cur, uint32_t seed, uint32_t frame, cudaStream_t st) {
    const size_t smem = frame_smem_bytes(s);
#define X(W)                                                                                                   \
    if (NW == W) {                                                                                             \
        auto kern = deps ? k_taa_pt<NL, W, true> : k_taa_pt<NL, W, false>;                                     \
        cudaError_t e = prep_smem(kern, smem);                                                                 \
        if (e != cudaSuccess) return e;                                                                        \
        kern<<<grid_of(p.Np), BLOCK, smem, st>>>(s, g, grid, c, p, x, cur, seed, frame);                       \
        return cudaGetLastError();                                                                             \
    }
    RC_NW_LIST(X)
#undef X
    return cudaErrorInvalidValue;
}


template <int NL>
cudaError_t Ops<NL>::build(int NW, const DState& s, const DStatic& g, const Grid& grid, const float* L, const float* inten,
                           float4* AE, uint32_t* SV, int Np, unsigned* flags, cudaStream_t st) {
    const size_t smem = frame_smem_bytes(s);
#define X(W)                                                                                     \
    if (NW == W) {                                                                               \
        cudaError_t e = prep_smem(k_build<NL, W>, smem);                                         \
        if (e != cudaSuccess) return e;                                                          \
        k_build<NL, W><<<grid_of(Np), BLOCK, smem, st>>>(s, g, grid, L, inten, AE, SV, Np, flags); \
        return cudaGetLastError();                                                               \
    }
    RC_NW_LIST(X)
#undef X
    return cudaErrorInvalidValue;
}

// Blocks of `kern` (BLOCK threads, `smem` dynamic shared bytes) resident on the whole current
// device at once, looked up once per device, kernel and shared-memory size.
static cudaError_t resident_grid(const void* kern, size_t smem, int& out, int threads) {
    struct Entry { int dev; const void* kern; size_t smem; int threads; int blocks; };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    for (const Entry& x : cache)
        if (x.dev == dev && x.kern == kern && x.smem == smem && x.threads == threads) { out = x.blocks; return cudaSuccess; }
    int per_sm = 0, sms = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    cache.push_back({dev, kern, smem, threads, per_sm * sms});
    out = per_sm * sms;
    return cudaSuccess;
}

template <int NL, int NW, bool DEPS, bool FUSED>
static cudaError_t frame_t(const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                           cudaStream_t st) {
    const size_t smem = frame_smem_bytes(s);
    cudaError_t e = prep_smem(k_frame<NL, NW, DEPS, FUSED>, smem);
    if (e != cudaSuccess) return e;
    int resident = 0;
    if ((e = resident_grid((const void*)k_frame<NL, NW, DEPS, FUSED>, smem, resident, BLOCK)) != cudaSuccess) return e;
    const int blocks = std::min(grid_of(p.Np), resident);
    k_frame<NL, NW, DEPS, FUSED><<<blocks, BLOCK, smem, st>>>(s, g, grid, c, p);
    return cudaGetLastError();
}

template <int NL>
cudaError_t Ops<NL>::frame(int NW, bool deps, bool fused, const DState& s, const DStatic& g, const Grid& grid,
                           const DevCache& c, const FrameParams& p, cudaStream_t st) {
#define X(W)                                                                        \
    if (NW == W) {                                                                  \
        if (deps) return fused ? frame_t<NL, W, true, true>(s, g, grid, c, p, st)   \
                               : frame_t<NL, W, true, false>(s, g, grid, c, p, st); \
        return fused ? frame_t<NL, W, false, true>(s, g, grid, c, p, st)            \
                     : frame_t<NL, W, false, false>(s, g, grid, c, p, st);          \
    }
    RC_NW_LIST(X)
#undef X
    return cudaErrorInvalidValue;
}

template <int NL>
cudaError_t Ops<NL>::update(const DState& s, const DStatic& g, const DevCache& c, const FrameParams& p, cudaStream_t st) {
    k_update<NL><<<grid_of(p.Np), BLOCK, 0, st>>>(s, g, c, p);
    return cudaGetLastError();
}

template <int NL>
cudaError_t Ops<NL>::event(const EvProgram& ev, const DevCache& c, cudaStream_t st) {
    k_event<NL><<<grid_of(ev.Np), BLOCK, 0, st>>>(ev, c);
    return cudaGetLastError();
}

template <int NL>
cudaError_t Ops<NL>::error(const DState& s, const DevCache& c, const FrameParams& p, cudaStream_t st) {
    k_error<NL><<<grid_of(p.Np), BLOCK, 0, st>>>(s, c, p);
    return cudaGetLastError();
}

template <int NL>
cudaError_t Ops<NL>::proj_apply(const DevCache& c, const DStatic& g, const FrameParams& p, cudaStream_t st) {
    k_proj_apply<NL><<<grid_of(p.Np), BLOCK, 0, st>>>(c, g, p);
    return cudaGetLastError();
}

template <int NL>
cudaError_t Ops<NL>::camera(const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                            const CameraD& cam, float* img, cudaStream_t st) {
    const size_t smem = frame_smem_bytes(s);
    cudaError_t e = prep_smem(k_camera<NL>, smem);
    if (e != cudaSuccess) return e;
    dim3 grd((cam.w + 15) / 16, (cam.h + 15) / 16);
    k_camera<NL><<<grd, BLOCK, smem, st>>>(s, g, grid, c, p, cam, img);
    return cudaGetLastError();
}

template <int NL>
cudaError_t Ops<NL>::paths(const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p, const CameraD& cam,
                           const PathD& pd, float* pos, float* nrm, float* rgb, void* vtx, int* len, float* img, cudaStream_t st) {
    const size_t smem = frame_smem_bytes(s);
    cudaError_t e = prep_smem(k_paths<NL>, smem);
    if (e != cudaSuccess) return e;
    dim3 grd((cam.w + 15) / 16, (cam.h + 15) / 16);
    k_paths<NL><<<grd, BLOCK, smem, st>>>(s, g, grid, c, p, cam, pd, pos, nrm, rgb, (rc_hg_vertex*)vtx, len, img);
    return cudaGetLastError();
}

template <int NL>
cudaError_t Ops<NL>::probe(int NW, const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                           const int* pts, int npts, void* recs, int maxrec, int* nrec, cudaStream_t st) {
    const size_t smem = frame_smem_bytes(s);
#define X(W)                                                                                                   \
    if (NW == W) {                                                                                             \
        cudaError_t e = prep_smem(k_probe<NL, W>, smem);                                                       \
        if (e != cudaSuccess) return e;                                                                        \
        k_probe<NL, W><<<grid_of(npts), BLOCK, smem, st>>>(s, g, grid, c, p, pts, npts, (RayRecD*)recs, maxrec, nrec); \
        return cudaGetLastError();                                                                             \
    }
    RC_NW_LIST(X)
#undef X
    return cudaErrorInvalidValue;
}

template <int NL>
cudaError_t Ops<NL>::preload(int NW) {
    cudaFuncAttributes a;
    cudaError_t e = cudaSuccess;
    auto touch = [&](const void* f) { if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, f); };
#define X(W)                                                 \
    if (NW == W) {                                           \
        touch((const void*)k_frame<NL, W, true, true>);      \
        touch((const void*)k_frame<NL, W, true, false>);     \
        touch((const void*)k_frame<NL, W, false, true>);     \
        touch((const void*)k_frame<NL, W, false, false>);    \
        touch((const void*)k_build<NL, W>);                  \
        touch((const void*)k_probe<NL, W>);                  \
    }
    RC_NW_LIST(X)
#undef X
    touch((const void*)k_update<NL>);
    touch((const void*)k_event<NL>);
    touch((const void*)k_pretrace<NL>);
    touch((const void*)k_ray_queue<NL>);
    touch((const void*)k_trace_queue<false>);
    touch((const void*)k_trace_queue<true>);
    touch((const void*)k_ref<NL>);
    touch((const void*)k_error<NL>);
    touch((const void*)k_proj_apply<NL>);
    touch((const void*)k_camera<NL>);
    return e;
}

#ifdef RC_NL_ONE
template struct Ops<RC_NL_ONE>;
#endif

#if RC_NL_ONE == 3   // compiled once: the preparation's probe, caller-given rays
// k_probe of the reference's preparation (prep_mesh.cuh:160-178): from each candidate point, 64
// Fibonacci directions through the static mesh; out = (closest hit, fraction of hits closer than
// diag, fraction of single-sided back faces hit).
// Free-space probe of the scene preparation: 48 directions of a spherical Fibonacci lattice
// from each candidate point through the static mesh.  out = (clearance: the nearest hit, 1e30
// when every ray escapes; the fraction of rays that hit; the fraction that meet a one-sided
// face from behind, i.e. the candidate is inside closed geometry).
__global__ void __launch_bounds__(BLOCK) k_prep_probe(const DStatic g, const float* __restrict__ C, int nc, float* __restrict__ out,
                                                      unsigned* flags) {
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    if (i >= nc) return;
    const f3 o = mk(C[3 * i], C[3 * i + 1], C[3 * i + 2]);
    constexpr int ND = 48;
    float clr = 1e30f;
    int hits = 0, behind = 0;
    for (int k = 0; k < ND; ++k) {
        const float z = 1.f - (2.f * k + 1.f) * (1.f / ND);
        const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
        float sp, cp;
        sincosf(2.39996323f * (float)k, &sp, &cp);   // golden angle
        const f3 d = mk(r * cp, r * sp, z);
        float t = 1e30f;
        int q = -1;
        trace_bvh(g, o, d, t, q, flags);
        if (q == -1) continue;
        ++hits;
        clr = fminf(clr, t);
        const float4 n4 = __ldg(g.STN + (-2 - q));
        if (n4.x * d.x + n4.y * d.y + n4.z * d.z > 0.f && !(__float_as_int(n4.w) & 1)) ++behind;
    }
    out[3 * i] = clr;
    out[3 * i + 1] = (float)hits / ND;
    out[3 * i + 2] = (float)behind / ND;
}

cudaError_t prep_probe(const DStatic& g, const float* C, int nc, float diag, float* out, unsigned* flags, cudaStream_t st) {
    (void)diag;
    k_prep_probe<<<(nc + BLOCK - 1) / BLOCK, BLOCK, 0, st>>>(g, C, nc, out, flags);
    return cudaGetLastError();
}

// Closest hit of caller-given rays against one state's geometry: the dynamic triangles, then
// the static mesh (trace_full, poc_gpu.cu:340-344).  rays = (origin, direction) per ray.
__global__ void __launch_bounds__(BLOCK) k_trace_rays(const DState s, const DStatic g, int brute, const float* __restrict__ rays,
                                                      int n, int* __restrict__ prim, float* __restrict__ tout, unsigned* flags) {
    extern __shared__ float4 sm[];
    stage_smem(sm, s);
    __syncthreads();
    const TraceSmem tsm = smem_view(sm, s);
    const int i = blockIdx.x * BLOCK + threadIdx.x;
    if (i >= n) return;
    const float* r = rays + 6 * (size_t)i;
    const f3 o = mk(r[0], r[1], r[2]), d = mk(r[3], r[4], r[5]);
    float t;
    int q, jb;
    trace_dyn(tsm, s, brute != 0, o, d, t, q, jb);
    if (g.has_bvh) trace_bvh(g, o, d, t, q, flags);
    prim[i] = q;
    tout[i] = q != -1 ? t : __int_as_float(0x7f800000);
}

cudaError_t trace_rays(const DState& s, const DStatic& g, int brute, const float* rays, int n, int* prim, float* t,
                       unsigned* flags, cudaStream_t st) {
    const size_t smem = frame_smem_bytes(s);
    cudaError_t e = prep_smem(k_trace_rays, smem);
    if (e != cudaSuccess) return e;
    k_trace_rays<<<(n + BLOCK - 1) / BLOCK, BLOCK, smem, st>>>(s, g, brute, rays, n, prim, t, flags);
    return cudaGetLastError();
}
#endif

}  // namespace rc
