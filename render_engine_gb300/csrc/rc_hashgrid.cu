// Hash-grid radiance cache with per-entry dependency masks (include/rc_hashgrid.h).
//
// The dependency part follows falcon123212/render_engine's windows/patch/rtxgi_bench.patch
// (bench A's HLSL): zone marking of points and segments, the per-path propagation of masks
// into the cache entries of the path, two banks rotated by the host, invalidation of the
// entries an event touches at resolve time, and compact snapshots.  Float expressions are
// evaluated in the order the HLSL writes them with explicitly rounded operations (no fused
// multiply-add), so the CPU oracle reproduces every mask bit.
//
// The cache itself (insert / accumulate / resolve / evict) is this library's: the patch calls
// the SHaRC SDK for it, which is not part of the reference.  All per-entry arrays are
// structure-of-arrays, 16-byte records per entry, so every kernel reads and writes whole
// 128-bit words; the resolve is one pass over the table (HBM-bound integer work) and writes a
// word only when it changes.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/rc_hashgrid.h"

struct rc_hg {
    rc_hg_config cfg{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    unsigned long long* keys = nullptr;
    uint4* accum = nullptr;
    uint4* resolved = nullptr;
    uint4* bank[2] = {nullptr, nullptr};
    int bank_sel = 0;
    uint32_t* scratch = nullptr;   // counters (4) + per-block snapshot counts
    size_t scratch_words = 0;
    unsigned long long* vox = nullptr;   // per-voxel light masks, vres^3 (rc_hg_voxels_init)
    unsigned long long* vox_out = nullptr;
    int vres = 0;
    std::string err;
};

namespace {

constexpr int ZX = RC_HG_ZONES_X, ZY = RC_HG_ZONES_Y, ZZ = RC_HG_ZONES_Z;
constexpr int HG_BLOCK = 256;
constexpr int SNAP_BLOCK = 1024;   // entries per block of the snapshot compaction
constexpr unsigned long long TOMB = ~0ull;   // evicted entry: probing goes on past it

struct HgDev {
    float zlo[3], zhi[3], org[3];
    float ih;            // 1 / cell (host quotient)
    uint32_t mask;       // capacity - 1
    uint32_t cap;
    int depth;
    int acc_frames, stale_frames;
    float td;
};

rc_status fail(rc_hg* hg, rc_status s, const char* fmt, ...) {
    char buf[512];
    va_list a;
    va_start(a, fmt);
    vsnprintf(buf, sizeof buf, fmt, a);
    va_end(a);
    if (hg) hg->err = buf;
    return s;
}
#define HGCK(x)                                                                                                 \
    do {                                                                                                        \
        cudaError_t e_ = (x);                                                                                   \
        if (e_ != cudaSuccess) return fail(hg, RC_ERR_CUDA, "CUDA %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

HgDev dev_of(const rc_hg* hg) {
    HgDev d;
    for (int k = 0; k < 3; ++k) {
        d.zlo[k] = hg->cfg.zone_lo[k];
        d.zhi[k] = hg->cfg.zone_hi[k];
        d.org[k] = hg->cfg.origin[k];
    }
    d.ih = 1.f / hg->cfg.cell;
    d.cap = hg->cfg.capacity;
    d.mask = hg->cfg.capacity - 1u;
    d.depth = std::min(std::max(hg->cfg.max_depth, 1), RC_HG_MAX_DEPTH);
    d.acc_frames = hg->cfg.acc_frames;
    d.stale_frames = hg->cfg.stale_frames;
    d.td = hg->cfg.tracing_distance;
    return d;
}

int grid_for(size_t n, int block) { return (int)std::min<size_t>((n + block - 1) / block, 1u << 20); }

// ------------------------------------------------------------------ dependency zones
__device__ __forceinline__ float mn(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float mx(float a, float b) { return a > b ? a : b; }

// rtxgi_bench.patch:825-837 DepMarkPoint
__device__ __forceinline__ void mark_point(const HgDev& c, uint32_t (&m)[3], float px, float py, float pz) {
    const float p[3] = {px, py, pz};
    const float G[3] = {(float)ZX, (float)ZY, (float)ZZ};
    float cc[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) cc[k] = __fmul_rn(__fdiv_rn(__fsub_rn(p[k], c.zlo[k]), __fsub_rn(c.zhi[k], c.zlo[k])), G[k]);
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (cc[k] < 0.0f || cc[k] >= G[k]) return;
    const uint32_t b = (uint32_t)cc[0] + ZX * ((uint32_t)cc[1] + ZY * (uint32_t)cc[2]);
    const uint32_t bit = 1u << (b & 31u);
    if (b < 32u) m[0] |= bit;
    else if (b < 64u) m[1] |= bit;
    else m[2] |= bit;
}

// rtxgi_bench.patch:839-858 DepMarkSegment: the segment clipped to the zone box, sampled every
// half of the smallest zone edge (at most 49 points); lerp(a, b, s) = a + s (b - a).
__device__ void mark_segment(const HgDev& c, uint32_t (&m)[3], const float (&a)[3], const float (&b)[3]) {
    float d[3], tn[3], tf[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        d[k] = __fsub_rn(b[k], a[k]);
        const float sd = fabsf(d[k]) > 1e-7f ? d[k] : 1e-7f;
        const float t0 = __fdiv_rn(__fsub_rn(c.zlo[k], a[k]), sd);
        const float t1 = __fdiv_rn(__fsub_rn(c.zhi[k], a[k]), sd);
        tn[k] = mn(t0, t1);
        tf[k] = mx(t0, t1);
    }
    const float tmin = mx(mx(tn[0], tn[1]), mx(tn[2], 0.0f));
    const float tmax = mn(mn(tf[0], tf[1]), mn(tf[2], 1.0f));
    if (tmin > tmax) return;
    const float c0 = __fdiv_rn(__fsub_rn(c.zhi[0], c.zlo[0]), (float)ZX);
    const float c1 = __fdiv_rn(__fsub_rn(c.zhi[1], c.zlo[1]), (float)ZY);
    const float c2 = __fdiv_rn(__fsub_rn(c.zhi[2], c.zlo[2]), (float)ZZ);
    const float dd = __fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1]));
    const float len = __fmul_rn(__fsqrt_rn(__fadd_rn(dd, __fmul_rn(d[2], d[2]))), __fsub_rn(tmax, tmin));
    const float q = ceilf(__fdiv_rn(len, __fmul_rn(0.5f, mn(c0, mn(c1, c2)))));
    const uint32_t n = q >= 47.0f ? 48u : (uint32_t)q + 1u;
    const float span = __fsub_rn(tmax, tmin);
    for (uint32_t i = 0; i <= n; ++i) {
        const float s = __fdiv_rn((float)i, (float)n);
        const float t = __fadd_rn(tmin, __fmul_rn(s, span));
        mark_point(c, m, __fadd_rn(a[0], __fmul_rn(d[0], t)), __fadd_rn(a[1], __fmul_rn(d[1], t)),
                   __fadd_rn(a[2], __fmul_rn(d[2], t)));
    }
}

// rtxgi_bench.patch:860-880 DepOr: OR into the bank being filled, only the words with new bits
__device__ __forceinline__ void dep_or(uint4* bank, uint32_t e, uint4 m) {
    if (e == RC_HG_INVALID || (m.x | m.y | m.z | m.w) == 0u) return;
    const uint4 cur = __ldcg(bank + e);
    unsigned* w = reinterpret_cast<unsigned*>(bank + e);
    if (m.x & ~cur.x) atomicOr(w + 0, m.x);
    if (m.y & ~cur.y) atomicOr(w + 1, m.y);
    if (m.z & ~cur.z) atomicOr(w + 2, m.z);
    if (m.w & ~cur.w) atomicOr(w + 3, m.w);
}

// rtxgi_bench.patch:904-1006: the dependency part of the path loop, one thread per path.  A
// vertex answered from the cache (RC_HG_STOP) passes that entry's masks, as they are when the
// thread reads them, to the earlier vertices (the reference reads them the same way, racing
// with other paths' updates of that entry).
// bw is one of b0 / b1 (no __restrict__ on them: they alias).
// Paths are either contiguous (ps = npaths + 1 offsets) or in fixed slots (ps = NULL, path p is
// v[p * stride .. p * stride + plen[p])).
__global__ void __launch_bounds__(HG_BLOCK) k_hg_mark(const HgDev c, const rc_hg_vertex* __restrict__ v,
                                                      const int* __restrict__ ps, const int* __restrict__ plen, int stride, int npaths,
                                                      uint4* bw, const uint4* b0, const uint4* b1) {
    const int p = blockIdx.x * HG_BLOCK + threadIdx.x;
    if (p >= npaths) return;
    uint32_t idx[RC_HG_MAX_DEPTH];
    int len = 0;
    const int D = c.depth;
    const long long j0 = ps ? ps[p] : (long long)p * stride;
    const long long j1 = ps ? ps[p + 1] : j0 + plen[p];
    for (long long j = j0; j < j1; ++j) {
        const rc_hg_vertex x = v[j];
        const float o[3] = {x.origin[0], x.origin[1], x.origin[2]};
        if (x.flags & RC_HG_MISS) {
            uint32_t sm[3] = {0u, 0u, 0u};
            const float e[3] = {__fadd_rn(o[0], __fmul_rn(x.dir[0], c.td)), __fadd_rn(o[1], __fmul_rn(x.dir[1], c.td)),
                                __fadd_rn(o[2], __fmul_rn(x.dir[2], c.td))};
            mark_segment(c, sm, o, e);
            const uint4 dm = make_uint4(sm[0], sm[1], sm[2], RC_HG_SKY_BIT);
            for (int di = 0; di < len; ++di) dep_or(bw, idx[di], dm);
            break;
        }
        const float h[3] = {x.hit[0], x.hit[1], x.hit[2]};
        uint32_t din[3] = {0u, 0u, 0u}, dloc[3] = {0u, 0u, 0u}, lights = 0u;
        mark_segment(c, din, o, h);
        mark_point(c, dloc, h[0], h[1], h[2]);
        if (x.light_index >= 0) {
            const float r = mn(x.light_dist, c.td);
            const float e[3] = {__fadd_rn(h[0], __fmul_rn(x.to_light[0], r)), __fadd_rn(h[1], __fmul_rn(x.to_light[1], r)),
                                __fadd_rn(h[2], __fmul_rn(x.to_light[2], r))};
            mark_segment(c, dloc, h, e);
            if (x.flags & RC_HG_LIGHT_VISIBLE) lights |= 1u << min(x.light_index, 30);
        }
        const int prev = len;
        for (int k = min(len, D - 1); k > 0; --k) idx[k] = idx[k - 1];
        idx[0] = x.entry;
        len = min(len + 1, D);
        const uint4 cur = make_uint4(dloc[0], dloc[1], dloc[2], lights);
        uint4 prv = make_uint4(dloc[0] | din[0], dloc[1] | din[1], dloc[2] | din[2], lights);
        const bool stop = (x.flags & RC_HG_STOP) != 0u;
        if (stop && x.entry != RC_HG_INVALID) {
            const uint4 a = __ldcg(b0 + x.entry), b = __ldcg(b1 + x.entry);
            prv.x |= a.x | b.x; prv.y |= a.y | b.y; prv.z |= a.z | b.z; prv.w |= a.w | b.w;
        }
        dep_or(bw, idx[0], cur);
        const int last = min(prev, D - 1);
        for (int di = 1; di <= last; ++di) dep_or(bw, idx[di], prv);
        if (stop) break;
    }
}

// ------------------------------------------------------------------ per-voxel light masks
// A res^3 grid over the zone box: voxel of a point per axis int((x - lo) * scale), clamped, with
// scale = res / (hi - lo) rounded once on the host; explicitly rounded operations.
struct VoxDev {
    float lo[3], scale[3];
    int res;
};
VoxDev vox_dev(const rc_hg* hg) {
    VoxDev v;
    for (int k = 0; k < 3; ++k) {
        v.lo[k] = hg->cfg.zone_lo[k];
        volatile float ext = hg->cfg.zone_hi[k] - hg->cfg.zone_lo[k];
        v.scale[k] = (float)hg->vres / ext;
    }
    v.res = hg->vres;
    return v;
}
__device__ __forceinline__ int vox_axis(float x, float lo, float scale, int res) {
    const int i = (int)__fmul_rn(__fsub_rn(x, lo), scale);
    return min(max(i, 0), res - 1);
}
// sample positions k / 19 of a shadow segment (20 samples, k_build's rasterisation)
__constant__ float c_seg19[20] = {0.f / 19.f,  1.f / 19.f,  2.f / 19.f,  3.f / 19.f,  4.f / 19.f,  5.f / 19.f,  6.f / 19.f,
                                  7.f / 19.f,  8.f / 19.f,  9.f / 19.f,  10.f / 19.f, 11.f / 19.f, 12.f / 19.f, 13.f / 19.f,
                                  14.f / 19.f, 15.f / 19.f, 16.f / 19.f, 17.f / 19.f, 18.f / 19.f, 19.f / 19.f};

// Bit l of every voxel on the shadow segment of a vertex whose sampled light l (< 64) was
// visible: 20 evenly spaced samples from the hit to the light (at most tracing_distance), as
// k_build rasterises its shadow rays (poc_gpu.cu:192-197).  A bit already set is not written.
__global__ void __launch_bounds__(HG_BLOCK) k_vox_mark(const HgDev c, const VoxDev g, const rc_hg_vertex* __restrict__ v,
                                                       const int* __restrict__ plen, int stride, int npaths,
                                                       unsigned long long* __restrict__ vox) {
    const int res = g.res;
    const int p = blockIdx.x * HG_BLOCK + threadIdx.x;
    if (p >= npaths) return;
    const long long j0 = (long long)p * stride;
    for (long long j = j0; j < j0 + plen[p]; ++j) {
        const rc_hg_vertex x = v[j];
        if ((x.flags & RC_HG_MISS) || x.light_index < 0 || x.light_index >= 64 || !(x.flags & RC_HG_LIGHT_VISIBLE)) continue;
        const unsigned long long bit = 1ull << x.light_index;
        const float r = mn(x.light_dist, c.td);
        float a[3], d[3];
        for (int k = 0; k < 3; ++k) {
            a[k] = x.hit[k];
            d[k] = __fmul_rn(x.to_light[k], r);
        }
        size_t last = ~(size_t)0;   // consecutive samples in one voxel mark it once
#pragma unroll 4
        for (int k = 0; k < 20; ++k) {
            const float t = c_seg19[k];
            const int ix = vox_axis(__fadd_rn(a[0], __fmul_rn(d[0], t)), g.lo[0], g.scale[0], res);
            const int iy = vox_axis(__fadd_rn(a[1], __fmul_rn(d[1], t)), g.lo[1], g.scale[1], res);
            const int iz = vox_axis(__fadd_rn(a[2], __fmul_rn(d[2], t)), g.lo[2], g.scale[2], res);
            const size_t vi = ((size_t)iz * res + iy) * res + ix;
            if (vi == last) continue;
            last = vi;
            unsigned long long* w = vox + vi;
            if (!(__ldcg(w) & bit)) atomicOr(w, bit);
        }
    }
}

// OR of the masks of the voxels [i0, i1] (inclusive, per axis)
__global__ void __launch_bounds__(HG_BLOCK) k_vox_box(const unsigned long long* __restrict__ vox, int res, int3 i0, int3 i1,
                                                      unsigned long long* out) {
    const int nx = i1.x - i0.x + 1, ny = i1.y - i0.y + 1, nz = i1.z - i0.z + 1;
    const long long n = (long long)nx * ny * nz;
    unsigned long long m = 0ull;
    for (long long t = blockIdx.x * (long long)HG_BLOCK + threadIdx.x; t < n; t += (long long)gridDim.x * HG_BLOCK) {
        const int x = i0.x + (int)(t % nx), y = i0.y + (int)((t / nx) % ny), z = i0.z + (int)(t / ((long long)nx * ny));
        m |= vox[((size_t)z * res + y) * res + x];
    }
    for (int o = 16; o > 0; o >>= 1) m |= __shfl_xor_sync(0xffffffffu, m, o);
    if ((threadIdx.x & 31) == 0 && m) atomicOr(out, m);
}

// ------------------------------------------------------------------ hash grid
// The reference's cache-point hash (poc_gpu.cu:251-262)
__device__ __forceinline__ unsigned long long hg_mix64(unsigned long long x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull; x ^= x >> 27; x *= 0x94d049bb133111ebull; x ^= x >> 31;
    return x;
}
__device__ __forceinline__ int hg_bucket(float nx, float ny, float nz) {
    const float ax = fabsf(nx), ay = fabsf(ny), az = fabsf(nz);
    if (ax >= ay && ax >= az) return nx > 0.f ? 0 : 1;
    if (ay >= az) return ny > 0.f ? 2 : 3;
    return nz > 0.f ? 4 : 5;
}
__device__ __forceinline__ unsigned long long hg_key(const HgDev& c, float px, float py, float pz, float nx, float ny, float nz) {
    const int cx = (int)floorf(__fmul_rn(__fsub_rn(px, c.org[0]), c.ih));
    const int cy = (int)floorf(__fmul_rn(__fsub_rn(py, c.org[1]), c.ih));
    const int cz = (int)floorf(__fmul_rn(__fsub_rn(pz, c.org[2]), c.ih));
    unsigned long long k = (unsigned long long)(cx & 0xFFFFF);
    k = (k << 20) | (unsigned long long)(cy & 0xFFFFF);
    k = (k << 20) | (unsigned long long)(cz & 0xFFFFF);
    return ((k << 3) | (unsigned long long)hg_bucket(nx, ny, nz)) + 1ull;
}

// Insert or find: linear probing from mix64(key) over at most 64 slots.  An evicted slot does
// not end the probe (so a key placed past it stays reachable, whatever order the inserts ran
// in); a missing key claims, by compare-and-swap, the first evicted slot it passed or else the
// empty slot that ended the probe.  A lost claim re-reads the same slot.
__global__ void __launch_bounds__(HG_BLOCK) k_hg_insert(const HgDev c, const float* __restrict__ pos, const float* __restrict__ nrm,
                                                        int n, unsigned long long* __restrict__ keys, uint32_t* __restrict__ entry) {
    const int i = blockIdx.x * HG_BLOCK + threadIdx.x;
    if (i >= n) return;
    const float nx = nrm[3 * (size_t)i], ny = nrm[3 * (size_t)i + 1], nz = nrm[3 * (size_t)i + 2];
    if (nx == 0.f && ny == 0.f && nz == 0.f) {   // no surface point: no entry
        entry[i] = RC_HG_INVALID;
        return;
    }
    const unsigned long long key = hg_key(c, pos[3 * (size_t)i], pos[3 * (size_t)i + 1], pos[3 * (size_t)i + 2], nx, ny, nz);
    uint32_t h = (uint32_t)hg_mix64(key) & c.mask;
    uint32_t out = RC_HG_INVALID, tomb = RC_HG_INVALID;
    for (int probe = 0; probe < 64 && out == RC_HG_INVALID; ++probe) {
        const unsigned long long k = __ldcg(keys + h);
        if (k == key) {
            out = h;
        } else if (k == TOMB) {
            if (tomb == RC_HG_INVALID) tomb = h;
            h = (h + 1u) & c.mask;
        } else if (k == 0ull) {
            const uint32_t slot = tomb != RC_HG_INVALID ? tomb : h;
            const unsigned long long expect = tomb != RC_HG_INVALID ? TOMB : 0ull;
            const unsigned long long prev = atomicCAS(keys + slot, expect, key);
            if (prev == expect || prev == key) out = slot;
            else if (slot == tomb) tomb = RC_HG_INVALID;   // taken by another key: go on from h
        } else {
            h = (h + 1u) & c.mask;
        }
    }
    if (out == RC_HG_INVALID && tomb != RC_HG_INVALID) {
        const unsigned long long prev = atomicCAS(keys + tomb, TOMB, key);
        if (prev == TOMB || prev == key) out = tomb;
    }
    entry[i] = out;
}

__device__ __forceinline__ uint32_t to_fixed(float x) {
    float y = __fmul_rn(x, 1024.f);
    if (!(y > 0.f)) return 0u;
    if (y > 2147483648.f) y = 2147483648.f;
    return __float2uint_rn(y);
}

// Radiance samples in 1/1024 units and a sample count, added with integer atomics; lanes of a
// warp that share an entry add theirs first (integer sums: the result does not depend on it).
__global__ void __launch_bounds__(HG_BLOCK) k_hg_accum(const uint32_t* __restrict__ entry, const float* __restrict__ rgb, int n,
                                                       uint4* __restrict__ accum) {
    const int i = blockIdx.x * HG_BLOCK + threadIdx.x;
    const uint32_t e = i < n ? entry[i] : RC_HG_INVALID;
    uint32_t r = 0u, g = 0u, b = 0u;
    if (e != RC_HG_INVALID) {
        r = to_fixed(rgb[3 * (size_t)i]);
        g = to_fixed(rgb[3 * (size_t)i + 1]);
        b = to_fixed(rgb[3 * (size_t)i + 2]);
    }
    // lanes with the same entry (each group reduces over its own mask)
    const unsigned peers = __match_any_sync(0xffffffffu, e);
    const int lane = threadIdx.x & 31, lead = __ffs(peers) - 1;
    const uint32_t sr = __reduce_add_sync(peers, r), sg = __reduce_add_sync(peers, g), sb = __reduce_add_sync(peers, b);
    const uint32_t sc = (uint32_t)__popc(peers);
    if (e == RC_HG_INVALID || lane != lead) return;
    unsigned* w = reinterpret_cast<unsigned*>(accum + e);
    if (sr) atomicAdd(w + 0, sr);
    if (sg) atomicAdd(w + 1, sg);
    if (sb) atomicAdd(w + 2, sb);
    atomicAdd(w + 3, sc);
}

__device__ __forceinline__ float h2f(uint32_t bits) { return __half2float(__ushort_as_half((unsigned short)bits)); }
__device__ __forceinline__ uint32_t f2h(float f) { return (uint32_t)__half_as_ushort(__float2half_rn(f)); }

// One pass over the table: rtxgi_bench.patch:1028-1050 (an entry whose masks are empty or
// meet the event mask is zeroed; an empty or evicted entry's masks are cleared) around the
// cache's resolve (the frame's samples folded into the mean, capped at acc_frames samples;
// an entry without samples for more than stale_frames frames is evicted).
__global__ void __launch_bounds__(HG_BLOCK) k_hg_resolve(const HgDev c, const uint4 inv, unsigned long long* __restrict__ keys,
                                                         uint4* __restrict__ accum, uint4* __restrict__ resolved,
                                                         uint4* __restrict__ b0, uint4* __restrict__ b1, uint32_t* __restrict__ counts) {
    __shared__ uint32_t cnt[3];
    if (threadIdx.x < 3) cnt[threadIdx.x] = 0u;
    __syncthreads();
    uint32_t n_inv = 0, n_evict = 0, n_valid = 0;
    const bool any_inv = (inv.x | inv.y | inv.z | inv.w) != 0u;
    for (uint32_t e = blockIdx.x * HG_BLOCK + threadIdx.x; e < c.cap; e += gridDim.x * HG_BLOCK) {
        // all five loads issued together: an empty or evicted slot holds no data (its arrays are
        // zero: cleared when the entry is evicted, below, and not written while the slot has no
        // key), but reading the key first and skipping the rest put a dependent load in front of
        // every live entry and measured slower (0.268 against 0.235 ms at 2^24 slots, 47 % live)
        const unsigned long long key0 = keys[e];
        const uint4 m0 = b0[e], m1 = b1[e];
        uint4 a = accum[e], r = resolved[e];
        const uint4 a_in = a, r_in = r;
        const uint4 dep = make_uint4(m0.x | m1.x, m0.y | m1.y, m0.z | m1.z, m0.w | m1.w);
        if (any_inv && ((dep.x | dep.y | dep.z | dep.w) == 0u ||
                        ((dep.x & inv.x) | (dep.y & inv.y) | (dep.z & inv.z) | (dep.w & inv.w)) != 0u)) {
            a = make_uint4(0u, 0u, 0u, 0u);
            r = make_uint4(0u, 0u, 0u, 0u);
            if (key0 != 0ull && key0 != TOMB) ++n_inv;
        }
        unsigned long long key = key0;
        const bool live = key0 != 0ull && key0 != TOMB;
        if (live) {
            const uint32_t nold = r.z & 0xFFFFu;
            uint32_t stale = r.z >> 16;
            if (a.w > 0u) {
                const float sc = 0.0009765625f;
                const uint32_t n = nold + a.w;
                const float fn = (float)nold, fd = __uint2float_rn(n);
                const float mr = __fdiv_rn(__fadd_rn(__fmul_rn(h2f(r.x & 0xFFFFu), fn), __fmul_rn(__uint2float_rn(a.x), sc)), fd);
                const float mg = __fdiv_rn(__fadd_rn(__fmul_rn(h2f(r.x >> 16), fn), __fmul_rn(__uint2float_rn(a.y), sc)), fd);
                const float mb = __fdiv_rn(__fadd_rn(__fmul_rn(h2f(r.y & 0xFFFFu), fn), __fmul_rn(__uint2float_rn(a.z), sc)), fd);
                const uint32_t nn = min(n, (uint32_t)c.acc_frames);
                r = make_uint4(f2h(mr) | f2h(mg) << 16, f2h(mb) | f2h(__uint2float_rn(nn)) << 16, nn, 0u);
            } else {
                ++stale;
                if (stale > (uint32_t)c.stale_frames) {
                    key = TOMB;
                    r = make_uint4(0u, 0u, 0u, 0u);
                    ++n_evict;
                } else {
                    r.z = nold | stale << 16;
                }
            }
            a = make_uint4(0u, 0u, 0u, 0u);
        }
        if (key != key0) keys[e] = key;
        if (a.x != a_in.x || a.y != a_in.y || a.z != a_in.z || a.w != a_in.w) accum[e] = a;
        if (r.x != r_in.x || r.y != r_in.y || r.z != r_in.z || r.w != r_in.w) resolved[e] = r;
        if (key == 0ull || key == TOMB) {
            if ((m0.x | m0.y | m0.z | m0.w) != 0u) b0[e] = make_uint4(0u, 0u, 0u, 0u);
            if ((m1.x | m1.y | m1.z | m1.w) != 0u) b1[e] = make_uint4(0u, 0u, 0u, 0u);
        } else if ((r.y >> 16) != 0u) {
            ++n_valid;
        }
    }
    if (counts) {
        n_inv = __reduce_add_sync(0xffffffffu, n_inv);
        n_evict = __reduce_add_sync(0xffffffffu, n_evict);
        n_valid = __reduce_add_sync(0xffffffffu, n_valid);
        if ((threadIdx.x & 31) == 0) {
            if (n_inv) atomicAdd(&cnt[0], n_inv);
            if (n_evict) atomicAdd(&cnt[1], n_evict);
            if (n_valid) atomicAdd(&cnt[2], n_valid);
        }
        __syncthreads();
        if (threadIdx.x < 3 && cnt[threadIdx.x]) atomicAdd(counts + threadIdx.x, cnt[threadIdx.x]);
    }
}

// ------------------------------------------------------------------ snapshots
// BenchSnap.hlsl (rtxgi_bench.patch:1283-1345).  The reference packs records in the order
// its atomic counter hands out slots; here the records are in entry order (count per block,
// one scan of the block counts, write at block offset + rank in block), so a snapshot is
// reproducible.
__device__ __forceinline__ bool snap_valid(const unsigned long long* keys, const uint4* resolved, uint32_t e) {
    const unsigned long long k = keys[e];
    return k != 0ull && k != TOMB && (resolved[e].y >> 16) != 0u;
}

__global__ void __launch_bounds__(SNAP_BLOCK) k_snap_count(const unsigned long long* __restrict__ keys, const uint4* __restrict__ resolved,
                                                           uint32_t cap, uint32_t* __restrict__ blk) {
    const uint32_t e = blockIdx.x * SNAP_BLOCK + threadIdx.x;
    const int v = e < cap && snap_valid(keys, resolved, e);
    const int n = __syncthreads_count(v);
    if (threadIdx.x == 0) blk[blockIdx.x] = (uint32_t)n;
}

// Exclusive scan of nblk block counts in place, total into *total (one block).
__global__ void __launch_bounds__(SNAP_BLOCK) k_snap_scan(uint32_t* __restrict__ blk, int nblk, uint32_t* __restrict__ total) {
    __shared__ uint32_t warp_sum[SNAP_BLOCK / 32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int base = 0; base < nblk; base += SNAP_BLOCK) {
        const int i = base + threadIdx.x;
        const uint32_t x = i < nblk ? blk[i] : 0u;
        uint32_t incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_sum[w] = incl;
        __syncthreads();
        if (w == 0) {
            uint32_t s = warp_sum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            warp_sum[lane] = s;   // inclusive over warps
        }
        __syncthreads();
        const uint32_t before = carry + (w > 0 ? warp_sum[w - 1] : 0u) + incl - x;
        if (i < nblk) blk[i] = before;
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_sum[SNAP_BLOCK / 32 - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(SNAP_BLOCK) k_snap_write(const unsigned long long* __restrict__ keys, const uint4* __restrict__ resolved,
                                                           uint32_t cap, const uint32_t* __restrict__ blk_off,
                                                           rc_hg_snap_rec* __restrict__ out, uint32_t out_cap) {
    __shared__ uint32_t warp_n[SNAP_BLOCK / 32];
    const uint32_t e = blockIdx.x * SNAP_BLOCK + threadIdx.x;
    const bool v = e < cap && snap_valid(keys, resolved, e);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, v);
    if (lane == 0) warp_n[w] = __popc(bal);
    __syncthreads();
    if (!v) return;
    uint32_t off = blk_off[blockIdx.x];
    for (int k = 0; k < w; ++k) off += warp_n[k];
    off += __popc(bal & ((1u << lane) - 1u));
    if (off >= out_cap) return;
    const uint4 r = resolved[e];
    const unsigned long long key = keys[e];
    rc_hg_snap_rec rec;
    rec.index = e;
    rec.sample_data = r.z;
    rec.key[0] = (uint32_t)key;
    rec.key[1] = (uint32_t)(key >> 32);
    rec.radiance[0] = r.x;
    rec.radiance[1] = r.y;
    out[off] = rec;
}

__global__ void __launch_bounds__(HG_BLOCK) k_snap_restore(const rc_hg_snap_rec* __restrict__ recs, uint32_t count, uint32_t cap,
                                                           unsigned long long* __restrict__ keys, uint4* __restrict__ resolved) {
    const uint32_t i = blockIdx.x * HG_BLOCK + threadIdx.x;
    if (i >= count) return;
    const rc_hg_snap_rec rec = recs[i];
    if (rec.index >= cap) return;
    keys[rec.index] = (unsigned long long)rec.key[0] | (unsigned long long)rec.key[1] << 32;
    resolved[rec.index] = make_uint4(rec.radiance[0], rec.radiance[1], rec.sample_data & 0xFFFFu, 0u);
}

// rtxgi_bench.patch:592-615 BenchObjVoxels (host)
void obj_zones(const rc_hg_config* c, const float* obj, uint32_t inv[4]) {
    const int G[3] = {ZX, ZY, ZZ};
    const float margin = 0.25f;
    float lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        const float half = 0.5f * obj[3 + k];
        lo[k] = obj[k] - half - margin;
        hi[k] = obj[k] + half + margin;
    }
    for (int z = 0; z < G[2]; ++z)
        for (int y = 0; y < G[1]; ++y)
            for (int x = 0; x < G[0]; ++x) {
                const int v[3] = {x, y, z};
                bool overlap = true;
                for (int k = 0; k < 3; ++k) {
                    const float cs = (c->zone_hi[k] - c->zone_lo[k]) / (float)G[k];
                    const float c0 = c->zone_lo[k] + cs * (float)v[k], c1 = c0 + cs;
                    if (hi[k] < c0 || lo[k] > c1) overlap = false;
                }
                if (overlap) {
                    const int b = x + G[0] * (y + G[1] * z);
                    inv[b / 32] |= 1u << (b % 32);
                }
            }
}

}  // namespace

// ============================================================================ C ABI
extern "C" {

rc_status rc_hg_create(const rc_hg_config* cfg, rc_hg** out) {
    if (!cfg || !out) return RC_ERR_ARG;
    *out = nullptr;
    const uint32_t cap = cfg->capacity;
    if (cap < 32 || (cap & (cap - 1)) || cap > (1u << 28)) return RC_ERR_ARG;
    if (!(cfg->cell > 0.f) || cfg->max_depth < 1 || cfg->max_depth > RC_HG_MAX_DEPTH || cfg->acc_frames < 1 ||
        cfg->acc_frames > 0xFFFF || cfg->stale_frames < 0 || cfg->stale_frames > 0xFFFE || !(cfg->tracing_distance > 0.f))
        return RC_ERR_ARG;
    for (int k = 0; k < 3; ++k)
        if (!(cfg->zone_hi[k] > cfg->zone_lo[k])) return RC_ERR_ARG;
    rc_hg* hg = new rc_hg();
    hg->cfg = *cfg;
    auto bad = [&](rc_status s) { rc_hg_destroy(hg); return s; };
    if (cudaSetDevice(cfg->device) != cudaSuccess) return bad(RC_ERR_CUDA);
    if (cfg->stream) hg->stream = (cudaStream_t)cfg->stream;
    else {
        if (cudaStreamCreateWithFlags(&hg->stream, cudaStreamNonBlocking) != cudaSuccess) return bad(RC_ERR_CUDA);
        hg->own_stream = true;
    }
    const size_t nblk = (cap + SNAP_BLOCK - 1) / SNAP_BLOCK;
    hg->scratch_words = 4 + nblk;
    if (cudaMalloc(&hg->keys, 8 * (size_t)cap) != cudaSuccess || cudaMalloc(&hg->accum, 16 * (size_t)cap) != cudaSuccess ||
        cudaMalloc(&hg->resolved, 16 * (size_t)cap) != cudaSuccess || cudaMalloc(&hg->bank[0], 16 * (size_t)cap) != cudaSuccess ||
        cudaMalloc(&hg->bank[1], 16 * (size_t)cap) != cudaSuccess || cudaMalloc(&hg->scratch, 4 * hg->scratch_words) != cudaSuccess)
        return bad(RC_ERR_NOMEM);
    rc_status s = rc_hg_clear(hg);
    if (s != RC_OK) return bad(s);
    if (cudaStreamSynchronize(hg->stream) != cudaSuccess) return bad(RC_ERR_CUDA);
    *out = hg;
    return RC_OK;
}

void rc_hg_destroy(rc_hg* hg) {
    if (!hg) return;
    if (hg->stream) cudaStreamSynchronize(hg->stream);
    cudaFree(hg->keys);
    cudaFree(hg->accum);
    cudaFree(hg->resolved);
    cudaFree(hg->bank[0]);
    cudaFree(hg->bank[1]);
    cudaFree(hg->scratch);
    cudaFree(hg->vox);
    cudaFree(hg->vox_out);
    if (hg->own_stream && hg->stream) cudaStreamDestroy(hg->stream);
    delete hg;
}

const char* rc_hg_last_error(const rc_hg* hg) { return hg ? hg->err.c_str() : "no cache"; }

rc_status rc_hg_array(rc_hg* hg, int which, void** d_ptr, size_t* bytes) {
    if (!hg) return RC_ERR_ARG;
    const size_t cap = hg->cfg.capacity;
    void* p = nullptr;
    size_t b = 16 * cap;
    switch (which) {
        case RC_HG_A_KEYS: p = hg->keys; b = 8 * cap; break;
        case RC_HG_A_ACCUM: p = hg->accum; break;
        case RC_HG_A_RESOLVED: p = hg->resolved; break;
        case RC_HG_A_BANK0: p = hg->bank[0]; break;
        case RC_HG_A_BANK1: p = hg->bank[1]; break;
        default: return fail(hg, RC_ERR_ARG, "array %d", which);
    }
    if (d_ptr) *d_ptr = p;
    if (bytes) *bytes = b;
    return RC_OK;
}

rc_status rc_hg_array_copy(rc_hg* hg, int which, void* host, size_t bytes, int to_device) {
    void* d = nullptr;
    size_t n = 0;
    rc_status s = rc_hg_array(hg, which, &d, &n);
    if (s != RC_OK) return s;
    if (!host || bytes != n) return fail(hg, RC_ERR_ARG, "array %d holds %zu bytes, not %zu", which, n, bytes);
    HGCK(cudaMemcpyAsync(to_device ? d : host, to_device ? host : d, n, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                         hg->stream));
    HGCK(cudaStreamSynchronize(hg->stream));
    return RC_OK;
}

rc_status rc_hg_clear(rc_hg* hg) {
    if (!hg) return RC_ERR_ARG;
    const size_t cap = hg->cfg.capacity;
    HGCK(cudaMemsetAsync(hg->keys, 0, 8 * cap, hg->stream));
    HGCK(cudaMemsetAsync(hg->accum, 0, 16 * cap, hg->stream));
    HGCK(cudaMemsetAsync(hg->resolved, 0, 16 * cap, hg->stream));
    HGCK(cudaMemsetAsync(hg->bank[0], 0, 16 * cap, hg->stream));
    HGCK(cudaMemsetAsync(hg->bank[1], 0, 16 * cap, hg->stream));
    hg->bank_sel = 0;
    return RC_OK;
}

rc_status rc_hg_insert(rc_hg* hg, const float* d_pos, const float* d_nrm, int n, uint32_t* d_entry) {
    if (!hg || n < 0 || (n > 0 && (!d_pos || !d_nrm || !d_entry))) return RC_ERR_ARG;
    if (n == 0) return RC_OK;
    k_hg_insert<<<grid_for(n, HG_BLOCK), HG_BLOCK, 0, hg->stream>>>(dev_of(hg), d_pos, d_nrm, n, hg->keys, d_entry);
    HGCK(cudaGetLastError());
    return RC_OK;
}

rc_status rc_hg_accumulate(rc_hg* hg, const uint32_t* d_entry, const float* d_rgb, int n) {
    if (!hg || n < 0 || (n > 0 && (!d_entry || !d_rgb))) return RC_ERR_ARG;
    if (n == 0) return RC_OK;
    k_hg_accum<<<grid_for(n, HG_BLOCK), HG_BLOCK, 0, hg->stream>>>(d_entry, d_rgb, n, hg->accum);
    HGCK(cudaGetLastError());
    return RC_OK;
}

rc_status rc_hg_begin_frame(rc_hg* hg, uint32_t dep_frame, uint32_t period) {
    if (!hg) return RC_ERR_ARG;
    const uint32_t P = period > 0 ? period : 16u;
    if (dep_frame % P == 0) {
        hg->bank_sel = (int)((dep_frame / P) % 2);
        HGCK(cudaMemsetAsync(hg->bank[hg->bank_sel], 0, 16 * (size_t)hg->cfg.capacity, hg->stream));
    }
    return RC_OK;
}

rc_status rc_hg_mark_paths(rc_hg* hg, const rc_hg_vertex* d_vertices, const int* d_path_start, int npaths) {
    if (!hg || npaths < 0 || (npaths > 0 && (!d_vertices || !d_path_start))) return RC_ERR_ARG;
    if (npaths == 0) return RC_OK;
    k_hg_mark<<<grid_for(npaths, HG_BLOCK), HG_BLOCK, 0, hg->stream>>>(dev_of(hg), d_vertices, d_path_start, nullptr, 0, npaths,
                                                                        hg->bank[hg->bank_sel], hg->bank[0], hg->bank[1]);
    HGCK(cudaGetLastError());
    return RC_OK;
}

rc_status rc_hg_mark_paths_strided(rc_hg* hg, const rc_hg_vertex* d_vertices, const int* d_len, int stride, int npaths) {
    if (!hg || npaths < 0 || stride < 1 || (npaths > 0 && (!d_vertices || !d_len))) return RC_ERR_ARG;
    if (npaths == 0) return RC_OK;
    k_hg_mark<<<grid_for(npaths, HG_BLOCK), HG_BLOCK, 0, hg->stream>>>(dev_of(hg), d_vertices, nullptr, d_len, stride, npaths,
                                                                        hg->bank[hg->bank_sel], hg->bank[0], hg->bank[1]);
    HGCK(cudaGetLastError());
    return RC_OK;
}

rc_status rc_hg_voxels_init(rc_hg* hg, int res) {
    if (!hg || res < 1 || res > 256) return RC_ERR_ARG;
    HGCK(cudaStreamSynchronize(hg->stream));
    cudaFree(hg->vox);
    cudaFree(hg->vox_out);
    hg->vox = nullptr;
    hg->vox_out = nullptr;
    hg->vres = 0;
    const size_t n = (size_t)res * res * res;
    if (cudaMalloc(&hg->vox, 8 * n) != cudaSuccess || cudaMalloc(&hg->vox_out, 8) != cudaSuccess)
        return fail(hg, RC_ERR_NOMEM, "voxel masks of %d^3", res);
    hg->vres = res;
    return rc_hg_voxels_clear(hg);
}

rc_status rc_hg_voxels_clear(rc_hg* hg) {
    if (!hg) return RC_ERR_ARG;
    if (!hg->vres) return fail(hg, RC_ERR_STATE, "no voxel masks (rc_hg_voxels_init)");
    HGCK(cudaMemsetAsync(hg->vox, 0, 8 * (size_t)hg->vres * hg->vres * hg->vres, hg->stream));
    return RC_OK;
}

rc_status rc_hg_voxels_mark(rc_hg* hg, const rc_hg_vertex* d_vertices, const int* d_len, int stride, int npaths) {
    if (!hg || npaths < 0 || stride < 1 || (npaths > 0 && (!d_vertices || !d_len))) return RC_ERR_ARG;
    if (!hg->vres) return fail(hg, RC_ERR_STATE, "no voxel masks (rc_hg_voxels_init)");
    if (npaths == 0) return RC_OK;
    k_vox_mark<<<grid_for(npaths, HG_BLOCK), HG_BLOCK, 0, hg->stream>>>(dev_of(hg), vox_dev(hg), d_vertices, d_len, stride, npaths,
                                                                         hg->vox);
    HGCK(cudaGetLastError());
    return RC_OK;
}

rc_status rc_hg_voxels_box_lights(rc_hg* hg, const float lo[3], const float hi[3], uint64_t* lights) {
    if (!hg || !lo || !hi || !lights) return RC_ERR_ARG;
    if (!hg->vres) return fail(hg, RC_ERR_STATE, "no voxel masks (rc_hg_voxels_init)");
    const int res = hg->vres;
    const VoxDev g = vox_dev(hg);
    int a[3], b[3];
    for (int k = 0; k < 3; ++k) {   // the host restatement of vox_axis
        volatile float d0 = lo[k] - g.lo[k], d1 = hi[k] - g.lo[k];
        volatile float f0 = d0 * g.scale[k], f1 = d1 * g.scale[k];
        a[k] = std::min(std::max((int)f0, 0), res - 1);
        b[k] = std::min(std::max((int)f1, 0), res - 1);
        if (b[k] < a[k]) std::swap(a[k], b[k]);
    }
    HGCK(cudaMemsetAsync(hg->vox_out, 0, 8, hg->stream));
    const long long n = (long long)(b[0] - a[0] + 1) * (b[1] - a[1] + 1) * (b[2] - a[2] + 1);
    const int blocks = (int)std::min<long long>((n + HG_BLOCK - 1) / HG_BLOCK, 4096);
    k_vox_box<<<blocks, HG_BLOCK, 0, hg->stream>>>(hg->vox, res, make_int3(a[0], a[1], a[2]), make_int3(b[0], b[1], b[2]), hg->vox_out);
    HGCK(cudaGetLastError());
    unsigned long long m = 0ull;
    HGCK(cudaMemcpyAsync(&m, hg->vox_out, 8, cudaMemcpyDeviceToHost, hg->stream));
    HGCK(cudaStreamSynchronize(hg->stream));
    *lights = m;
    return RC_OK;
}

rc_status rc_hg_voxels_copy(rc_hg* hg, uint64_t* host, size_t count) {
    if (!hg || !host) return RC_ERR_ARG;
    if (!hg->vres) return fail(hg, RC_ERR_STATE, "no voxel masks (rc_hg_voxels_init)");
    const size_t n = (size_t)hg->vres * hg->vres * hg->vres;
    if (count != n) return fail(hg, RC_ERR_ARG, "the voxel masks hold %zu words", n);
    HGCK(cudaMemcpyAsync(host, hg->vox, 8 * n, cudaMemcpyDeviceToHost, hg->stream));
    HGCK(cudaStreamSynchronize(hg->stream));
    return RC_OK;
}

rc_status rc_hg_resolve(rc_hg* hg, const uint32_t inv[4], uint32_t* d_counts) {
    if (!hg) return RC_ERR_ARG;
    const uint4 iv = inv ? make_uint4(inv[0], inv[1], inv[2], inv[3]) : make_uint4(0u, 0u, 0u, 0u);
    if (d_counts) HGCK(cudaMemsetAsync(d_counts, 0, 3 * sizeof(uint32_t), hg->stream));
    int sms = 0, dev = 0;
    HGCK(cudaGetDevice(&dev));
    HGCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = std::min(grid_for(hg->cfg.capacity, HG_BLOCK), sms * 8);
    k_hg_resolve<<<grid, HG_BLOCK, 0, hg->stream>>>(dev_of(hg), iv, hg->keys, hg->accum, hg->resolved, hg->bank[0], hg->bank[1],
                                                     d_counts);
    HGCK(cudaGetLastError());
    return RC_OK;
}

void rc_hg_event_mask(const rc_hg_config* cfg, const float* la, const float* lb, int nlights, int sky_a, int sky_b,
                      const float* obj_a, const float* obj_b, uint32_t inv[4]) {
    if (!inv) return;
    inv[0] = inv[1] = inv[2] = inv[3] = 0;
    if (!cfg) return;
    for (int i = 0; i < nlights && i < 31; ++i)
        if (la && lb && la[i] != lb[i]) inv[3] |= 1u << i;
    if (sky_a != sky_b) inv[3] |= RC_HG_SKY_BIT;
    bool moved = (obj_a == nullptr) != (obj_b == nullptr);
    if (obj_a && obj_b)
        for (int k = 0; k < 6; ++k)
            if (obj_a[k] != obj_b[k]) moved = true;
    if (moved) {
        if (obj_a) obj_zones(cfg, obj_a, inv);
        if (obj_b) obj_zones(cfg, obj_b, inv);
    }
}

rc_status rc_hg_snapshot(rc_hg* hg, rc_hg_snap_rec* d_recs, uint32_t cap, uint32_t* count) {
    if (!hg || !count || (cap > 0 && !d_recs)) return RC_ERR_ARG;
    const uint32_t n = hg->cfg.capacity;
    const int nblk = (int)((n + SNAP_BLOCK - 1) / SNAP_BLOCK);
    uint32_t* total = hg->scratch;
    uint32_t* blk = hg->scratch + 4;
    k_snap_count<<<nblk, SNAP_BLOCK, 0, hg->stream>>>(hg->keys, hg->resolved, n, blk);
    k_snap_scan<<<1, SNAP_BLOCK, 0, hg->stream>>>(blk, nblk, total);
    if (cap > 0) k_snap_write<<<nblk, SNAP_BLOCK, 0, hg->stream>>>(hg->keys, hg->resolved, n, blk, d_recs, cap);
    HGCK(cudaGetLastError());
    HGCK(cudaMemcpyAsync(count, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, hg->stream));
    HGCK(cudaStreamSynchronize(hg->stream));
    return RC_OK;
}

rc_status rc_hg_restore(rc_hg* hg, const rc_hg_snap_rec* d_recs, uint32_t count) {
    if (!hg || (count > 0 && !d_recs)) return RC_ERR_ARG;
    if (count == 0) return RC_OK;
    k_snap_restore<<<grid_for(count, HG_BLOCK), HG_BLOCK, 0, hg->stream>>>(d_recs, count, hg->cfg.capacity, hg->keys, hg->resolved);
    HGCK(cudaGetLastError());
    return RC_OK;
}

}  // extern "C"

namespace {
__global__ void k_set_entries(rc_hg_vertex* __restrict__ v, const uint32_t* __restrict__ entry, long long n) {
    const long long i = blockIdx.x * (long long)HG_BLOCK + threadIdx.x;
    if (i < n) v[i].entry = entry[i];
}
}  // namespace

namespace rc {
cudaStream_t hg_stream(rc_hg* hg) { return hg->stream; }
const rc_hg_config& hg_config(const rc_hg* hg) { return hg->cfg; }
bool hg_has_voxels(const rc_hg* hg) { return hg->vres > 0; }
cudaError_t hg_set_entries(rc_hg* hg, rc_hg_vertex* v, const uint32_t* entry, long long n) {
    if (n <= 0) return cudaSuccess;
    k_set_entries<<<(unsigned)((n + HG_BLOCK - 1) / HG_BLOCK), HG_BLOCK, 0, hg->stream>>>(v, entry, n);
    return cudaGetLastError();
}
}  // namespace rc
