// Scene preparation on the GPU: an MSH1 triangle mesh becomes a format-3 scene with converged
// references, the input the reference's `prep` mode produces (cuda/prep_mesh.cuh:303-531) for
// its mesh scenes.  This file's own design, every heavy step a kernel:
//   1. BVH: linear BVH over 63-bit Morton codes of the triangle centroids (Karras, "Maximizing
//      Parallelism in the Construction of BVHs, Octrees, and k-d Trees", HPG 2012), boxes and
//      SAH costs fitted bottom-up, subtrees of at most four triangles collapsed into leaves
//      where the SAH says so, then laid out in the format's order (children of a node adjacent,
//      subtrees contiguous) by each node's walk to the root;
//   2. cache points: every triangle sampled by the R2 low-discrepancy sequence (about three
//      samples per cell area), samples binned into cells of side h and one normal bucket in a
//      GPU hash table (64-bit CAS), each cell keeping the sample nearest its centre (a 64-bit
//      atomic minimum over distance and sample id) and the area-weighted albedo (fixed-point
//      integer sums, so the result does not depend on the order of the atomics); h is scaled
//      until the cell count is within 5 % of the target; points in Morton order;
//   3. verification zones: blocks of 4 x 4 x 4 cells of one normal bucket, numbered by a sort;
//   4. the lookup table (HK, HV): linear probing from mix64(key), placed in canonical order by
//      a sort on the home slot and a prefix maximum, so the table is the same on every run;
//   5. lamps and the movable cube placed in free space found by probe rays (48 directions from
//      each point of a jittered grid), the five states and the events' transit voxels, each
//      lamp's intensity set so that it lights the points with a mean direct light of 1 / NL;
//   6. converged references by rc_reference_build.
// Sorting, scans and the unique pass use CUB.
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/rc_api.h"
#include "rc_internal.h"

namespace rc {
// defined with the context (rc_runtime.cu)
rc_status ctx_fail(rc_ctx* ctx, rc_status s, const char* fmt, ...);
}  // namespace rc

namespace {

constexpr int MAX_LEAF = 4;          // triangles per leaf at most (the traversal tests a leaf's triangles in a loop)
constexpr float C_TRAV = 1.0f;       // SAH cost of visiting an inner node, relative to one triangle test
constexpr float SAMPLES_PER_CELL = 3.0f;   // samples drawn per h^2 of triangle area
constexpr int PB = 256;              // threads per block of the preparation kernels

struct Mesh {
    int nt = 0;
    std::vector<float> V;      // 9 per triangle
    std::vector<float> alb;
    std::vector<uint8_t> ds;   // double-sided
};

// MSH1 (the reference's mesh input, prep_mesh.cuh:22-29): "MSH1", int32 triangle count, 9 floats
// per triangle, one albedo per triangle, one double-sided byte per triangle
bool read_msh1(const char* path, Mesh& M, std::string& err) {
    FILE* f = fopen(path, "rb");
    if (!f) { err = std::string("mesh ") + path + " cannot be read"; return false; }
    char magic[4];
    int nt = 0;
    bool ok = fread(magic, 1, 4, f) == 4 && memcmp(magic, "MSH1", 4) == 0 && fread(&nt, 4, 1, f) == 1 && nt > 0 && nt < (1 << 27);
    if (ok) {
        M.nt = nt;
        M.V.resize(9 * (size_t)nt);
        M.alb.resize(nt);
        M.ds.resize(nt);
        ok = fread(M.V.data(), 4, M.V.size(), f) == M.V.size() && fread(M.alb.data(), 4, M.alb.size(), f) == M.alb.size() &&
             fread(M.ds.data(), 1, M.ds.size(), f) == M.ds.size();
    }
    fclose(f);
    if (!ok) err = std::string("mesh ") + path + ": not an MSH1 file or truncated";
    for (size_t k = 0; ok && k < M.V.size(); ++k)
        if (!std::isfinite(M.V[k])) { err = "mesh: non-finite vertex coordinate"; ok = false; }
    return ok;
}

// ---------------------------------------------------------------- shared arithmetic
// The cell key and its hash are the ones the frame kernels look points up with
// (poc_gpu.cu:251-262): they are part of the format.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull; x ^= x >> 27; x *= 0x94d049bb133111ebull; x ^= x >> 31;
    return x;
}
__host__ __device__ __forceinline__ int normal_bucket(float nx, float ny, float nz) {
    const float ax = fabsf(nx), ay = fabsf(ny), az = fabsf(nz);
    if (ax >= ay && ax >= az) return nx > 0.f ? 0 : 1;
    if (ay >= az) return ny > 0.f ? 2 : 3;
    return nz > 0.f ? 4 : 5;
}
__host__ __device__ __forceinline__ uint64_t cell_key(int cx, int cy, int cz, int b) {
    uint64_t k = (uint64_t)(cx & 0xFFFFF);
    k = (k << 20) | (uint64_t)(cy & 0xFFFFF);
    k = (k << 20) | (uint64_t)(cz & 0xFFFFF);
    return ((k << 3) | (uint64_t)b) + 1ull;
}
// every third bit: 21 bits -> 63
__host__ __device__ __forceinline__ uint64_t spread3(uint64_t x) {
    x &= 0x1fffffull;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}
__device__ __forceinline__ uint32_t wang(uint32_t x) {   // a 32-bit integer mix (lowbias32 constants)
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
// float <-> unsigned with the order of the floats (for atomic minimum / maximum)
__device__ __forceinline__ unsigned f2o(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float o2f(unsigned u) {
    u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    memcpy(&f, &u, 4);
    return f;
}
// every product and sum rounded on its own (no contraction), so a CPU restatement builds the same tree
__device__ __forceinline__ float box_area(float3 lo, float3 hi) {
    const float dx = fmaxf(__fsub_rn(hi.x, lo.x), 0.f), dy = fmaxf(__fsub_rn(hi.y, lo.y), 0.f), dz = fmaxf(__fsub_rn(hi.z, lo.z), 0.f);
    return __fmul_rn(2.f, __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx)));
}

// ---------------------------------------------------------------- 1. BVH
// Per triangle: bounds (for the tree), centroid bounds and mesh bounds (ordered-int atomics).
__global__ void k_tri_bounds(const float* __restrict__ V, int n, float4* __restrict__ tlo, float4* __restrict__ thi,
                             unsigned* __restrict__ bounds /* 0-5 centroid min/max, 6-11 mesh min/max */) {
    const int t = blockIdx.x * PB + threadIdx.x;
    if (t >= n) return;
    const float* v = V + 9 * (size_t)t;
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = fminf(v[a], fminf(v[3 + a], v[6 + a]));
        hi[a] = fmaxf(v[a], fmaxf(v[3 + a], v[6 + a]));
        const float c = __fmul_rn(0.5f, __fadd_rn(lo[a], hi[a]));
        atomicMin(bounds + a, f2o(c));
        atomicMax(bounds + 3 + a, f2o(c));
        atomicMin(bounds + 6 + a, f2o(lo[a]));
        atomicMax(bounds + 9 + a, f2o(hi[a]));
    }
    tlo[t] = make_float4(lo[0], lo[1], lo[2], 0.f);
    thi[t] = make_float4(hi[0], hi[1], hi[2], 0.f);
}

__global__ void k_morton(const float4* __restrict__ tlo, const float4* __restrict__ thi, int n, const unsigned* __restrict__ bounds,
                         uint64_t* __restrict__ code, int* __restrict__ id) {
    const int t = blockIdx.x * PB + threadIdx.x;
    if (t >= n) return;
    const float4 a = tlo[t], b = thi[t];
    const float c[3] = {__fmul_rn(0.5f, __fadd_rn(a.x, b.x)), __fmul_rn(0.5f, __fadd_rn(a.y, b.y)), __fmul_rn(0.5f, __fadd_rn(a.z, b.z))};
    uint64_t q[3];
    for (int k = 0; k < 3; ++k) {
        const float lo = o2f(bounds[k]), hi = o2f(bounds[3 + k]);
        const float e = __fsub_rn(hi, lo);
        const float u = e > 0.f ? __fdiv_rn(__fsub_rn(c[k], lo), e) : 0.f;
        q[k] = (uint64_t)fminf(fmaxf(__fmul_rn(u, 2097152.f), 0.f), 2097151.f);
    }
    code[t] = spread3(q[0]) | spread3(q[1]) << 1 | spread3(q[2]) << 2;
    id[t] = t;
}

// Radix tree over the sorted codes: inner nodes 0 .. n-2 (root 0), leaf k is node n-1+k.
// Equal codes are ordered by their index (the code is extended by the index).
__device__ __forceinline__ int lcp(const uint64_t* c, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t x = c[i] ^ c[j];
    return x ? __clzll((long long)x) : 64 + __clz(i ^ j);
}
__global__ void k_radix_tree(const uint64_t* __restrict__ c, int n, int2* __restrict__ child, int* __restrict__ parent,
                             int* __restrict__ first) {
    const int i = blockIdx.x * PB + threadIdx.x;
    if (i >= n - 1) return;
    const int d = lcp(c, n, i, i + 1) - lcp(c, n, i, i - 1) > 0 ? 1 : -1;
    const int dmin = lcp(c, n, i, i - d);
    int lmax = 2;
    while (lcp(c, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (lcp(c, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = lcp(c, n, i, j);
    int s = 0;
    for (int div = 2;; div *= 2) {
        const int t = (l + div - 1) / div;
        if (lcp(c, n, i, i + (s + t) * d) > dnode) s += t;
        if (t <= 1) break;
    }
    const int g = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int left = lo == g ? n - 1 + g : g;
    const int right = hi == g + 1 ? n - 1 + g + 1 : g + 1;
    child[i] = make_int2(left, right);
    parent[left] = i;
    parent[right] = i;
    first[i] = lo;
    if (i == 0) parent[0] = -1;
}

struct FitNode {   // per node of the radix tree, filled bottom-up
    float4 lo, hi;  // box; lo.w = SAH cost, hi.w unused
    int count;      // triangles below
    int desc;       // nodes below it in the output tree (0 for a leaf or a collapsed subtree)
    int collapsed;  // 1: emitted as a leaf of its whole range
    int pad;
};

__device__ __forceinline__ FitNode load_fit(const FitNode* p) {
    const float4* q = reinterpret_cast<const float4*>(p);
    FitNode f;
    f.lo = __ldcg(q);
    f.hi = __ldcg(q + 1);
    const int4 r = __ldcg(reinterpret_cast<const int4*>(q + 2));
    f.count = r.x;
    f.desc = r.y;
    f.collapsed = r.z;
    f.pad = r.w;
    return f;
}
static_assert(sizeof(FitNode) == 48, "FitNode: three 16-byte words");

// Bottom-up pass: each leaf climbs while it is the second child to arrive at its parent.
__global__ void k_fit(const float4* __restrict__ tlo, const float4* __restrict__ thi, const int* __restrict__ sid, int n,
                      const int2* __restrict__ child, const int* __restrict__ parent, FitNode* nodes, unsigned* arrive) {
    const int k = blockIdx.x * PB + threadIdx.x;
    if (k >= n) return;
    int x = n - 1 + k;
    {
        const int t = sid[k];
        const float4 a = tlo[t], b = thi[t];
        FitNode f;
        f.lo = make_float4(a.x, a.y, a.z, box_area(make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z)));
        f.hi = make_float4(b.x, b.y, b.z, 0.f);
        f.count = 1;
        f.desc = 0;
        f.collapsed = 0;
        f.pad = 0;
        nodes[x] = f;
    }
    while (true) {
        const int p = parent[x];
        if (p < 0) return;
        __threadfence();
        if (atomicAdd(arrive + p, 1u) == 0u) return;   // the sibling is not done yet: it will carry on
        __threadfence();
        const int2 ch = child[p];
        const FitNode L = load_fit(nodes + ch.x), R = load_fit(nodes + ch.y);   // written by other threads: read through L2
        FitNode f;
        const float3 lo = make_float3(fminf(L.lo.x, R.lo.x), fminf(L.lo.y, R.lo.y), fminf(L.lo.z, R.lo.z));
        const float3 hi = make_float3(fmaxf(L.hi.x, R.hi.x), fmaxf(L.hi.y, R.hi.y), fmaxf(L.hi.z, R.hi.z));
        const float A = box_area(lo, hi);
        f.count = L.count + R.count;
        const float split = __fadd_rn(__fadd_rn(__fmul_rn(C_TRAV, A), L.lo.w), R.lo.w);
        const float leaf = __fmul_rn((float)f.count, A);
        f.collapsed = f.count <= MAX_LEAF && leaf <= split;
        f.desc = f.collapsed ? 0 : 2 + L.desc + R.desc;
        f.lo = make_float4(lo.x, lo.y, lo.z, f.collapsed ? leaf : split);
        f.hi = make_float4(hi.x, hi.y, hi.z, 0.f);
        f.pad = 0;
        nodes[p] = f;
        x = p;
    }
}

// Output layout: the root at 0; the children of a node at c and c + 1, where c is the start of
// its children's block; the left child's descendants follow at c + 2, the right child's after
// them.  A node's block start is 1 + the sum, over the edges from the root down to it, of
// 2 plus (for a right child) its left sibling's descendant count.
__global__ void k_layout(int n, const int2* __restrict__ child, const int* __restrict__ parent, const int* __restrict__ first,
                         const FitNode* __restrict__ nodes, float4* __restrict__ out, int* __restrict__ stats /* 0 nodes, 1 depth */) {
    const int x = blockIdx.x * PB + threadIdx.x;
    if (x >= 2 * n - 1) return;
    int cb = 1, depth = 0, y = x, rx = 0;
    bool first_edge = true;
    int sib_desc = 0;
    while (y != 0) {
        const int p = parent[y];
        if (nodes[p].collapsed) return;   // inside a collapsed subtree: not emitted
        const int2 ch = child[p];
        const int right = ch.y == y;
        const int sd = right ? nodes[ch.x].desc : 0;
        cb += 2 + sd;
        if (first_edge) { rx = right; sib_desc = sd; first_edge = false; }
        ++depth;
        y = p;
    }
    const int pos = x == 0 ? 0 : cb - 2 - sib_desc + rx;
    const FitNode f = nodes[x];
    const bool leaf = x >= n - 1 || f.collapsed;
    const int lf = leaf ? (x >= n - 1 ? x - (n - 1) : first[x]) : cb;
    const int cnt = leaf ? f.count : 0;
    out[2 * pos] = make_float4(f.lo.x, f.lo.y, f.lo.z, __int_as_float(lf));
    out[2 * pos + 1] = make_float4(f.hi.x, f.hi.y, f.hi.z, __int_as_float(cnt));
    atomicAdd(stats, 1);
    atomicMax(stats + 1, depth);
}

// Triangles in leaf order: ST (v0, e1, e2), STN (unit normal, w = 1 when double-sided), the
// traversal's padded copy ST4, and the albedo.
__global__ void k_write_tris(const float* __restrict__ V, const float* __restrict__ alb, const uint8_t* __restrict__ ds,
                             const int* __restrict__ sid, int n, float* __restrict__ ST, float4* __restrict__ STN, float4* __restrict__ ST4,
                             float* __restrict__ salb, uint8_t* __restrict__ sds) {
    const int j = blockIdx.x * PB + threadIdx.x;
    if (j >= n) return;
    const int t = sid[j];
    const float* v = V + 9 * (size_t)t;
    float T[12];
    for (int a = 0; a < 3; ++a) {
        T[a] = v[a];
        T[3 + a] = __fsub_rn(v[3 + a], v[a]);
        T[6 + a] = __fsub_rn(v[6 + a], v[a]);
    }
    T[9] = T[10] = T[11] = 0.f;
    for (int a = 0; a < 9; ++a) ST[9 * (size_t)j + a] = T[a];
    ST4[3 * (size_t)j] = make_float4(T[0], T[1], T[2], T[3]);
    ST4[3 * (size_t)j + 1] = make_float4(T[4], T[5], T[6], T[7]);
    ST4[3 * (size_t)j + 2] = make_float4(T[8], 0.f, 0.f, 0.f);
    const float cx = __fsub_rn(__fmul_rn(T[4], T[8]), __fmul_rn(T[5], T[7]));
    const float cy = __fsub_rn(__fmul_rn(T[5], T[6]), __fmul_rn(T[3], T[8]));
    const float cz = __fsub_rn(__fmul_rn(T[3], T[7]), __fmul_rn(T[4], T[6]));
    float l = sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy)), __fmul_rn(cz, cz)));
    l = l > 0.f ? l : 1.f;
    STN[j] = make_float4(__fdiv_rn(cx, l), __fdiv_rn(cy, l), __fdiv_rn(cz, l), __int_as_float(ds[t] ? 1 : 0));
    salb[j] = alb[t];
    sds[j] = ds[t];
}

// ---------------------------------------------------------------- 2. cache points
__global__ void k_tri_samples(const float* __restrict__ ST, int n, float h, float* __restrict__ area, int* __restrict__ ns) {
    const int j = blockIdx.x * PB + threadIdx.x;
    if (j >= n) return;
    const float* T = ST + 9 * (size_t)j;
    const double cx = (double)T[4] * T[8] - (double)T[5] * T[7];
    const double cy = (double)T[5] * T[6] - (double)T[3] * T[8];
    const double cz = (double)T[3] * T[7] - (double)T[4] * T[6];
    const double a = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
    area[j] = (float)a;
    ns[j] = a < 1e-12 ? 0 : (int)fmin(1048576.0, fmax(1.0, ceil(SAMPLES_PER_CELL * a / ((double)h * h))));
}

struct CellTable {
    uint64_t* key;    // 0 = empty
    uint64_t* best;   // (distance to the cell centre as ordered bits) << 32 | (sample << 1 | side)
    uint64_t* asum;   // albedo x weight, fixed point
    uint64_t* wsum;   // weight, fixed point
    uint64_t mask;
};

// Sample k of triangle j: the R2 sequence (Roberts 2018, the plastic number's powers) from a
// per-triangle offset, folded into the triangle.
__device__ __forceinline__ float3 sample_point(const float* T, int j, int k, uint32_t seed) {
    const uint32_t hsh = wang(seed ^ wang((uint32_t)j * 0x9E3779B9u + 0x632BE5ABu));
    const float o1 = (float)(hsh >> 8) * (1.f / 16777216.f), o2 = (float)(wang(hsh) >> 8) * (1.f / 16777216.f);
    const double a1 = 0.7548776662466927, a2 = 0.5698402909980532;   // 1/g, 1/g^2, g = 1.32471795724...
    float u = (float)fmod((double)o1 + a1 * (k + 1), 1.0);
    float v = (float)fmod((double)o2 + a2 * (k + 1), 1.0);
    if (u + v > 1.f) { u = 1.f - u; v = 1.f - v; }
    return make_float3(__fadd_rn(T[0], __fadd_rn(__fmul_rn(T[3], u), __fmul_rn(T[6], v))),
                       __fadd_rn(T[1], __fadd_rn(__fmul_rn(T[4], u), __fmul_rn(T[7], v))),
                       __fadd_rn(T[2], __fadd_rn(__fmul_rn(T[5], u), __fmul_rn(T[8], v))));
}
__device__ __forceinline__ void cell_of(float3 P, float3 lo, float h, int c[3], float& d2) {
    const float p[3] = {P.x, P.y, P.z}, l[3] = {lo.x, lo.y, lo.z};
    d2 = 0.f;
    for (int a = 0; a < 3; ++a) {
        c[a] = (int)floorf(__fdiv_rn(__fsub_rn(p[a], l[a]), h));
        const float cc = __fadd_rn(l[a], __fmul_rn(__fadd_rn((float)c[a], 0.5f), h));
        const float d = __fsub_rn(p[a], cc);
        d2 = __fadd_rn(d2, __fmul_rn(d, d));
    }
}
__device__ __forceinline__ int upper_tri(const int* off, int n, int s) {   // triangle whose sample range holds s
    int lo = 0, hi = n;   // first index with off > s, minus one
    while (lo < hi) {
        const int m = (lo + hi) >> 1;
        if (off[m] <= s) lo = m + 1;
        else hi = m;
    }
    return lo - 1;
}
__global__ void k_cell_samples(const float* __restrict__ ST, const float4* __restrict__ STN, const float* __restrict__ salb,
                               const uint8_t* __restrict__ sds, const float* __restrict__ area, const int* __restrict__ ns,
                               const int* __restrict__ off, int n, int S, float h, float3 lo, uint32_t seed, CellTable tab,
                               unsigned* __restrict__ cells, unsigned* __restrict__ overflow) {
    const int s = blockIdx.x * PB + threadIdx.x;
    if (s >= S) return;
    const int j = upper_tri(off, n, s);
    const int k = s - off[j];
    const float* T = ST + 9 * (size_t)j;
    const float3 P = sample_point(T, j, k, seed);
    int c[3];
    float d2;
    cell_of(P, lo, h, c, d2);
    const float4 nn = STN[j];
    // weights in units of h^2 / 2^32 (a sample's area is at most h^2 / 3)
    const double w = (double)area[j] / ns[j] / ((double)h * h) * 4294967296.0;
    const uint64_t wf = (uint64_t)w, af = (uint64_t)(w * salb[j]);
    const int sides = sds[j] ? 2 : 1;
    for (int sd = 0; sd < sides; ++sd) {
        const float sg = sd ? -1.f : 1.f;
        const uint64_t key = cell_key(c[0], c[1], c[2], normal_bucket(sg * nn.x, sg * nn.y, sg * nn.z));
        uint64_t slot = mix64(key) & tab.mask;
        int probes = 0;
        while (true) {
            const unsigned long long old = atomicCAS((unsigned long long*)tab.key + slot, 0ull, (unsigned long long)key);
            if (old == 0ull) { atomicAdd(cells, 1u); break; }
            if (old == key) break;
            slot = (slot + 1) & tab.mask;
            if (++probes > 4096) { atomicOr(overflow, 1u); return; }
        }
        atomicMin((unsigned long long*)tab.best + slot, (unsigned long long)((uint64_t)__float_as_uint(d2) << 32 | (uint64_t)(2u * (unsigned)s + sd)));
        atomicAdd((unsigned long long*)tab.asum + slot, (unsigned long long)af);
        atomicAdd((unsigned long long*)tab.wsum + slot, (unsigned long long)wf);
    }
}

struct PointOut {
    uint64_t* order;   // Morton order key: morton(cx, cy, cz) << 3 | bucket
    uint64_t* key;     // cell key
    float* P;          // 3 per point
    float* N;
    float* A;
};
__global__ void k_cell_points(CellTable tab, uint64_t cap, const float* __restrict__ ST, const float4* __restrict__ STN,
                              const int* __restrict__ off, int n, float h, float3 lo, uint32_t seed, PointOut out,
                              unsigned* __restrict__ count) {
    const uint64_t slot = (uint64_t)blockIdx.x * PB + threadIdx.x;
    if (slot >= cap) return;
    const uint64_t key = tab.key[slot];
    if (!key) return;
    const unsigned id = (unsigned)(tab.best[slot] & 0xffffffffull);
    const int s = (int)(id >> 1), sd = (int)(id & 1u);
    const int j = upper_tri(off, n, s);
    const float3 P = sample_point(ST + 9 * (size_t)j, j, s - off[j], seed);
    const float4 nn = STN[j];
    const float sg = sd ? -1.f : 1.f;
    const uint64_t kk = key - 1ull;
    const uint64_t b = kk & 7ull, cz = (kk >> 3) & 0xFFFFFull, cy = (kk >> 23) & 0xFFFFFull, cx = (kk >> 43) & 0xFFFFFull;
    const unsigned i = atomicAdd(count, 1u);
    out.order[i] = (spread3(cx) | spread3(cy) << 1 | spread3(cz) << 2) << 3 | b;
    out.key[i] = key;
    out.P[3 * (size_t)i] = P.x;
    out.P[3 * (size_t)i + 1] = P.y;
    out.P[3 * (size_t)i + 2] = P.z;
    out.N[3 * (size_t)i] = sg * nn.x;
    out.N[3 * (size_t)i + 1] = sg * nn.y;
    out.N[3 * (size_t)i + 2] = sg * nn.z;
    const uint64_t ws = tab.wsum[slot];
    out.A[i] = ws ? (float)((double)tab.asum[slot] / (double)ws) : 0.5f;
}

template <typename T>
__global__ void k_gather(const T* __restrict__ src, const int* __restrict__ idx, int n, int width, T* __restrict__ dst) {
    const size_t e = (size_t)blockIdx.x * PB + threadIdx.x;
    if (e >= (size_t)n * width) return;
    const size_t i = e / width, c = e % width;
    dst[e] = src[(size_t)idx[i] * width + c];
}

// ---------------------------------------------------------------- 3./4. zones and lookup table
__global__ void k_zone_keys(const uint64_t* __restrict__ key, int n, uint64_t* __restrict__ z) {
    const int i = blockIdx.x * PB + threadIdx.x;
    if (i >= n) return;
    const uint64_t k = key[i] - 1ull;
    const int b = (int)(k & 7ull), cz = (int)((k >> 3) & 0xFFFFFull), cy = (int)((k >> 23) & 0xFFFFFull), cx = (int)((k >> 43) & 0xFFFFFull);
    z[i] = cell_key(cx >> 2, cy >> 2, cz >> 2, b);
}
__global__ void k_zone_ids(const uint64_t* __restrict__ z, int n, const uint64_t* __restrict__ uniq, int nu, int* __restrict__ region) {
    const int i = blockIdx.x * PB + threadIdx.x;
    if (i >= n) return;
    const uint64_t v = z[i];
    int lo = 0, hi = nu;
    while (lo < hi) {
        const int m = (lo + hi) >> 1;
        if (uniq[m] < v) lo = m + 1;
        else hi = m;
    }
    region[i] = lo;
}
__global__ void k_home(const uint64_t* __restrict__ key, int n, uint64_t mask, unsigned* __restrict__ home, int* __restrict__ id) {
    const int i = blockIdx.x * PB + threadIdx.x;
    if (i >= n) return;
    home[i] = (unsigned)(mix64(key[i]) & mask);
    id[i] = i;
}
__global__ void k_home_minus_rank(const unsigned* __restrict__ home, int n, long long* __restrict__ v) {
    const int j = blockIdx.x * PB + threadIdx.x;
    if (j >= n) return;
    v[j] = (long long)home[j] - j;
}
// slot_j = j + max_{i <= j}(home_i - i): every slot from an entry's home to its slot is taken by
// an earlier entry, so linear probing from the home finds it.  Entries whose slot would pass the
// table's end are left to k_hash_tail.
__global__ void k_hash_place(const unsigned* __restrict__ home, const int* __restrict__ id, const long long* __restrict__ pm, int n,
                             const uint64_t* __restrict__ key, uint64_t hs, uint64_t* __restrict__ HK, int* __restrict__ HV,
                             unsigned* __restrict__ maxdisp, int* __restrict__ tail_from) {
    const int j = blockIdx.x * PB + threadIdx.x;
    if (j >= n) return;
    const long long slot = j + pm[j];
    if (slot >= (long long)hs) { atomicMin(tail_from, j); return; }
    HK[slot] = key[id[j]];
    HV[slot] = id[j];
    atomicMax(maxdisp, (unsigned)(slot - home[j]));
}
__global__ void k_hash_tail(const unsigned* __restrict__ home, const int* __restrict__ id, int n, const int* __restrict__ tail_from,
                            const uint64_t* __restrict__ key, uint64_t mask, uint64_t* __restrict__ HK, int* __restrict__ HV,
                            unsigned* __restrict__ maxdisp) {
    for (int j = *tail_from; j < n; ++j) {   // one thread, in order
        uint64_t s = home[j];
        while (HK[s] != 0ull) s = (s + 1) & mask;
        HK[s] = key[id[j]];
        HV[s] = id[j];
        const unsigned d = (unsigned)((s - home[j]) & mask);
        if (d > *maxdisp) *maxdisp = d;
    }
}

struct MaxOp {
    __host__ __device__ __forceinline__ long long operator()(long long a, long long b) const { return a > b ? a : b; }
};

// ---------------------------------------------------------------- host helpers
struct DevPool {
    std::vector<void*> p;
    ~DevPool() { for (void* x : p) cudaFree(x); }
    template <typename T>
    T* get(size_t n) {
        void* x = nullptr;
        if (cudaMalloc(&x, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        p.push_back(x);
        return static_cast<T*>(x);
    }
};
inline unsigned grid_of(size_t n) { return (unsigned)((n + PB - 1) / PB); }

#define PK(x)                                                                                           \
    do {                                                                                                \
        cudaError_t e_ = (x);                                                                           \
        if (e_ != cudaSuccess) return rc::ctx_fail(ctx, RC_ERR_CUDA, "prep: %s", cudaGetErrorString(e_)); \
    } while (0)
#define PA(ptr) \
    do { if (!(ptr)) return rc::ctx_fail(ctx, RC_ERR_NOMEM, "prep: out of device memory"); } while (0)

template <typename K, typename V>
cudaError_t sort_pairs(DevPool& pool, const K* kin, K* kout, const V* vin, V* vout, int n, cudaStream_t st, int end_bit = sizeof(K) * 8) {
    size_t bytes = 0;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, bytes, kin, kout, vin, vout, n, 0, end_bit, st);
    if (e != cudaSuccess) return e;
    void* tmp = pool.get<uint8_t>(bytes);
    if (!tmp) return cudaErrorMemoryAllocation;
    return cub::DeviceRadixSort::SortPairs(tmp, bytes, kin, kout, vin, vout, n, 0, end_bit, st);
}

struct Prepared {
    float lo[3], ext[3], h = 0.f;
    int nt = 0, nnodes = 0, depth = 0;
    std::vector<float> ST, STN, BN;   // BN: 8 floats per node
    std::vector<uint64_t> HK;
    std::vector<int> HV;
    int npst = 0, nbox = 0, NR = 0, bnu = 0, NL = 3;
    std::vector<float> L, A;
    std::vector<int> region;
    std::vector<float> Pst, Nst;
    std::vector<std::vector<float>> inten;
    std::vector<int> boxpos;
    float boxc[2][3], boxe = 0.f;
    std::vector<std::vector<float>> ref, Pw;
    std::vector<std::vector<uint8_t>> valid;
};

constexpr int GVX = 8, GVY = 4, GVZ = 4;   // transit grid of the reference build, which the event voxels index

int host_vox_axis(float p, float lo, float ext, int G) {   // vox_of's per-axis rule (poc_gpu.cu:192-197)
    return std::min(std::max((int)((p - lo) / ext * G), 0), G - 1);
}

// the cube's six faces as (o, u, v, n), u x v along the outward normal
void cube_quads(const float c[3], float e, float Q[72]) {
    const float E = 2.f * e;
    const float F[6][12] = {{c[0] + e, c[1] - e, c[2] - e, 0, E, 0, 0, 0, E, 1, 0, 0},
                            {c[0] - e, c[1] - e, c[2] - e, 0, 0, E, 0, E, 0, -1, 0, 0},
                            {c[0] - e, c[1] + e, c[2] - e, 0, 0, E, E, 0, 0, 0, 1, 0},
                            {c[0] - e, c[1] - e, c[2] - e, E, 0, 0, 0, 0, E, 0, -1, 0},
                            {c[0] - e, c[1] - e, c[2] + e, E, 0, 0, 0, E, 0, 0, 0, 1},
                            {c[0] - e, c[1] - e, c[2] - e, 0, E, 0, E, 0, 0, 0, 0, -1}};
    memcpy(Q, F, sizeof F);
}

// Format-3 scene bytes (the layout poc_gpu.cu:751-801 reads).
std::vector<uint8_t> scene_bytes(const Prepared& m, bool with_ref) {
    std::vector<uint8_t> out;
    auto W = [&](const void* p, size_t n) { out.insert(out.end(), (const uint8_t*)p, (const uint8_t*)p + n); };
    const int NS = (int)m.inten.size(), Np = m.npst + m.nbox, NL = m.NL;
    const int hdr[8] = {Np, 6, 12, NS, NL, m.NR, with_ref ? 1 : 0, 3};
    W(hdr, 32);
    W(m.lo, 12);
    W(m.ext, 12);
    W(&m.h, 4);
    const int mm[4] = {m.nt, m.nnodes, (int)m.HK.size(), m.npst};
    W(mm, 16);
    W(m.ST.data(), m.ST.size() * 4);
    W(m.STN.data(), m.STN.size() * 4);
    W(m.BN.data(), m.BN.size() * 4);
    W(m.HK.data(), m.HK.size() * 8);
    W(m.HV.data(), m.HV.size() * 4);
    W(m.L.data(), m.L.size() * 4);
    W(m.A.data(), m.A.size() * 4);
    W(m.region.data(), m.region.size() * 4);
    for (int si = 0; si < NS; ++si) {
        std::vector<float> P(m.Pst), N(m.Nst);
        float Q[72];
        cube_quads(m.boxc[m.boxpos[si]], m.boxe, Q);
        std::vector<int> dims, off;
        for (int q = 0; q < 6; ++q) {
            dims.push_back(m.bnu);
            dims.push_back(m.bnu);
            off.push_back(m.npst + q * m.bnu * m.bnu);
            for (int iv = 0; iv < m.bnu; ++iv)
                for (int iu = 0; iu < m.bnu; ++iu)
                    for (int x = 0; x < 3; ++x) {
                        P.push_back(Q[12 * q + x] + Q[12 * q + 3 + x] * ((iu + 0.5f) / m.bnu) + Q[12 * q + 6 + x] * ((iv + 0.5f) / m.bnu));
                        N.push_back(Q[12 * q + 9 + x]);
                    }
        }
        std::vector<float> T;
        std::vector<int> TQ;
        for (int q = 0; q < 6; ++q) {   // the face split along its diagonal: (o, o+u, o+u+v), (o, o+u+v, o+v)
            const float* o = &Q[12 * q];
            const float* u = o + 3;
            const float* v = o + 6;
            for (int x = 0; x < 3; ++x) T.push_back(o[x]);
            for (int x = 0; x < 3; ++x) T.push_back(u[x]);
            for (int x = 0; x < 3; ++x) T.push_back(u[x] + v[x]);
            for (int x = 0; x < 3; ++x) T.push_back(o[x]);
            for (int x = 0; x < 3; ++x) T.push_back(u[x] + v[x]);
            for (int x = 0; x < 3; ++x) T.push_back(v[x]);
            TQ.push_back(q);
            TQ.push_back(q);
        }
        W(m.inten[si].data(), (size_t)NL * 4);
        W(P.data(), P.size() * 4);
        W(N.data(), N.size() * 4);
        W(Q, sizeof Q);
        W(dims.data(), dims.size() * 4);
        W(off.data(), off.size() * 4);
        W(T.data(), T.size() * 4);
        W(TQ.data(), TQ.size() * 4);
        if (with_ref) {
            W(m.ref[si].data(), (size_t)Np * 4);
            W(m.valid[si].data(), (size_t)Np);
            W(m.Pw[si].data(), (size_t)NL * Np * 4);
        }
    }
    // events: the transit voxels that either cube position overlaps (a box / voxel overlap on
    // the grid), and the voxel of each lamp that comes on
    for (int a = 0; a < NS; ++a)
        for (int b = 0; b < NS; ++b) {
            std::vector<int> occ;
            if (a != b && m.boxpos[a] != m.boxpos[b]) {
                for (int p = 0; p < 2; ++p) {
                    int i0[3], i1[3];
                    const int G[3] = {GVX, GVY, GVZ};
                    for (int x = 0; x < 3; ++x) {
                        i0[x] = host_vox_axis(m.boxc[p][x] - m.boxe, m.lo[x], m.ext[x], G[x]);
                        i1[x] = host_vox_axis(m.boxc[p][x] + m.boxe, m.lo[x], m.ext[x], G[x]);
                    }
                    for (int k = i0[2]; k <= i1[2]; ++k)
                        for (int j = i0[1]; j <= i1[1]; ++j)
                            for (int i = i0[0]; i <= i1[0]; ++i) occ.push_back((k * GVY + j) * GVX + i);
                }
                std::sort(occ.begin(), occ.end());
                occ.erase(std::unique(occ.begin(), occ.end()), occ.end());
            }
            const int no = (int)occ.size();
            W(&no, 4);
            W(occ.data(), occ.size() * 4);
            for (int l = 0; l < NL; ++l) {
                std::vector<int> em;
                if (a != b && m.inten[a][l] == 0.f && m.inten[b][l] > 0.f) {
                    const float* p = &m.L[3 * l];
                    em.push_back((host_vox_axis(p[2], m.lo[2], m.ext[2], GVZ) * GVY + host_vox_axis(p[1], m.lo[1], m.ext[1], GVY)) * GVX +
                                 host_vox_axis(p[0], m.lo[0], m.ext[0], GVX));
                }
                const int ne = (int)em.size();
                W(&ne, 4);
                W(em.data(), em.size() * 4);
            }
        }
    return out;
}

bool write_file(const char* path, const std::vector<uint8_t>& b) {
    FILE* f = fopen(path, "wb");
    if (!f) return false;
    const bool ok = fwrite(b.data(), 1, b.size(), f) == b.size();
    return fclose(f) == 0 && ok;
}

double since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

float dist3(const float* a, const float* b) {
    return sqrtf((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
}

}  // namespace

// The state table of prepared scenes is an interface: the reference's scenario files for its mesh
// scenes (cuda/scenes/scenarios_publiques.txt) name these states by index.  Lamps 0 and 1 and the
// cube: 0 = lamps 0, 1 on, cube at A; 1 = lamp 0 off; 2 = cube at B; 3 = lamp 2 on as well (its
// first appearance); 4 = lamp 0 off, cube at B.  Lamps beyond the third stay on in every state.
static const float STATE_LAMPS[5][3] = {{1, 1, 0}, {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 0}};
static const int STATE_CUBE[5] = {0, 0, 1, 0, 1};

extern "C" rc_status rc_prep_mesh_params(rc_ctx* ctx, const char* mesh_path, const char* scene_path, const rc_prep_params* prm,
                                         rc_prep_report* rep) {
    if (!ctx || !mesh_path || !scene_path || !prm || prm->target_points < 16 || prm->lamps < 1 || prm->lamps > 32) return RC_ERR_ARG;
    const auto t0 = std::chrono::steady_clock::now();
    const int NL = prm->lamps;
    const uint32_t seed = prm->seed;
    Mesh M;
    std::string err;
    if (!read_msh1(mesh_path, M, err)) return rc::ctx_fail(ctx, RC_ERR_IO, err.c_str());
    const int n = M.nt;
    cudaStream_t st = nullptr;
    PK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamFree { cudaStream_t s; ~StreamFree() { cudaStreamSynchronize(s); cudaStreamDestroy(s); } } stream_free{st};
    DevPool pool;
    float* dV = pool.get<float>(9 * (size_t)n);
    float* dalb = pool.get<float>(n);
    uint8_t* dds = pool.get<uint8_t>(n);
    float4* tlo = pool.get<float4>(n);
    float4* thi = pool.get<float4>(n);
    unsigned* dbounds = pool.get<unsigned>(12);
    unsigned* dflag = pool.get<unsigned>(8);
    PA(dV); PA(dalb); PA(dds); PA(tlo); PA(thi); PA(dbounds); PA(dflag);
    PK(cudaMemcpyAsync(dV, M.V.data(), M.V.size() * 4, cudaMemcpyHostToDevice, st));
    PK(cudaMemcpyAsync(dalb, M.alb.data(), M.alb.size() * 4, cudaMemcpyHostToDevice, st));
    PK(cudaMemcpyAsync(dds, M.ds.data(), M.ds.size(), cudaMemcpyHostToDevice, st));
    {
        unsigned init[12];
        for (int a = 0; a < 3; ++a) { init[a] = init[6 + a] = 0xFFFFFFFFu; init[3 + a] = init[9 + a] = 0u; }
        PK(cudaMemcpyAsync(dbounds, init, sizeof init, cudaMemcpyHostToDevice, st));
        PK(cudaStreamSynchronize(st));
    }
    k_tri_bounds<<<grid_of(n), PB, 0, st>>>(dV, n, tlo, thi, dbounds);
    PK(cudaGetLastError());
    unsigned hb[12];
    PK(cudaMemcpyAsync(hb, dbounds, sizeof hb, cudaMemcpyDeviceToHost, st));
    PK(cudaStreamSynchronize(st));
    Prepared m;
    m.NL = NL;
    m.nt = n;
    float hi[3];
    for (int a = 0; a < 3; ++a) { m.lo[a] = o2f(hb[6 + a]); hi[a] = o2f(hb[9 + a]); }
    float diag = 0.f;
    for (int a = 0; a < 3; ++a) diag += (hi[a] - m.lo[a]) * (hi[a] - m.lo[a]);
    diag = sqrtf(diag);
    // the scene box: the mesh's bounds grown by 2 % of the diagonal on every side, at least 10 cm
    for (int a = 0; a < 3; ++a) {
        const float pad = std::max(0.02f * diag, 0.1f);
        m.lo[a] -= pad;
        hi[a] += pad;
        m.ext[a] = hi[a] - m.lo[a];
    }
    // ---- 1. BVH
    uint64_t* code = pool.get<uint64_t>(n);
    uint64_t* scode = pool.get<uint64_t>(n);
    int* id = pool.get<int>(n);
    int* sid = pool.get<int>(n);
    PA(code); PA(scode); PA(id); PA(sid);
    k_morton<<<grid_of(n), PB, 0, st>>>(tlo, thi, n, dbounds, code, id);
    PK(cudaGetLastError());
    PK(sort_pairs(pool, code, scode, id, sid, n, st, 63));
    float4* dBN = pool.get<float4>(2 * (size_t)(2 * n - 1));
    int* dstats = pool.get<int>(2);
    PA(dBN); PA(dstats);
    PK(cudaMemsetAsync(dstats, 0, 8, st));
    if (n == 1) {   // one triangle: the root is a leaf
        float lo[3], hi1[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(M.V[a], std::min(M.V[3 + a], M.V[6 + a]));
            hi1[a] = std::max(M.V[a], std::max(M.V[3 + a], M.V[6 + a]));
        }
        m.BN = {lo[0], lo[1], lo[2], 0.f, hi1[0], hi1[1], hi1[2], 0.f};
        const int zero = 0, one = 1;
        memcpy(&m.BN[3], &zero, 4);
        memcpy(&m.BN[7], &one, 4);
        m.nnodes = 1;
        PK(cudaMemcpyAsync(dBN, m.BN.data(), 32, cudaMemcpyHostToDevice, st));
    } else {
        int2* child = pool.get<int2>(n - 1);
        int* parent = pool.get<int>(2 * n - 1);
        int* first = pool.get<int>(n - 1);
        FitNode* nodes = pool.get<FitNode>(2 * n - 1);
        unsigned* arrive = pool.get<unsigned>(n - 1);
        PA(child); PA(parent); PA(first); PA(nodes); PA(arrive);
        k_radix_tree<<<grid_of(n - 1), PB, 0, st>>>(scode, n, child, parent, first);
        PK(cudaGetLastError());
        PK(cudaMemsetAsync(arrive, 0, 4 * (size_t)(n - 1), st));
        k_fit<<<grid_of(n), PB, 0, st>>>(tlo, thi, sid, n, child, parent, nodes, arrive);
        PK(cudaGetLastError());
        k_layout<<<grid_of(2 * (size_t)n - 1), PB, 0, st>>>(n, child, parent, first, nodes, dBN, dstats);
        PK(cudaGetLastError());
        int hs2[2];
        PK(cudaMemcpyAsync(hs2, dstats, 8, cudaMemcpyDeviceToHost, st));
        FitNode root;
        PK(cudaMemcpyAsync(&root, nodes, sizeof root, cudaMemcpyDeviceToHost, st));
        PK(cudaStreamSynchronize(st));
        m.nnodes = hs2[0];
        m.depth = hs2[1];
        if (m.nnodes != 1 + root.desc) return rc::ctx_fail(ctx, RC_ERR_DEVICE, "prep: BVH layout wrote %d nodes, expected %d", m.nnodes, 1 + root.desc);
        // the traversals keep at most 64 deferred nodes; a deeper tree could lose hits
        if (m.depth > 60) return rc::ctx_fail(ctx, RC_ERR_UNSUPPORTED, "prep: BVH depth %d above 60", m.depth);
        m.BN.resize(8 * (size_t)m.nnodes);
        PK(cudaMemcpyAsync(m.BN.data(), dBN, m.BN.size() * 4, cudaMemcpyDeviceToHost, st));
    }
    float* dST = pool.get<float>(9 * (size_t)n);
    float4* dSTN = pool.get<float4>(n);
    float4* dST4 = pool.get<float4>(3 * (size_t)n);
    float* salb = pool.get<float>(n);
    uint8_t* sds = pool.get<uint8_t>(n);
    PA(dST); PA(dSTN); PA(dST4); PA(salb); PA(sds);
    k_write_tris<<<grid_of(n), PB, 0, st>>>(dV, dalb, dds, sid, n, dST, dSTN, dST4, salb, sds);
    PK(cudaGetLastError());
    m.ST.resize(9 * (size_t)n);
    m.STN.resize(4 * (size_t)n);
    PK(cudaMemcpyAsync(m.ST.data(), dST, m.ST.size() * 4, cudaMemcpyDeviceToHost, st));
    PK(cudaMemcpyAsync(m.STN.data(), dSTN, m.STN.size() * 4, cudaMemcpyDeviceToHost, st));
    // ---- 2. cache points
    float* darea = pool.get<float>(n);
    int* dns = pool.get<int>(n + 1);   // n counts and a zero past the end: the scan's n + 1 inputs
    int* doff = pool.get<int>(n + 1);
    PA(darea); PA(dns); PA(doff);
    std::vector<float> harea(n);
    std::vector<uint8_t> hsds(n);
    k_tri_samples<<<grid_of(n), PB, 0, st>>>(dST, n, 1.f, darea, dns);
    PK(cudaGetLastError());
    PK(cudaMemcpyAsync(harea.data(), darea, 4 * (size_t)n, cudaMemcpyDeviceToHost, st));
    PK(cudaMemcpyAsync(hsds.data(), sds, n, cudaMemcpyDeviceToHost, st));
    PK(cudaStreamSynchronize(st));
    double atot = 0;   // surface area, two-sided triangles counted twice (in leaf order, a fixed order)
    for (int t = 0; t < n; ++t) atot += (double)harea[t] * (hsds[t] ? 2 : 1);
    const float3 lo3 = make_float3(m.lo[0], m.lo[1], m.lo[2]);
    float h = (float)sqrt(atot / prm->target_points);
    size_t ex_bytes = 0;
    PK(cub::DeviceScan::ExclusiveSum(nullptr, ex_bytes, dns, doff, n + 1, st));
    void* ex_tmp = pool.get<uint8_t>(ex_bytes);
    PA(ex_tmp);
    CellTable tab{};
    uint64_t cap = 0;
    unsigned ncells = 0;
    int S = 0;
    unsigned* dcount = pool.get<unsigned>(2);
    PA(dcount);
    std::vector<int> hns(n);
    for (int it = 0; it < 6; ++it) {
        k_tri_samples<<<grid_of(n), PB, 0, st>>>(dST, n, h, darea, dns);
        PK(cudaGetLastError());
        PK(cudaMemcpyAsync(hns.data(), dns, 4 * (size_t)n, cudaMemcpyDeviceToHost, st));
        PK(cudaStreamSynchronize(st));
        long long tot = 0;
        for (int t = 0; t < n; ++t) tot += hns[t];
        if (tot >= (1ll << 30)) return rc::ctx_fail(ctx, RC_ERR_UNSUPPORTED, "prep: %lld samples (cells too small for the mesh)", tot);
        S = (int)tot;
        PK(cudaMemsetAsync(dns + n, 0, 4, st));
        PK(cub::DeviceScan::ExclusiveSum(ex_tmp, ex_bytes, dns, doff, n + 1, st));
        const uint64_t want = std::max<uint64_t>(2048, 4ull * (uint64_t)S);
        if (want > cap) {
            cap = 1;
            while (cap < want) cap <<= 1;
            tab.key = pool.get<uint64_t>(cap);
            tab.best = pool.get<uint64_t>(cap);
            tab.asum = pool.get<uint64_t>(cap);
            tab.wsum = pool.get<uint64_t>(cap);
            PA(tab.key); PA(tab.best); PA(tab.asum); PA(tab.wsum);
            tab.mask = cap - 1;
        }
        PK(cudaMemsetAsync(tab.key, 0, 8 * cap, st));
        PK(cudaMemsetAsync(tab.best, 0xFF, 8 * cap, st));
        PK(cudaMemsetAsync(tab.asum, 0, 8 * cap, st));
        PK(cudaMemsetAsync(tab.wsum, 0, 8 * cap, st));
        PK(cudaMemsetAsync(dcount, 0, 8, st));
        k_cell_samples<<<grid_of(S), PB, 0, st>>>(dST, dSTN, salb, sds, darea, dns, doff, n, S, h, lo3, seed, tab, dcount, dcount + 1);
        PK(cudaGetLastError());
        unsigned hc[2];
        PK(cudaMemcpyAsync(hc, dcount, 8, cudaMemcpyDeviceToHost, st));
        PK(cudaStreamSynchronize(st));
        if (hc[1]) return rc::ctx_fail(ctx, RC_ERR_DEVICE, "prep: cell table overflow");
        ncells = hc[0];
        const double ratio = (double)ncells / prm->target_points;
        if (fabs(ratio - 1.0) < 0.05 || it == 5) break;
        h *= (float)std::min(2.0, std::max(0.5, sqrt(ratio)));
    }
    m.h = h;
    const int np = (int)ncells;
    PointOut po{};
    po.order = pool.get<uint64_t>(np);
    po.key = pool.get<uint64_t>(np);
    po.P = pool.get<float>(3 * (size_t)np);
    po.N = pool.get<float>(3 * (size_t)np);
    po.A = pool.get<float>(np);
    PA(po.order); PA(po.key); PA(po.P); PA(po.N); PA(po.A);
    PK(cudaMemsetAsync(dcount, 0, 4, st));
    k_cell_points<<<grid_of(cap), PB, 0, st>>>(tab, cap, dST, dSTN, doff, n, h, lo3, seed, po, dcount);
    PK(cudaGetLastError());
    // Morton order (the order keys are unique, so the permutation does not depend on the atomics)
    uint64_t* sorder = pool.get<uint64_t>(np);
    int* iota = pool.get<int>(np);
    int* perm = pool.get<int>(np);
    PA(sorder); PA(iota); PA(perm);
    {
        std::vector<int> hi0(np);
        for (int i = 0; i < np; ++i) hi0[i] = i;
        PK(cudaMemcpyAsync(iota, hi0.data(), 4 * (size_t)np, cudaMemcpyHostToDevice, st));
        PK(sort_pairs(pool, po.order, sorder, iota, perm, np, st, 63));
        PK(cudaStreamSynchronize(st));
    }
    uint64_t* key = pool.get<uint64_t>(np);
    float* P = pool.get<float>(3 * (size_t)np);
    float* Nn = pool.get<float>(3 * (size_t)np);
    float* A = pool.get<float>(np);
    PA(key); PA(P); PA(Nn); PA(A);
    k_gather<uint64_t><<<grid_of(np), PB, 0, st>>>(po.key, perm, np, 1, key);
    k_gather<float><<<grid_of(3 * (size_t)np), PB, 0, st>>>(po.P, perm, np, 3, P);
    k_gather<float><<<grid_of(3 * (size_t)np), PB, 0, st>>>(po.N, perm, np, 3, Nn);
    k_gather<float><<<grid_of(np), PB, 0, st>>>(po.A, perm, np, 1, A);
    PK(cudaGetLastError());
    // ---- 3. zones
    uint64_t* zk = pool.get<uint64_t>(np);
    uint64_t* zs = pool.get<uint64_t>(np);
    uint64_t* zu = pool.get<uint64_t>(np);
    int* dnu = pool.get<int>(1);
    int* dreg = pool.get<int>(np);
    PA(zk); PA(zs); PA(zu); PA(dnu); PA(dreg);
    k_zone_keys<<<grid_of(np), PB, 0, st>>>(key, np, zk);
    PK(cudaGetLastError());
    {
        size_t b = 0;
        PK(cub::DeviceRadixSort::SortKeys(nullptr, b, zk, zs, np, 0, 64, st));
        void* t = pool.get<uint8_t>(b);
        PA(t);
        PK(cub::DeviceRadixSort::SortKeys(t, b, zk, zs, np, 0, 64, st));
        size_t b2 = 0;
        PK(cub::DeviceSelect::Unique(nullptr, b2, zs, zu, dnu, np, st));
        void* t2 = pool.get<uint8_t>(b2);
        PA(t2);
        PK(cub::DeviceSelect::Unique(t2, b2, zs, zu, dnu, np, st));
    }
    int nzones = 0;
    PK(cudaMemcpyAsync(&nzones, dnu, 4, cudaMemcpyDeviceToHost, st));
    PK(cudaStreamSynchronize(st));
    k_zone_ids<<<grid_of(np), PB, 0, st>>>(zk, np, zu, nzones, dreg);
    PK(cudaGetLastError());
    // ---- 4. lookup table: at most half full; rebuilt twice as large if a probe run passes 63
    uint64_t HS = 64;
    while (HS < 2 * (uint64_t)np) HS <<= 1;
    std::vector<uint64_t> HK;
    std::vector<int> HV;
    for (int tries = 0;; ++tries) {
        unsigned* home = pool.get<unsigned>(np);
        unsigned* shome = pool.get<unsigned>(np);
        int* hid = pool.get<int>(np);
        int* shid = pool.get<int>(np);
        long long* v = pool.get<long long>(np);
        long long* pm = pool.get<long long>(np);
        uint64_t* dHK = pool.get<uint64_t>(HS);
        int* dHV = pool.get<int>(HS);
        unsigned* dmax = pool.get<unsigned>(1);
        int* dtail = pool.get<int>(1);
        PA(home); PA(shome); PA(hid); PA(shid); PA(v); PA(pm); PA(dHK); PA(dHV); PA(dmax); PA(dtail);
        k_home<<<grid_of(np), PB, 0, st>>>(key, np, HS - 1, home, hid);
        PK(cudaGetLastError());
        PK(sort_pairs(pool, home, shome, hid, shid, np, st));
        k_home_minus_rank<<<grid_of(np), PB, 0, st>>>(shome, np, v);
        PK(cudaGetLastError());
        size_t b = 0;
        PK(cub::DeviceScan::InclusiveScan(nullptr, b, v, pm, MaxOp(), np, st));
        void* t = pool.get<uint8_t>(b);
        PA(t);
        PK(cub::DeviceScan::InclusiveScan(t, b, v, pm, MaxOp(), np, st));
        PK(cudaMemsetAsync(dHK, 0, 8 * HS, st));
        PK(cudaMemsetAsync(dHV, 0xFF, 4 * HS, st));
        PK(cudaMemsetAsync(dmax, 0, 4, st));
        const int big = np;
        PK(cudaMemcpyAsync(dtail, &big, 4, cudaMemcpyHostToDevice, st));
        k_hash_place<<<grid_of(np), PB, 0, st>>>(shome, shid, pm, np, key, HS, dHK, dHV, dmax, dtail);
        k_hash_tail<<<1, 1, 0, st>>>(shome, shid, np, dtail, key, HS - 1, dHK, dHV, dmax);
        PK(cudaGetLastError());
        unsigned maxd = 0;
        PK(cudaMemcpyAsync(&maxd, dmax, 4, cudaMemcpyDeviceToHost, st));
        PK(cudaStreamSynchronize(st));
        if (maxd < 63 || tries >= 3) {
            if (maxd >= 63) return rc::ctx_fail(ctx, RC_ERR_DEVICE, "prep: lookup table probe run %u", maxd);
            HK.resize(HS);
            HV.resize(HS);
            PK(cudaMemcpyAsync(HK.data(), dHK, 8 * HS, cudaMemcpyDeviceToHost, st));
            PK(cudaMemcpyAsync(HV.data(), dHV, 4 * HS, cudaMemcpyDeviceToHost, st));
            break;
        }
        HS <<= 1;
    }
    m.npst = np;
    m.NR = nzones;
    m.Pst.resize(3 * (size_t)np);
    m.Nst.resize(3 * (size_t)np);
    m.A.resize(np);
    m.region.resize(np);
    PK(cudaMemcpyAsync(m.Pst.data(), P, 12 * (size_t)np, cudaMemcpyDeviceToHost, st));
    PK(cudaMemcpyAsync(m.Nst.data(), Nn, 12 * (size_t)np, cudaMemcpyDeviceToHost, st));
    PK(cudaMemcpyAsync(m.A.data(), A, 4 * (size_t)np, cudaMemcpyDeviceToHost, st));
    PK(cudaMemcpyAsync(m.region.data(), dreg, 4 * (size_t)np, cudaMemcpyDeviceToHost, st));
    PK(cudaStreamSynchronize(st));
    m.HK = std::move(HK);
    m.HV = std::move(HV);
    // ---- 5. free space: a jittered grid of about 16k candidates, 48 probe rays each
    std::vector<float> C, O;
    {
        const double vol = (double)m.ext[0] * m.ext[1] * m.ext[2];
        const float cs = (float)cbrt(vol / 16384.0);
        int g[3];
        for (int a = 0; a < 3; ++a) g[a] = std::max(2, (int)(m.ext[a] / cs));
        uint64_t r = mix64(0x5eedull ^ seed);
        auto u01 = [&]() { r = mix64(r + 0x9E3779B97F4A7C15ull); return (float)(r >> 40) * (1.f / 16777216.f); };
        for (int k = 0; k < g[2]; ++k)
            for (int j = 0; j < g[1]; ++j)
                for (int i = 0; i < g[0]; ++i) {
                    const int ijk[3] = {i, j, k};
                    for (int a = 0; a < 3; ++a) C.push_back(m.lo[a] + m.ext[a] * ((ijk[a] + 0.15f + 0.7f * u01()) / g[a]));
                }
    }
    const int NC = (int)(C.size() / 3);
    {
        float* dC = pool.get<float>(C.size());
        float* dO = pool.get<float>(3 * (size_t)NC);
        PA(dC); PA(dO);
        PK(cudaMemcpyAsync(dC, C.data(), C.size() * 4, cudaMemcpyHostToDevice, st));
        rc::DStatic g{};
        g.ST = dST;
        g.ST4 = dST4;
        g.STN = dSTN;
        g.BN = dBN;
        g.has_bvh = 1;
        g.nnodes = m.nnodes;
        g.max_visits = 4 * m.nnodes + 64;
        PK(cudaMemsetAsync(dflag, 0, 4, st));
        PK(rc::prep_probe(g, dC, NC, diag, dO, dflag, st));
        O.resize(3 * (size_t)NC);
        unsigned fl = 0;
        PK(cudaMemcpyAsync(O.data(), dO, O.size() * 4, cudaMemcpyDeviceToHost, st));
        PK(cudaMemcpyAsync(&fl, dflag, 4, cudaMemcpyDeviceToHost, st));
        PK(cudaStreamSynchronize(st));
        if (fl) return rc::ctx_fail(ctx, RC_ERR_DEVICE, "prep: BVH traversal guard tripped (flags %u)", fl);
    }
    // free candidates: outside closed geometry (fewer than a quarter of the rays meet a one-sided
    // face from behind) with clearance; the clearance asked for relaxes until there are enough
    std::vector<int> fr;
    float need = 0.03f * diag;
    for (int tries = 0; tries < 8; ++tries, need *= 0.7f) {
        fr.clear();
        for (int i = 0; i < NC; ++i)
            if (O[3 * i + 2] < 0.25f && O[3 * i] >= need) fr.push_back(i);
        if ((int)fr.size() >= NL + 8) break;
    }
    if ((int)fr.size() < NL + 2) return rc::ctx_fail(ctx, RC_ERR_FORMAT, "prep: not enough free space for %d lamps and the cube", NL);
    // lamps: the candidate with the most clearance in the band of 20-70 % of the scene's height,
    // then farthest-point sampling among the band's better-cleared half
    std::vector<int> band;
    for (int i : fr) {
        const float zr = (C[3 * i + 2] - m.lo[2]) / m.ext[2];
        if (zr >= 0.2f && zr <= 0.7f) band.push_back(i);
    }
    if ((int)band.size() < NL) band = fr;
    std::vector<float> cl;
    for (int i : band) cl.push_back(O[3 * i]);
    std::sort(cl.begin(), cl.end());
    const float cmid = cl[cl.size() / 2];
    std::vector<int> lamps;
    {
        int best = band[0];
        for (int i : band) if (O[3 * i] > O[3 * best]) best = i;
        lamps.push_back(best);
    }
    while ((int)lamps.size() < NL) {
        int best = -1;
        float bd = -1.f;
        for (int i : band) {
            if (O[3 * i] < cmid) continue;
            float d = 1e30f;
            for (int j : lamps) d = std::min(d, dist3(&C[3 * i], &C[3 * j]));
            if (d > bd) { bd = d; best = i; }
        }
        if (best < 0 || bd <= 0.f) return rc::ctx_fail(ctx, RC_ERR_FORMAT, "prep: no place for lamp %d", (int)lamps.size());
        lamps.push_back(best);
    }
    for (int j : lamps)
        for (int x = 0; x < 3; ++x) m.L.push_back(C[3 * j + x]);
    // the movable cube (edge b): position A near lamp 0, B near lamp 1 (so that both events
    // change the light), each with room for the cube and away from the lamps and each other
    float b = std::min(2.0f, std::max(0.3f, 0.05f * diag));
    int ia = -1, ib = -1;
    for (int tries = 0; tries < 10; ++tries) {
        ia = ib = -1;
        auto fits = [&](int i) {
            if (O[3 * i] < 0.9f * b) return false;
            for (int l = 0; l < NL; ++l)
                if (dist3(&C[3 * i], &m.L[3 * l]) < 1.5f * b) return false;
            return true;
        };
        float da = 1e30f, db = 1e30f;
        for (int i : fr)
            if (fits(i) && dist3(&C[3 * i], &m.L[0]) < da) { da = dist3(&C[3 * i], &m.L[0]); ia = i; }
        const float* lb = NL > 1 ? &m.L[3] : &m.L[0];
        if (ia >= 0)
            for (int i : fr)
                if (fits(i) && dist3(&C[3 * i], &C[3 * ia]) >= 2.5f * b && dist3(&C[3 * i], lb) < db) { db = dist3(&C[3 * i], lb); ib = i; }
        if (ia >= 0 && ib >= 0) break;
        b *= 0.8f;
    }
    if (ia < 0 || ib < 0) return rc::ctx_fail(ctx, RC_ERR_FORMAT, "prep: no place for the movable cube");
    m.boxe = 0.5f * b;
    for (int x = 0; x < 3; ++x) { m.boxc[0][x] = C[3 * ia + x]; m.boxc[1][x] = C[3 * ib + x]; }
    m.bnu = std::max(2, (int)ceilf(b / m.h));
    m.nbox = 6 * m.bnu * m.bnu;
    for (int k = 0; k < m.nbox; ++k) m.A.push_back(0.5f);
    for (int q = 0; q < 6; ++q)   // one verification zone per cube face
        for (int k = 0; k < m.bnu * m.bnu; ++k) m.region.push_back(m.NR + q);
    m.NR += 6;
    // ---- states
    for (int si = 0; si < 5; ++si) {
        std::vector<float> in(NL, 1.f);
        for (int l = 0; l < std::min(NL, 3); ++l) in[l] = STATE_LAMPS[si][l];
        m.inten.push_back(in);
        m.boxpos.push_back(STATE_CUBE[si]);
    }
    // each lamp's intensity: a mean direct light of 1 / NL over the points of state 0's geometry
    const int Np = m.npst + m.nbox;
    rc_status stt;
    {
        Prepared probe = m;
        for (auto& v : probe.inten) std::fill(v.begin(), v.end(), 1.f);
        std::vector<uint8_t> sb = scene_bytes(probe, false);
        if ((stt = rc_scene_load_memory(ctx, sb.data(), sb.size())) != RC_OK) return stt;
        std::vector<float> Ed((size_t)NL * Np);
        if ((stt = rc_state_array_copy(ctx, 0, RC_SA_EDIR, Ed.data(), Ed.size() * 4)) != RC_OK) return stt;
        for (int l = 0; l < NL; ++l) {
            double sm = 0;
            for (int i = 0; i < Np; ++i) sm += Ed[(size_t)i * NL + l];
            const float s = sm > 0 ? (float)((double)Np / NL / sm) : 1.f;
            for (auto& v : m.inten) v[l] *= s;
        }
        sb = scene_bytes(m, false);
        if ((stt = rc_scene_load_memory(ctx, sb.data(), sb.size())) != RC_OK) return stt;
    }
    // references (the preparation's parameters; PREP_BRUIT_CIBLE / PREP_ITER_MAX as the reference reads them)
    rc_ref_params rp{32, 16, 64, 2048, 0.03};
    if (const char* e = getenv("PREP_BRUIT_CIBLE")) rp.noise_target = atof(e);
    if (const char* e = getenv("PREP_ITER_MAX")) rp.max_iter = std::max(rp.block, atoi(e));
    if (prm->ref_iterations > 0) rp.max_iter = std::max(rp.block, prm->ref_iterations);
    const bool with_ref = prm->ref_iterations >= 0;
    double noise[5] = {0, 0, 0, 0, 0};
    int iters[5] = {0, 0, 0, 0, 0};
    if (with_ref && (stt = rc_reference_build(ctx, &rp, noise, iters)) != RC_OK) return stt;
    double vfrac = 0;
    for (int si = 0; si < 5 && with_ref; ++si) {
        std::vector<float> ref(Np), pw((size_t)NL * Np);
        std::vector<uint8_t> val(Np);
        if ((stt = rc_state_array_copy(ctx, si, RC_SA_REF, ref.data(), ref.size() * 4)) != RC_OK ||
            (stt = rc_state_array_copy(ctx, si, RC_SA_VALID, val.data(), val.size())) != RC_OK ||
            (stt = rc_state_array_copy(ctx, si, RC_SA_PW, pw.data(), pw.size() * 4)) != RC_OK)
            return stt;
        long long nv = 0;
        for (uint8_t x : val) nv += x != 0;
        vfrac += (double)nv / Np / 5;
        m.ref.push_back(std::move(ref));
        m.valid.push_back(std::move(val));
        m.Pw.push_back(std::move(pw));
    }
    if (!write_file(scene_path, scene_bytes(m, with_ref))) return rc::ctx_fail(ctx, RC_ERR_IO, "prep: cannot write %s", scene_path);
    if (rep) {
        memset(rep, 0, sizeof *rep);
        rep->triangles = n;
        rep->np = Np;
        rep->zones = m.NR;
        rep->bvh_nodes = m.nnodes;
        rep->bvh_depth = m.depth;
        rep->cell_m = m.h;
        rep->diag_m = diag;
        rep->cube_m = b;
        rep->valid_fraction = vfrac;
        rep->ns = 5;
        rep->nl = NL;
        for (int si = 0; si < 5; ++si) { rep->noise[si] = noise[si]; rep->iterations[si] = iters[si]; }
        for (int l = 0; l < NL; ++l)
            for (int x = 0; x < 3; ++x) rep->lights[l][x] = m.L[3 * l + x];
        rep->seconds = since(t0);
    }
    return RC_OK;
}

extern "C" rc_status rc_prep_mesh(rc_ctx* ctx, const char* mesh_path, const char* scene_path, int target, rc_prep_report* rep) {
    rc_prep_params p{target, 3, 1u, 0};
    return rc_prep_mesh_params(ctx, mesh_path, scene_path, &p, rep);
}
