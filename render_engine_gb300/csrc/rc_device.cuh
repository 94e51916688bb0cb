// Device-side building blocks of the radiance-cache frame loop (sm_103a).
//
// The arithmetic of every function that decides a hit, a cache point or a voxel bit is
// written expression by expression like the reference (cuda/poc_gpu.cu of
// falcon123212/render_engine), so that the GPU results are bit-identical to the
// reference kernels built with the same compiler: hit primitive ids, cache-point ids,
// dependency masks and invalidation sets are integer results of that arithmetic.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rc {

constexpr int KSNAP = 6;
constexpr int NEQ = 28;
constexpr int BLOCK = 256;          // points per block; also the fixed reduction tree
constexpr int MAX_GROUPS = 64;      // plane-culling groups per state (64-bit candidate mask)
constexpr int MAX_EV_OPS = 40;

struct f3 { float x, y, z; };
__device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ f3 xyz(float4 a) { return {a.x, a.y, a.z}; }

// poc_gpu.cu:127-135
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float rnd(uint32_t& s) {
    s = s * 747796405u + 2891336453u;
    uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    w = (w >> 22u) ^ w;
    return (w >> 8) * (1.0f / 16777216.0f);
}
// poc_gpu.cu:260-262, 251-259
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull; x ^= x >> 27; x *= 0x94d049bb133111ebull; x ^= x >> 31;
    return x;
}
__device__ __forceinline__ int normal_bucket(float nx, float ny, float nz) {
    float ax = fabsf(nx), ay = fabsf(ny), az = fabsf(nz);
    if (ax >= ay && ax >= az) return nx > 0.f ? 0 : 1;
    if (ay >= az) return ny > 0.f ? 2 : 3;
    return nz > 0.f ? 4 : 5;
}
__device__ __forceinline__ unsigned long long cell_key(int cx, int cy, int cz, int b) {
    unsigned long long k = (unsigned long long)(cx & 0xFFFFF);
    k = (k << 20) | (unsigned long long)(cy & 0xFFFFF);
    k = (k << 20) | (unsigned long long)(cz & 0xFFFFF);
    return ((k << 3) | (unsigned long long)b) + 1ull;
}

// Transit voxel grid: bounds and resolution (the reference keeps them in __constant__
// c_lo/c_ext and compile-time VX/VY/VZ, poc_gpu.cu:98-114).
struct Grid {
    float lo[3], ext[3];
    int vx, vy, vz;
    float scale[3];   // vx / ext[0], vy / ext[1], vz / ext[2] as float quotients (set by set_grid_scale)
};

// The float quotients every DDA walk starts from, computed once on the host (IEEE division
// rounds the same on host and device).
inline void set_grid_scale(Grid& g) {
    g.scale[0] = (float)g.vx / g.ext[0];
    g.scale[1] = (float)g.vy / g.ext[1];
    g.scale[2] = (float)g.vz / g.ext[2];
}

// One axis of vox_of (poc_gpu.cu:137-142): int((x - lo) / ext * n), clamped to [0, n - 1].  The
// reference's quotient q = (x - lo) / ext * n is only needed to the integer: qf = (x - lo) * s,
// s = n / ext rounded, and q each carry two roundings, so |qf - q| <= 2.4e-7 |q|, forty times
// less than the 1e-5 |qf| (or 1e-5) margin asked of qf's distance to the nearest integer; when qf
// is that far from one, truncating it gives q's integer.  Otherwise (and for a NaN or an infinity,
// whose comparisons are false) the reference's own IEEE division decides.  The result is the
// reference's, without the division in all but a few samples.
__device__ __forceinline__ int vox_axis(float x, float lo, float ext, float s, int n) {
    const float d = x - lo;
    const float qf = d * s;
    const float r = rintf(qf);
    const int v = fabsf(qf - r) > 1e-5f * fmaxf(1.f, fabsf(qf)) ? int(qf) : int(d / ext * n);
    return min(max(v, 0), n - 1);
}
__device__ __forceinline__ int vox_of(const Grid& g, f3 p) {
    const int i = vox_axis(p.x, g.lo[0], g.ext[0], g.scale[0], g.vx);
    const int j = vox_axis(p.y, g.lo[1], g.ext[1], g.scale[1], g.vy);
    const int k = vox_axis(p.z, g.lo[2], g.ext[2], g.scale[2], g.vz);
    return (k * g.vy + j) * g.vx + i;
}

template <int NW>
__device__ __forceinline__ void set_bit(uint32_t (&m)[NW], int v) {
    const uint32_t bit = 1u << (v & 31);
    const int w0 = v >> 5;
#pragma unroll
    for (int w = 0; w < NW; ++w) m[w] |= (w == w0) ? bit : 0u;
}

// Amanatides-Woo walk of segment a->b over the transit grid, same float sequence as
// dda_reg (poc_gpu.cu:171-190).  The loop bound vx+vy+vz is the reference's.
//
// Every product and sum is rounded on its own (__fmul_rn / __fadd_rn / __fsub_rn are never
// fused into an FMA): the grid coordinate ax = (a.x - lo) * sx must be rounded before ix is
// subtracted from it.  A fused (a.x - lo) * sx - ix keeps the product's low bits, and a
// cache point lying on a voxel face (z = 2.25 with sz = 4/3: the product is 3.0000001,
// rounded 3.0) then starts with tmz = 1e-7 * tdz instead of 0 and breaks the tie at a voxel
// edge the other way.
template <int NW>
__device__ __forceinline__ void dda_walk(const Grid& g, f3 a, f3 b, uint32_t (&m)[NW]) {
    const int VX = g.vx, VY = g.vy, VZ = g.vz;
    const float sx = g.scale[0], sy = g.scale[1], sz = g.scale[2];
    const float ax = __fmul_rn(__fsub_rn(a.x, g.lo[0]), sx), ay = __fmul_rn(__fsub_rn(a.y, g.lo[1]), sy),
                az = __fmul_rn(__fsub_rn(a.z, g.lo[2]), sz);
    const float bx = __fmul_rn(__fsub_rn(b.x, g.lo[0]), sx), by = __fmul_rn(__fsub_rn(b.y, g.lo[1]), sy),
                bz = __fmul_rn(__fsub_rn(b.z, g.lo[2]), sz);
    int ix = min(max(int(ax), 0), VX - 1), iy = min(max(int(ay), 0), VY - 1), iz = min(max(int(az), 0), VZ - 1);
    int ex = min(max(int(bx), 0), VX - 1), ey = min(max(int(by), 0), VY - 1), ez = min(max(int(bz), 0), VZ - 1);
    const float dx = __fsub_rn(bx, ax), dy = __fsub_rn(by, ay), dz = __fsub_rn(bz, az);
    int stx = dx > 0 ? 1 : -1, sty = dy > 0 ? 1 : -1, stz = dz > 0 ? 1 : -1;
    float tdx = dx != 0 ? fabsf(1.f / dx) : 1e30f, tdy = dy != 0 ? fabsf(1.f / dy) : 1e30f, tdz = dz != 0 ? fabsf(1.f / dz) : 1e30f;
    float tmx = dx != 0 ? __fmul_rn(dx > 0 ? __fsub_rn((float)(ix + 1), ax) : __fsub_rn(ax, (float)ix), tdx) : 1e30f;
    float tmy = dy != 0 ? __fmul_rn(dy > 0 ? __fsub_rn((float)(iy + 1), ay) : __fsub_rn(ay, (float)iy), tdy) : 1e30f;
    float tmz = dz != 0 ? __fmul_rn(dz > 0 ? __fsub_rn((float)(iz + 1), az) : __fsub_rn(az, (float)iz), tdz) : 1e30f;
    const int steps = VX + VY + VZ;
    // The voxel index v and the steps left before each axis leaves the grid are carried along
    // instead of the three coordinates: the same voxels in the same order, and the same exits
    // (at the end voxel, or when the chosen axis would step out of the grid).
    int v = (iz * VY + iy) * VX + ix;
    const int ve = (ez * VY + ey) * VX + ex;
    int rx = stx > 0 ? VX - 1 - ix : ix, ry = sty > 0 ? VY - 1 - iy : iy, rz = stz > 0 ? VZ - 1 - iz : iz;
    const int dvx = stx, dvy = sty * VX, dvz = stz * VX * VY;
    unsigned long long lo = 0ull, hi = 0ull;   // the 128 mask bits while NW == 4
    for (int s = 0; s < steps; ++s) {
        if (NW == 4) {
            const unsigned long long bit = 1ull << (v & 63);
            lo |= v < 64 ? bit : 0ull;
            hi |= v < 64 ? 0ull : bit;
        } else {
            set_bit<NW>(m, v);
        }
        if (v == ve) break;
        // one axis steps per iteration, chosen like the reference's if / else-if chain; written
        // with selects so the lanes of a warp do not split three ways
        const bool sx = tmx < tmy && tmx < tmz;
        const bool sy = !sx && tmy < tmz;
        const int left = sx ? rx : (sy ? ry : rz);
        if (left == 0) break;
        rx -= sx ? 1 : 0;
        ry -= sy ? 1 : 0;
        rz -= (!sx && !sy) ? 1 : 0;
        v += sx ? dvx : (sy ? dvy : dvz);
        tmx = sx ? __fadd_rn(tmx, tdx) : tmx;
        tmy = sy ? __fadd_rn(tmy, tdy) : tmy;
        tmz = (!sx && !sy) ? __fadd_rn(tmz, tdz) : tmz;
    }
    if (NW == 4) {
        m[0] |= (uint32_t)lo;
        m[1] |= (uint32_t)(lo >> 32);
        m[2] |= (uint32_t)hi;
        m[3 % NW] |= (uint32_t)(hi >> 32);
    }
}

// poc_gpu.cu:360-366
__device__ __forceinline__ f3 cosine_dir(f3 N, float u1, float u2) {
    float r = sqrtf(u1), phi = 6.28318530718f * u2;
    f3 a = fabsf(N.x) > 0.9f ? mk(0, 1, 0) : mk(1, 0, 0);
    f3 T = cross(N, a); T = T * rsqrtf(dot(T, T));
    f3 B = cross(N, T);
    return T * (r * cosf(phi)) + B * (r * sinf(phi)) + N * sqrtf(fmaxf(0.f, 1.f - u1));
}

// ---------------------------------------------------------------------------- triangles
// Dynamic triangles live in shared memory as 3 float4 each: (v0, quad id bits), (e1, 0), (e2, 0).
//
// Möller-Trumbore of one triangle, the reference's expression order (poc_gpu.cu:203-217).
// Accepts when t is smaller, or equal with a smaller triangle index: over any visiting order
// this selects what the reference's in-order scan selects.
__device__ __forceinline__ void mt_tri(const float4* __restrict__ tri, int j, f3 o, f3 d,
                                       float& tmin, int& q, int& jbest) {
    const float4 A = tri[3 * j], B = tri[3 * j + 1], C = tri[3 * j + 2];
    const f3 v0 = xyz(A), e1 = xyz(B), e2 = xyz(C);
    f3 p = cross(d, e2);
    float det = dot(e1, p);
    if (fabsf(det) <= 1e-9f) return;
    float inv = 1.f / det;
    f3 tv = o - v0;
    float u = dot(tv, p) * inv;
    if (u < 0.f) return;
    f3 qv = cross(tv, e1);
    float v = dot(d, qv) * inv;
    if (v < 0.f || u + v > 1.f) return;
    float t = dot(e2, qv) * inv;
    if (t > 1e-4f && (t < tmin || (t == tmin && j < jbest))) { tmin = t; q = __float_as_int(A.w); jbest = j; }
}

// Plane-culling group: the axis-aligned triangles of one quad lying in one plane k = c.
// 3 float4: (c, centre_a, half_a, centre_b) (half_b, first triangle bits, count bits, 0)
// (n_a, n_b, w, eps) -- the last is the line between the group's two triangles -- where
// a, b are the two other axes in increasing order and the box is the triangles' bounding box
// grown by a margin far above the rounding error of the exact test, so the filter never drops
// the triangle the exact scan would pick.  Each axis holds an even number of groups (a
// padding group has c = NaN and no triangles), and after the 3 ng group records come the
// pass-1 records of each pair (g, g + 1), g even, packed for paired FP32 arithmetic and
// negated: (-c_g, -c_g+1, -centre_a_g, -centre_a_g+1) (-half_a_g, -half_a_g+1, -centre_b_g,
// -centre_b_g+1) (-half_b_g, -half_b_g+1, 0, 0).
struct GroupRanges { int g0[4]; };  // groups of axis 0 in [g0[0], g0[1]), axis 1 [g0[1], g0[2]), axis 2 [g0[2], g0[3])

}  // namespace rc
