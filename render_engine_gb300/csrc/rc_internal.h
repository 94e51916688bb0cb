// Structures shared by the host runtime and the kernels (plain data, passed by value).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "rc_device.cuh"

namespace rc {

// Per-state scene data on the device.
struct DState {
    const float4* P4;          // point position (xyz, 0)
    const float4* N4;          // point normal (xyz, 0)
    const float4* AE;          // gather record per point: A, Edir[0..NL-1], zero padded to AES floats
    const uint32_t* SV;        // static shadow-voxel mask, NW words per point
    const float* Q;            // quads: o, u, v, n (12 floats each)
    const int* dims;           // nu, nv per quad
    const int* off;            // first point of each quad
    const float4* tri;         // dynamic triangles, 3 float4 each (v0 + quad id bits, e1, e2)
    const float4* grp;         // plane-culling groups, 3 float4 each, then the pair records (grp_float4s)
    const int* misc;           // dynamic triangles outside any group (always tested exactly)
    const float* ref;          // converged reference per point (scenes with references)
    const uint8_t* valid;
    int nt, ng, nmisc;
    GroupRanges gr;
};

// State-independent scene data (format 3 static mesh and spatial hash, per-point albedo/regions).
struct DStatic {
    const float* ST;           // static triangles v0, e1, e2
    const float4* ST4;         // the same, three float4 per triangle: (v0, e1.x), (e1.yz, e2.xy), (e2.z, 0, 0, 0)
    const float4* STN;         // geometric normal + flags (w bit 0 = double sided)
    const float4* BN;          // BVH nodes, 2 float4 each
    const unsigned long long* HK;
    const int* HV;
    const int* region;
    const float* A;            // albedo per point
    unsigned hmask;
    float hcell;
    int has_bvh;
    int nnodes;
    int max_visits;            // traversal guard (4 x nodes)
    int watertight;            // static triangles by the watertight test (RC_FLAG_WATERTIGHT)
};

struct DevCache {
    float* Lc;                 // LCS floats per point
    float* Lc2;
    float* m;                  // LCS floats per point (trace output on split frames)
    float* n;
    float* c0;
    int* kk;
    uint8_t* pending;
    uint32_t* cur;             // word-major masks
    uint32_t* prev;
    uint32_t* stale;
    float* age;
    float* snap;               // KSNAP x Np x LCS
    float* neq;                // NR x NEQ
    float* coef;               // NR x KSNAP
    float* rstat;              // NR x 4
    float* dstat;              // NR x 3
    float4* pre_hit;           // static-mesh scenes: hits traced ahead, PRE_K per point
    float4* rayq;              // static-mesh scenes: the ray queue of the traced-ahead rays, 2 float4 per ray
    unsigned* rayctr;          // [0] rays in the queue, [1] the next ray to hand out
    float* sumpr;              // 2 slots
    int* npend;                // [0] current, [1] accumulator
    double* err;               // 3 doubles per frame of the run
    float* partf;              // block partials (float)
    double* partd;             // block partials (3 doubles per block)
    int* parti;                // block partials (int)
    unsigned* ticket;          // last-block counters: [0] Sum 1/(n+1), [1] error sums, [2] pending count
    unsigned* flags;           // device guard flags
    unsigned long long* check; // [0] trace disagreements, [1] rays checked
    unsigned long long* rays;  // rays traced since the run began
    unsigned long long* pracc; // fixed-point accumulator of Sum 1/(n+1) (zero between kernels)
    unsigned long long* npacc; // pending-count accumulator (zero between kernels)
};

enum MaskOp { MASK_NONE = 0, MASK_OR = 1, MASK_FRESH = 2, MASK_ZERO = 3 };
enum DevFlag { FLAG_BVH_VISITS = 1u, FLAG_BAD_INDEX = 2u };

struct FrameParams {
    int Np, NR, mode;
    float budget, nmax;
    uint32_t seed, frame;
    int pend_left, dormant, resp_mask;
    float nmax_resp;
    int ddgi;
    float ddgi_h, ddgi_thr;
    int ddgi_clamp, ramp, proj_left, projK;
    int slot[KSNAP];
    float rays;
    int mask_op;
    int want_err, err_frame;   // error sums of this frame go to err[3*err_frame]
    int sum_in, sum_out;       // sumpr slots read / written
    int decide;                // split update: run the verification decision first
    int brute, check;          // trace options
    float half_inv_np;         // 0.5f / Np, the float quotient the ray count uses
    const float4* pre_hit;     // rays traced ahead by k_pretrace (pre_k per point), or null
    int pre_k;
    int wavefront;             // traced-ahead rays through the ray queue (k_trace_queue) instead of k_pretrace
};

// Pinhole camera of the image pass: pixel (x, y) looks along
// fwd + right * ((x + 0.5) / w * 2 - 1) * tx + up * (1 - (y + 0.5) / h * 2) * ty.
struct CameraD {
    float eye[3], fwd[3], right[3], up[3];
    float tx, ty;
    int w, h;
};

// Camera-path pass feeding the hash-grid cache (rc_hg_camera_paths): lights and path shape.
struct PathD {
    int bounces, slots;          // slots = bounces + 1 vertices per path
    uint32_t seed, frame;
    float td;                    // length of the sun's shadow rays
    int nl;
    float lpos[32][3], lrgb[32][3], lint[32];   // point lights: position, colour, intensity of the state
    int area_on;
    float ac[3], au[3], av[3], an[3], aarea, argb[3];   // rectangle: corner, edges, unit normal, area, radiance
    int sun_on;
    float sdir[3], srgb[3];
    float sky[3];
};

// Event program: the per-point kernels of one event of Runner::run, in launch order.
enum EvKind { EV_SNAP_SAVE = 0, EV_ORACLE, EV_RESCALE, EV_WAKE, EV_TOUCHED, EV_SNAP_RESTORE, EV_RESTORED };
struct EvOp {
    int kind;
    int a;            // slot / light / touched kind / verify
    int b;            // verify (wake) / list length (touched)
    int count;        // pending count of this op reaches npend
    int dormant;      // host dormant mask when the reference launches the op
    float x;          // rescale ratio
    const int* list;  // touched voxel list
    const float* r0;  // oracle: reference before / after
    const float* r1;
};
struct EvProgram {
    int nops;
    int npend_mode;   // 0 keep, 1 publish the counted ops, 2 set to zero
    int zero_rstat, zero_neq;
    int want_sumpr;   // mode 1: recompute Sum 1/(n+1) into sumpr[sum_slot]
    int sum_slot;
    float nmax;       // restored history
    int Np, NR;
    EvOp ops[MAX_EV_OPS];
};

// Launch wrappers (rc_kernels.cu), one instantiation per light count, each compiled in its
// own translation unit (-DRC_NL_ONE=n) so the build runs in parallel.
template <int NL>
struct Ops {
    static cudaError_t build(int NW, const DState& s, const DStatic& g, const Grid& grid, const float* L, const float* inten,
                             float4* AE, uint32_t* SV, int Np, unsigned* flags, cudaStream_t st);
    static cudaError_t frame(int NW, bool deps, bool fused, const DState& s, const DStatic& g, const Grid& grid,
                             const DevCache& c, const FrameParams& p, cudaStream_t st);
    static cudaError_t update(const DState& s, const DStatic& g, const DevCache& c, const FrameParams& p, cudaStream_t st);
    static cudaError_t event(const EvProgram& ev, const DevCache& c, cudaStream_t st);
    static cudaError_t error(const DState& s, const DevCache& c, const FrameParams& p, cudaStream_t st);
    static cudaError_t proj_apply(const DevCache& c, const DStatic& g, const FrameParams& p, cudaStream_t st);
    static cudaError_t camera(const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                              const CameraD& cam, float* img, cudaStream_t st);
    // load every kernel of this light count and mask width now, so the first event or
    // verification frame does not pay for loading its kernels
    static cudaError_t preload(int NW);
    static cudaError_t probe(int NW, const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                             const int* pts, int npts, void* recs, int maxrec, int* nrec, cudaStream_t st);
    // one iteration of the converged-reference solve (scene preparation)
    static cudaError_t ref_iter(const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                                const float* Lin, float* Lout, float* acc, float* closec, uint32_t seed, int K, int accumulate,
                                int count_close, cudaStream_t st);
    // one taa-mode sample per point (x), with deps the rays' dependency masks or-ed into cur
    static cudaError_t taa_sample(int NW, bool deps, const DState& s, const DStatic& g, const Grid& grid, const DevCache& c,
                                  const FrameParams& p, float* x, uint32_t* cur, uint32_t seed, uint32_t frame, cudaStream_t st);
    // one camera path per pixel (vertex records in `vtx`, which is an rc_hg_vertex array)
    static cudaError_t paths(const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                             const CameraD& cam, const PathD& pd, float* pos, float* nrm, float* rgb, void* vtx, int* len, float* img,
                             cudaStream_t st);
    // K frozen rays per point (the rays of one reference iteration with `seed`): hit cache point or -1
    static cudaError_t frozen_hits(const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                                   uint32_t seed, int K, int* hits, cudaStream_t st);
    // the first p.pre_k rays of every point traced ahead of the frame kernel (static-mesh scenes)
    static cudaError_t pretrace(const DState& s, const DStatic& g, const Grid& grid, const DevCache& c, const FrameParams& p,
                                float4* out, cudaStream_t st);
};
// Free-space probe of the scene preparation (48 directions per candidate point through the
// static mesh of g): out[3 i] = closest hit (1e30 when none), out[3 i + 1] = fraction of rays
// that hit, out[3 i + 2] = fraction that meet a one-sided face from behind.
cudaError_t prep_probe(const DStatic& g, const float* C, int nc, float diag, float* out, unsigned* flags, cudaStream_t st);
// Closest hit of n caller-given rays (6 floats each: origin, direction) against state s's
// dynamic triangles and g's static mesh: prim = quad id, -2 - static triangle or -1; t = hit
// distance (+inf when none).
cudaError_t trace_rays(const DState& s, const DStatic& g, int brute, const float* rays, int n, int* prim, float* t,
                       unsigned* flags, cudaStream_t st);

// Light counts and mask widths with compiled kernels.
#define RC_NL_VALUES(X) X(1) X(2) X(3) X(4) X(8) X(16) X(32)
inline bool supported_nl_nw(int NL, int NW) {
    bool nl = false;
#define X(n) nl = nl || NL == n;
    RC_NL_VALUES(X)
#undef X
    return nl && (NW == 4 || NW == 24);
}
#define X(n) extern template struct Ops<n>;
RC_NL_VALUES(X)
#undef X
// The group buffer: 3 float4 per group, then 3 float4 per pair of groups (pass-1 records).
__host__ __device__ inline int grp_float4s(int ng) { return 3 * ng + 3 * (ng / 2); }
__host__ __device__ inline size_t frame_smem_bytes(const DState& s) {
    return sizeof(float4) * (3 * (size_t)s.nt + (size_t)grp_float4s(s.ng)) + sizeof(int) * (size_t)s.nmisc + 16;
}
__host__ __device__ constexpr int lcs_of(int NL) { return (NL + 3) / 4 * 4; }
__host__ __device__ constexpr int aes_of(int NL) { return (NL + 1 + 3) / 4 * 4; }

}  // namespace rc
