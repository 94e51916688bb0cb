// Host runtime behind include/rc_api.h: scene loading, device buffers, and the frame driver.
//
// The frame driver follows Runner::run of the reference (cuda/poc_gpu.cu:826-1016) step by
// step — the same event rules, the same order of operations on the cache — but issues the
// work differently: one kernel per ordinary frame, one kernel per event, no host
// synchronisation except where the reference's projection solve needs the region sums on
// the host, and no per-frame memsets or device-to-device copies (counters and sums live in
// ping-pong slots written by the kernels' last block).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rc_api.h"
#include "../../include/rc_hashgrid.h"
#include "rc_adjoint.h"
#include "rc_hg_internal.h"
#include "rc_internal.h"
#include "rc_taa.h"

using namespace rc;

// Dispatch on the light count to the per-count kernel instantiations.
#define RC_DISPATCH(NL, call)                       \
    [&]() -> cudaError_t {                          \
        switch (NL) {                               \
            case 1: return Ops<1>::call;            \
            case 2: return Ops<2>::call;            \
            case 3: return Ops<3>::call;            \
            case 4: return Ops<4>::call;            \
            case 8: return Ops<8>::call;            \
            case 16: return Ops<16>::call;          \
            case 32: return Ops<32>::call;          \
        }                                           \
        return cudaErrorInvalidValue;               \
    }()

namespace {

constexpr int VERIF_FRAMES = 4;   // poc_gpu.cu:115
constexpr int PROJ_FRAMES = 4;    // poc_gpu.cu:424
constexpr int PRE_K = 4;          // rays per point traced ahead on static-mesh scenes (more are traced inline)

struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;   // the stream the buffer was allocated on (and is freed on)
};

// Device memory of contexts comes from one stream-ordered pool per device that keeps the pages
// it has mapped (release threshold: never): a context that is destroyed and created again, or
// a scene loaded after another, reuses them instead of mapping fresh memory (mapping costs
// about as much as copying the scene).
cudaMemPool_t device_pool(int dev) {
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!pools[dev]) {
        cudaMemPoolProps pp{};
        pp.allocType = cudaMemAllocationTypePinned;
        pp.handleTypes = cudaMemHandleTypeNone;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = dev;
        cudaMemPool_t p = nullptr;
        if (cudaMemPoolCreate(&p, &pp) != cudaSuccess) return nullptr;
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        pools[dev] = p;
    }
    return pools[dev];
}

struct HostState {
    std::vector<float> inten;
    const float* pw = nullptr;      // device warm start (padded cache layout)
    DState d{};
    // Built on first use (ensure_state): until then the state's positions, normals and warm
    // start wait on the device as the file lays them out (xyz triples, NL floats per point).
    bool built = false;             // build issued (on the side stream ahead of use, or on the context's stream)
    bool wait = false;              // the context's stream has yet to wait for the side stream's build
    const float* raw = nullptr;     // 6 Np floats (P, N) then NL Np (Pw, scenes with references)
    const float* dint = nullptr;    // device light intensities
    size_t raw_buf = 0;             // index of the raw buffer in the scene's pool
    bool copies_side = false;       // its per-point arrays were copied on the side stream (RC_FLAG_LOAD_ASYNC)
};

struct Scene {
    int Np = 0, Nq = 0, Nt = 0, NS = 0, NL = 0, NR = 0, has_ref = 0, fmt = 2;
    int nst = 0, nnodes = 0, hsize = 0, npst = 0;
    float hcell = 0.f;
    Grid grid{};
    std::vector<HostState> st;
    DStatic g{};
    const float* L = nullptr;       // device light positions, 3 floats per light
    std::vector<float> hL;          // host copies: light positions, state 0's quad grids
    std::vector<int> hdims, hoff;
    // events: [pair * (1 + NL) + 0] = occluder voxels, [.. + 1 + l] = voxels of light l
    std::vector<std::vector<int>> ev;
    std::vector<const int*> ev_dev;
    double scene_bytes = 0;
};

// State of the taa mode (run_taa_mode, poc_gpu.cu:1175-1282).
struct TaaRun {
    bool active = false;
    rc_taa_method M{};
    uint32_t seed = 0;
    int f = 0, prev_state = 0, verify_left = 0;
    float *x = nullptr, *H = nullptr, *H2 = nullptr, *mu = nullptr, *sg = nullptr, *rs = nullptr, *cnt = nullptr;
    int *qid = nullptr, *react = nullptr;   // quad of each point (-1: none)
    const int4* quad = nullptr;              // per quad: first point, nu, nv
    uint8_t* pend = nullptr;
    uint32_t *cur = nullptr, *prev = nullptr;
    double *part = nullptr, *out = nullptr;
    std::vector<const int*> dV;     // event voxels per state pair (device), and their counts
    std::vector<int> nV;
    // per state: the sum of the references over the valid points and their count (the error's
    // denominators), computed once per run and state
    std::vector<double> ref_sum, ref_cnt;
    std::vector<char> have_sums;
};

struct Run {
    bool active = false;
    rc_method M{};
    FrameParams p{};
    int dormant = 0;
    float ilearn[32] = {0};
    int pend_left = 0, nslots = 0, slot_state[KSNAP], slot_next = 0, last_event_f = 0, proj_left = 0, projK = 0;
    int slot[KSNAP] = {0};
    int prev_state = 0, f = 0, sum_cur = 0, nerr = 0;
    float nmax = 0.f;
    int last_kernels = 0, last_fused = 0, last_event = 0;
};

}  // namespace

struct rc_ctx {
    rc_config cfg{};
    int NW = 4;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    std::vector<DevBuf> scene_bufs, cache_bufs, adj_bufs, taa_bufs, cam_bufs;
    TaaRun taa;
    // camera-path pass (rc_hg_camera_paths): per slot and per pixel buffers of the last pass
    struct CamPass {
        size_t slots_cap = 0, pix_cap = 0;
        float *pos = nullptr, *nrm = nullptr, *rgb = nullptr;
        rc_hg_vertex* vtx = nullptr;
        uint32_t* entry = nullptr;
        int* len = nullptr;
        int stride = 0, npaths = 0;
        cudaEvent_t ready = nullptr;
    } cam;
    cudaStream_t side = nullptr;                // state builds issued ahead of use (prebuild_state)
    std::vector<cudaEvent_t> state_ev;          // per state: its build on the side stream is done
    cudaEvent_t load_ev = nullptr;              // the load's copies, which the side stream waits for
    std::vector<cudaEvent_t> copies_ev;         // per state: its copies on the side stream are done (RC_FLAG_LOAD_ASYNC)
    int adj_np = 0, adj_k = 0;                  // sizes of the last rc_adjoint (0: none)
    int adj_cap_np = 0, adj_cap_k = 0, adj_cap_nl = 0;   // sizes the adjoint buffers were allocated for
    float4* adj_aeu = nullptr;                  // unit-emission direct light of the last adjoint
    int adj_aeu_state = -1;                     // the state adj_aeu holds (-1: none)
    const float* adj_ones = nullptr;
    rc::adj::Bufs adj{};
    Scene S;
    bool have_scene = false;
    DevCache c{};
    size_t err_cap = 0;         // frames of error sums allocated
    Run run;
    double cache_bytes = 0;
    long long launches = 0;
    // device guard words: [0] raised by the run's kernels (read and cleared by rc_device_flags),
    // [1] by one-shot calls that trace (rc_trace_rays), [2] the loader's checks
    unsigned* flags_dev = nullptr;
    float* img = nullptr;
    size_t img_cap = 0;
    cudaEvent_t ev[8] = {};
    double* pinned = nullptr;   // page-locked scratch for per-frame scalar read-backs (8 doubles)
    void* stage = nullptr;      // device staging of padded arrays packed for one host copy
    size_t stage_cap = 0;
};

namespace {

rc_status fail(rc_ctx* ctx, rc_status s, const char* fmt, ...) {
    char buf[512];
    va_list a;
    va_start(a, fmt);
    vsnprintf(buf, sizeof buf, fmt, a);
    va_end(a);
    if (ctx) ctx->err = buf;
    return s;
}
#define CKR(x)                                                                                          \
    do {                                                                                                \
        cudaError_t e_ = (x);                                                                           \
        if (e_ != cudaSuccess) return fail(ctx, RC_ERR_CUDA, "CUDA %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

// A buffer of n elements from the device's pool, ordered on the context's stream (usable on it
// at once, on other streams after they wait for it).
template <class T>
rc_status dalloc(rc_ctx* ctx, std::vector<DevBuf>& pool, T** out, size_t n, cudaStream_t on = nullptr) {
    void* p = nullptr;
    size_t bytes = n * sizeof(T) + 16;
    cudaMemPool_t mp = device_pool(ctx->cfg.device);
    if (!mp) return fail(ctx, RC_ERR_CUDA, "no memory pool on device %d", ctx->cfg.device);
    cudaStream_t st = on ? on : ctx->stream;
    cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, mp, st);
    if (e != cudaSuccess) return fail(ctx, RC_ERR_NOMEM, "device allocation of %zu bytes: %s", bytes, cudaGetErrorString(e));
    pool.push_back({p, bytes, st});
    *out = (T*)p;
    return RC_OK;
}
template <class T>
rc_status dput(rc_ctx* ctx, std::vector<DevBuf>& pool, const T** out, const std::vector<T>& v) {
    T* p = nullptr;
    rc_status s = dalloc(ctx, pool, &p, v.size());
    if (s != RC_OK) return s;
    if (!v.empty()) CKR(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    *out = p;
    return RC_OK;
}
// Back to the device's pool once the work queued on the buffer's stream so far is done.
void free_pool(std::vector<DevBuf>& pool) {
    for (auto& b : pool)
        if (b.p) cudaFreeAsync(b.p, b.s);
    pool.clear();
}

struct Reader {
    const uint8_t* p;
    size_t n, off = 0;
    bool bad = false;
    template <class T>
    void get(T* dst, size_t cnt) {
        size_t b = cnt * sizeof(T);
        if (bad || b / sizeof(T) != cnt || off + b > n) { bad = true; return; }
        if (b) memcpy(dst, p + off, b);
        off += b;
    }
    template <class T>
    std::vector<T> vec(size_t cnt) {
        if (bad || cnt > (n - off) / sizeof(T)) { bad = true; return {}; }
        std::vector<T> v(cnt);
        get(v.data(), cnt);
        return v;
    }
    // The next cnt elements of type T, left in place (no host copy; possibly unaligned, so read
    // them on the host with memcpy only).
    template <class T>
    const uint8_t* raw(size_t cnt) {
        if (bad || cnt > (n - off) / sizeof(T)) { bad = true; return nullptr; }
        const uint8_t* q = p + off;
        off += cnt * sizeof(T);
        return q;
    }
};

// Load-time kernels: the scene's large per-point arrays are copied to the device as they lie
// in the file and re-laid out there.
__global__ void k_load_pack4(const float* __restrict__ src, float4* __restrict__ dst, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = make_float4(src[3 * i], src[3 * i + 1], src[3 * i + 2], 0.f);
}
// static triangles (9 floats: v0, e1, e2) as three float4 each, for 16-byte loads
__global__ void k_load_tri4(const float* __restrict__ src, float4* __restrict__ dst, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float* t = src + 9 * i;
        dst[3 * i] = make_float4(t[0], t[1], t[2], t[3]);
        dst[3 * i + 1] = make_float4(t[4], t[5], t[6], t[7]);
        dst[3 * i + 2] = make_float4(t[8], 0.f, 0.f, 0.f);
    }
}
__global__ void k_load_pad(const float* __restrict__ src, float* __restrict__ dst, size_t n, int nl, int lcs) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        for (int l = 0; l < lcs; ++l) dst[(size_t)lcs * i + l] = l < nl ? src[(size_t)nl * i + l] : 0.f;
}
__global__ void k_load_check(const int* __restrict__ v, size_t n, int lo, int hi, unsigned* __restrict__ bad, unsigned bit) {
    bool out = false;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out |= v[i] < lo || v[i] >= hi;
    if (__any_sync(0xffffffffu, out) && (threadIdx.x & 31) == 0) atomicOr(bad, bit);
}
__global__ void k_fill(float* __restrict__ dst, size_t n, float v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) dst[i] = v;
}
// Rows of 4-byte elements between a padded device layout (ss per row) and a packed one (ds per
// row, ds <= ss): one contiguous host copy of the packed rows instead of a 2-D copy of
// millions of 12-byte rows.  Unpacking leaves the padding of each row as it was.
__global__ void k_pack_rows(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, size_t rows, int ds, int ss) {
    const size_t n = rows * (size_t)ds;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const size_t r = t / (size_t)ds, k = t - r * ds;
        dst[t] = src[r * ss + k];
    }
}
__global__ void k_unpack_rows(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, size_t rows, int ds, int ss) {
    const size_t n = rows * (size_t)ds;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const size_t r = t / (size_t)ds, k = t - r * ds;
        dst[r * ss + k] = src[t];
    }
}
constexpr unsigned LOAD_BAD_REGION = 1u, LOAD_BAD_HASH = 2u;
int load_grid(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 4096); }

// Device copy of `bytes` bytes at `src` (host) into a new buffer of the pool.
template <class T>
rc_status dput_raw(rc_ctx* ctx, std::vector<DevBuf>& pool, const T** out, const uint8_t* src, size_t cnt, cudaStream_t on = nullptr) {
    T* p = nullptr;
    rc_status s = dalloc(ctx, pool, &p, cnt, on);
    if (s != RC_OK) return s;
    if (cnt) CKR(cudaMemcpyAsync(p, src, cnt * sizeof(T), cudaMemcpyHostToDevice, on ? on : ctx->stream));
    *out = p;
    return RC_OK;
}

// The small host arrays of a scene (lights, quads, triangles, groups, intensities, event lists),
// gathered into one host block and sent with one copy per flush into one buffer of the pool: about a
// hundred small copies from pageable memory cost more than the 139 MB of per-point arrays.
struct Stage {
    struct Item { void** slot; size_t off; };
    std::vector<uint8_t> host;
    std::vector<Item> items;
    template <class T>
    void add(const T** out, const std::vector<T>& v) {
        const size_t off = (host.size() + 255) & ~(size_t)255;
        host.resize(off + v.size() * sizeof(T));
        if (!v.empty()) memcpy(host.data() + off, v.data(), v.size() * sizeof(T));
        items.push_back({reinterpret_cast<void**>(const_cast<T**>(out)), off});
    }
    rc_status flush(rc_ctx* ctx, std::vector<DevBuf>& pool) {
        if (items.empty()) return RC_OK;
        uint8_t* p = nullptr;
        rc_status s = dalloc(ctx, pool, &p, host.size());
        if (s != RC_OK) return s;
        if (!host.empty()) CKR(cudaMemcpyAsync(p, host.data(), host.size(), cudaMemcpyHostToDevice, ctx->stream));
        for (const Item& it : items) *it.slot = p + it.off;
        items.clear();
        host.clear();   // a copy from pageable memory has taken the bytes when it returns
        return RC_OK;
    }
};

// poc_gpu.cu:720-735: fine event grid (16 x 8 x 6 over the 8 x 4 x 3 m box) -> transit grid.
std::vector<int> to_grid(const std::vector<int>& fine, int VX, int VY, int VZ) {
    const int FX = 16, FY = 8, FZ = 6;
    const float X1 = 8.f, Y1 = 4.f, Z1 = 3.f;
    std::vector<char> mark((size_t)VX * VY * VZ, 0);
    for (int v : fine) {
        int i = v % FX, j = (v / FX) % FY, k = v / (FX * FY);
        float x0 = i * X1 / FX, x1 = (i + 1) * X1 / FX, y0 = j * Y1 / FY, y1 = (j + 1) * Y1 / FY;
        float z0 = k * Z1 / FZ, z1 = (k + 1) * Z1 / FZ;
        int a0 = std::min(int(x0 / X1 * VX + 1e-4f), VX - 1), a1 = std::min(int(x1 / X1 * VX - 1e-4f), VX - 1);
        int b0 = std::min(int(y0 / Y1 * VY + 1e-4f), VY - 1), b1 = std::min(int(y1 / Y1 * VY - 1e-4f), VY - 1);
        int c0 = std::min(int(z0 / Z1 * VZ + 1e-4f), VZ - 1), c1 = std::min(int(z1 / Z1 * VZ - 1e-4f), VZ - 1);
        for (int a = a0; a <= a1; ++a)
            for (int b = b0; b <= b1; ++b)
                for (int c = c0; c <= c1; ++c) mark[((size_t)c * VY + b) * VX + a] = 1;
    }
    std::vector<int> out;
    for (size_t v = 0; v < mark.size(); ++v)
        if (mark[v]) out.push_back((int)v);
    return out;
}

// Plane-culling groups of one state's dynamic triangles: consecutive triangles of one quad
// lying in the same axis-aligned plane (a quad's two triangles) form a group whose box is
// their bounding box grown by a margin; triangles that are not axis-aligned stay outside any
// group and are always tested exactly.  Groups are ordered by plane axis.
struct Groups {
    std::vector<float4> grp;
    std::vector<int> misc;
    GroupRanges gr{};
};
Groups build_groups(const std::vector<float>& T, const std::vector<int>& TQ, int nt) {
    struct G { int axis, j0, cnt; float c, lo[2], hi[2]; float line[4]; };
    std::vector<G> gs;
    std::vector<int> misc;
    auto axis_of = [&](int j) {
        const float* t = &T[9 * (size_t)j];
        for (int k = 0; k < 3; ++k)
            if (t[3 + k] == 0.f && t[6 + k] == 0.f) return k;
        return -1;
    };
    // in-plane axes in increasing order, as the kernel's filter reads them
    auto box = [&](int j, int k, float lo[2], float hi[2]) {
        const float* t = &T[9 * (size_t)j];
        const int ax[2] = {k == 0 ? 1 : 0, k == 2 ? 1 : 2};
        for (int u = 0; u < 2; ++u) {
            float v0 = t[ax[u]], v1 = t[ax[u]] + t[3 + ax[u]], v2 = t[ax[u]] + t[6 + ax[u]];
            lo[u] = std::min(v0, std::min(v1, v2));
            hi[u] = std::max(v0, std::max(v1, v2));
        }
    };
    // The line separating the two triangles of a group, in the in-plane axes (a, b):
    // n . (a, b) + w > eps holds on the first triangle's side, < -eps on the second's, with
    // eps far above the rounding of the crossing point the trace computes.  Groups whose
    // triangles do not share an edge with the third vertices on opposite sides get eps = inf.
    auto split_line = [&](int j, int k, float line[4]) {
        line[0] = line[1] = line[2] = 0.f;
        line[3] = INFINITY;
        const int ax[2] = {k == 0 ? 1 : 0, k == 2 ? 1 : 2};
        double V[2][3][2];
        double scale = 0.0;
        for (int t = 0; t < 2; ++t) {
            const float* tr = &T[9 * (size_t)(j + t)];
            for (int u = 0; u < 2; ++u) {
                V[t][0][u] = tr[ax[u]];
                V[t][1][u] = (double)(tr[ax[u]] + tr[3 + ax[u]]);
                V[t][2][u] = (double)(tr[ax[u]] + tr[6 + ax[u]]);
            }
            for (int v = 0; v < 3; ++v) scale = std::max(scale, std::max(fabs(V[t][v][0]), fabs(V[t][v][1])));
        }
        const double tol = 1e-6 * (1.0 + scale);
        int sa[2], sb[2], ns = 0;
        for (int x = 0; x < 3 && ns < 3; ++x)
            for (int y = 0; y < 3; ++y)
                if (fabs(V[0][x][0] - V[1][y][0]) <= tol && fabs(V[0][x][1] - V[1][y][1]) <= tol) {
                    if (ns < 2) { sa[ns] = x; sb[ns] = y; }
                    ++ns;
                    break;
                }
        if (ns != 2) return;
        const double* e0 = V[0][sa[0]];
        const double* e1 = V[0][sa[1]];
        double na = -(e1[1] - e0[1]), nb = e1[0] - e0[0];
        const double len = sqrt(na * na + nb * nb);
        if (!(len > tol)) return;
        na /= len; nb /= len;
        double w = -(na * e0[0] + nb * e0[1]);
        const int ta = 3 - sa[0] - sa[1], tb = 3 - sb[0] - sb[1];
        double da = na * V[0][ta][0] + nb * V[0][ta][1] + w, db = na * V[1][tb][0] + nb * V[1][tb][1] + w;
        if (da < 0) { na = -na; nb = -nb; w = -w; da = -da; db = -db; }
        if (!(da > tol && db < -tol)) return;
        line[0] = (float)na;
        line[1] = (float)nb;
        line[2] = (float)w;
        line[3] = (float)(2e-3 + 1e-4 * len + 1e-5 * scale);
    };
    int j = 0;
    while (j < nt) {
        const int k = axis_of(j);
        if (k < 0) { misc.push_back(j); ++j; continue; }
        G g{};
        g.line[3] = INFINITY;
        g.axis = k;
        g.j0 = j;
        g.c = T[9 * (size_t)j + k];
        g.cnt = 1;
        box(j, k, g.lo, g.hi);
        if (j + 1 < nt && TQ[j + 1] == TQ[j] && axis_of(j + 1) == k && T[9 * (size_t)(j + 1) + k] == g.c) {
            float lo2[2], hi2[2];
            box(j + 1, k, lo2, hi2);
            for (int u = 0; u < 2; ++u) { g.lo[u] = std::min(g.lo[u], lo2[u]); g.hi[u] = std::max(g.hi[u], hi2[u]); }
            g.cnt = 2;
            split_line(j, k, g.line);
        }
        gs.push_back(g);
        j += g.cnt;
    }
    Groups out;
    // up to 3 padding groups (one per axis) must still fit in the candidate mask
    constexpr int MAX_REAL = MAX_GROUPS - 3;
    if ((int)gs.size() > MAX_REAL) {
        std::stable_sort(gs.begin(), gs.end(), [](const G& a, const G& b) {
            return (a.hi[0] - a.lo[0]) * (a.hi[1] - a.lo[1]) > (b.hi[0] - b.lo[0]) * (b.hi[1] - b.lo[1]);
        });
        for (size_t x = MAX_REAL; x < gs.size(); ++x)
            for (int t = 0; t < gs[x].cnt; ++t) misc.push_back(gs[x].j0 + t);
        gs.resize(MAX_REAL);
    }
    std::stable_sort(gs.begin(), gs.end(), [](const G& a, const G& b) { return a.axis < b.axis; });
    int cnt[3] = {0, 0, 0};
    for (auto& g : gs) cnt[g.axis]++;
    {
        // pad every axis to an even count: the filter tests groups two at a time
        std::vector<G> padded;
        size_t x = 0;
        for (int k = 0; k < 3; ++k) {
            for (int n = 0; n < cnt[k]; ++n) padded.push_back(gs[x++]);
            if (cnt[k] & 1) {
                G pad{};
                pad.axis = k;
                pad.c = NAN;
                pad.line[3] = INFINITY;
                padded.push_back(pad);
                cnt[k]++;
            }
        }
        gs.swap(padded);
    }
    out.gr.g0[0] = 0;
    out.gr.g0[1] = cnt[0];
    out.gr.g0[2] = cnt[0] + cnt[1];
    out.gr.g0[3] = cnt[0] + cnt[1] + cnt[2];
    for (auto& g : gs) {
        // centre and half extent of the box grown by the margin, in double so the float box
        // still contains the grown box
        float ctr[2], half[2];
        for (int u = 0; u < 2; ++u) {
            const double m = 2e-3 + 1e-4 * ((double)g.hi[u] - g.lo[u]) + 1e-6 * (fabs((double)g.lo[u]) + fabs((double)g.hi[u]));
            const double lo = (double)g.lo[u] - m, hi = (double)g.hi[u] + m;
            ctr[u] = (float)(0.5 * (lo + hi));
            half[u] = (float)(0.5 * (hi - lo) + 1e-6 * (fabs(lo) + fabs(hi)));
        }
        int j0 = g.j0, c = g.cnt, z = 0;
        float fj0, fc, fz;
        memcpy(&fj0, &j0, 4); memcpy(&fc, &c, 4); memcpy(&fz, &z, 4);
        out.grp.push_back(make_float4(g.c, ctr[0], half[0], ctr[1]));
        out.grp.push_back(make_float4(half[1], fj0, fc, fz));
        out.grp.push_back(make_float4(g.line[0], g.line[1], g.line[2], g.line[3]));
    }
    for (size_t x = 0; x + 1 < gs.size(); x += 2) {
        const float4 a0 = out.grp[3 * x], a1 = out.grp[3 * x + 1], b0 = out.grp[3 * x + 3], b1 = out.grp[3 * x + 4];
        out.grp.push_back(make_float4(-a0.x, -b0.x, -a0.y, -b0.y));
        out.grp.push_back(make_float4(-a0.z, -b0.z, -a0.w, -b0.w));
        out.grp.push_back(make_float4(-a1.x, -b1.x, 0.f, 0.f));
    }
    std::sort(misc.begin(), misc.end());
    out.misc = misc;
    return out;
}

rc_status build_state(rc_ctx* ctx, Scene& S, int k, cudaStream_t st);
rc_status ensure_side(rc_ctx* ctx, int ns);
rc_status side_after_stream(rc_ctx* ctx);

rc_status load_scene(rc_ctx* ctx, const uint8_t* data, size_t n) {
    Reader r{data, n};
    int h[8];
    r.get(h, 8);
    if (r.bad) return fail(ctx, RC_ERR_FORMAT, "scene: truncated header");
    if (h[7] != 2 && h[7] != 3) return fail(ctx, RC_ERR_FORMAT, "scene format %d not supported (2 or 3)", h[7]);
    if (h[0] <= 0 || h[1] < 0 || h[2] < 0 || h[3] <= 0 || h[4] <= 0 || h[5] <= 0)
        return fail(ctx, RC_ERR_FORMAT, "scene: bad header");
    if (ctx->cfg.expect_lights > 0 && h[4] != ctx->cfg.expect_lights)
        return fail(ctx, RC_ERR_LIGHTS, "scene has %d lights, this build expects %d", h[4], ctx->cfg.expect_lights);
    if (!supported_nl_nw(h[4], ctx->NW)) return fail(ctx, RC_ERR_UNSUPPORTED, "%d lights with %d mask words not built", h[4], ctx->NW);
    Scene S;
    S.Np = h[0]; S.Nq = h[1]; S.Nt = h[2]; S.NS = h[3]; S.NL = h[4]; S.NR = h[5]; S.has_ref = h[6]; S.fmt = h[7];
    const int NL = S.NL, NW = ctx->NW;
    const size_t Np = (size_t)S.Np;
    S.grid.lo[0] = S.grid.lo[1] = S.grid.lo[2] = 0.f;
    S.grid.ext[0] = 8.f; S.grid.ext[1] = 4.f; S.grid.ext[2] = 3.f;
    S.grid.vx = ctx->cfg.grid[0]; S.grid.vy = ctx->cfg.grid[1]; S.grid.vz = ctx->cfg.grid[2];
    auto& pool = ctx->scene_bufs;
    DStatic& g = S.g;
    memset(&g, 0, sizeof g);
    CKR(cudaMemsetAsync(ctx->flags_dev + 2, 0, sizeof(unsigned), ctx->stream));   // load checks
    if (S.fmt == 3) {
        int m[4];
        r.get(S.grid.lo, 3); r.get(S.grid.ext, 3); r.get(&S.hcell, 1); r.get(m, 4);
        if (r.bad || m[0] < 0 || m[1] <= 0 || m[2] <= 0 || (m[2] & (m[2] - 1)) || m[3] < 0)
            return fail(ctx, RC_ERR_FORMAT, "scene: bad mesh block");
        S.nst = m[0]; S.nnodes = m[1]; S.hsize = m[2]; S.npst = m[3];
        const uint8_t* ST = r.raw<float>(9 * (size_t)m[0]);
        const uint8_t* STN = r.raw<float>(4 * (size_t)m[0]);
        const uint8_t* BN = r.raw<float>(8 * (size_t)m[1]);
        const uint8_t* HK = r.raw<unsigned long long>((size_t)m[2]);
        const uint8_t* HV = r.raw<int>((size_t)m[2]);
        if (r.bad) return fail(ctx, RC_ERR_FORMAT, "scene: truncated mesh block");
        // every node link and leaf range must stay inside the arrays the traversal reads (the
        // state build traverses the tree, so this is checked before anything runs)
        for (int k = 0; k < m[1]; ++k) {
            int lf, cnt;
            memcpy(&lf, BN + 4 * (8 * (size_t)k + 3), 4);
            memcpy(&cnt, BN + 4 * (8 * (size_t)k + 7), 4);
            if (cnt > 0) { if (lf < 0 || (long long)lf + cnt > m[0]) return fail(ctx, RC_ERR_FORMAT, "BVH leaf %d out of range", k); }
            else if (lf < 0 || lf + 1 >= m[1]) return fail(ctx, RC_ERR_FORMAT, "BVH node %d child out of range", k);
        }
        if (!(S.hcell > 0.f)) return fail(ctx, RC_ERR_FORMAT, "hash cell size");
        rc_status s;
        if ((s = dput_raw(ctx, pool, &g.ST, ST, 9 * (size_t)m[0])) || (s = dput_raw(ctx, pool, (const float**)&g.STN, STN, 4 * (size_t)m[0])) ||
            (s = dput_raw(ctx, pool, (const float**)&g.BN, BN, 8 * (size_t)m[1])) ||
            (s = dput_raw(ctx, pool, &g.HK, HK, (size_t)m[2])) || (s = dput_raw(ctx, pool, &g.HV, HV, (size_t)m[2])))
            return s;
        {
            float4* st4 = nullptr;
            if ((s = dalloc(ctx, pool, &st4, 3 * (size_t)m[0]))) return s;
            k_load_tri4<<<load_grid((size_t)m[0]), 256, 0, ctx->stream>>>(g.ST, st4, (size_t)m[0]);
            CKR(cudaGetLastError());
            g.ST4 = st4;
        }
        // hash values are cache point ids or -1; checked on the device, read back before the load returns
        k_load_check<<<load_grid((size_t)m[2]), 256, 0, ctx->stream>>>(g.HV, (size_t)m[2], -1, S.Np, ctx->flags_dev + 2, LOAD_BAD_HASH);
        CKR(cudaGetLastError());
        g.hmask = (unsigned)m[2] - 1u;
        g.hcell = S.hcell;
        g.has_bvh = 1;
        g.nnodes = m[1];
        g.max_visits = 4 * m[1] + 64;
        g.watertight = (ctx->cfg.flags & RC_FLAG_WATERTIGHT) != 0;
    }
    set_grid_scale(S.grid);
    auto L = r.vec<float>(3 * (size_t)NL);
    S.hL = L;
    const uint8_t* A = r.raw<float>(Np);
    const uint8_t* region = r.raw<int>(Np);
    if (r.bad) return fail(ctx, RC_ERR_FORMAT, "scene: truncated");
    rc_status s;
    CKR(RC_DISPATCH(NL, preload(NW)));
    Stage stage;
    stage.add(&S.L, L);
    if ((s = dput_raw(ctx, pool, &g.A, A, Np)) || (s = dput_raw(ctx, pool, &g.region, region, Np))) return s;
    // region ids index the per-region statistics; checked on the device (no frame runs before
    // the load has read the result back)
    k_load_check<<<load_grid(Np), 256, 0, ctx->stream>>>(g.region, Np, 0, S.NR, ctx->flags_dev + 2, LOAD_BAD_REGION);
    CKR(cudaGetLastError());
    S.st.resize(S.NS);
    // RC_FLAG_LOAD_ASYNC: every state's per-point arrays go on the side stream (the load returns
    // once the global arrays are checked; the caller keeps its buffer until rc_sync)
    const bool async = (ctx->cfg.flags & RC_FLAG_LOAD_ASYNC) != 0;
    if (async && (s = ensure_side(ctx, S.NS))) return s;
    for (int k = 0; k < S.NS; ++k) {
        HostState& hs = S.st[k];
        hs.inten = r.vec<float>(NL);
        const uint8_t* P = r.raw<float>(3 * Np);
        const uint8_t* N = r.raw<float>(3 * Np);
        auto Q = r.vec<float>(12 * (size_t)S.Nq);
        auto dims = r.vec<int>(2 * (size_t)S.Nq), off = r.vec<int>((size_t)S.Nq);
        if (k == 0) { S.hdims = dims; S.hoff = off; }
        auto T = r.vec<float>(9 * (size_t)S.Nt);
        auto TQ = r.vec<int>((size_t)S.Nt);
        const uint8_t *ref = nullptr, *valid = nullptr, *Pw = nullptr;
        if (S.has_ref) { ref = r.raw<float>(Np); valid = r.raw<uint8_t>(Np); Pw = r.raw<float>((size_t)NL * Np); }
        if (r.bad) return fail(ctx, RC_ERR_FORMAT, "scene: truncated state %d", k);
        for (int q = 0; q < S.Nq; ++q)
            if (dims[2 * q] <= 0 || dims[2 * q + 1] <= 0 || off[q] < 0 ||
                (long long)off[q] + (long long)dims[2 * q] * dims[2 * q + 1] > S.Np)
                return fail(ctx, RC_ERR_FORMAT, "quad %d grid out of range", q);
        for (int t : TQ) if (t < 0 || t >= S.Nq) return fail(ctx, RC_ERR_FORMAT, "triangle quad id out of range");
        std::vector<float4> tri(3 * (size_t)S.Nt);
        for (int j = 0; j < S.Nt; ++j) {
            float qb;
            memcpy(&qb, &TQ[j], 4);
            const float* t = &T[9 * (size_t)j];
            tri[3 * j] = make_float4(t[0], t[1], t[2], qb);
            tri[3 * j + 1] = make_float4(t[3], t[4], t[5], 0.f);
            tri[3 * j + 2] = make_float4(t[6], t[7], t[8], 0.f);
        }
        Groups G = build_groups(T, TQ, S.Nt);
        DState& d = hs.d;
        memset(&d, 0, sizeof d);
        stage.add(&d.Q, Q);
        stage.add(&d.dims, dims);
        stage.add(&d.off, off);
        stage.add(&d.tri, tri);
        stage.add(&d.grp, G.grp);
        stage.add(&d.misc, G.misc);
        stage.add(&hs.dint, hs.inten);
        {
            // the per-point arrays are copied now and re-laid out when the state is built; with
            // RC_FLAG_LOAD_ASYNC they are copied on the side stream (state 0's first, then its
            // build, then the other states') and the load does not wait for them
            const bool side = async;
            cudaStream_t cs = side ? ctx->side : ctx->stream;
            float* raw = nullptr;
            const size_t nraw = (size_t)(6 + (S.has_ref ? NL : 0)) * Np;
            if ((s = dalloc(ctx, pool, &raw, nraw, cs))) return s;
            hs.raw_buf = pool.size() - 1;
            CKR(cudaMemcpyAsync(raw, P, 12 * Np, cudaMemcpyHostToDevice, cs));
            CKR(cudaMemcpyAsync(raw + 3 * Np, N, 12 * Np, cudaMemcpyHostToDevice, cs));
            if (S.has_ref) CKR(cudaMemcpyAsync(raw + 6 * Np, Pw, 4 * (size_t)NL * Np, cudaMemcpyHostToDevice, cs));
            hs.raw = raw;
            if (S.has_ref)
                if ((s = dput_raw(ctx, pool, &d.ref, ref, Np, cs)) || (s = dput_raw(ctx, pool, &d.valid, valid, Np, cs))) return s;
            if (side) {
                CKR(cudaEventRecord(ctx->copies_ev[k], cs));
                hs.copies_side = true;
            }
        }
        d.nt = S.Nt;
        d.ng = G.gr.g0[3];
        d.nmisc = (int)G.misc.size();
        d.gr = G.gr;
        size_t smem = frame_smem_bytes(d);
        if (smem > 200 * 1024) return fail(ctx, RC_ERR_UNSUPPORTED, "%d dynamic triangles exceed shared memory", S.Nt);
        if (k == 0) {
            // state 0's build (where runs usually begin) starts on the side stream as soon as its
            // arrays are on the device, while the other states' copies stream in
            if ((s = stage.flush(ctx, pool)) || (s = ensure_side(ctx, S.NS)) || (s = side_after_stream(ctx)) ||
                (s = build_state(ctx, S, 0, ctx->side)))
                return s;
            CKR(cudaEventRecord(ctx->state_ev[0], ctx->side));
            hs.wait = true;
        }
    }
    const int npairs = S.NS * S.NS;
    S.ev.resize((size_t)npairs * (1 + NL));
    for (int e = 0; e < npairs; ++e) {
        for (int kind = 0; kind <= NL; ++kind) {
            int cnt = 0;
            r.get(&cnt, 1);
            if (r.bad || cnt < 0) return fail(ctx, RC_ERR_FORMAT, "scene: truncated event lists");
            auto raw = r.vec<int>((size_t)cnt);
            if (r.bad) return fail(ctx, RC_ERR_FORMAT, "scene: truncated event lists");
            auto& dst = S.ev[(size_t)e * (1 + NL) + kind];
            if (S.fmt == 3) dst = raw;
            else {
                for (int v : raw) if (v < 0 || v >= 16 * 8 * 6) return fail(ctx, RC_ERR_FORMAT, "event voxel out of range");
                dst = to_grid(raw, S.grid.vx, S.grid.vy, S.grid.vz);
            }
            for (int v : dst) if (v < 0 || v >= S.grid.vx * S.grid.vy * S.grid.vz) return fail(ctx, RC_ERR_FORMAT, "event voxel out of range");
        }
    }
    S.ev_dev.assign(S.ev.size(), nullptr);
    for (size_t e = 0; e < S.ev.size(); ++e)
        if (!S.ev[e].empty()) stage.add(&S.ev_dev[e], S.ev[e]);
    if ((s = stage.flush(ctx, pool))) return s;
    unsigned bad = 0;
    CKR(cudaMemcpyAsync(&bad, ctx->flags_dev + 2, sizeof bad, cudaMemcpyDeviceToHost, ctx->stream));
    CKR(cudaStreamSynchronize(ctx->stream));
    if (bad & LOAD_BAD_REGION) return fail(ctx, RC_ERR_FORMAT, "region index out of range");
    if (bad & LOAD_BAD_HASH) return fail(ctx, RC_ERR_FORMAT, "hash value out of range");
    ctx->S = std::move(S);
    return RC_OK;
}

}  // namespace

namespace {

// A state's device build: positions and normals packed to float4, the warm start padded like
// the cache, the direct light and shadow-voxel masks (k_build); the raw copy is then released.
// Issued on stream `st`.
rc_status build_state(rc_ctx* ctx, Scene& S, int k, cudaStream_t st) {
    HostState& hs = S.st[k];
    const int NL = S.NL, NW = ctx->NW;
    const size_t Np = (size_t)S.Np;
    auto& pool = ctx->scene_bufs;
    DState& d = hs.d;
    float4 *P4 = nullptr, *N4 = nullptr, *AE = nullptr;
    uint32_t* SV = nullptr;
    rc_status s;
    if ((s = dalloc(ctx, pool, &P4, Np, st)) || (s = dalloc(ctx, pool, &N4, Np, st)) ||
        (s = dalloc(ctx, pool, &AE, (size_t)aes_of(NL) / 4 * Np, st)) || (s = dalloc(ctx, pool, &SV, (size_t)NW * Np, st)))
        return s;
    k_load_pack4<<<load_grid(Np), 256, 0, st>>>(hs.raw, P4, Np);
    k_load_pack4<<<load_grid(Np), 256, 0, st>>>(hs.raw + 3 * Np, N4, Np);
    CKR(cudaGetLastError());
    d.P4 = P4;
    d.N4 = N4;
    if (S.has_ref) {
        // warm start of every run beginning in this state (poc_gpu.cu:832), padded like the cache
        float* pw = nullptr;
        if ((s = dalloc(ctx, pool, &pw, (size_t)lcs_of(NL) * Np, st))) return s;
        k_load_pad<<<load_grid(Np), 256, 0, st>>>(hs.raw + 6 * Np, pw, Np, NL, lcs_of(NL));
        CKR(cudaGetLastError());
        hs.pw = pw;
    }
    CKR(RC_DISPATCH(NL, build(NW, d, S.g, S.grid, S.L, hs.dint, AE, SV, S.Np, ctx->flags_dev, st)));
    d.AE = AE;
    d.SV = SV;
    DevBuf& rb = pool[hs.raw_buf];
    if (rb.p == hs.raw) {
        cudaFreeAsync(rb.p, st);
        rb.p = nullptr;
        rb.n = 0;
    }
    hs.raw = nullptr;
    hs.built = true;
    ctx->launches += 3 + (S.has_ref ? 1 : 0);
    return RC_OK;
}
// State k's build issued on the side stream (behind the load's copies, which the side stream
// waits for once, at the load), unless it is built or issued already; the context's stream waits
// for its event at first use.
rc_status prebuild_state(rc_ctx* ctx, int k) {
    HostState& hs = ctx->S.st[k];
    if (hs.built || !ctx->side) return RC_OK;
    rc_status s = build_state(ctx, ctx->S, k, ctx->side);
    if (s != RC_OK) return s;
    CKR(cudaEventRecord(ctx->state_ev[k], ctx->side));
    hs.wait = true;
    return RC_OK;
}
// Before the context's stream uses state k: wait for its build on the side stream, or build it;
// then issue the next state's build on the side stream, so that a run moving through the states
// in order finds each one built (a state that is never used is never built).
rc_status ensure_state(rc_ctx* ctx, int k) {
    Scene& S = ctx->S;
    if (k < 0 || k >= S.NS) return fail(ctx, RC_ERR_ARG, "state %d out of range", k);
    HostState& hs = S.st[k];
    if (hs.built) {
        if (hs.wait) {
            CKR(cudaStreamWaitEvent(ctx->stream, ctx->state_ev[k], 0));
            hs.wait = false;
        }
    } else {
        if (hs.copies_side) CKR(cudaStreamWaitEvent(ctx->stream, ctx->copies_ev[k], 0));
        rc_status s = build_state(ctx, S, k, ctx->stream);
        if (s != RC_OK) return s;
    }
    return S.NS > 1 ? prebuild_state(ctx, (k + 1) % S.NS) : RC_OK;
}
rc_status ensure_all_states(rc_ctx* ctx) {
    for (int k = 0; k < ctx->S.NS; ++k) {
        rc_status s = ensure_state(ctx, k);
        if (s != RC_OK) return s;
    }
    return RC_OK;
}
// The side stream and the per-state events (created once per context, grown with the scene).
rc_status ensure_side(rc_ctx* ctx, int ns) {
    if (!ctx->side) CKR(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
    if (!ctx->load_ev) CKR(cudaEventCreateWithFlags(&ctx->load_ev, cudaEventDisableTiming));
    while ((int)ctx->state_ev.size() < ns) {
        cudaEvent_t e = nullptr, c = nullptr;
        CKR(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->state_ev.push_back(e);
        CKR(cudaEventCreateWithFlags(&c, cudaEventDisableTiming));
        ctx->copies_ev.push_back(c);
    }
    return RC_OK;
}
// The side stream waits for everything the context's stream has queued (the load's copies).
rc_status side_after_stream(rc_ctx* ctx) {
    CKR(cudaEventRecord(ctx->load_ev, ctx->stream));
    CKR(cudaStreamWaitEvent(ctx->side, ctx->load_ev, 0));
    return RC_OK;
}
// After a load: the side stream waits for all of the load's copies (state 0's build was issued
// by the load itself, behind its own copies); the other states are built ahead of first use.
rc_status issue_state_builds(rc_ctx* ctx) {
    rc_status s = ensure_side(ctx, ctx->S.NS);
    if (s != RC_OK) return s;
    if ((s = side_after_stream(ctx)) != RC_OK) return s;
    return prebuild_state(ctx, 0);
}

rc_status alloc_cache(rc_ctx* ctx) {
    free_pool(ctx->cache_bufs);
    ctx->err_cap = 0;
    const Scene& S = ctx->S;
    const size_t Np = (size_t)S.Np, LCS = (size_t)lcs_of(S.NL), NW = (size_t)ctx->NW, NR = (size_t)S.NR;
    const size_t G = (Np + BLOCK - 1) / BLOCK;
    DevCache& c = ctx->c;
    auto& pool = ctx->cache_bufs;
    rc_status s;
    if ((s = dalloc(ctx, pool, &c.Lc, LCS * Np)) || (s = dalloc(ctx, pool, &c.Lc2, LCS * Np)) ||
        (s = dalloc(ctx, pool, &c.m, LCS * Np)) || (s = dalloc(ctx, pool, &c.n, Np)) || (s = dalloc(ctx, pool, &c.c0, Np)) ||
        (s = dalloc(ctx, pool, &c.kk, Np)) || (s = dalloc(ctx, pool, &c.pending, Np)) || (s = dalloc(ctx, pool, &c.cur, NW * Np)) ||
        (s = dalloc(ctx, pool, &c.prev, NW * Np)) || (s = dalloc(ctx, pool, &c.stale, Np)) || (s = dalloc(ctx, pool, &c.age, Np)) ||
        (s = dalloc(ctx, pool, &c.snap, (size_t)KSNAP * Np * LCS)) || (s = dalloc(ctx, pool, &c.neq, NR * NEQ)) ||
        (s = dalloc(ctx, pool, &c.coef, NR * KSNAP)) || (s = dalloc(ctx, pool, &c.rstat, 4 * NR)) ||
        (s = dalloc(ctx, pool, &c.dstat, 3 * NR)) || (s = dalloc(ctx, pool, &c.sumpr, 2)) || (s = dalloc(ctx, pool, &c.npend, 2)) ||
        (s = dalloc(ctx, pool, &c.partf, G)) || (s = dalloc(ctx, pool, &c.partd, 3 * G)) || (s = dalloc(ctx, pool, &c.parti, G)) ||
        (s = dalloc(ctx, pool, &c.ticket, 4)) || (s = dalloc(ctx, pool, &c.check, 2)) || (s = dalloc(ctx, pool, &c.rays, 1)) ||
        (s = dalloc(ctx, pool, &c.pracc, 1)) || (s = dalloc(ctx, pool, &c.npacc, 1)))
        return s;
    c.pre_hit = nullptr;
    c.rayq = nullptr;
    c.rayctr = nullptr;
    // the traced-ahead hits and the traversal's work counters; the ray queue only when asked for
    if (S.g.has_bvh && ((s = dalloc(ctx, pool, &c.pre_hit, (size_t)PRE_K * Np)) || (s = dalloc(ctx, pool, &c.rayctr, 2)) ||
                        ((ctx->cfg.flags & RC_FLAG_RAY_QUEUE) && (s = dalloc(ctx, pool, &c.rayq, 2 * (size_t)PRE_K * Np)))))
        return s;
    CKR(cudaMemsetAsync(c.ticket, 0, 16, ctx->stream));
    CKR(cudaMemsetAsync(c.check, 0, 16, ctx->stream));
    CKR(cudaMemsetAsync(c.pracc, 0, 8, ctx->stream));
    CKR(cudaMemsetAsync(c.npacc, 0, 8, ctx->stream));
    CKR(cudaMemsetAsync(c.snap, 0, (size_t)KSNAP * Np * LCS * 4, ctx->stream));
    CKR(cudaMemsetAsync(c.m, 0, LCS * Np * 4, ctx->stream));
    CKR(cudaMemsetAsync(c.kk, 0, Np * 4, ctx->stream));
    CKR(cudaMemsetAsync(c.c0, 0, Np * 4, ctx->stream));
    CKR(cudaMemsetAsync(c.neq, 0, NR * NEQ * 4, ctx->stream));
    CKR(cudaMemsetAsync(c.coef, 0, NR * KSNAP * 4, ctx->stream));
    CKR(cudaMemsetAsync(c.rstat, 0, 4 * NR * 4, ctx->stream));
    CKR(cudaMemsetAsync(c.dstat, 0, 3 * NR * 4, ctx->stream));
    c.flags = ctx->flags_dev;
    c.err = nullptr;
    double b = 0;
    for (auto& x : pool) b += (double)x.n;
    ctx->cache_bytes = b;
    return RC_OK;
}

rc_status ensure_err(rc_ctx* ctx, size_t frames) {
    if (frames <= ctx->err_cap) return RC_OK;
    size_t cap = std::max<size_t>(1024, frames * 2);
    double* p = nullptr;
    std::vector<DevBuf> fresh;
    rc_status s = dalloc(ctx, fresh, &p, cap * 3);
    if (s != RC_OK) return s;
    if (ctx->c.err) {
        CKR(cudaMemcpyAsync(p, ctx->c.err, ctx->err_cap * 3 * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        for (auto it = ctx->cache_bufs.begin(); it != ctx->cache_bufs.end(); ++it)
            if (it->p == ctx->c.err) { cudaFreeAsync(it->p, it->s); ctx->cache_bufs.erase(it); break; }
    }
    ctx->cache_bufs.push_back(fresh[0]);
    ctx->c.err = p;
    ctx->err_cap = cap;
    return RC_OK;
}

// One event of Runner::run (poc_gpu.cu:856-943) as an event program for k_event.
struct EvBuilder {
    EvProgram ev{};
    // pending-count bookkeeping of the reference: every verification step resets the count
    // (cudaMemset of npend) and publishes its own count; a restore without verification
    // leaves it at zero
    int last_reset = -1;
    bool any_count = false;
    bool zero_after = false;
    bool ok = true;
    EvOp& add(int kind) {
        if (ev.nops >= MAX_EV_OPS) { ok = false; return ev.ops[MAX_EV_OPS - 1]; }
        EvOp& o = ev.ops[ev.nops++];
        memset(&o, 0, sizeof o);
        o.kind = kind;
        return o;
    }
    void counting_op(EvOp& o) {
        last_reset = ev.nops - 1;
        any_count = true;
        zero_after = false;
        o.count = 1;
    }
    void finish() {
        for (int k = 0; k < ev.nops; ++k)
            if (ev.ops[k].count && k != last_reset) ev.ops[k].count = 0;
        ev.npend_mode = zero_after ? 2 : (any_count ? 1 : 0);
    }
};

rc_status do_event(rc_ctx* ctx, int e, int si) {
    Scene& S = ctx->S;
    Run& R = ctx->run;
    const rc_method& M = R.M;
    const int NL = S.NL, f = R.f;
    const int pe = e * S.NS + si;
    EvBuilder B;
    B.ev.Np = S.Np;
    B.ev.NR = S.NR;
    B.ev.nmax = R.nmax;
    if (M.snaps && f - R.last_event_f >= 20) {
        int k = -1;
        for (int a = 0; a < R.nslots; ++a) if (R.slot_state[a] == e) k = a;
        if (k < 0) { if (R.nslots < KSNAP) k = R.nslots++; else { k = R.slot_next; R.slot_next = (R.slot_next + 1) % KSNAP; } }
        R.slot_state[k] = e;
        EvOp& o = B.add(EV_SNAP_SAVE);
        o.a = k;
    }
    if (M.oracle && S.has_ref) {
        EvOp& o = B.add(EV_ORACLE);
        o.r0 = S.st[e].d.ref;
        o.r1 = S.st[si].d.ref;
    }
    auto rescale = [&](int l, float ratio) {
        EvOp& o = B.add(EV_RESCALE);
        o.a = l;
        o.x = ratio;
    };
    if (M.rescale && !M.deps) {
        for (int l = 0; l < NL; ++l) {
            float a = S.st[e].inten[l], b = S.st[si].inten[l];
            if (a == b) continue;
            if (M.memory && a > 0 && b == 0) { R.dormant |= 1 << l; R.ilearn[l] = a; }
            else if (M.memory && a == 0 && b > 0 && ((R.dormant >> l) & 1)) { rescale(l, b / R.ilearn[l]); R.dormant &= ~(1 << l); }
            else if (a > 0) rescale(l, b / a);
        }
    }
    if (M.deps) {
        int woke = 0;
        for (int l = 0; l < NL; ++l) {
            float a = S.st[e].inten[l], b = S.st[si].inten[l];
            if (a == b) continue;
            if (M.memory && a > 0 && b == 0) { R.dormant |= 1 << l; R.ilearn[l] = a; }
            else if (M.memory && a == 0 && b > 0 && ((R.dormant >> l) & 1)) {
                rescale(l, b / R.ilearn[l]);
                R.dormant &= ~(1 << l);
                woke |= 1 << l;
                EvOp& o = B.add(EV_WAKE);
                o.a = l;
                o.b = M.wake_verify ? 1 : 0;
                o.dormant = R.dormant;
                if (M.wake_verify) {
                    B.counting_op(o);
                    B.ev.zero_rstat = 1;
                    R.pend_left = VERIF_FRAMES;
                }
            } else if (a > 0) rescale(l, b / a);
        }
        for (int l = 0; l < NL; ++l) {
            const auto& V = S.ev[(size_t)pe * (1 + NL) + 1 + l];
            if (!V.empty() && !((woke >> l) & 1)) {
                EvOp& o = B.add(EV_TOUCHED);
                o.a = 0;
                o.b = (int)V.size();
                o.list = S.ev_dev[(size_t)pe * (1 + NL) + 1 + l];
                o.dormant = R.dormant;
            }
        }
        const auto& occ = S.ev[(size_t)pe * (1 + NL)];
        if (!occ.empty()) {
            if (M.verify) {
                EvOp& o = B.add(EV_TOUCHED);
                o.a = 1;
                o.b = (int)occ.size();
                o.list = S.ev_dev[(size_t)pe * (1 + NL)];
                o.dormant = R.dormant;
                B.counting_op(o);
                B.ev.zero_rstat = 1;
                R.pend_left = VERIF_FRAMES;
            } else if (R.dormant) {
                EvOp& o = B.add(EV_TOUCHED);
                o.a = 2;
                o.b = (int)occ.size();
                o.list = S.ev_dev[(size_t)pe * (1 + NL)];
                o.dormant = R.dormant;
            }
        }
    }
    if (M.snaps) {
        int hit = -1;
        for (int a = 0; a < R.nslots; ++a) if (R.slot_state[a] == si) hit = a;
        if (hit >= 0) {
            EvOp& o = B.add(EV_SNAP_RESTORE);
            o.a = hit;
            EvOp& r = B.add(EV_RESTORED);
            r.a = M.snap_verify ? 1 : 0;
            r.dormant = R.dormant;
            if (M.snap_verify) {
                B.counting_op(r);
                B.ev.zero_rstat = 1;
                R.pend_left = VERIF_FRAMES;
            } else {
                B.zero_after = true;
                B.any_count = false;
                B.last_reset = -1;
                R.pend_left = 0;
            }
            R.proj_left = 0;
        } else if (M.proj && R.nslots >= 2) {
            R.projK = R.nslots;
            for (int a = 0; a < R.nslots; ++a) R.slot[a] = a;
            B.ev.zero_neq = 1;
            R.proj_left = PROJ_FRAMES;
        }
    }
    R.last_event_f = f;
    B.ev.want_sumpr = M.mode == 1 ? 1 : 0;
    B.ev.sum_slot = R.sum_cur;
    B.finish();
    if (!B.ok) return fail(ctx, RC_ERR_UNSUPPORTED, "event needs more than %d kernel steps", MAX_EV_OPS);
    if (B.ev.nops == 0 && !B.ev.want_sumpr && B.ev.npend_mode == 0 && !B.ev.zero_rstat && !B.ev.zero_neq) return RC_OK;
    CKR(RC_DISPATCH(NL, event(B.ev, ctx->c, ctx->stream)));
    ctx->run.last_kernels++;
    return RC_OK;
}

// poc_gpu.cu:966-988: per-region FP64 least squares of the snapshot projection (host).
void proj_solve(const std::vector<float>& q, std::vector<float>& cf, int NR, int K) {
    for (int r = 0; r < NR; ++r) {
        const float* Q = &q[(size_t)r * NEQ];
        if (Q[27] < 24.f) continue;
        double A[KSNAP][KSNAP + 1];
        int ix = 0;
        double tr = 0;
        for (int a = 0; a < K; ++a) for (int b = a; b < K; ++b) { A[a][b] = A[b][a] = Q[ix++]; }
        for (int a = 0; a < K; ++a) { A[a][K] = Q[21 + a]; tr += A[a][a]; }
        for (int a = 0; a < K; ++a) A[a][a] += 1e-3 * tr / K + 1e-9;
        bool ok = true;
        for (int a = 0; a < K && ok; ++a) {
            int pv = a;
            for (int b = a + 1; b < K; ++b) if (fabs(A[b][a]) > fabs(A[pv][a])) pv = b;
            if (fabs(A[pv][a]) < 1e-12) { ok = false; break; }
            for (int t = 0; t <= K; ++t) std::swap(A[a][t], A[pv][t]);
            for (int b = 0; b < K; ++b)
                if (b != a) { double m = A[b][a] / A[a][a]; for (int t = a; t <= K; ++t) A[b][t] -= m * A[a][t]; }
        }
        if (!ok) continue;
        bool sane = true;
        double x[KSNAP];
        for (int a = 0; a < K; ++a) { x[a] = A[a][K] / A[a][a]; if (!std::isfinite(x[a]) || fabs(x[a]) > 4.0) sane = false; }
        if (sane) for (int a = 0; a < K; ++a) cf[(size_t)r * KSNAP + a] = (float)x[a];
    }
}

FrameParams base_params(rc_ctx* ctx) {
    const Run& R = ctx->run;
    const rc_method& M = R.M;
    FrameParams p{};
    p.Np = ctx->S.Np;
    p.NR = ctx->S.NR;
    p.mode = M.mode;
    p.budget = M.budget * M.rays;
    p.nmax = R.nmax;
    p.seed = R.p.seed;
    p.frame = (uint32_t)R.f;
    p.pend_left = R.pend_left;
    p.dormant = R.dormant;
    p.resp_mask = M.resp_mask;
    p.nmax_resp = M.nmax_resp * M.rays;
    p.ddgi = M.ddgi ? 1 : 0;
    p.ddgi_h = M.ddgi_h;
    p.ddgi_thr = M.ddgi_thr;
    p.ddgi_clamp = M.ddgi_clamp ? 1 : 0;
    p.ramp = M.ramp ? 1 : 0;
    p.proj_left = R.proj_left;
    p.projK = R.projK;
    for (int a = 0; a < KSNAP; ++a) p.slot[a] = R.slot[a];
    p.rays = M.rays;
    p.sum_in = R.sum_cur;
    p.sum_out = 1 - R.sum_cur;
    p.brute = (ctx->cfg.flags & RC_FLAG_BRUTE_FORCE) ? 1 : 0;
    p.check = (ctx->cfg.flags & RC_FLAG_CHECK_TRACE) ? 1 : 0;
    p.half_inv_np = 0.5f / (float)ctx->S.Np;
    return p;
}

rc_status frame_impl(rc_ctx* ctx, int si, int want_err, rc_timers* tm) {
    if (rc_status es = ensure_state(ctx, si)) return es;
    Scene& S = ctx->S;
    Run& R = ctx->run;
    const rc_method& M = R.M;
    const int f = R.f;
    cudaStream_t st = ctx->stream;
    rc_status s;
    R.last_kernels = 0;
    R.last_event = 0;
    if (f > 0 && R.prev_state != si) {
        R.last_event = 1;
        if (tm) CKR(cudaEventRecord(ctx->ev[4], st));
        if ((s = do_event(ctx, R.prev_state, si)) != RC_OK) return s;
        if (tm) {
            CKR(cudaEventRecord(ctx->ev[5], st));
            CKR(cudaEventSynchronize(ctx->ev[5]));
            float ms;
            cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]);
            tm->event += ms;
            tm->events++;
        }
    }
    R.prev_state = si;
    const DState& d = S.st[si].d;
    FrameParams p = base_params(ctx);
    const bool rec_err = want_err && S.has_ref;
    if (rec_err && (s = ensure_err(ctx, (size_t)R.nerr + 1)) != RC_OK) return s;
    p.want_err = rec_err ? 1 : 0;
    p.err_frame = R.nerr;
    if (M.ddgi) CKR(cudaMemsetAsync(ctx->c.dstat, 0, 3 * (size_t)S.NR * 4, st));
    if (tm) CKR(cudaEventRecord(ctx->ev[0], st));
    const bool track = M.deps && (f % (M.track_every > 0 ? M.track_every : 1) == 0);
    if (M.deps && f % 32 == 0) {
        std::swap(ctx->c.cur, ctx->c.prev);
        p.mask_op = track ? MASK_FRESH : MASK_ZERO;
    } else {
        p.mask_op = track ? MASK_OR : MASK_NONE;
    }
    if (tm) CKR(cudaEventRecord(ctx->ev[1], st));
    const bool proj_apply_now = R.proj_left == 1;
    const bool fused = R.pend_left == 0 && R.proj_left == 0 && !M.ddgi;
    if (ctx->c.pre_hit && !(ctx->cfg.flags & RC_FLAG_CHECK_TRACE)) {
        // static-mesh scene: the traversal runs ahead in its own kernel
        p.pre_hit = ctx->c.pre_hit;
        p.pre_k = PRE_K;
        p.wavefront = (ctx->cfg.flags & RC_FLAG_RAY_QUEUE) != 0;
        CKR(RC_DISPATCH(S.NL, pretrace(d, S.g, S.grid, ctx->c, p, ctx->c.pre_hit, st)));
        R.last_kernels += p.wavefront ? 2 : 1;
    }
    if (fused) {
        CKR(RC_DISPATCH(S.NL, frame(ctx->NW, track, true, d, S.g, S.grid, ctx->c, p, st)));
        R.last_kernels += 1;
        if (tm) { CKR(cudaEventRecord(ctx->ev[2], st)); CKR(cudaEventRecord(ctx->ev[3], st)); }
    } else {
        CKR(RC_DISPATCH(S.NL, frame(ctx->NW, track, false, d, S.g, S.grid, ctx->c, p, st)));
        if (tm) CKR(cudaEventRecord(ctx->ev[2], st));
        FrameParams pu = p;
        pu.decide = R.pend_left > 0 ? 1 : 0;
        if (tm) CKR(cudaEventRecord(ctx->ev[3], st));
        if (proj_apply_now) pu.want_err = 0;
        CKR(RC_DISPATCH(S.NL, update(d, S.g, ctx->c, pu, st)));
        R.last_kernels += 2;
        if (R.pend_left > 0) R.pend_left--;
    }
    R.sum_cur = 1 - R.sum_cur;
    std::swap(ctx->c.Lc, ctx->c.Lc2);
    if (R.proj_left > 0 && --R.proj_left == 0) {
        const size_t nq = (size_t)S.NR * NEQ;
        std::vector<float> q(nq), cf((size_t)S.NR * KSNAP, NAN);
        CKR(cudaMemcpyAsync(q.data(), ctx->c.neq, nq * 4, cudaMemcpyDeviceToHost, st));
        CKR(cudaStreamSynchronize(st));
        proj_solve(q, cf, S.NR, R.projK);
        CKR(cudaMemcpyAsync(ctx->c.coef, cf.data(), cf.size() * 4, cudaMemcpyHostToDevice, st));
        FrameParams pp = base_params(ctx);
        CKR(RC_DISPATCH(S.NL, proj_apply(ctx->c, S.g, pp, st)));
        R.last_kernels += 1;
        CKR(cudaStreamSynchronize(st));   // cf lives on this stack frame
        R.pend_left = VERIF_FRAMES;
        if (rec_err) {
            FrameParams pe = base_params(ctx);
            pe.err_frame = R.nerr;
            CKR(RC_DISPATCH(S.NL, error(d, ctx->c, pe, st)));
            R.last_kernels += 1;
        }
    }
    if (tm) {
        CKR(cudaEventRecord(ctx->ev[6], st));
        CKR(cudaEventSynchronize(ctx->ev[6]));
        float a, b, dd, u;
        cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
        cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]);
        cudaEventElapsedTime(&dd, ctx->ev[2], ctx->ev[3]);
        cudaEventElapsedTime(&u, ctx->ev[3], ctx->ev[6]);
        tm->swap += a; tm->trace += b; tm->decide += dd; tm->update += u;
        tm->frames++;
    }
    if (rec_err) R.nerr++;
    R.last_fused = fused ? 1 : 0;
    ctx->launches += R.last_kernels;
    R.f = f + 1;
    return RC_OK;
}

}  // namespace

// ============================================================================ C ABI
namespace {

constexpr float TAA_ALPHA_R = 0.5f;   // poc_gpu.cu:1231
constexpr int TAA_RF = 4;

// fine event voxel of a light (host_vox_fine, poc_gpu.cu:1170-1173)
int taa_vox_fine(const float* p) {
    const int i = std::min(std::max(int(p[0] / 8.f * 16), 0), 15), j = std::min(std::max(int(p[1] / 4.f * 8), 0), 7),
              k = std::min(std::max(int(p[2] / 3.f * 6), 0), 5);
    return (k * 8 + j) * 16 + i;
}

// buffers, neighbourhoods and event voxel lists (run_taa_mode's set-up, poc_gpu.cu:1189-1222)
rc_status taa_alloc(rc_ctx* ctx) {
    free_pool(ctx->taa_bufs);
    TaaRun& t = ctx->taa;
    t = TaaRun{};
    const Scene& S = ctx->S;
    const size_t Np = (size_t)S.Np, NW = (size_t)ctx->NW;
    auto& pool = ctx->taa_bufs;
    // the quad grid of each point (state 0's grids, as the reference's neighbourhood table);
    // a point listed by two quads keeps the later one, as the table's rows would
    std::vector<int> qid(Np, -1);
    std::vector<int4> quad((size_t)std::max(S.Nq, 1));
    for (int q = 0; q < S.Nq; ++q) {
        const int nu = S.hdims[2 * q], nv = S.hdims[2 * q + 1], o = S.hoff[q];
        quad[q] = make_int4(o, nu, nv, 0);
        for (size_t i = (size_t)o; i < (size_t)o + (size_t)nu * nv; ++i) qid[i] = q;
    }
    const int* dq = nullptr;
    const int4* dquad = nullptr;
    rc_status s;
    if ((s = dalloc(ctx, pool, &t.x, Np)) || (s = dalloc(ctx, pool, &t.H, Np)) || (s = dalloc(ctx, pool, &t.H2, Np)) ||
        (s = dalloc(ctx, pool, &t.mu, Np)) || (s = dalloc(ctx, pool, &t.sg, Np)) || (s = dalloc(ctx, pool, &t.react, Np)) ||
        (s = dalloc(ctx, pool, &t.pend, Np)) || (s = dalloc(ctx, pool, &t.cur, NW * Np)) || (s = dalloc(ctx, pool, &t.prev, NW * Np)) ||
        (s = dalloc(ctx, pool, &t.rs, 3 * (size_t)S.NR)) || (s = dalloc(ctx, pool, &t.cnt, (size_t)S.NR)) ||
        (s = dalloc(ctx, pool, &t.part, 3 * (size_t)taa::post_blocks(S.Np))) || (s = dalloc(ctx, pool, &t.out, 3)) ||
        (s = dput(ctx, pool, &dq, qid)) || (s = dput(ctx, pool, &dquad, quad)))
        return s;
    t.qid = const_cast<int*>(dq);
    t.quad = dquad;
    const int NS = S.NS, NL = S.NL;
    t.dV.assign((size_t)NS * NS, nullptr);
    t.nV.assign((size_t)NS * NS, 0);
    for (int a = 0; a < NS; ++a)
        for (int b = 0; b < NS; ++b) {
            if (a == b) continue;
            std::vector<int> fine;
            for (int l = 0; l < NL; ++l)
                if (S.st[a].inten[l] != S.st[b].inten[l]) fine.push_back(taa_vox_fine(&S.hL[3 * (size_t)l]));
            std::vector<int> v = to_grid(fine, S.grid.vx, S.grid.vy, S.grid.vz);
            for (int x : S.ev[((size_t)a * NS + b) * (1 + NL)]) v.push_back(x);
            std::sort(v.begin(), v.end());
            v.erase(std::unique(v.begin(), v.end()), v.end());
            t.nV[(size_t)a * NS + b] = (int)v.size();
            const int* dv = nullptr;
            if ((s = dput(ctx, pool, &dv, v.empty() ? std::vector<int>{0} : v)) != RC_OK) return s;
            t.dV[(size_t)a * NS + b] = dv;
        }
    return RC_OK;
}

}  // namespace

extern "C" {

int rc_abi_version(void) { return RC_ABI_VERSION; }

const char* rc_status_string(rc_status s) {
    switch (s) {
        case RC_OK: return "ok";
        case RC_ERR_ARG: return "bad argument";
        case RC_ERR_IO: return "i/o error";
        case RC_ERR_FORMAT: return "bad scene format";
        case RC_ERR_CUDA: return "CUDA error";
        case RC_ERR_NOMEM: return "out of memory";
        case RC_ERR_STATE: return "call out of order";
        case RC_ERR_DEVICE: return "device guard tripped";
        case RC_ERR_UNSUPPORTED: return "unsupported configuration";
        case RC_ERR_LIGHTS: return "light count mismatch";
    }
    return "unknown status";
}

rc_status rc_create(const rc_config* cfg, rc_ctx** out) {
    if (!out) return RC_ERR_ARG;
    *out = nullptr;
    rc_ctx* ctx = new rc_ctx();
    if (cfg) ctx->cfg = *cfg;
    if (ctx->cfg.grid[0] <= 0 || ctx->cfg.grid[1] <= 0 || ctx->cfg.grid[2] <= 0) {
        ctx->cfg.grid[0] = 8; ctx->cfg.grid[1] = 4; ctx->cfg.grid[2] = 4;
    }
    const int nv = ctx->cfg.grid[0] * ctx->cfg.grid[1] * ctx->cfg.grid[2];
    if (nv % 128 != 0 || nv > 32 * 128) { delete ctx; return RC_ERR_UNSUPPORTED; }
    ctx->NW = nv / 32;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= ctx->cfg.device || ctx->cfg.device < 0) {
        cudaGetLastError();
        delete ctx;
        return RC_ERR_CUDA;
    }
    if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) { delete ctx; return RC_ERR_CUDA; }
    if (ctx->cfg.stream) ctx->stream = (cudaStream_t)ctx->cfg.stream;
    else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { delete ctx; return RC_ERR_CUDA; }
        ctx->own_stream = true;
    }
    for (auto& e : ctx->ev) cudaEventCreate(&e);
    if (cudaMalloc(&ctx->flags_dev, 16) != cudaSuccess || cudaMemset(ctx->flags_dev, 0, 16) != cudaSuccess) {
        rc_destroy(ctx);
        return RC_ERR_CUDA;
    }
    *out = ctx;
    return RC_OK;
}

void rc_destroy(rc_ctx* ctx) {
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    free_pool(ctx->cache_bufs);
    free_pool(ctx->scene_bufs);
    free_pool(ctx->adj_bufs);
    free_pool(ctx->taa_bufs);
    free_pool(ctx->cam_bufs);
    if (ctx->cam.ready) cudaEventDestroy(ctx->cam.ready);
    if (ctx->flags_dev) cudaFree(ctx->flags_dev);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->stage) cudaFree(ctx->stage);
    if (ctx->img) cudaFree(ctx->img);
    for (auto& e : ctx->ev) if (e) cudaEventDestroy(e);
    for (auto& e : ctx->state_ev) cudaEventDestroy(e);
    if (ctx->load_ev) cudaEventDestroy(ctx->load_ev);
    for (auto& e : ctx->copies_ev) cudaEventDestroy(e);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* rc_last_error(const rc_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

rc_status rc_device_info_get(rc_ctx* ctx, rc_device_info* out) {
    if (!ctx || !out) return RC_ERR_ARG;
    cudaDeviceProp pr;
    CKR(cudaGetDeviceProperties(&pr, ctx->cfg.device));
    memset(out, 0, sizeof *out);
    snprintf(out->name, sizeof out->name, "%s", pr.name);
    out->sm_count = pr.multiProcessorCount;
    out->cc_major = pr.major;
    out->cc_minor = pr.minor;
    size_t fr = 0, tot = 0;
    CKR(cudaMemGetInfo(&fr, &tot));
    out->mem_used_mb = (double)(tot - fr) / 1048576.0;
    out->mem_total_mb = (double)tot / 1048576.0;
    return RC_OK;
}

rc_status rc_scene_load_memory(rc_ctx* ctx, const void* data, size_t nbytes) {
    if (!ctx || !data) return RC_ERR_ARG;
    CKR(cudaSetDevice(ctx->cfg.device));
    CKR(cudaStreamSynchronize(ctx->stream));
    if (ctx->side) CKR(cudaStreamSynchronize(ctx->side));
    free_pool(ctx->cache_bufs);
    free_pool(ctx->scene_bufs);
    free_pool(ctx->adj_bufs);
    free_pool(ctx->taa_bufs);
    ctx->taa = TaaRun{};
    ctx->adj_np = ctx->adj_k = 0;
    ctx->adj_cap_np = ctx->adj_cap_k = ctx->adj_cap_nl = 0;
    ctx->have_scene = false;
    ctx->run.active = false;
    ctx->c = DevCache{};
    ctx->err_cap = 0;
    rc_status s = load_scene(ctx, (const uint8_t*)data, nbytes);
    // copies from the caller's buffer may still be in flight after a failed load
    if (s != RC_OK) { cudaStreamSynchronize(ctx->stream); free_pool(ctx->scene_bufs); return s; }
    // the cache's buffers and their clearing are ordered on the context's stream before any frame
    // (no host wait: with RC_FLAG_LOAD_ASYNC the copy engine is still busy with the other states)
    if ((s = alloc_cache(ctx)) != RC_OK) return s;
    CKR(cudaGetLastError());
    ctx->have_scene = true;
    // the states' device builds run behind the load on the side stream
    if ((s = issue_state_builds(ctx)) != RC_OK) { ctx->have_scene = false; return s; }
    double b = 0;
    for (auto& x : ctx->scene_bufs) b += (double)x.n;
    ctx->S.scene_bytes = b;
    return RC_OK;
}

rc_status rc_scene_load(rc_ctx* ctx, const char* path) {
    if (!ctx || !path) return RC_ERR_ARG;
    FILE* f = fopen(path, "rb");
    if (!f) return fail(ctx, RC_ERR_IO, "cannot open scene file %s", path);
    std::vector<uint8_t> buf;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (n < 0) { fclose(f); return fail(ctx, RC_ERR_IO, "cannot size %s", path); }
    buf.resize((size_t)n);
    size_t got = n ? fread(buf.data(), 1, (size_t)n, f) : 0;
    fclose(f);
    if (got != (size_t)n) return fail(ctx, RC_ERR_IO, "short read on %s", path);
    return rc_scene_load_memory(ctx, buf.data(), buf.size());
}

rc_status rc_scene_info_get(const rc_ctx* ctx, rc_scene_info* out) {
    if (!ctx || !out) return RC_ERR_ARG;
    if (!ctx->have_scene) return RC_ERR_STATE;
    const Scene& S = ctx->S;
    out->np = S.Np; out->nq = S.Nq; out->nt = S.Nt; out->ns = S.NS; out->nl = S.NL; out->nr = S.NR;
    out->has_ref = S.has_ref; out->fmt = S.fmt; out->nw = ctx->NW; out->nst = S.nst; out->nnodes = S.nnodes; out->hsize = S.hsize;
    out->scene_bytes = S.scene_bytes;
    out->cache_bytes = ctx->cache_bytes;
    return RC_OK;
}

rc_status rc_state_lights(const rc_ctx* ctx, int state, float* inten, int nl) {
    if (!ctx || !inten) return RC_ERR_ARG;
    if (!ctx->have_scene) return RC_ERR_STATE;
    if (state < 0 || state >= ctx->S.NS || nl != ctx->S.NL) return RC_ERR_ARG;
    memcpy(inten, ctx->S.st[state].inten.data(), sizeof(float) * (size_t)nl);
    return RC_OK;
}

rc_status rc_run_begin(rc_ctx* ctx, const rc_method* m, int s0, uint32_t seed) {
    if (!ctx || !m) return RC_ERR_ARG;
    if (!ctx->have_scene) return fail(ctx, RC_ERR_STATE, "no scene loaded");
    Scene& S = ctx->S;
    if (s0 < 0 || s0 >= S.NS) return fail(ctx, RC_ERR_ARG, "state %d out of range", s0);
    if (!(m->rays > 0.f)) return fail(ctx, RC_ERR_ARG, "rays must be > 0");
    rc_status es = ensure_state(ctx, s0);
    if (es != RC_OK) return es;
    Run& R = ctx->run;
    R = Run{};
    R.M = *m;
    if (R.M.track_every <= 0) R.M.track_every = 1;
    cudaStream_t st = ctx->stream;
    const size_t Np = (size_t)S.Np, LCS = (size_t)lcs_of(S.NL);
    DevCache& c = ctx->c;
    // poc_gpu.cu:832-841
    if (S.has_ref) CKR(cudaMemcpyAsync(c.Lc, S.st[s0].pw, LCS * Np * 4, cudaMemcpyDeviceToDevice, st));
    else CKR(cudaMemsetAsync(c.Lc, 0, LCS * Np * 4, st));
    R.nmax = m->nmax * m->rays;
    {
        k_fill<<<load_grid(Np), 256, 0, st>>>(c.n, Np, R.nmax);
        k_fill<<<load_grid(Np), 256, 0, st>>>(c.age, Np, 1e4f);
        CKR(cudaGetLastError());
        CKR(cudaMemsetAsync(c.pending, 0, Np, st));
        CKR(cudaMemsetAsync(c.cur, 0, (size_t)ctx->NW * Np * 4, st));
        CKR(cudaMemsetAsync(c.prev, 0, (size_t)ctx->NW * Np * 4, st));
        CKR(cudaMemsetAsync(c.stale, 0, Np * 4, st));
        float sp[2] = {float(S.Np) / (R.nmax + 1.f), 0.f};
        int z2[2] = {0, 0};
        CKR(cudaMemcpyAsync(c.sumpr, sp, 8, cudaMemcpyHostToDevice, st));
        CKR(cudaMemcpyAsync(c.npend, z2, 8, cudaMemcpyHostToDevice, st));
        CKR(cudaMemsetAsync(c.rays, 0, 8, st));
        CKR(cudaStreamSynchronize(st));   // sp and z2 are about to go out of scope
    }
    R.p.seed = seed;
    for (int k = 0; k < KSNAP; ++k) R.slot_state[k] = -1;
    R.prev_state = s0;
    R.active = true;
    return RC_OK;
}

rc_status rc_frame(rc_ctx* ctx, int state, int want_err) {
    if (!ctx) return RC_ERR_ARG;
    if (!ctx->run.active) return fail(ctx, RC_ERR_STATE, "no run begun");
    if (state < 0 || state >= ctx->S.NS) return fail(ctx, RC_ERR_ARG, "state %d out of range", state);
    return frame_impl(ctx, state, want_err, nullptr);
}

rc_status rc_errors(rc_ctx* ctx, float* out, int max, int* n) {
    if (!ctx || !n) return RC_ERR_ARG;
    const int k = ctx->run.nerr;
    *n = k;
    if (!out || k == 0) return RC_OK;
    std::vector<double> h(3 * (size_t)k);
    CKR(cudaMemcpyAsync(h.data(), ctx->c.err, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CKR(cudaStreamSynchronize(ctx->stream));
    for (int f = 0; f < k && f < max; ++f) out[f] = float(sqrt(h[3 * f] / h[3 * f + 2]) / (h[3 * f + 1] / h[3 * f + 2]));
    return RC_OK;
}

rc_status rc_run(rc_ctx* ctx, const rc_method* m, const int* seq, int nframes, uint32_t seed, int want_err, float* errs,
                 rc_timers* tm) {
    if (!ctx || !m || !seq || nframes <= 0) return RC_ERR_ARG;
    for (int f = 0; f < nframes; ++f)
        if (seq[f] < 0 || (ctx->have_scene && seq[f] >= ctx->S.NS)) return fail(ctx, RC_ERR_ARG, "state out of range");
    rc_status s = rc_run_begin(ctx, m, seq[0], seed);
    if (s != RC_OK) return s;
    for (int f = 0; f < nframes; ++f)
        if ((s = frame_impl(ctx, seq[f], want_err, tm)) != RC_OK) return s;
    if (errs) {
        int n = 0;
        if ((s = rc_errors(ctx, errs, nframes, &n)) != RC_OK) return s;
    }
    CKR(cudaStreamSynchronize(ctx->stream));
    return RC_OK;
}

rc_status rc_sync(rc_ctx* ctx) {
    if (!ctx) return RC_ERR_ARG;
    CKR(cudaStreamSynchronize(ctx->stream));
    if (ctx->side) CKR(cudaStreamSynchronize(ctx->side));
    return RC_OK;
}

rc_status rc_scene_build_states(rc_ctx* ctx) {
    if (!ctx) return RC_ERR_ARG;
    if (!ctx->have_scene) return fail(ctx, RC_ERR_STATE, "no scene loaded");
    CKR(cudaSetDevice(ctx->cfg.device));
    for (int k = 0; k < ctx->S.NS; ++k) {
        rc_status s = prebuild_state(ctx, k);
        if (s != RC_OK) return s;
    }
    return RC_OK;
}

static rc_status camera_basis(rc_ctx* ctx, const rc_camera* cam, CameraD* out) {
    // camera frame: forward to the target, right = forward x up, up re-orthogonalised
    double f[3], r[3], u[3];
    for (int k = 0; k < 3; ++k) f[k] = (double)cam->at[k] - cam->eye[k];
    double fl = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(fl > 0)) return fail(ctx, RC_ERR_ARG, "camera eye equals target");
    for (int k = 0; k < 3; ++k) f[k] /= fl;
    r[0] = f[1] * cam->up[2] - f[2] * cam->up[1];
    r[1] = f[2] * cam->up[0] - f[0] * cam->up[2];
    r[2] = f[0] * cam->up[1] - f[1] * cam->up[0];
    double rl = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (!(rl > 0)) return fail(ctx, RC_ERR_ARG, "camera up is parallel to the view direction");
    for (int k = 0; k < 3; ++k) r[k] /= rl;
    u[0] = r[1] * f[2] - r[2] * f[1];
    u[1] = r[2] * f[0] - r[0] * f[2];
    u[2] = r[0] * f[1] - r[1] * f[0];
    CameraD& cd = *out;
    for (int k = 0; k < 3; ++k) { cd.eye[k] = cam->eye[k]; cd.fwd[k] = (float)f[k]; cd.right[k] = (float)r[k]; cd.up[k] = (float)u[k]; }
    cd.ty = (float)tan(0.5 * cam->fov_y_deg * 3.14159265358979323846 / 180.0);
    cd.tx = cd.ty * (float)cam->width / (float)cam->height;
    cd.w = cam->width;
    cd.h = cam->height;
    return RC_OK;
}

rc_status rc_render(rc_ctx* ctx, int state, const rc_camera* cam, float* image, size_t image_floats) {
    if (!ctx || !cam) return RC_ERR_ARG;
    if (!ctx->run.active) return fail(ctx, RC_ERR_STATE, "no run begun");
    const Scene& S = ctx->S;
    if (state < 0 || state >= S.NS) return fail(ctx, RC_ERR_ARG, "state %d out of range", state);
    if (cam->width <= 0 || cam->height <= 0 || cam->width > 16384 || cam->height > 16384 || !(cam->fov_y_deg > 0.f && cam->fov_y_deg < 179.f))
        return fail(ctx, RC_ERR_ARG, "bad camera");
    const size_t npx = (size_t)cam->width * cam->height;
    if (image && image_floats != npx) return fail(ctx, RC_ERR_ARG, "image holds %zu floats, not %zu", image_floats, npx);
    if (rc_status es = ensure_state(ctx, state)) return es;
    if (npx > ctx->img_cap) {
        if (ctx->img) { CKR(cudaStreamSynchronize(ctx->stream)); cudaFree(ctx->img); ctx->img = nullptr; }
        cudaError_t e = cudaMalloc(&ctx->img, npx * sizeof(float));
        if (e != cudaSuccess) { ctx->img_cap = 0; return fail(ctx, RC_ERR_NOMEM, "image buffer: %s", cudaGetErrorString(e)); }
        ctx->img_cap = npx;
    }
    CameraD cd;
    rc_status cs = camera_basis(ctx, cam, &cd);
    if (cs != RC_OK) return cs;
    FrameParams p = base_params(ctx);
    CKR(RC_DISPATCH(S.NL, camera(S.st[state].d, S.g, S.grid, ctx->c, p, cd, ctx->img, ctx->stream)));
    ctx->launches++;
    if (image) {
        CKR(cudaMemcpyAsync(image, ctx->img, npx * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CKR(cudaStreamSynchronize(ctx->stream));
    }
    return RC_OK;
}


static bool array_geom(rc_ctx* ctx, int which, size_t* elem, size_t* count, size_t* src_stride, size_t* dst_stride, void** dev) {
    const Scene& S = ctx->S;
    const size_t Np = (size_t)S.Np, NL = (size_t)S.NL, LCS = (size_t)lcs_of(S.NL), NR = (size_t)S.NR, NW = (size_t)ctx->NW;
    DevCache& c = ctx->c;
    *src_stride = *dst_stride = 0;
    switch (which) {
        case RC_A_LC: *elem = 4; *count = NL * Np; *dev = c.Lc; *src_stride = LCS; *dst_stride = NL; return true;
        case RC_A_LC2: *elem = 4; *count = NL * Np; *dev = c.Lc2; *src_stride = LCS; *dst_stride = NL; return true;
        case RC_A_M: *elem = 4; *count = NL * Np; *dev = c.m; *src_stride = LCS; *dst_stride = NL; return true;
        case RC_A_N: *elem = 4; *count = Np; *dev = c.n; return true;
        case RC_A_C0: *elem = 4; *count = Np; *dev = c.c0; return true;
        case RC_A_KK: *elem = 4; *count = Np; *dev = c.kk; return true;
        case RC_A_PENDING: *elem = 1; *count = Np; *dev = c.pending; return true;
        case RC_A_CUR: *elem = 4; *count = NW * Np; *dev = c.cur; return true;
        case RC_A_PREV: *elem = 4; *count = NW * Np; *dev = c.prev; return true;
        case RC_A_STALE: *elem = 4; *count = Np; *dev = c.stale; return true;
        case RC_A_AGE: *elem = 4; *count = Np; *dev = c.age; return true;
        case RC_A_SNAP: *elem = 4; *count = (size_t)KSNAP * Np * NL; *dev = c.snap; *src_stride = LCS; *dst_stride = NL; return true;
        case RC_A_NEQ: *elem = 4; *count = NR * NEQ; *dev = c.neq; return true;
        case RC_A_COEF: *elem = 4; *count = NR * KSNAP; *dev = c.coef; return true;
        case RC_A_RSTAT: *elem = 4; *count = 4 * NR; *dev = c.rstat; return true;
        case RC_A_DSTAT: *elem = 4; *count = 3 * NR; *dev = c.dstat; return true;
        case RC_A_SUMPR: *elem = 4; *count = 2; *dev = c.sumpr; return true;
        case RC_A_NPEND: *elem = 4; *count = 2; *dev = c.npend; return true;
    }
    return false;
}

rc_status rc_array_info(rc_ctx* ctx, int which, size_t* nbytes, void** dev_ptr) {
    if (!ctx || !nbytes) return RC_ERR_ARG;
    if (!ctx->have_scene) return RC_ERR_STATE;
    size_t elem, count, ss, ds;
    void* dev;
    if (!array_geom(ctx, which, &elem, &count, &ss, &ds, &dev)) return RC_ERR_ARG;
    *nbytes = elem * count;
    if (dev_ptr) *dev_ptr = dev;
    return RC_OK;
}

// `rows` rows of 4-byte elements between host (ds per row, packed) and device (ss per row,
// the first ds copied): packed on the device into the staging buffer, then one contiguous copy
// (or the reverse).  Asynchronous on the context's stream.
static rc_status copy_rows(rc_ctx* ctx, void* host, void* dev, size_t rows, int ds, int ss, bool to_device) {
    const size_t nbytes = rows * (size_t)ds * 4;
    cudaStream_t st = ctx->stream;
    if (ctx->stage_cap < nbytes) {
        CKR(cudaStreamSynchronize(st));
        if (ctx->stage) cudaFree(ctx->stage);
        ctx->stage = nullptr;
        ctx->stage_cap = 0;
        CKR(cudaMalloc(&ctx->stage, nbytes));
        ctx->stage_cap = nbytes;
    }
    uint32_t* sb = static_cast<uint32_t*>(ctx->stage);
    if (to_device) {
        CKR(cudaMemcpyAsync(sb, host, nbytes, cudaMemcpyHostToDevice, st));
        k_unpack_rows<<<load_grid(rows * ds), 256, 0, st>>>(sb, static_cast<uint32_t*>(dev), rows, ds, ss);
        CKR(cudaGetLastError());
    } else {
        k_pack_rows<<<load_grid(rows * ds), 256, 0, st>>>(static_cast<const uint32_t*>(dev), sb, rows, ds, ss);
        CKR(cudaGetLastError());
        CKR(cudaMemcpyAsync(host, sb, nbytes, cudaMemcpyDeviceToHost, st));
    }
    return RC_OK;
}

rc_status rc_array_copy(rc_ctx* ctx, int which, void* host, size_t nbytes, int to_device) {
    if (!ctx || !host) return RC_ERR_ARG;
    if (!ctx->have_scene) return RC_ERR_STATE;
    size_t elem, count, ss, ds;
    void* dev;
    if (!array_geom(ctx, which, &elem, &count, &ss, &ds, &dev)) return RC_ERR_ARG;
    if (nbytes != elem * count) return fail(ctx, RC_ERR_ARG, "array %d is %zu bytes, not %zu", which, elem * count, nbytes);
    if (which == RC_A_SUMPR && to_device) {
        // logical slot 0 = the value the next frame reads
        float v[2];
        memcpy(v, host, 8);
        float d[2];
        d[ctx->run.sum_cur] = v[0];
        d[1 - ctx->run.sum_cur] = v[1];
        CKR(cudaMemcpyAsync(dev, d, 8, cudaMemcpyHostToDevice, ctx->stream));
        CKR(cudaStreamSynchronize(ctx->stream));
        return RC_OK;
    }
    if (ss) {
        // padded device rows of ss elements, packed host rows of ds elements
        const size_t rows = count / ds;
        rc_status s2;
        if (elem == 4) {
            if ((s2 = copy_rows(ctx, host, dev, rows, (int)ds, (int)ss, to_device != 0)) != RC_OK) return s2;
        } else if (to_device) {
            CKR(cudaMemcpy2DAsync(dev, ss * elem, host, ds * elem, ds * elem, rows, cudaMemcpyHostToDevice, ctx->stream));
        } else {
            CKR(cudaMemcpy2DAsync(host, ds * elem, dev, ss * elem, ds * elem, rows, cudaMemcpyDeviceToHost, ctx->stream));
        }
    } else {
        CKR(cudaMemcpyAsync(to_device ? dev : host, to_device ? host : dev, nbytes,
                            to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, ctx->stream));
    }
    CKR(cudaStreamSynchronize(ctx->stream));
    if (which == RC_A_SUMPR && !to_device) {
        float v[2];
        memcpy(v, host, 8);
        float o[2] = {v[ctx->run.sum_cur], v[1 - ctx->run.sum_cur]};
        memcpy(host, o, 8);
    }
    return RC_OK;
}

rc_status rc_scalar_get(rc_ctx* ctx, int which, int* value) {
    if (!ctx || !value) return RC_ERR_ARG;
    const Run& R = ctx->run;
    switch (which) {
        case RC_S_PEND_LEFT: *value = R.pend_left; return RC_OK;
        case RC_S_DORMANT: *value = R.dormant; return RC_OK;
        case RC_S_PROJ_LEFT: *value = R.proj_left; return RC_OK;
        case RC_S_FRAME: *value = R.f; return RC_OK;
        case RC_S_NSLOTS: *value = R.nslots; return RC_OK;
        case RC_S_LAST_EVENT: *value = R.last_event_f; return RC_OK;
        case RC_S_PROJK: *value = R.projK; return RC_OK;
        case RC_S_LAST_FRAME_KERNELS: *value = R.last_kernels; return RC_OK;
        case RC_S_LAST_FRAME_FUSED: *value = R.last_fused; return RC_OK;
    }
    return RC_ERR_ARG;
}

rc_status rc_scalar_set(rc_ctx* ctx, int which, int value) {
    if (!ctx) return RC_ERR_ARG;
    Run& R = ctx->run;
    switch (which) {
        case RC_S_PEND_LEFT: R.pend_left = value; return RC_OK;
        case RC_S_DORMANT: R.dormant = value; return RC_OK;
        case RC_S_PROJ_LEFT: R.proj_left = value; return RC_OK;
        case RC_S_FRAME: R.f = value; return RC_OK;
        case RC_S_NSLOTS: R.nslots = value; return RC_OK;
        case RC_S_LAST_EVENT: R.last_event_f = value; return RC_OK;
        case RC_S_PROJK: R.projK = value; return RC_OK;
    }
    return RC_ERR_ARG;
}

rc_status rc_state_array_copy(rc_ctx* ctx, int state, int which, void* host, size_t nbytes) {
    if (!ctx || !host) return RC_ERR_ARG;
    if (!ctx->have_scene) return RC_ERR_STATE;
    const Scene& S = ctx->S;
    if (state < 0 || state >= S.NS) return RC_ERR_ARG;
    const size_t Np = (size_t)S.Np, NL = (size_t)S.NL, AES = (size_t)aes_of(S.NL);
    if (rc_status es = ensure_state(ctx, state)) return es;
    const DState& d = S.st[state].d;
    cudaStream_t st = ctx->stream;
    switch (which) {
        case RC_SA_EDIR:
            if (nbytes != 4 * NL * Np) return RC_ERR_ARG;
            {
                rc_status s2 = copy_rows(ctx, host, const_cast<float*>(reinterpret_cast<const float*>(d.AE)) + 1, Np, (int)NL, (int)AES, false);
                if (s2 != RC_OK) return s2;
            }
            break;
        case RC_SA_SV:
            if (nbytes != 4 * (size_t)ctx->NW * Np) return RC_ERR_ARG;
            CKR(cudaMemcpyAsync(host, d.SV, nbytes, cudaMemcpyDeviceToHost, st));
            break;
        case RC_SA_REF:
            if (!S.has_ref || nbytes != 4 * Np) return RC_ERR_ARG;
            CKR(cudaMemcpyAsync(host, d.ref, nbytes, cudaMemcpyDeviceToHost, st));
            break;
        case RC_SA_VALID:
            if (!S.has_ref || nbytes != Np) return RC_ERR_ARG;
            CKR(cudaMemcpyAsync(host, d.valid, nbytes, cudaMemcpyDeviceToHost, st));
            break;
        case RC_SA_PW:
            if (!S.has_ref || nbytes != 4 * NL * Np) return RC_ERR_ARG;
            {
                rc_status s2 = copy_rows(ctx, host, const_cast<float*>(S.st[state].pw), Np, (int)NL, lcs_of(S.NL), false);
                if (s2 != RC_OK) return s2;
            }
            break;
        default:
            return RC_ERR_ARG;
    }
    CKR(cudaStreamSynchronize(st));
    return RC_OK;
}

rc_status rc_probe_rays(rc_ctx* ctx, int state, const int* points, int npoints, rc_ray_rec* out, int maxrec, int* nrec) {
    if (!ctx || !points || !out || !nrec || npoints < 0 || maxrec < 0) return RC_ERR_ARG;
    if (!ctx->run.active) return fail(ctx, RC_ERR_STATE, "no run begun");
    const Scene& S = ctx->S;
    if (state < 0 || state >= S.NS) return RC_ERR_ARG;
    *nrec = 0;
    if (npoints == 0) return RC_OK;
    if (rc_status es = ensure_state(ctx, state)) return es;
    int* dpts = nullptr;
    int* dn = nullptr;
    void* drec = nullptr;
    CKR(cudaMalloc(&dpts, sizeof(int) * (size_t)npoints));
    CKR(cudaMalloc(&dn, sizeof(int)));
    CKR(cudaMalloc(&drec, sizeof(rc_ray_rec) * (size_t)(maxrec > 0 ? maxrec : 1)));
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(dpts, points, sizeof(int) * (size_t)npoints, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(dn, 0, sizeof(int), st);
    FrameParams p = base_params(ctx);
    cudaError_t e = RC_DISPATCH(S.NL, probe(ctx->NW, S.st[state].d, S.g, S.grid, ctx->c, p, dpts, npoints, drec, maxrec, dn, st));
    int n = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&n, dn, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && n > 0) e = cudaMemcpy(out, drec, sizeof(rc_ray_rec) * (size_t)std::min(n, maxrec), cudaMemcpyDeviceToHost);
    cudaFree(dpts);
    cudaFree(dn);
    cudaFree(drec);
    if (e != cudaSuccess) return fail(ctx, RC_ERR_CUDA, "probe: %s", cudaGetErrorString(e));
    *nrec = std::min(n, maxrec);
    return RC_OK;
}

rc_status rc_trace_rays(rc_ctx* ctx, int state, const float* rays, int nrays, int* prim, float* t) {
    if (!ctx || nrays < 0 || (nrays > 0 && (!rays || !prim || !t))) return RC_ERR_ARG;
    if (!ctx->have_scene) return fail(ctx, RC_ERR_STATE, "no scene loaded");
    const Scene& S = ctx->S;
    if (state < 0 || state >= S.NS) return RC_ERR_ARG;
    if (nrays == 0) return RC_OK;
    CKR(cudaSetDevice(ctx->cfg.device));
    if (rc_status es = ensure_state(ctx, state)) return es;
    std::vector<DevBuf> tmp;
    struct TmpFree { std::vector<DevBuf>& p; ~TmpFree() { free_pool(p); } } tmp_free{tmp};
    float* dr = nullptr;
    float* dt = nullptr;
    int* dq = nullptr;
    rc_status s;
    if ((s = dalloc(ctx, tmp, &dr, 6 * (size_t)nrays)) || (s = dalloc(ctx, tmp, &dq, (size_t)nrays)) ||
        (s = dalloc(ctx, tmp, &dt, (size_t)nrays)))
        return s;
    cudaStream_t st = ctx->stream;
    unsigned flags = 0;
    CKR(cudaMemcpyAsync(dr, rays, 24 * (size_t)nrays, cudaMemcpyHostToDevice, st));
    // word 1 is this call's own guard word: word 0 keeps what the run's frames raised
    CKR(cudaMemsetAsync(ctx->flags_dev + 1, 0, 4, st));
    CKR(trace_rays(S.st[state].d, S.g, (ctx->cfg.flags & RC_FLAG_BRUTE_FORCE) != 0, dr, nrays, dq, dt, ctx->flags_dev + 1, st));
    CKR(cudaMemcpyAsync(prim, dq, 4 * (size_t)nrays, cudaMemcpyDeviceToHost, st));
    CKR(cudaMemcpyAsync(t, dt, 4 * (size_t)nrays, cudaMemcpyDeviceToHost, st));
    CKR(cudaMemcpyAsync(&flags, ctx->flags_dev + 1, 4, cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    if (flags) return fail(ctx, RC_ERR_DEVICE, "trace: BVH traversal guard tripped (flags %u)", flags);
    return RC_OK;
}

rc_status rc_trace_check_count(rc_ctx* ctx, long long* mismatches, long long* rays) {
    if (!ctx || !mismatches || !rays) return RC_ERR_ARG;
    if (!ctx->have_scene) return RC_ERR_STATE;
    unsigned long long h[2];
    CKR(cudaMemcpyAsync(h, ctx->c.check, 16, cudaMemcpyDeviceToHost, ctx->stream));
    CKR(cudaMemsetAsync(ctx->c.check, 0, 16, ctx->stream));
    CKR(cudaStreamSynchronize(ctx->stream));
    *mismatches = (long long)h[0];
    *rays = (long long)h[1];
    return RC_OK;
}

rc_status rc_run_stats_get(rc_ctx* ctx, rc_run_stats* out) {
    if (!ctx || !out) return RC_ERR_ARG;
    memset(out, 0, sizeof *out);
    out->launches = ctx->launches;
    if (!ctx->have_scene) return RC_OK;
    unsigned long long r = 0;
    CKR(cudaMemcpyAsync(&r, ctx->c.rays, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CKR(cudaStreamSynchronize(ctx->stream));
    out->rays = (long long)r;
    out->frames = ctx->run.f;
    out->last_frame_kernels = ctx->run.last_kernels;
    out->last_frame_fused = ctx->run.last_fused;
    out->last_frame_event = ctx->run.last_event;
    return RC_OK;
}

rc_status rc_reference_build(rc_ctx* ctx, const rc_ref_params* prm, double* noise, int* iters) {
    if (!ctx || !prm || prm->K < 1 || prm->warmup < 0 || prm->block < 1 || prm->max_iter < prm->block) return RC_ERR_ARG;
    if (!ctx->have_scene) return fail(ctx, RC_ERR_STATE, "no scene loaded");
    Scene& S = ctx->S;
    const size_t Np = (size_t)S.Np;
    const int NL = S.NL, LCS = lcs_of(NL);
    cudaStream_t st = ctx->stream;
    if (rc_status es = ensure_all_states(ctx)) return es;
    // the references change: a taa run recomputes its per-state error denominators
    std::fill(ctx->taa.have_sums.begin(), ctx->taa.have_sums.end(), (char)0);
    std::vector<DevBuf> tmp;
    struct TmpFree { std::vector<DevBuf>& p; ~TmpFree() { free_pool(p); } } tmp_free{tmp};
    float *chain[2], *acc[2], *out = nullptr, *closec = nullptr;
    rc_status s;
    for (int ch = 0; ch < 2; ++ch)
        if ((s = dalloc(ctx, tmp, &chain[ch], LCS * Np)) || (s = dalloc(ctx, tmp, &acc[ch], LCS * Np))) return s;
    if ((s = dalloc(ctx, tmp, &out, LCS * Np)) || (s = dalloc(ctx, tmp, &closec, Np))) return s;
    FrameParams p{};
    p.Np = S.Np;
    auto mix = [](unsigned long long x) {   // poc_gpu.cu:260-262
        x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull; x ^= x >> 27; x *= 0x94d049bb133111ebull; x ^= x >> 31;
        return x;
    };
    std::vector<float> a0(LCS * Np), a1(LCS * Np), cc(Np);
    for (int si = 0; si < S.NS; ++si) {
        HostState& hs = S.st[si];
        const DState& d = hs.d;
        CKR(cudaMemsetAsync(closec, 0, Np * 4, st));
        for (int ch = 0; ch < 2; ++ch) {
            CKR(cudaMemsetAsync(chain[ch], 0, LCS * Np * 4, st));
            CKR(cudaMemsetAsync(acc[ch], 0, LCS * Np * 4, st));
        }
        int done = 0, T = 0;
        double nz = 1.0;
        std::vector<float> ref(Np), pw(LCS * Np, 0.f);
        std::vector<uint8_t> val(Np);
        while (true) {
            const int n_it = done == 0 ? prm->warmup + prm->block : prm->block;
            for (int ch = 0; ch < 2; ++ch) {
                float* a = chain[ch];
                float* b = out;
                for (int k = 0; k < n_it; ++k) {
                    const int it = done + k;
                    const uint32_t seed = (uint32_t)mix(0x51ull + 7919ull * (unsigned long long)si + 104729ull * (unsigned long long)ch +
                                                        31ull * (unsigned long long)it);
                    CKR(RC_DISPATCH(NL, ref_iter(d, S.g, S.grid, ctx->c, p, a, b, acc[ch], closec, seed, prm->K, it >= prm->warmup,
                                                 ch == 0, st)));
                    std::swap(a, b);
                }
                if (a != chain[ch]) {   // the last iterate is in `out`: keep it as the chain's state
                    CKR(cudaMemcpyAsync(chain[ch], a, LCS * Np * 4, cudaMemcpyDeviceToDevice, st));
                }
            }
            done += n_it;
            T = done - prm->warmup;
            CKR(cudaMemcpyAsync(a0.data(), acc[0], a0.size() * 4, cudaMemcpyDeviceToHost, st));
            CKR(cudaMemcpyAsync(a1.data(), acc[1], a1.size() * 4, cudaMemcpyDeviceToHost, st));
            CKR(cudaMemcpyAsync(cc.data(), closec, Np * 4, cudaMemcpyDeviceToHost, st));
            CKR(cudaStreamSynchronize(st));
            double d2 = 0, rs = 0;
            int nv = 0;
            for (size_t i = 0; i < Np; ++i) {
                float e0 = 0, e1 = 0;
                for (int l = 0; l < NL; ++l) {
                    const float x0 = a0[LCS * i + l] / T, x1 = a1[LCS * i + l] / T;
                    pw[LCS * i + l] = 0.5f * (x0 + x1);
                    e0 += x0;
                    e1 += x1;
                }
                ref[i] = 0.5f * (e0 + e1);
                val[i] = cc[i] / ((double)prm->K * done) < 0.3;
                if (val[i]) { d2 += 0.25 * (e0 - e1) * (e0 - e1); rs += ref[i]; nv++; }
            }
            nz = nv && rs > 0 ? sqrt(d2 / nv) / (rs / nv) : 0.0;
            if (nz <= prm->noise_target || T >= prm->max_iter) break;
        }
        if (noise) noise[si] = nz;
        if (iters) iters[si] = T;
        DState& dm = hs.d;
        if (!dm.ref) {
            float* r = nullptr;
            uint8_t* v = nullptr;
            float* w = nullptr;
            if ((s = dalloc(ctx, ctx->scene_bufs, &r, Np)) || (s = dalloc(ctx, ctx->scene_bufs, &v, Np)) ||
                (s = dalloc(ctx, ctx->scene_bufs, &w, LCS * Np)))
                return s;
            dm.ref = r;
            dm.valid = v;
            hs.pw = w;
        }
        CKR(cudaMemcpyAsync((void*)dm.ref, ref.data(), Np * 4, cudaMemcpyHostToDevice, st));
        CKR(cudaMemcpyAsync((void*)dm.valid, val.data(), Np, cudaMemcpyHostToDevice, st));
        CKR(cudaMemcpyAsync((void*)hs.pw, pw.data(), LCS * Np * 4, cudaMemcpyHostToDevice, st));
        CKR(cudaStreamSynchronize(st));
    }
    S.has_ref = 1;
    return RC_OK;
}

rc_status rc_adjoint(rc_ctx* ctx, const rc_adjoint_params* prm, const float* weights, float* dJ_dE, rc_adjoint_result* res) {
    if (!ctx || !prm || !weights || !dJ_dE || prm->K < 1 || prm->K > 1024 || prm->iterations < 0) return RC_ERR_ARG;
    if (!ctx->have_scene) return fail(ctx, RC_ERR_STATE, "no scene loaded");
    Scene& S = ctx->S;
    if (prm->state < 0 || prm->state >= S.NS) return fail(ctx, RC_ERR_ARG, "state %d out of range", prm->state);
    if ((long long)S.Np * prm->K >= (1ll << 31)) return fail(ctx, RC_ERR_ARG, "Np * K must stay below 2^31");
    if (S.NL + 1 > adj::MAX_COLS) return fail(ctx, RC_ERR_UNSUPPORTED, "%d lights", S.NL);
    CKR(cudaSetDevice(ctx->cfg.device));
    if (rc_status es = ensure_state(ctx, prm->state)) return es;
    cudaStream_t st = ctx->stream;
    const size_t Np = (size_t)S.Np, K = (size_t)prm->K;
    const int NL = S.NL, AES = aes_of(NL), iters = prm->iterations ? prm->iterations : 64;
    adj::Bufs b = ctx->adj;
    rc_status s;
    // buffers kept from call to call while the point count, K and the light count stay
    if (ctx->adj_cap_np != S.Np || ctx->adj_cap_k != prm->K || ctx->adj_cap_nl != NL) {
        CKR(cudaStreamSynchronize(st));
        free_pool(ctx->adj_bufs);
        ctx->adj_np = ctx->adj_k = 0;
        ctx->adj_cap_np = ctx->adj_cap_k = ctx->adj_cap_nl = 0;
        auto& pool = ctx->adj_bufs;
        b = adj::Bufs{};
        float4* AEu = nullptr;
        const float* ones = nullptr;
        if ((s = dalloc(ctx, pool, &b.hits, Np * K)) || (s = dalloc(ctx, pool, &b.cnt, Np + 1)) || (s = dalloc(ctx, pool, &b.off, Np + 1)) ||
            (s = dalloc(ctx, pool, &b.fill, Np)) || (s = dalloc(ctx, pool, &b.src, Np * K)) || (s = dalloc(ctx, pool, &b.unordered, Np * K)) ||
            (s = dalloc(ctx, pool, &b.scratch, adj::scan_scratch_ints((long long)Np + 1))) || (s = dalloc(ctx, pool, &b.da, Np)) ||
            (s = dalloc(ctx, pool, &b.L[0], Np)) || (s = dalloc(ctx, pool, &b.L[1], Np)) || (s = dalloc(ctx, pool, &b.g[0], Np)) ||
            (s = dalloc(ctx, pool, &b.g[1], Np)) || (s = dalloc(ctx, pool, &b.u[0], Np)) ||
            (s = dalloc(ctx, pool, &b.u[1], Np)) || (s = dalloc(ctx, pool, &b.w, Np)) ||
            (s = dalloc(ctx, pool, &b.part, (size_t)adj::GRAD_BLOCKS * (NL + 1))) || (s = dalloc(ctx, pool, &b.stats, 1)) ||
            (s = dalloc(ctx, pool, &AEu, (size_t)AES / 4 * Np)) || (s = dput(ctx, pool, &ones, std::vector<float>((size_t)NL, 1.f))))
            return s;
        ctx->adj_aeu = AEu;
        ctx->adj_aeu_state = -1;
        ctx->adj_ones = ones;
        ctx->adj_cap_np = S.Np;
        ctx->adj_cap_k = prm->K;
        ctx->adj_cap_nl = NL;
    }
    float4* AEu = ctx->adj_aeu;
    const float* ones = ctx->adj_ones;
    const DState& d = S.st[prm->state].d;
    FrameParams p{};
    p.Np = S.Np;
    CKR(cudaMemcpyAsync(b.w, weights, Np * 4, cudaMemcpyHostToDevice, st));
    CKR(RC_DISPATCH(NL, frozen_hits(d, S.g, S.grid, ctx->c, p, prm->seed, prm->K, b.hits, st)));
    int launched = 0;
    if (ctx->adj_aeu_state != prm->state) {
        // G_l, the direct light of every light at unit emission, depends only on the state's
        // geometry and the light positions: built once per state (no voxel masks)
        CKR(RC_DISPATCH(NL, build(ctx->NW, d, S.g, S.grid, S.L, ones, AEu, nullptr, S.Np, ctx->flags_dev, st)));
        ctx->adj_aeu_state = prm->state;
        launched = 1;
    }
    CKR(adj::build_transpose(b, S.Np, prm->K, st));
    // the emissions of the forward solve: the state's, or the caller's
    std::vector<float> E = S.st[prm->state].inten;
    std::vector<DevBuf> tmp;
    struct TmpFree { std::vector<DevBuf>& p; ~TmpFree() { free_pool(p); } } tmp_free{tmp};
    const float* dem = nullptr;
    if (prm->emission) {
        for (int l = 0; l < NL; ++l) {
            if (!std::isfinite(prm->emission[l])) return fail(ctx, RC_ERR_ARG, "emission %d not finite", l);
            E[l] = prm->emission[l];
        }
        if ((s = dput(ctx, tmp, &dem, E))) return s;
    }
    CKR(adj::solve(&b, S.Np, prm->K, NL, AES, reinterpret_cast<const float*>(d.AE), reinterpret_cast<const float*>(AEu), dem, iters,
                   st));
    adj::Stats hs{};
    CKR(cudaMemcpyAsync(&hs, b.stats, sizeof hs, cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    ctx->launches += 9 + launched + 2 * iters;
    double jg = 0.0;
    for (int l = 0; l < NL; ++l) {
        dJ_dE[l] = (float)hs.out[l];
        jg += (double)E[l] * hs.out[l];
    }
    if (res) {
        auto f = [](unsigned x) { float v; memcpy(&v, &x, 4); return (double)v; };
        res->J = hs.out[NL];
        res->J_grad = jg;
        res->fwd_change = f(hs.chg[1]) > 0 ? f(hs.chg[0]) / f(hs.chg[1]) : 0.0;
        res->adj_change = f(hs.chg[3]) > 0 ? f(hs.chg[2]) / f(hs.chg[3]) : 0.0;
        res->rays = (long long)(Np * K);
        res->back = (long long)hs.back;
        res->max_incoming = hs.max_incoming;
    }
    ctx->adj = b;
    ctx->adj_np = S.Np;
    ctx->adj_k = prm->K;
    return RC_OK;
}

rc_status rc_adjoint_arrays(rc_ctx* ctx, float* L, float* u, int* hits) {
    if (!ctx) return RC_ERR_ARG;
    if (!ctx->adj_np) return fail(ctx, RC_ERR_STATE, "no adjoint computed");
    const size_t Np = (size_t)ctx->adj_np, K = (size_t)ctx->adj_k;
    cudaStream_t st = ctx->stream;
    if (L) CKR(cudaMemcpyAsync(L, ctx->adj.L_final, Np * 4, cudaMemcpyDeviceToHost, st));
    if (u) CKR(cudaMemcpyAsync(u, ctx->adj.u_final, Np * 4, cudaMemcpyDeviceToHost, st));
    if (hits) CKR(cudaMemcpyAsync(hits, ctx->adj.hits, Np * K * 4, cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    return RC_OK;
}


rc_status rc_taa_begin(rc_ctx* ctx, const rc_taa_method* m, int first_state, uint32_t seed) {
    if (!ctx || !m || m->mask < 0 || m->mask > 4) return RC_ERR_ARG;
    if (!ctx->have_scene) return fail(ctx, RC_ERR_STATE, "no scene loaded");
    const Scene& S = ctx->S;
    if (S.fmt != 2) return fail(ctx, RC_ERR_UNSUPPORTED, "taa mode: format-2 scenes only (as the reference)");
    if (!S.has_ref) return fail(ctx, RC_ERR_STATE, "taa mode needs a scene with references");
    if (first_state < 0 || first_state >= S.NS) return fail(ctx, RC_ERR_ARG, "state %d out of range", first_state);
    CKR(cudaSetDevice(ctx->cfg.device));
    rc_status s;
    if ((s = ensure_state(ctx, first_state))) return s;
    if (!ctx->taa.x && (s = taa_alloc(ctx))) return s;
    TaaRun& t = ctx->taa;
    const size_t Np = (size_t)S.Np, NW = (size_t)ctx->NW;
    cudaStream_t st = ctx->stream;
    // poc_gpu.cu:1241-1245: converged history, masks and counters cleared
    CKR(cudaMemcpyAsync(t.H, S.st[first_state].d.ref, Np * 4, cudaMemcpyDeviceToDevice, st));
    CKR(cudaMemsetAsync(t.react, 0, Np * 4, st));
    CKR(cudaMemsetAsync(t.pend, 0, Np, st));
    CKR(cudaMemsetAsync(t.cur, 0, NW * Np * 4, st));
    CKR(cudaMemsetAsync(t.prev, 0, NW * Np * 4, st));
    t.M = *m;
    t.seed = seed;
    t.f = 0;
    t.ref_sum.assign(S.NS, 0.0);
    t.ref_cnt.assign(S.NS, 0.0);
    t.have_sums.assign(S.NS, 0);
    t.prev_state = first_state;
    t.verify_left = 0;
    t.active = true;
    return RC_OK;
}

// One frame of run_taa_mode's loop (poc_gpu.cu:1246-1274).
rc_status rc_taa_frame(rc_ctx* ctx, int state, float* err) {
    if (!ctx) return RC_ERR_ARG;
    TaaRun& t = ctx->taa;
    if (!t.active) return fail(ctx, RC_ERR_STATE, "no taa run begun");
    const Scene& S = ctx->S;
    if (state < 0 || state >= S.NS) return fail(ctx, RC_ERR_ARG, "state %d out of range", state);
    if (rc_status es = ensure_state(ctx, state)) return es;
    const int Np = S.Np, NW = ctx->NW, f = t.f;
    const size_t nbytes_mask = (size_t)NW * Np * 4;
    cudaStream_t st = ctx->stream;
    const rc_taa_method& M = t.M;
    const bool deps = M.mask == 2 || M.mask == 3;
    if (deps && f % 32 == 0) {
        std::swap(t.cur, t.prev);
        CKR(cudaMemsetAsync(t.cur, 0, nbytes_mask, st));
    }
    const DState& d = S.st[state].d;
    FrameParams p{};
    p.Np = Np;
    p.NR = S.NR;
    CKR(RC_DISPATCH(S.NL, taa_sample(NW, deps, d, S.g, S.grid, ctx->c, p, t.x, t.cur, t.seed, (uint32_t)f, st)));
    int kernels = 1;
    if (f > 0 && t.prev_state != state) {
        const size_t pe = (size_t)t.prev_state * S.NS + state;
        if (M.mask == 2) { CKR(taa::touch(t.cur, t.prev, Np, t.dV[pe], t.nV[pe], t.react, t.pend, TAA_RF, 0, st)); ++kernels; }
        if (M.mask == 3) {
            CKR(taa::touch(t.cur, t.prev, Np, t.dV[pe], t.nV[pe], t.react, t.pend, TAA_RF, 1, st));
            t.verify_left = 2;
            CKR(cudaMemsetAsync(t.rs, 0, 3 * (size_t)S.NR * 4, st));
            CKR(cudaMemsetAsync(t.cnt, 0, (size_t)S.NR * 4, st));
            ++kernels;
        }
        if (M.mask == 4) { CKR(taa::oracle(S.st[t.prev_state].d.ref, d.ref, Np, t.react, TAA_RF, st)); ++kernels; }
    }
    if (M.mask == 1) {   // blind detection every frame
        CKR(cudaMemsetAsync(t.rs, 0, 3 * (size_t)S.NR * 4, st));
        CKR(cudaMemsetAsync(t.cnt, 0, (size_t)S.NR * 4, st));
        CKR(taa::zone_acc(t.x, t.H, t.pend, S.g.region, Np, t.rs, t.cnt, 0, st));
        CKR(taa::zone_decide(t.rs, t.cnt, t.pend, S.g.region, Np, t.react, 0, TAA_RF, 0, st));
        kernels += 2;
    }
    if (M.mask == 3 && t.verify_left > 0) {   // verification over the flagged points, two frames
        CKR(taa::zone_acc(t.x, t.H, t.pend, S.g.region, Np, t.rs, t.cnt, 1, st));
        ++kernels;
        if (--t.verify_left == 0) {
            CKR(taa::zone_decide(t.rs, t.cnt, t.pend, S.g.region, Np, t.react, 1, TAA_RF, 1, st));
            ++kernels;
        }
    }
    if (err && !t.have_sums[state]) {
        double h[3];
        CKR(taa::ref_sums(d.ref, d.valid, Np, t.part, t.out, st));
        kernels += 2;
        CKR(cudaMemcpyAsync(h, t.out, sizeof h, cudaMemcpyDeviceToHost, st));
        CKR(cudaStreamSynchronize(st));
        t.ref_sum[state] = h[1];
        t.ref_cnt[state] = h[2];
        t.have_sums[state] = 1;
    }
    CKR(taa::post(t.x, t.qid, t.quad, t.H, t.H2, t.mu, t.sg, t.react, Np, M.alpha, TAA_ALPHA_R, M.gamma, d.ref, d.valid, err ? t.part : nullptr,
                  t.out, st));
    kernels += err ? 2 : 1;
    std::swap(t.H, t.H2);
    ctx->launches += kernels;
    t.prev_state = state;
    t.f = f + 1;
    if (err) {
        // the squared error through page-locked memory: one DMA, no staging copy
        if (!ctx->pinned) CKR(cudaMallocHost(&ctx->pinned, 8 * sizeof(double)));
        CKR(cudaMemcpyAsync(ctx->pinned, t.out, sizeof(double), cudaMemcpyDeviceToHost, st));
        CKR(cudaStreamSynchronize(st));
        const double d2 = ctx->pinned[0];
        const double rs = t.ref_sum[state], cn = t.ref_cnt[state];
        *err = (float)(cn > 0 && rs > 0 ? std::sqrt(d2 / cn) / (rs / cn) : 0.0);
    }
    return RC_OK;
}

rc_status rc_taa_array_copy(rc_ctx* ctx, int which, void* host, size_t nbytes, int to_device) {
    if (!ctx || !host) return RC_ERR_ARG;
    TaaRun& t = ctx->taa;
    if (!t.x) return fail(ctx, RC_ERR_STATE, "no taa run begun");
    const size_t Np = (size_t)ctx->S.Np, NW = (size_t)ctx->NW;
    void* p = nullptr;
    size_t n = 0;
    switch (which) {
        case RC_T_X: p = t.x; n = 4 * Np; break;
        case RC_T_H: p = t.H; n = 4 * Np; break;
        case RC_T_MU: p = t.mu; n = 4 * Np; break;
        case RC_T_SG: p = t.sg; n = 4 * Np; break;
        case RC_T_REACT: p = t.react; n = 4 * Np; break;
        case RC_T_PEND: p = t.pend; n = Np; break;
        case RC_T_CUR: p = t.cur; n = 4 * NW * Np; break;
        case RC_T_PREV: p = t.prev; n = 4 * NW * Np; break;
        default: return fail(ctx, RC_ERR_ARG, "taa array %d", which);
    }
    if (nbytes != n) return fail(ctx, RC_ERR_ARG, "taa array %d holds %zu bytes", which, n);
    CKR(cudaMemcpyAsync(to_device ? p : host, to_device ? host : p, n, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                        ctx->stream));
    CKR(cudaStreamSynchronize(ctx->stream));
    return RC_OK;
}

rc_status rc_hg_camera_paths(rc_hg* hg, rc_ctx* ctx, int state, const rc_hg_path_params* prm, float* d_image) {
    if (!hg || !ctx || !prm) return RC_ERR_ARG;
    if (!ctx->have_scene) return fail(ctx, RC_ERR_STATE, "no scene loaded");
    const Scene& S = ctx->S;
    if (state < 0 || state >= S.NS) return fail(ctx, RC_ERR_ARG, "state %d out of range", state);
    if (prm->bounces < 0 || prm->bounces >= RC_HG_MAX_DEPTH) return fail(ctx, RC_ERR_ARG, "bounces %d", prm->bounces);
    const rc_camera* cam = &prm->cam;
    if (cam->width <= 0 || cam->height <= 0 || cam->width > 16384 || cam->height > 16384 || !(cam->fov_y_deg > 0.f && cam->fov_y_deg < 179.f))
        return fail(ctx, RC_ERR_ARG, "bad camera");
    if (S.NL > 32) return fail(ctx, RC_ERR_UNSUPPORTED, "%d lights", S.NL);
    CameraD cd;
    rc_status st = camera_basis(ctx, cam, &cd);
    if (st != RC_OK) return st;
    const size_t npix = (size_t)cam->width * cam->height, S1 = (size_t)prm->bounces + 1, nslots = npix * S1;
    auto& C = ctx->cam;
    CKR(cudaSetDevice(ctx->cfg.device));
    cudaStream_t hs = rc::hg_stream(hg);
    if ((st = ensure_state(ctx, state))) return st;
    if (nslots > C.slots_cap || npix > C.pix_cap) {
        CKR(cudaStreamSynchronize(hs));
        CKR(cudaStreamSynchronize(ctx->stream));
        free_pool(ctx->cam_bufs);
        C.slots_cap = C.pix_cap = 0;
        auto& pool = ctx->cam_bufs;
        if ((st = dalloc(ctx, pool, &C.pos, 3 * nslots)) || (st = dalloc(ctx, pool, &C.nrm, 3 * nslots)) ||
            (st = dalloc(ctx, pool, &C.rgb, 3 * nslots)) || (st = dalloc(ctx, pool, &C.vtx, nslots)) ||
            (st = dalloc(ctx, pool, &C.entry, nslots)) || (st = dalloc(ctx, pool, &C.len, npix)))
            return st;
        C.slots_cap = nslots;
        C.pix_cap = npix;
    }
    if (!C.ready) CKR(cudaEventCreateWithFlags(&C.ready, cudaEventDisableTiming));
    // lights and path shape
    PathD pd{};
    pd.bounces = prm->bounces;
    pd.slots = (int)S1;
    pd.seed = prm->seed;
    pd.frame = prm->frame;
    pd.td = rc::hg_config(hg).tracing_distance;
    pd.nl = S.NL;
    bool white = true;
    for (int l = 0; l < S.NL; ++l)
        for (int k = 0; k < 3; ++k) white = white && prm->light_rgb[l][k] == 0.f;
    for (int l = 0; l < S.NL; ++l) {
        for (int k = 0; k < 3; ++k) {
            pd.lpos[l][k] = S.hL[3 * (size_t)l + k];
            pd.lrgb[l][k] = white ? 1.f : prm->light_rgb[l][k];
        }
        pd.lint[l] = S.st[state].inten[l];
    }
    const float* ar = prm->area_rgb;
    pd.area_on = ar[0] > 0.f || ar[1] > 0.f || ar[2] > 0.f;
    if (pd.area_on) {
        const float* u = prm->area_u;
        const float* v = prm->area_v;
        const double n[3] = {(double)u[1] * v[2] - (double)u[2] * v[1], (double)u[2] * v[0] - (double)u[0] * v[2],
                             (double)u[0] * v[1] - (double)u[1] * v[0]};
        const double a = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (!(a > 0)) return fail(ctx, RC_ERR_ARG, "degenerate rectangle light");
        for (int k = 0; k < 3; ++k) {
            pd.ac[k] = prm->area_corner[k];
            pd.au[k] = u[k];
            pd.av[k] = v[k];
            pd.an[k] = (float)(n[k] / a);
            pd.argb[k] = ar[k];
        }
        pd.aarea = (float)a;
    }
    const float* sr = prm->sun_rgb;
    pd.sun_on = sr[0] > 0.f || sr[1] > 0.f || sr[2] > 0.f;
    if (pd.sun_on) {
        const double d[3] = {prm->sun_dir[0], prm->sun_dir[1], prm->sun_dir[2]};
        const double l = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        if (!(l > 0)) return fail(ctx, RC_ERR_ARG, "sun direction is zero");
        for (int k = 0; k < 3; ++k) {
            pd.sdir[k] = (float)(d[k] / l);
            pd.srgb[k] = sr[k];
        }
    }
    for (int k = 0; k < 3; ++k) pd.sky[k] = prm->sky_rgb[k];
    // after the context's own work, on the cache's stream
    CKR(cudaEventRecord(C.ready, ctx->stream));
    CKR(cudaStreamWaitEvent(hs, C.ready, 0));
    FrameParams p{};
    p.Np = S.Np;
    p.NR = S.NR;
    CKR(RC_DISPATCH(S.NL, paths(S.st[state].d, S.g, S.grid, ctx->c, p, cd, pd, C.pos, C.nrm, C.rgb, C.vtx, C.len, d_image, hs)));
    const int n = (int)nslots, np = (int)npix;
    if ((st = rc_hg_insert(hg, C.pos, C.nrm, n, C.entry))) return fail(ctx, st, "insert: %s", rc_hg_last_error(hg));
    CKR(rc::hg_set_entries(hg, C.vtx, C.entry, (long long)nslots));
    if ((st = rc_hg_accumulate(hg, C.entry, C.rgb, n))) return fail(ctx, st, "accumulate: %s", rc_hg_last_error(hg));
    if ((st = rc_hg_mark_paths_strided(hg, C.vtx, C.len, (int)S1, np))) return fail(ctx, st, "mark: %s", rc_hg_last_error(hg));
    if (rc::hg_has_voxels(hg) && (st = rc_hg_voxels_mark(hg, C.vtx, C.len, (int)S1, np)))
        return fail(ctx, st, "voxels: %s", rc_hg_last_error(hg));
    // the context's later work waits for this pass
    CKR(cudaEventRecord(C.ready, hs));
    CKR(cudaStreamWaitEvent(ctx->stream, C.ready, 0));
    C.stride = (int)S1;
    C.npaths = np;
    ctx->launches += 6;
    return RC_OK;
}

rc_status rc_hg_camera_arrays(rc_ctx* ctx, const rc_hg_vertex** d_vertices, const float** d_rgb, const uint32_t** d_entry,
                              const int** d_len, int* stride, int* npaths) {
    if (!ctx) return RC_ERR_ARG;
    const auto& C = ctx->cam;
    if (!C.npaths) return fail(ctx, RC_ERR_STATE, "no camera pass");
    if (d_vertices) *d_vertices = C.vtx;
    if (d_rgb) *d_rgb = C.rgb;
    if (d_entry) *d_entry = C.entry;
    if (d_len) *d_len = C.len;
    if (stride) *stride = C.stride;
    if (npaths) *npaths = C.npaths;
    return RC_OK;
}

}  // extern "C"

namespace rc {

rc_status ctx_fail(rc_ctx* ctx, rc_status s, const char* fmt, ...) {
    char buf[512];
    va_list a;
    va_start(a, fmt);
    vsnprintf(buf, sizeof buf, fmt, a);
    va_end(a);
    if (ctx) ctx->err = buf;
    return s;
}

}  // namespace rc

extern "C" {

rc_status rc_device_flags(rc_ctx* ctx, unsigned* flags) {
    if (!ctx || !flags) return RC_ERR_ARG;
    if (ctx->side) CKR(cudaStreamSynchronize(ctx->side));   // state builds raise guards too
    CKR(cudaMemcpyAsync(flags, ctx->flags_dev, 4, cudaMemcpyDeviceToHost, ctx->stream));
    CKR(cudaMemsetAsync(ctx->flags_dev, 0, 4, ctx->stream));
    CKR(cudaStreamSynchronize(ctx->stream));
    return RC_OK;
}

}  // extern "C"
