// Driver for the reference's own kernels — TEST AND BASELINE INFRASTRUCTURE ONLY.
//
// oracle/build_ref.sh compiles the reference's cuda/poc_gpu.cu (unchanged, from the
// reference checkout) into a device-only cubin under oracle/_ref/.  This file loads that
// cubin with the CUDA driver API and runs its kernels (k_build, k_trace2<DEPS>, k_decide,
// k_update, k_sumpr, k_touched, k_wake, k_rescale, k_restored, k_proj_apply, k_oracle,
// k_error, and the taa mode's k_taa_*) with the host logic of the reference's load(),
// Runner::run and run_taa_mode (poc_gpu.cu:751-801, 826-1016, 1175-1282) restated here,
// including its per-frame event timing.
// The kernel argument structs below mirror the reference's DevState / Cache / Params
// (poc_gpu.cu:222-237, 394-422) field for field, since the kernels read them by value.
//
// Used by the GPU parity tests (bit-exact comparison of the product kernels with the
// reference kernels from identical state) and by the reference arm of the benchmark.
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr int KSNAP = 6, NEQ = 28, VERIF_FRAMES = 4, PROJ_FRAMES = 4, MAXNL = 32;

struct float4_ { float x, y, z, w; };

// poc_gpu.cu:222-237 (inten sized for the largest light count this driver supports; the
// struct is rebuilt per light count in dev_state_bytes()).
struct RefMethod {
    int mode; float nmax, budget; int deps, verify, oracle, track_every, rescale, resp_mask; float nmax_resp;
    int ddgi; float ddgi_h, ddgi_thr; int ddgi_clamp, memory, ramp, wake_verify, snaps, proj, snap_verify; float rays;
};

struct Cache {   // poc_gpu.cu:394-409
    float *Lc, *Lc2, *m, *n, *c0;
    int* kk;
    uint8_t* pending;
    uint32_t *cur, *prev;
    float* rstat;
    float* dstat;
    uint8_t* stale;
    float* snap;
    float* neq;
    float* coef;
    float* age;
    float* sumpr;
    int* npend;
    double* err;
};

struct Params {  // poc_gpu.cu:411-422
    int Np, NR, mode;
    float budget, nmax;
    uint32_t seed, frame;
    int pend_left, deps;
    int resp_mask; float nmax_resp;
    int ddgi; float ddgi_h, ddgi_thr; int ddgi_clamp;
    int dormant;
    int ramp;
    int proj_left, projK; int slot[6];
    float rays;
};

struct HostState {
    std::vector<float> inten;
    CUdeviceptr P = 0, N = 0, Q = 0, T = 0, Edir = 0, ref = 0, Pw = 0, dims = 0, off = 0, TQ = 0, SV = 0, valid = 0;
};

struct Timers { double trace = 0, decide = 0, update = 0, swap = 0, event = 0; int frames = 0, events = 0; };

struct Taa {   // poc_gpu.cu:1051-1060
    float *x, *H, *H2, *mu, *sg;
    int* nb;
    int* react;
    uint8_t* pend;
    uint32_t *cur, *prev;
    float* rs;
    double* err;
};

}  // namespace

struct ref_ctx {
    int NL = 3, NW = 4, VX = 8, VY = 4, VZ = 4;
    CUcontext cu = nullptr;
    CUmodule mod = nullptr;
    CUfunction f_build, f_trace[2], f_decide, f_update, f_sumpr, f_touched, f_wake, f_rescale, f_restored, f_proj, f_oracle, f_error;
    CUdeviceptr c_lo = 0, c_ext = 0;
    std::string err;
    std::vector<CUdeviceptr> bufs;
    // scene
    int Np = 0, Nq = 0, Nt = 0, NS = 0, NR = 0, has_ref = 0, fmt = 2, nst = 0;
    CUdeviceptr ST = 0, STN = 0, BN = 0, HK = 0, HV = 0;
    unsigned hmask = 0; float hcell = 0.f;
    CUdeviceptr dL = 0, dA = 0, dRegion = 0;
    std::vector<HostState> st;
    std::vector<std::vector<int>> occ, em;
    std::vector<CUdeviceptr> dOcc, dEm;
    Cache c{};
    // run
    RefMethod M{};
    Params p{};
    int dormant = 0; float ilearn[32] = {0};
    int pend_left = 0, nslots = 0, slot_state[KSNAP], slot_next = 0, last_event_f = 0, proj_left = 0;
    int prev_state = 0, f = 0;
    float nmax = 0.f;
    CUevent ev[6] = {};
    bool loaded = false;
    // taa mode (run_taa_mode, poc_gpu.cu:1175-1282)
    CUfunction f_taa_pt[2], f_taa_stats, f_taa_zacc, f_taa_zdec, f_taa_count, f_taa_touch, f_taa_oracle, f_taa_update, f_taa_err;
    std::vector<float> hL;
    std::vector<int> hdims, hoff;
    Taa taa{};
    float* taa_cnt = nullptr;
    std::vector<std::vector<int>> taaV;
    std::vector<CUdeviceptr> dTaaV;
    float taa_alpha = 0.1f, taa_gamma = 1.f;
    int taa_mask = 0, taa_f = 0, taa_prev = 0, taa_verify = 0;
    uint32_t taa_seed = 0;
};

namespace {

int fail(ref_ctx* r, const char* what, CUresult e) {
    const char* s = nullptr;
    cuGetErrorString(e, &s);
    char b[512];
    snprintf(b, sizeof b, "%s: %s", what, s ? s : "?");
    r->err = b;
    return -1;
}
#define CKD(x, what) do { CUresult e_ = (x); if (e_ != CUDA_SUCCESS) return fail(r, what, e_); } while (0)

CUdeviceptr alloc(ref_ctx* r, size_t bytes) {
    CUdeviceptr p = 0;
    if (cuMemAlloc(&p, bytes + 16) != CUDA_SUCCESS) return 0;
    r->bufs.push_back(p);
    return p;
}
template <class T>
CUdeviceptr put(ref_ctx* r, const std::vector<T>& v) {
    CUdeviceptr p = alloc(r, v.size() * sizeof(T));
    if (p && !v.empty()) cuMemcpyHtoD(p, v.data(), v.size() * sizeof(T));
    return p;
}

// DevState (poc_gpu.cu:222-237) laid out as the device compiler does for this light count.
std::vector<uint8_t> dev_state_bytes(const ref_ctx* r, const HostState& h) {
    std::vector<uint8_t> b;
    auto pad = [&](size_t a) { while (b.size() % a) b.push_back(0); };
    auto ptr = [&](CUdeviceptr p) { pad(8); uint64_t v = p; b.insert(b.end(), (uint8_t*)&v, (uint8_t*)&v + 8); };
    auto i32 = [&](int v) { pad(4); b.insert(b.end(), (uint8_t*)&v, (uint8_t*)&v + 4); };
    auto f32 = [&](float v) { pad(4); b.insert(b.end(), (uint8_t*)&v, (uint8_t*)&v + 4); };
    ptr(h.P); ptr(h.N); ptr(h.Q); ptr(h.T); ptr(h.Edir); ptr(h.ref); ptr(h.Pw);
    ptr(h.dims); ptr(h.off); ptr(h.TQ);
    ptr(h.SV);
    ptr(h.valid);
    for (int l = 0; l < r->NL; ++l) f32(h.inten[l]);
    i32(r->Nt);
    ptr(r->ST); ptr(r->STN); ptr(r->BN); ptr(r->HK); ptr(r->HV);
    uint32_t hm = r->hmask;
    pad(4); b.insert(b.end(), (uint8_t*)&hm, (uint8_t*)&hm + 4);
    f32(r->hcell);
    pad(8);
    return b;
}

int launch(ref_ctx* r, CUfunction fn, int grid, unsigned smem, std::vector<void*> args, const char* what) {
    CKD(cuLaunchKernel(fn, grid, 1, 1, 256, 1, 1, smem, nullptr, args.data(), nullptr), what);
    return 0;
}

struct Rd {
    const uint8_t* p; size_t n, off = 0; bool bad = false;
    template <class T> std::vector<T> vec(size_t cnt) {
        if (bad || cnt > (n - off) / sizeof(T)) { bad = true; return {}; }
        std::vector<T> v(cnt);
        if (cnt) memcpy(v.data(), p + off, cnt * sizeof(T));
        off += cnt * sizeof(T);
        return v;
    }
};

std::vector<int> to_grid(const ref_ctx* r, const std::vector<int>& fine) {   // poc_gpu.cu:720-735
    const int FX = 16, FY = 8, FZ = 6, VX = r->VX, VY = r->VY, VZ = r->VZ;
    const float X1 = 8.f, Y1 = 4.f, Z1 = 3.f;
    std::vector<char> mark((size_t)VX * VY * VZ, 0);
    for (int v : fine) {
        int i = v % FX, j = (v / FX) % FY, k = v / (FX * FY);
        float x0 = i * X1 / FX, x1 = (i + 1) * X1 / FX, y0 = j * Y1 / FY, y1 = (j + 1) * Y1 / FY;
        float z0 = k * Z1 / FZ, z1 = (k + 1) * Z1 / FZ;
        int a0 = std::min(int(x0 / X1 * VX + 1e-4f), VX - 1), a1 = std::min(int(x1 / X1 * VX - 1e-4f), VX - 1);
        int b0 = std::min(int(y0 / Y1 * VY + 1e-4f), VY - 1), b1 = std::min(int(y1 / Y1 * VY - 1e-4f), VY - 1);
        int c0 = std::min(int(z0 / Z1 * VZ + 1e-4f), VZ - 1), c1 = std::min(int(z1 / Z1 * VZ - 1e-4f), VZ - 1);
        for (int a = a0; a <= a1; ++a) for (int b = b0; b <= b1; ++b) for (int c = c0; c <= c1; ++c) mark[(c * VY + b) * VX + a] = 1;
    }
    std::vector<int> out;
    for (size_t v = 0; v < mark.size(); ++v) if (mark[v]) out.push_back((int)v);
    return out;
}

int grid_of(const ref_ctx* r) { return (r->Np + 255) / 256; }

}  // namespace

extern "C" {

const char* ref_last_error(ref_ctx* r) { return r ? r->err.c_str() : "no context"; }

// The cubin's transit grid (its -DGX/-DGY/-DGZ) is vx x vy x vz; NW = vx vy vz / 32.
ref_ctx* ref_create_grid(const char* cubin, int nl, int vx, int vy, int vz, char* err, int errlen) {
    auto seterr = [&](const char* m) { if (err && errlen > 0) { strncpy(err, m, errlen - 1); err[errlen - 1] = 0; } };
    if (nl <= 0 || nl > MAXNL) { seterr("light count"); return nullptr; }
    if (vx <= 0 || vy <= 0 || vz <= 0 || (vx * vy * vz) % 128) { seterr("transit grid"); return nullptr; }
    if (cuInit(0) != CUDA_SUCCESS) { seterr("cuInit failed"); return nullptr; }
    ref_ctx* r = new ref_ctx();
    r->NL = nl;
    r->VX = vx;
    r->VY = vy;
    r->VZ = vz;
    r->NW = vx * vy * vz / 32;
    CUdevice dev;
    if (cuDeviceGet(&dev, 0) != CUDA_SUCCESS || cuDevicePrimaryCtxRetain(&r->cu, dev) != CUDA_SUCCESS ||
        cuCtxSetCurrent(r->cu) != CUDA_SUCCESS) { seterr("no CUDA context"); delete r; return nullptr; }
    if (cuModuleLoad(&r->mod, cubin) != CUDA_SUCCESS) { seterr("cannot load the reference cubin"); delete r; return nullptr; }
    struct { CUfunction* f; const char* n; } fns[] = {
        {&r->f_build, "_Z7k_build8DevStatePKfi"},
        {&r->f_trace[0], "_Z8k_trace2ILb0EEv8DevState5Cache6ParamsPKiPKf"},
        {&r->f_trace[1], "_Z8k_trace2ILb1EEv8DevState5Cache6ParamsPKiPKf"},
        {&r->f_decide, "_Z8k_decide5Cache6ParamsPKi"},
        {&r->f_update, "_Z8k_update5Cache6ParamsPKi"},
        {&r->f_sumpr, "_Z7k_sumpr5Cachei"},
        {&r->f_touched, "_Z9k_touched5CacheiPKiiii"},
        {&r->f_wake, "_Z6k_wake5Cacheiiii"},
        {&r->f_rescale, "_Z9k_rescale5Cacheiif"},
        {&r->f_restored, "_Z10k_restored5Cacheifii"},
        {&r->f_proj, "_Z12k_proj_apply5Cache6ParamsPKi"},
        {&r->f_oracle, "_Z8k_oracle5CacheiPKfS1_"},
        {&r->f_error, "_Z7k_error5CacheiPKfPKhi"},
        {&r->f_taa_pt[0], "_Z8k_taa_ptILb0EEv8DevState3TaaijjPKf"},
        {&r->f_taa_pt[1], "_Z8k_taa_ptILb1EEv8DevState3TaaijjPKf"},
        {&r->f_taa_stats, "_Z11k_taa_stats3Taai"},
        {&r->f_taa_zacc, "_Z14k_taa_zone_acc3TaaiPKii"},
        {&r->f_taa_zdec, "_Z17k_taa_zone_decide3TaaiPKiPKfiii"},
        {&r->f_taa_count, "_Z12k_count_zoneiPKiPKhiPf"},
        {&r->f_taa_touch, "_Z11k_taa_touch3TaaiPKiiii"},
        {&r->f_taa_oracle, "_Z12k_taa_oracle3TaaiPKfS1_i"},
        {&r->f_taa_update, "_Z12k_taa_update3Taaifff"},
        {&r->f_taa_err, "_Z9k_taa_err3TaaiPKfPKh"},
    };
    for (auto& x : fns)
        if (cuModuleGetFunction(x.f, r->mod, x.n) != CUDA_SUCCESS) { seterr(x.n); delete r; return nullptr; }
    size_t b1, b2;
    if (cuModuleGetGlobal(&r->c_lo, &b1, r->mod, "c_lo") != CUDA_SUCCESS || cuModuleGetGlobal(&r->c_ext, &b2, r->mod, "c_ext") != CUDA_SUCCESS) {
        seterr("bounds symbols"); delete r; return nullptr;
    }
    for (auto& e : r->ev) cuEventCreate(&e, CU_EVENT_DEFAULT);
    return r;
}

ref_ctx* ref_create(const char* cubin, int nl, char* err, int errlen) { return ref_create_grid(cubin, nl, 8, 4, 4, err, errlen); }

void ref_destroy(ref_ctx* r) {
    if (!r) return;
    cuCtxSynchronize();
    for (auto p : r->bufs) cuMemFree(p);
    for (auto& e : r->ev) if (e) cuEventDestroy(e);
    if (r->mod) cuModuleUnload(r->mod);
    delete r;
}

// load() + k_build (poc_gpu.cu:751-801)
int ref_load(ref_ctx* r, const void* data, size_t n) {
    cuCtxSetCurrent(r->cu);
    Rd rd{(const uint8_t*)data, n};
    auto h = rd.vec<int>(8);
    if (rd.bad || h[4] != r->NL || (h[7] != 2 && h[7] != 3)) { r->err = "scene header"; return -1; }
    r->Np = h[0]; r->Nq = h[1]; r->Nt = h[2]; r->NS = h[3]; r->NR = h[5]; r->has_ref = h[6]; r->fmt = h[7];
    const int NL = r->NL;
    const size_t Np = r->Np;
    float lo[3] = {0, 0, 0}, ext[3] = {8.f, 4.f, 3.f};
    if (r->fmt == 3) {
        auto l = rd.vec<float>(3), e = rd.vec<float>(3), hc = rd.vec<float>(1);
        auto m = rd.vec<int>(4);
        if (rd.bad) { r->err = "mesh block"; return -1; }
        memcpy(lo, l.data(), 12); memcpy(ext, e.data(), 12);
        r->hcell = hc[0];
        r->ST = put(r, rd.vec<float>(9 * (size_t)m[0])); r->STN = put(r, rd.vec<float>(4 * (size_t)m[0]));
        r->BN = put(r, rd.vec<float>(8 * (size_t)m[1])); r->HK = put(r, rd.vec<unsigned long long>((size_t)m[2]));
        r->HV = put(r, rd.vec<int>((size_t)m[2]));
        r->hmask = (unsigned)m[2] - 1; r->nst = m[0];
    }
    CKD(cuMemcpyHtoD(r->c_lo, lo, 12), "c_lo");
    CKD(cuMemcpyHtoD(r->c_ext, ext, 12), "c_ext");
    auto L = rd.vec<float>(3 * (size_t)NL);
    r->hL = L;
    auto A = rd.vec<float>(Np);
    auto region = rd.vec<int>(Np);
    r->st.assign(r->NS, HostState());
    for (int s = 0; s < r->NS; ++s) {
        HostState& d = r->st[s];
        d.inten = rd.vec<float>(NL);
        d.P = put(r, rd.vec<float>(3 * Np)); d.N = put(r, rd.vec<float>(3 * Np)); d.Q = put(r, rd.vec<float>(12 * (size_t)r->Nq));
        auto dims = rd.vec<int>(2 * (size_t)r->Nq), off = rd.vec<int>((size_t)r->Nq);
        if (s == 0) { r->hdims = dims; r->hoff = off; }   // poc_gpu.cu:783
        d.dims = put(r, dims); d.off = put(r, off);
        d.T = put(r, rd.vec<float>(9 * (size_t)r->Nt)); d.TQ = put(r, rd.vec<int>((size_t)r->Nt));
        if (r->has_ref) { d.ref = put(r, rd.vec<float>(Np)); d.valid = put(r, rd.vec<uint8_t>(Np)); d.Pw = put(r, rd.vec<float>((size_t)NL * Np)); }
        d.Edir = alloc(r, 4 * (size_t)NL * Np); d.SV = alloc(r, 4 * (size_t)r->NW * Np);
    }
    r->occ.clear(); r->em.clear();
    for (int e = 0; e < r->NS * r->NS; ++e) {
        auto no = rd.vec<int>(1);
        if (rd.bad) break;
        auto o = rd.vec<int>((size_t)no[0]);
        r->occ.push_back(r->fmt == 3 ? o : to_grid(r, o));
        for (int l = 0; l < NL; ++l) {
            auto ne = rd.vec<int>(1);
            if (rd.bad) break;
            auto m = rd.vec<int>((size_t)ne[0]);
            r->em.push_back(r->fmt == 3 ? m : to_grid(r, m));
        }
    }
    if (rd.bad) { r->err = "truncated scene"; return -1; }
    r->dL = put(r, L); r->dA = put(r, A); r->dRegion = put(r, region);
    for (auto& o : r->occ) r->dOcc.push_back(put(r, o.empty() ? std::vector<int>{0} : o));
    for (auto& m : r->em) r->dEm.push_back(put(r, m.empty() ? std::vector<int>{0} : m));
    // Runner constructor (poc_gpu.cu:812-823)
    Cache& c = r->c;
    c.Lc = (float*)alloc(r, 4 * NL * Np); c.Lc2 = (float*)alloc(r, 4 * NL * Np); c.m = (float*)alloc(r, 4 * NL * Np);
    c.n = (float*)alloc(r, 4 * Np); c.c0 = (float*)alloc(r, 4 * Np); c.kk = (int*)alloc(r, 4 * Np); c.pending = (uint8_t*)alloc(r, Np);
    c.cur = (uint32_t*)alloc(r, 4 * r->NW * Np); c.prev = (uint32_t*)alloc(r, 4 * r->NW * Np);
    c.stale = (uint8_t*)alloc(r, Np); c.age = (float*)alloc(r, 4 * Np);
    c.snap = (float*)alloc(r, 4 * (size_t)KSNAP * Np * NL); c.neq = (float*)alloc(r, 4 * (size_t)r->NR * NEQ);
    c.coef = (float*)alloc(r, 4 * (size_t)r->NR * KSNAP); c.rstat = (float*)alloc(r, 16 * (size_t)r->NR);
    c.dstat = (float*)alloc(r, 12 * (size_t)r->NR); c.sumpr = (float*)alloc(r, 8); c.npend = (int*)alloc(r, 8); c.err = (double*)alloc(r, 24);
    unsigned shm = r->Nt * 10 * 4;
    for (auto& d : r->st) {
        auto b = dev_state_bytes(r, d);
        CUdeviceptr dl = r->dL;
        int np = r->Np;
        if (launch(r, r->f_build, grid_of(r), shm, {b.data(), &dl, &np}, "k_build")) return -1;
    }
    CKD(cuCtxSynchronize(), "k_build");
    r->loaded = true;
    return 0;
}

int ref_begin(ref_ctx* r, const RefMethod* m, int s0, uint32_t seed) {
    if (!r->loaded) return -1;
    cuCtxSetCurrent(r->cu);
    const size_t Np = r->Np, NL = r->NL;
    Cache& c = r->c;
    r->M = *m;
    if (r->M.track_every <= 0) r->M.track_every = 1;
    // poc_gpu.cu:830-850
    if (r->has_ref) CKD(cuMemcpyDtoD((CUdeviceptr)c.Lc, r->st[s0].Pw, NL * Np * 4), "warm");
    else CKD(cuMemsetD8((CUdeviceptr)c.Lc, 0, NL * Np * 4), "warm");
    r->nmax = m->nmax * m->rays;
    std::vector<float> nm(Np, r->nmax), ag(Np, 1e4f);
    CKD(cuMemcpyHtoD((CUdeviceptr)c.n, nm.data(), Np * 4), "n");
    CKD(cuMemsetD8((CUdeviceptr)c.pending, 0, Np), "pending");
    CKD(cuMemsetD8((CUdeviceptr)c.cur, 0, r->NW * Np * 4), "cur");
    CKD(cuMemsetD8((CUdeviceptr)c.prev, 0, r->NW * Np * 4), "prev");
    CKD(cuMemsetD8((CUdeviceptr)c.stale, 0, Np), "stale");
    CKD(cuMemcpyHtoD((CUdeviceptr)c.age, ag.data(), Np * 4), "age");
    float sp[2] = {float(r->Np) / (r->nmax + 1.f), 0.f};
    int z2[2] = {0, 0};
    CKD(cuMemcpyHtoD((CUdeviceptr)c.sumpr, sp, 8), "sumpr");
    CKD(cuMemcpyHtoD((CUdeviceptr)c.npend, z2, 8), "npend");
    r->dormant = 0;
    for (auto& x : r->ilearn) x = 0.f;
    Params p{};
    p.Np = r->Np; p.NR = r->NR; p.mode = m->mode; p.budget = m->budget; p.nmax = m->nmax; p.seed = seed; p.frame = 0;
    p.pend_left = 0; p.deps = m->deps; p.resp_mask = m->resp_mask; p.nmax_resp = m->nmax_resp; p.ddgi = m->ddgi ? 1 : 0;
    p.ddgi_h = m->ddgi_h; p.ddgi_thr = m->ddgi_thr; p.ddgi_clamp = m->ddgi_clamp ? 1 : 0; p.dormant = 0; p.ramp = m->ramp ? 1 : 0;
    p.rays = m->rays; p.budget = m->budget * m->rays; p.nmax = r->nmax; p.nmax_resp = m->nmax_resp * m->rays;
    r->p = p;
    r->pend_left = 0; r->nslots = 0; r->slot_next = 0; r->last_event_f = 0; r->proj_left = 0;
    for (int k = 0; k < KSNAP; ++k) r->slot_state[k] = -1;
    r->prev_state = s0; r->f = 0;
    return 0;
}

static int dzero(ref_ctx* r, void* p, size_t bytes) { CKD(cuMemsetD8((CUdeviceptr)p, 0, bytes), "memset"); return 0; }
static int dcopy(ref_ctx* r, void* dst, const void* src, size_t bytes) { CKD(cuMemcpyDtoD((CUdeviceptr)dst, (CUdeviceptr)src, bytes), "copy"); return 0; }

// One frame of Runner::run (poc_gpu.cu:851-1011).  With ms != NULL the frame is timed like
// the reference's timing mode: ms[0..4] += swap, trace, decide, update, event.
int ref_frame(ref_ctx* r, int si, int want_err, float* errv, double* ms) {
    cuCtxSetCurrent(r->cu);
    const RefMethod& M = r->M;
    const int NL = r->NL, G = grid_of(r), f = r->f;
    const size_t Np = r->Np;
    Cache& c = r->c;
    Params& p = r->p;
    int Npi = r->Np;
    HostState& st = r->st[si];
    p.frame = (uint32_t)f;
    unsigned shm = r->Nt * 10 * 4;
    if (f > 0 && r->prev_state != si) {
        const int e = r->prev_state, pe = e * r->NS + si;
        if (ms) cuEventRecord(r->ev[4], nullptr);
        if (M.snaps && f - r->last_event_f >= 20) {
            int k = -1;
            for (int a = 0; a < r->nslots; ++a) if (r->slot_state[a] == e) k = a;
            if (k < 0) { if (r->nslots < KSNAP) k = r->nslots++; else { k = r->slot_next; r->slot_next = (r->slot_next + 1) % KSNAP; } }
            r->slot_state[k] = e;
            if (dcopy(r, c.snap + (size_t)k * Np * NL, c.Lc, Np * NL * 4)) return -1;
        }
        if (M.oracle && r->has_ref) {
            CUdeviceptr a = r->st[e].ref, b = st.ref;
            if (launch(r, r->f_oracle, G, 0, {&c, &Npi, &a, &b}, "k_oracle")) return -1;
        }
        auto rescale = [&](int l, float ratio) { return launch(r, r->f_rescale, G, 0, {&c, &Npi, &l, &ratio}, "k_rescale"); };
        if (M.rescale && !M.deps) {
            for (int l = 0; l < NL; ++l) {
                float a = r->st[e].inten[l], b = st.inten[l];
                if (a == b) continue;
                if (M.memory && a > 0 && b == 0) { r->dormant |= 1 << l; r->ilearn[l] = a; }
                else if (M.memory && a == 0 && b > 0 && ((r->dormant >> l) & 1)) { if (rescale(l, b / r->ilearn[l])) return -1; r->dormant &= ~(1 << l); }
                else if (a > 0) { if (rescale(l, b / a)) return -1; }
            }
        }
        if (M.deps) {
            int woke = 0;
            for (int l = 0; l < NL; ++l) {
                float a = r->st[e].inten[l], b = st.inten[l];
                if (a == b) continue;
                if (M.memory && a > 0 && b == 0) { r->dormant |= 1 << l; r->ilearn[l] = a; }
                else if (M.memory && a == 0 && b > 0 && ((r->dormant >> l) & 1)) {
                    if (rescale(l, b / r->ilearn[l])) return -1;
                    r->dormant &= ~(1 << l);
                    woke |= 1 << l;
                    int one = 1, zero = 0, dm = r->dormant, ll = l;
                    if (M.wake_verify) {
                        if (dzero(r, c.npend, 8) || dzero(r, c.rstat, 16 * (size_t)r->NR)) return -1;
                        if (launch(r, r->f_wake, G, 0, {&c, &Npi, &ll, &one, &dm}, "k_wake")) return -1;
                        if (dcopy(r, c.npend, c.npend + 1, 4)) return -1;
                        r->pend_left = VERIF_FRAMES;
                    } else if (launch(r, r->f_wake, G, 0, {&c, &Npi, &ll, &zero, &dm}, "k_wake")) return -1;
                } else if (a > 0) { if (rescale(l, b / a)) return -1; }
            }
            for (int l = 0; l < NL; ++l) {
                int ix = pe * NL + l;
                if (!r->em[ix].empty() && !((woke >> l) & 1)) {
                    CUdeviceptr V = r->dEm[ix];
                    int nv = (int)r->em[ix].size(), kind = 0, dm = r->dormant;
                    if (launch(r, r->f_touched, G, 0, {&c, &Npi, &V, &nv, &kind, &dm}, "k_touched")) return -1;
                }
            }
            if (!r->occ[pe].empty()) {
                CUdeviceptr V = r->dOcc[pe];
                int nv = (int)r->occ[pe].size(), dm = r->dormant;
                if (M.verify) {
                    int kind = 1;
                    if (dzero(r, c.npend, 8) || dzero(r, c.rstat, 16 * (size_t)r->NR)) return -1;
                    if (launch(r, r->f_touched, G, 0, {&c, &Npi, &V, &nv, &kind, &dm}, "k_touched")) return -1;
                    if (dcopy(r, c.npend, c.npend + 1, 4)) return -1;
                    r->pend_left = VERIF_FRAMES;
                } else if (r->dormant) {
                    int kind = 2;
                    if (launch(r, r->f_touched, G, 0, {&c, &Npi, &V, &nv, &kind, &dm}, "k_touched")) return -1;
                }
            }
        }
        if (M.snaps) {
            int hit = -1;
            for (int a = 0; a < r->nslots; ++a) if (r->slot_state[a] == si) hit = a;
            if (hit >= 0) {
                if (dcopy(r, c.Lc, c.snap + (size_t)hit * Np * NL, Np * NL * 4)) return -1;
                float nmax = r->nmax;
                int dm = r->dormant;
                if (M.snap_verify) {
                    int one = 1;
                    if (dzero(r, c.npend, 8) || dzero(r, c.rstat, 16 * (size_t)r->NR)) return -1;
                    if (launch(r, r->f_restored, G, 0, {&c, &Npi, &nmax, &dm, &one}, "k_restored")) return -1;
                    if (dcopy(r, c.npend, c.npend + 1, 4)) return -1;
                    r->pend_left = VERIF_FRAMES;
                } else {
                    int zero = 0;
                    if (launch(r, r->f_restored, G, 0, {&c, &Npi, &nmax, &dm, &zero}, "k_restored")) return -1;
                    if (dzero(r, c.npend, 8)) return -1;
                    r->pend_left = 0;
                }
                r->proj_left = 0;
            } else if (M.proj && r->nslots >= 2) {
                p.projK = r->nslots;
                for (int a = 0; a < r->nslots; ++a) p.slot[a] = a;
                if (dzero(r, c.neq, 4 * (size_t)r->NR * NEQ)) return -1;
                r->proj_left = PROJ_FRAMES;
            }
        }
        r->last_event_f = f;
        if (M.mode == 1) {
            if (dzero(r, c.sumpr, 4)) return -1;
            if (launch(r, r->f_sumpr, G, 0, {&c, &Npi}, "k_sumpr")) return -1;
        }
        if (ms) {
            cuEventRecord(r->ev[5], nullptr);
            cuEventSynchronize(r->ev[5]);
            float t;
            cuEventElapsedTime(&t, r->ev[4], r->ev[5]);
            ms[4] += t;
        }
    }
    r->prev_state = si;
    p.pend_left = r->pend_left;
    p.dormant = r->dormant;
    p.proj_left = r->proj_left;
    if (M.ddgi && dzero(r, c.dstat, 12 * (size_t)r->NR)) return -1;
    if (ms) cuEventRecord(r->ev[0], nullptr);
    if (M.deps && f % 32 == 0) {
        std::swap(c.cur, c.prev);
        if (dzero(r, c.cur, 4 * (size_t)r->NW * Np)) return -1;
    }
    if (ms) cuEventRecord(r->ev[1], nullptr);
    const bool track = M.deps && (f % M.track_every == 0);
    {
        auto b = dev_state_bytes(r, st);
        CUdeviceptr rg = r->dRegion, al = r->dA;
        if (launch(r, r->f_trace[track ? 1 : 0], G, shm, {b.data(), &c, &p, &rg, &al}, "k_trace2")) return -1;
    }
    if (ms) cuEventRecord(r->ev[2], nullptr);
    if (r->pend_left > 0) {
        CUdeviceptr rg = r->dRegion;
        if (dzero(r, c.npend + 1, 4)) return -1;
        if (launch(r, r->f_decide, G, 0, {&c, &p, &rg}, "k_decide")) return -1;
        if (dcopy(r, c.npend, c.npend + 1, 4)) return -1;
        r->pend_left--;
    }
    if (ms) cuEventRecord(r->ev[3], nullptr);
    {
        CUdeviceptr rg = r->dRegion;
        if (dzero(r, c.sumpr + 1, 4)) return -1;
        if (launch(r, r->f_update, G, 0, {&c, &p, &rg}, "k_update")) return -1;
        if (dcopy(r, c.sumpr, c.sumpr + 1, 4)) return -1;
    }
    std::swap(c.Lc, c.Lc2);
    if (r->proj_left > 0 && --r->proj_left == 0) {
        const int K = p.projK;
        std::vector<float> q((size_t)r->NR * NEQ), cf((size_t)r->NR * KSNAP, NAN);
        CKD(cuMemcpyDtoH(q.data(), (CUdeviceptr)c.neq, q.size() * 4), "neq");
        for (int rg = 0; rg < r->NR; ++rg) {   // poc_gpu.cu:970-988
            const float* Q = &q[(size_t)rg * NEQ];
            if (Q[27] < 24.f) continue;
            double A[KSNAP][KSNAP + 1]; int ix = 0; double tr = 0;
            for (int a = 0; a < K; ++a) for (int b = a; b < K; ++b) { A[a][b] = A[b][a] = Q[ix++]; }
            for (int a = 0; a < K; ++a) { A[a][K] = Q[21 + a]; tr += A[a][a]; }
            for (int a = 0; a < K; ++a) A[a][a] += 1e-3 * tr / K + 1e-9;
            bool ok = true;
            for (int a = 0; a < K && ok; ++a) {
                int pv = a; for (int b = a + 1; b < K; ++b) if (fabs(A[b][a]) > fabs(A[pv][a])) pv = b;
                if (fabs(A[pv][a]) < 1e-12) { ok = false; break; }
                for (int t = 0; t <= K; ++t) std::swap(A[a][t], A[pv][t]);
                for (int b = 0; b < K; ++b) if (b != a) { double mm = A[b][a] / A[a][a]; for (int t = a; t <= K; ++t) A[b][t] -= mm * A[a][t]; }
            }
            if (!ok) continue;
            bool sane = true; double x[KSNAP];
            for (int a = 0; a < K; ++a) { x[a] = A[a][K] / A[a][a]; if (!std::isfinite(x[a]) || fabs(x[a]) > 4.0) sane = false; }
            if (sane) for (int a = 0; a < K; ++a) cf[(size_t)rg * KSNAP + a] = (float)x[a];
        }
        CKD(cuMemcpyHtoD((CUdeviceptr)c.coef, cf.data(), cf.size() * 4), "coef");
        if (dzero(r, c.npend, 8) || dzero(r, c.rstat, 16 * (size_t)r->NR)) return -1;
        CUdeviceptr rg = r->dRegion;
        if (launch(r, r->f_proj, G, 0, {&c, &p, &rg}, "k_proj_apply")) return -1;
        if (dcopy(r, c.npend, c.npend + 1, 4)) return -1;
        r->pend_left = VERIF_FRAMES;
    }
    if (ms) {
        cuEventRecord(r->ev[5], nullptr);
        cuEventSynchronize(r->ev[5]);
        float a, b, d, u;
        cuEventElapsedTime(&a, r->ev[0], r->ev[1]);
        cuEventElapsedTime(&b, r->ev[1], r->ev[2]);
        cuEventElapsedTime(&d, r->ev[2], r->ev[3]);
        cuEventElapsedTime(&u, r->ev[3], r->ev[5]);
        ms[0] += a; ms[1] += b; ms[2] += d; ms[3] += u;
    }
    int have = 0;
    if (want_err && r->has_ref) {
        if (dzero(r, c.err, 24)) return -1;
        CUdeviceptr rf = st.ref, vl = st.valid;
        int dm = r->dormant;
        if (launch(r, r->f_error, G, 0, {&c, &Npi, &rf, &vl, &dm}, "k_error")) return -1;
        double hh[3];
        CKD(cuMemcpyDtoH(hh, (CUdeviceptr)c.err, 24), "err");
        if (errv) *errv = float(sqrt(hh[0] / hh[2]) / (hh[1] / hh[2]));
        have = 1;
    }
    r->f = f + 1;
    return have;
}

// ---------------------------------------------------------------- taa mode
// Set-up of run_taa_mode (poc_gpu.cu:1189-1222) and the per-seed reset (:1241-1245).
int ref_taa_begin(ref_ctx* r, float alpha, float gamma, int mask, int s0, uint32_t seed) {
    if (!r->loaded || !r->has_ref || r->fmt != 2) { r->err = "taa: format-2 scene with references needed"; return -1; }
    cuCtxSetCurrent(r->cu);
    const size_t Np = r->Np;
    Taa& t = r->taa;
    if (!t.x) {
        std::vector<int> nb(9 * Np, -1);
        for (int q = 0; q < r->Nq; ++q) {
            int nu = r->hdims[2 * q], nv = r->hdims[2 * q + 1], o = r->hoff[q];
            for (int iv = 0; iv < nv; ++iv) for (int iu = 0; iu < nu; ++iu) {
                size_t i = (size_t)o + (size_t)iv * nu + iu;
                int k = 0;
                for (int dv = -1; dv <= 1; ++dv) for (int du = -1; du <= 1; ++du) {
                    int a = iu + du, b = iv + dv;
                    nb[9 * i + k++] = (a >= 0 && a < nu && b >= 0 && b < nv) ? o + b * nu + a : -1;
                }
            }
        }
        t.x = (float*)alloc(r, 4 * Np); t.H = (float*)alloc(r, 4 * Np); t.H2 = (float*)alloc(r, 4 * Np);
        t.mu = (float*)alloc(r, 4 * Np); t.sg = (float*)alloc(r, 4 * Np); t.nb = (int*)put(r, nb);
        t.react = (int*)alloc(r, 4 * Np); t.pend = (uint8_t*)alloc(r, Np);
        t.cur = (uint32_t*)alloc(r, 4 * r->NW * Np); t.prev = (uint32_t*)alloc(r, 4 * r->NW * Np);
        t.rs = (float*)alloc(r, 12 * (size_t)r->NR); t.err = (double*)alloc(r, 24);
        r->taa_cnt = (float*)alloc(r, 4 * (size_t)r->NR);
        r->taaV.assign((size_t)r->NS * r->NS, {});
        r->dTaaV.assign((size_t)r->NS * r->NS, 0);
        for (int a = 0; a < r->NS; ++a) for (int b = 0; b < r->NS; ++b) {
            if (a == b) continue;
            std::vector<int> fine;
            for (int l = 0; l < r->NL; ++l)
                if (r->st[a].inten[l] != r->st[b].inten[l]) {   // host_vox_fine (poc_gpu.cu:1170-1173)
                    const float* pl = &r->hL[3 * (size_t)l];
                    int i = std::min(std::max(int(pl[0] / 8.f * 16), 0), 15), j = std::min(std::max(int(pl[1] / 4.f * 8), 0), 7),
                        k = std::min(std::max(int(pl[2] / 3.f * 6), 0), 5);
                    fine.push_back((k * 8 + j) * 16 + i);
                }
            std::vector<int> v = to_grid(r, fine);
            for (int x : r->occ[a * r->NS + b]) v.push_back(x);
            std::sort(v.begin(), v.end());
            v.erase(std::unique(v.begin(), v.end()), v.end());
            r->taaV[a * r->NS + b] = v;
            r->dTaaV[a * r->NS + b] = put(r, v.empty() ? std::vector<int>{0} : v);
        }
    }
    CKD(cuMemcpyDtoD((CUdeviceptr)t.H, r->st[s0].ref, Np * 4), "taa history");
    if (dzero(r, t.react, Np * 4) || dzero(r, t.pend, Np) || dzero(r, t.cur, r->NW * Np * 4) || dzero(r, t.prev, r->NW * Np * 4)) return -1;
    r->taa_alpha = alpha; r->taa_gamma = gamma; r->taa_mask = mask; r->taa_seed = seed;
    r->taa_f = 0; r->taa_prev = s0; r->taa_verify = 0;
    return 0;
}

// One frame of run_taa_mode's loop (poc_gpu.cu:1246-1274); err (may be NULL) receives the frame's error.
int ref_taa_frame(ref_ctx* r, int si, float* err) {
    cuCtxSetCurrent(r->cu);
    Taa& t = r->taa;
    if (!t.x) { r->err = "no taa run"; return -1; }
    const int G = grid_of(r), f = r->taa_f, mask = r->taa_mask, RF = 4;
    const float ALPHA_R = 0.5f;
    const size_t Np = r->Np;
    int Npi = r->Np;
    HostState& st = r->st[si];
    const bool deps = mask == 2 || mask == 3;
    if (deps && f % 32 == 0) { std::swap(t.cur, t.prev); if (dzero(r, t.cur, r->NW * Np * 4)) return -1; }
    auto b = dev_state_bytes(r, st);
    uint32_t seed = r->taa_seed, fr = (uint32_t)f;
    CUdeviceptr dA = r->dA, reg = r->dRegion;
    unsigned shm = r->Nt * 10 * 4;
    if (launch(r, r->f_taa_pt[deps ? 1 : 0], G, shm, {b.data(), &t, &Npi, &seed, &fr, &dA}, "k_taa_pt")) return -1;
    if (f > 0 && r->taa_prev != si) {
        int pe = r->taa_prev * r->NS + si, nv = (int)r->taaV[pe].size(), rf = RF;
        CUdeviceptr V = r->dTaaV[pe];
        if (mask == 2) { int tp = 0; if (launch(r, r->f_taa_touch, G, 0, {&t, &Npi, &V, &nv, &rf, &tp}, "k_taa_touch")) return -1; }
        if (mask == 3) {
            int tp = 1;
            if (launch(r, r->f_taa_touch, G, 0, {&t, &Npi, &V, &nv, &rf, &tp}, "k_taa_touch")) return -1;
            r->taa_verify = 2;
            if (dzero(r, t.rs, 12 * (size_t)r->NR) || dzero(r, r->taa_cnt, 4 * (size_t)r->NR)) return -1;
        }
        if (mask == 4) {
            CUdeviceptr ro = r->st[r->taa_prev].ref, rn = st.ref;
            if (launch(r, r->f_taa_oracle, G, 0, {&t, &Npi, &ro, &rn, &rf}, "k_taa_oracle")) return -1;
        }
    }
    CUdeviceptr cnt = (CUdeviceptr)r->taa_cnt, pend = (CUdeviceptr)t.pend;
    if (mask == 1) {
        int zero = 0, rf = RF;
        if (dzero(r, t.rs, 12 * (size_t)r->NR) || dzero(r, r->taa_cnt, 4 * (size_t)r->NR)) return -1;
        if (launch(r, r->f_taa_zacc, G, 0, {&t, &Npi, &reg, &zero}, "k_taa_zone_acc")) return -1;
        if (launch(r, r->f_taa_count, G, 0, {&Npi, &reg, &pend, &zero, &cnt}, "k_count_zone")) return -1;
        if (launch(r, r->f_taa_zdec, G, 0, {&t, &Npi, &reg, &cnt, &zero, &rf, &zero}, "k_taa_zone_decide")) return -1;
    }
    if (mask == 3 && r->taa_verify > 0) {
        int one = 1, rf = RF;
        if (launch(r, r->f_taa_zacc, G, 0, {&t, &Npi, &reg, &one}, "k_taa_zone_acc")) return -1;
        if (launch(r, r->f_taa_count, G, 0, {&Npi, &reg, &pend, &one, &cnt}, "k_count_zone")) return -1;
        if (--r->taa_verify == 0)
            if (launch(r, r->f_taa_zdec, G, 0, {&t, &Npi, &reg, &cnt, &one, &rf, &one}, "k_taa_zone_decide")) return -1;
    }
    if (launch(r, r->f_taa_stats, G, 0, {&t, &Npi}, "k_taa_stats")) return -1;
    float al = r->taa_alpha, ar = ALPHA_R, ga = r->taa_gamma;
    if (launch(r, r->f_taa_update, G, 0, {&t, &Npi, &al, &ar, &ga}, "k_taa_update")) return -1;
    std::swap(t.H, t.H2);
    if (dzero(r, t.err, 24)) return -1;
    CUdeviceptr ref = st.ref, valid = st.valid;
    if (launch(r, r->f_taa_err, G, 0, {&t, &Npi, &ref, &valid}, "k_taa_err")) return -1;
    double h[3];
    CKD(cuMemcpyDtoH(h, (CUdeviceptr)t.err, 24), "taa err");
    if (err) *err = (float)(sqrt(h[0] / h[2]) / (h[1] / h[2]));
    r->taa_prev = si;
    r->taa_f = f + 1;
    return 0;
}

// taa arrays: 0 x, 1 H, 2 mu, 3 sg, 4 react, 5 pend, 6 cur, 7 prev (layouts of rc_taa_array_copy)
int ref_taa_array(ref_ctx* r, int which, void* host, size_t nbytes, int to_device) {
    cuCtxSetCurrent(r->cu);
    Taa& t = r->taa;
    const size_t Np = r->Np, NW = r->NW;
    void* p = nullptr;
    size_t n = 0;
    switch (which) {
        case 0: p = t.x; n = 4 * Np; break;
        case 1: p = t.H; n = 4 * Np; break;
        case 2: p = t.mu; n = 4 * Np; break;
        case 3: p = t.sg; n = 4 * Np; break;
        case 4: p = t.react; n = 4 * Np; break;
        case 5: p = t.pend; n = Np; break;
        case 6: p = t.cur; n = 4 * NW * Np; break;
        case 7: p = t.prev; n = 4 * NW * Np; break;
        default: r->err = "taa array"; return -1;
    }
    if (!p || nbytes != n) { r->err = "taa array size"; return -1; }
    if (to_device) CKD(cuMemcpyHtoD((CUdeviceptr)p, host, n), "taa array");
    else CKD(cuMemcpyDtoH(host, (CUdeviceptr)p, n), "taa array");
    return 0;
}

int ref_sync(ref_ctx* r) { cuCtxSetCurrent(r->cu); CKD(cuCtxSynchronize(), "sync"); return 0; }

// Run-state arrays with the ids of include/rc_api.h (RC_A_*), in the reference layouts.
int ref_array(ref_ctx* r, int which, void* host, size_t nbytes, int to_device) {
    cuCtxSetCurrent(r->cu);
    const size_t Np = r->Np, NL = r->NL, NW = r->NW, NR = r->NR;
    Cache& c = r->c;
    void* dev = nullptr;
    size_t need = 0;
    switch (which) {
        case 0: dev = c.Lc; need = 4 * NL * Np; break;
        case 1: dev = c.Lc2; need = 4 * NL * Np; break;
        case 2: dev = c.m; need = 4 * NL * Np; break;
        case 3: dev = c.n; need = 4 * Np; break;
        case 4: dev = c.c0; need = 4 * Np; break;
        case 5: dev = c.kk; need = 4 * Np; break;
        case 6: dev = c.pending; need = Np; break;
        case 7: dev = c.cur; need = 4 * NW * Np; break;
        case 8: dev = c.prev; need = 4 * NW * Np; break;
        case 9: dev = c.stale; need = Np; break;   // 8 bits per point in the reference
        case 10: dev = c.age; need = 4 * Np; break;
        case 11: dev = c.snap; need = 4 * (size_t)KSNAP * Np * NL; break;
        case 12: dev = c.neq; need = 4 * NR * NEQ; break;
        case 13: dev = c.coef; need = 4 * NR * KSNAP; break;
        case 14: dev = c.rstat; need = 16 * NR; break;
        case 15: dev = c.dstat; need = 12 * NR; break;
        case 16: dev = c.sumpr; need = 8; break;
        case 17: dev = c.npend; need = 8; break;
        default: r->err = "array id"; return -1;
    }
    if (nbytes != need) { r->err = "array size"; return -1; }
    if (to_device) CKD(cuMemcpyHtoD((CUdeviceptr)dev, host, nbytes), "htod");
    else CKD(cuMemcpyDtoH(host, (CUdeviceptr)dev, nbytes), "dtoh");
    return 0;
}

// Scalars with the ids of RC_S_*.
int ref_scalar(ref_ctx* r, int which, int set, int value) {
    int* v = nullptr;
    switch (which) {
        case 0: v = &r->pend_left; break;
        case 1: v = &r->dormant; break;
        case 2: v = &r->proj_left; break;
        case 3: v = &r->f; break;
        case 4: v = &r->nslots; break;
        case 5: v = &r->last_event_f; break;
        case 6: v = &r->p.projK; break;
        default: return -1;
    }
    if (set) *v = value;
    return *v;
}

// k_build outputs of a state: 0 = Edir (NL floats per point), 1 = SV (NW words per point).
int ref_state_array(ref_ctx* r, int state, int which, void* host, size_t nbytes) {
    cuCtxSetCurrent(r->cu);
    const size_t Np = r->Np;
    if (state < 0 || state >= r->NS) return -1;
    if (which == 0 && nbytes == 4 * (size_t)r->NL * Np) CKD(cuMemcpyDtoH(host, r->st[state].Edir, nbytes), "edir");
    else if (which == 1 && nbytes == 4 * (size_t)r->NW * Np) CKD(cuMemcpyDtoH(host, r->st[state].SV, nbytes), "sv");
    else return -1;
    return 0;
}

}  // extern "C"
