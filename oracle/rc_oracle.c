/*
 * CPU oracle for the radiance-cache frame loop — TEST INFRASTRUCTURE ONLY (see rc_oracle.h).
 *
 * Restates cuda/poc_gpu.cu of falcon123212/render_engine in plain C, FP32 in the same
 * operation order.  Differences from the GPU reference that are inherent to a CPU build:
 *  - cosf / sinf / sqrtf come from the C library and rsqrtf(x) is 1/sqrtf(x); the CUDA
 *    versions differ by a few ulp, so ray directions match the GPU to ~1e-7 relative;
 *  - build with -ffp-contract=off: no fused multiply-add, identical results on x86 and Arm;
 *  - region sums (rstat, neq, dstat) are accumulated in point order (the reference uses
 *    float atomics, whose order is not defined); Sum 1/(n+1) is computed exactly (64-bit
 *    fixed point, one final rounding) and the FP64 error sums use the fixed reduction tree of
 *    the product kernels, so those sums are exact copies of what the product computes;
 *  - the per-point "stale" set of dormant lights is 32 bits wide (the reference stores it
 *    in 8 bits, which only differs for scenes with more than 8 lights).
 */
#include "rc_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KSNAP 6
#define NEQ 28
#define VERIF_FRAMES 4
#define PROJ_FRAMES 4
#define BLK 256

/* ------------------------------------------------------------------ small vector math */
typedef struct { float x, y, z; } v3;
static inline v3 V(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, float s) { return V(a.x * s, a.y * s, a.z * s); }
static inline float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) { return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline v3 vld(const float* p, long i) { return V(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int f2i(float f) { int i; memcpy(&i, &f, 4); return i; }

/* poc_gpu.cu:127-129 integer mixer */
static inline uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}
/* poc_gpu.cu:130-135 LCG step + output permutation -> 24-bit uniform */
static inline float rnd(uint32_t* s) {
    *s = *s * 747796405u + 2891336453u;
    uint32_t w = ((*s >> ((*s >> 28u) + 4u)) ^ *s) * 277803737u;
    w = (w >> 22u) ^ w;
    return (float)(w >> 8) * (1.0f / 16777216.0f);
}
/* poc_gpu.cu:260-262 splitmix64 finaliser */
static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull; x ^= x >> 27; x *= 0x94d049bb133111ebull; x ^= x >> 31;
    return x;
}
/* poc_gpu.cu:251-256 */
static inline int normal_bucket(float nx, float ny, float nz) {
    float ax = fabsf(nx), ay = fabsf(ny), az = fabsf(nz);
    if (ax >= ay && ax >= az) return nx > 0.f ? 0 : 1;
    if (ay >= az) return ny > 0.f ? 2 : 3;
    return nz > 0.f ? 4 : 5;
}
/* poc_gpu.cu:257-259 */
static inline uint64_t cell_key(int cx, int cy, int cz, int b) {
    uint64_t k = (uint64_t)(cx & 0xFFFFF);
    k = (k << 20) | (uint64_t)(cy & 0xFFFFF);
    k = (k << 20) | (uint64_t)(cz & 0xFFFFF);
    return ((k << 3) | (uint64_t)b) + 1ull;
}

/* ------------------------------------------------------------------ scene */
typedef struct {
    float* inten; float *P, *N, *Q, *T, *ref, *Pw; int *dims, *off, *TQ; uint8_t* valid;
    float* Edir; uint32_t* SV;
} ostate;

struct osc_scene {
    int Np, Nq, Nt, NS, NL, NR, has_ref, fmt;
    int VX, VY, VZ, NV, NW;
    float lo[3], ext[3];
    /* format 3 */
    float hcell; int nst, nnodes, hsize, npst;
    float *ST, *STN, *BN; uint64_t* HK; int* HV;
    float *L, *A; int* region;
    ostate* st;
    int** ev; int* nev;   /* NS*NS*(1+NL) lists on the transit grid: [pair*(1+NL)+0]=occluders, +1+l = light l */
};

typedef struct { const uint8_t* p; size_t n, off; int bad; } rdr;
static void rd_bytes(rdr* r, void* dst, size_t n) {
    if (r->bad || r->off + n > r->n) { r->bad = 1; if (dst && n) memset(dst, 0, n); return; }
    if (n) memcpy(dst, r->p + r->off, n);
    r->off += n;
}
static void* rd_arr(rdr* r, size_t elem, size_t cnt) {
    size_t n = elem * cnt;
    void* d = malloc(n ? n : 16);
    if (!d) { r->bad = 1; return NULL; }
    rd_bytes(r, d, n);
    return d;
}

/* poc_gpu.cu:720-735: fine event grid (16x8x6 over the 8x4x3 m box) -> transit grid */
static int* to_grid(const osc_scene* s, const int* fine, int nf, int* nout) {
    const int FX = 16, FY = 8, FZ = 6;
    const float X1 = 8.f, Y1 = 4.f, Z1 = 3.f;
    char* mark = (char*)calloc((size_t)s->NV, 1);
    for (int q = 0; q < nf; ++q) {
        int v = fine[q];
        int i = v % FX, j = (v / FX) % FY, k = v / (FX * FY);
        float x0 = (float)i * X1 / FX, x1 = (float)(i + 1) * X1 / FX;
        float y0 = (float)j * Y1 / FY, y1 = (float)(j + 1) * Y1 / FY;
        float z0 = (float)k * Z1 / FZ, z1 = (float)(k + 1) * Z1 / FZ;
        int a0 = imin((int)(x0 / X1 * s->VX + 1e-4f), s->VX - 1), a1 = imin((int)(x1 / X1 * s->VX - 1e-4f), s->VX - 1);
        int b0 = imin((int)(y0 / Y1 * s->VY + 1e-4f), s->VY - 1), b1 = imin((int)(y1 / Y1 * s->VY - 1e-4f), s->VY - 1);
        int c0 = imin((int)(z0 / Z1 * s->VZ + 1e-4f), s->VZ - 1), c1 = imin((int)(z1 / Z1 * s->VZ - 1e-4f), s->VZ - 1);
        for (int a = a0; a <= a1; ++a)
            for (int b = b0; b <= b1; ++b)
                for (int c = c0; c <= c1; ++c) mark[(c * s->VY + b) * s->VX + a] = 1;
    }
    int cnt = 0;
    for (int v = 0; v < s->NV; ++v) cnt += mark[v];
    int* out = (int*)malloc(sizeof(int) * (size_t)(cnt ? cnt : 1));
    cnt = 0;
    for (int v = 0; v < s->NV; ++v) if (mark[v]) out[cnt++] = v;
    free(mark);
    *nout = cnt;
    return out;
}

static void seterr(char* err, int errlen, const char* msg) {
    if (err && errlen > 0) { strncpy(err, msg, (size_t)errlen - 1); err[errlen - 1] = 0; }
}

/* poc_gpu.cu:751-801 scene loader (formats 2 and 3) */
osc_scene* osc_load_mem(const void* buf, size_t n, int vx, int vy, int vz, char* err, int errlen) {
    rdr r = {(const uint8_t*)buf, n, 0, 0};
    int h[8];
    rd_bytes(&r, h, 32);
    if (r.bad) { seterr(err, errlen, "truncated header"); return NULL; }
    if (h[7] != 2 && h[7] != 3) { seterr(err, errlen, "unsupported scene format"); return NULL; }
    if (h[0] <= 0 || h[1] < 0 || h[2] < 0 || h[3] <= 0 || h[4] <= 0 || h[4] > 32 || h[5] <= 0) {
        seterr(err, errlen, "bad header"); return NULL;
    }
    if (vx <= 0 || vy <= 0 || vz <= 0 || (vx * vy * vz) % 128 != 0) { seterr(err, errlen, "transit grid must be a multiple of 128 voxels"); return NULL; }
    osc_scene* s = (osc_scene*)calloc(1, sizeof(osc_scene));
    s->Np = h[0]; s->Nq = h[1]; s->Nt = h[2]; s->NS = h[3]; s->NL = h[4]; s->NR = h[5]; s->has_ref = h[6]; s->fmt = h[7];
    s->VX = vx; s->VY = vy; s->VZ = vz; s->NV = vx * vy * vz; s->NW = s->NV / 32;
    s->lo[0] = s->lo[1] = s->lo[2] = 0.f; s->ext[0] = 8.f; s->ext[1] = 4.f; s->ext[2] = 3.f;
    const int NL = s->NL; const size_t Np = (size_t)s->Np;
    if (s->fmt == 3) {
        int m[4];
        rd_bytes(&r, s->lo, 12); rd_bytes(&r, s->ext, 12); rd_bytes(&r, &s->hcell, 4); rd_bytes(&r, m, 16);
        if (r.bad || m[0] < 0 || m[1] <= 0 || m[2] <= 0 || (m[2] & (m[2] - 1))) { seterr(err, errlen, "bad format-3 block"); osc_free(s); return NULL; }
        s->nst = m[0]; s->nnodes = m[1]; s->hsize = m[2]; s->npst = m[3];
        s->ST = (float*)rd_arr(&r, 4, 9 * (size_t)m[0]);
        s->STN = (float*)rd_arr(&r, 4, 4 * (size_t)m[0]);
        s->BN = (float*)rd_arr(&r, 4, 8 * (size_t)m[1]);
        s->HK = (uint64_t*)rd_arr(&r, 8, (size_t)m[2]);
        s->HV = (int*)rd_arr(&r, 4, (size_t)m[2]);
    }
    s->L = (float*)rd_arr(&r, 4, 3 * (size_t)NL);
    s->A = (float*)rd_arr(&r, 4, Np);
    s->region = (int*)rd_arr(&r, 4, Np);
    s->st = (ostate*)calloc((size_t)s->NS, sizeof(ostate));
    for (int k = 0; k < s->NS && !r.bad; ++k) {
        ostate* t = &s->st[k];
        t->inten = (float*)rd_arr(&r, 4, (size_t)NL);
        t->P = (float*)rd_arr(&r, 4, 3 * Np);
        t->N = (float*)rd_arr(&r, 4, 3 * Np);
        t->Q = (float*)rd_arr(&r, 4, 12 * (size_t)s->Nq);
        t->dims = (int*)rd_arr(&r, 4, 2 * (size_t)s->Nq);
        t->off = (int*)rd_arr(&r, 4, (size_t)s->Nq);
        t->T = (float*)rd_arr(&r, 4, 9 * (size_t)s->Nt);
        t->TQ = (int*)rd_arr(&r, 4, (size_t)s->Nt);
        if (s->has_ref) {
            t->ref = (float*)rd_arr(&r, 4, Np);
            t->valid = (uint8_t*)rd_arr(&r, 1, Np);
            t->Pw = (float*)rd_arr(&r, 4, (size_t)NL * Np);
        }
        t->Edir = (float*)calloc((size_t)NL * Np, 4);
        t->SV = (uint32_t*)calloc((size_t)s->NW * Np, 4);
    }
    const int NE = s->NS * s->NS * (1 + NL);
    s->ev = (int**)calloc((size_t)NE, sizeof(int*));
    s->nev = (int*)calloc((size_t)NE, sizeof(int));
    for (int e = 0; e < s->NS * s->NS && !r.bad; ++e) {
        for (int kind = 0; kind <= NL; ++kind) {
            int cnt = 0;
            rd_bytes(&r, &cnt, 4);
            if (r.bad || cnt < 0 || (size_t)cnt > (n - r.off) / 4) { r.bad = 1; break; }
            int* raw = (int*)rd_arr(&r, 4, (size_t)cnt);
            int idx = e * (1 + NL) + kind;
            if (s->fmt == 3) { s->ev[idx] = raw; s->nev[idx] = cnt; }
            else { s->ev[idx] = to_grid(s, raw, cnt, &s->nev[idx]); free(raw); }
        }
    }
    if (r.bad) { seterr(err, errlen, "truncated scene"); osc_free(s); return NULL; }
    /* indices that the kernels dereference must be in range */
    for (size_t i = 0; i < Np; ++i)
        if (s->region[i] < 0 || s->region[i] >= s->NR) { seterr(err, errlen, "region index out of range"); osc_free(s); return NULL; }
    for (int k = 0; k < s->NS; ++k)
        for (int t = 0; t < s->Nt; ++t)
            if (s->st[k].TQ[t] < 0 || s->st[k].TQ[t] >= s->Nq) { seterr(err, errlen, "triangle quad index out of range"); osc_free(s); return NULL; }
    return s;
}

osc_scene* osc_load_file(const char* path, int vx, int vy, int vz, char* err, int errlen) {
    FILE* f = fopen(path, "rb");
    if (!f) { seterr(err, errlen, "cannot open scene file"); return NULL; }
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    void* b = malloc((size_t)(n > 0 ? n : 1));
    size_t got = fread(b, 1, (size_t)n, f);
    fclose(f);
    osc_scene* s = got == (size_t)n ? osc_load_mem(b, (size_t)n, vx, vy, vz, err, errlen) : NULL;
    if (got != (size_t)n) seterr(err, errlen, "short read");
    free(b);
    return s;
}

void osc_free(osc_scene* s) {
    if (!s) return;
    free(s->ST); free(s->STN); free(s->BN); free(s->HK); free(s->HV);
    free(s->L); free(s->A); free(s->region);
    if (s->st)
        for (int k = 0; k < s->NS; ++k) {
            ostate* t = &s->st[k];
            free(t->inten); free(t->P); free(t->N); free(t->Q); free(t->dims); free(t->off); free(t->T); free(t->TQ);
            free(t->ref); free(t->valid); free(t->Pw); free(t->Edir); free(t->SV);
        }
    free(s->st);
    if (s->ev) for (int e = 0; e < s->NS * s->NS * (1 + s->NL); ++e) free(s->ev[e]);
    free(s->ev); free(s->nev);
    free(s);
}

void osc_info(const osc_scene* s, int out[10]) {
    out[0] = s->Np; out[1] = s->Nq; out[2] = s->Nt; out[3] = s->NS; out[4] = s->NL; out[5] = s->NR;
    out[6] = s->has_ref; out[7] = s->fmt; out[8] = s->NW; out[9] = s->nst;
}

void* osc_state_array(osc_scene* s, int k, int which, size_t* nbytes) {
    ostate* t = &s->st[k];
    size_t Np = (size_t)s->Np;
    switch (which) {
        case 0: *nbytes = 4 * (size_t)s->NL * Np; return t->Edir;
        case 1: *nbytes = 4 * (size_t)s->NW * Np; return t->SV;
        case 2: *nbytes = t->ref ? 4 * Np : 0; return t->ref;
        case 3: *nbytes = t->valid ? Np : 0; return t->valid;
        case 4: *nbytes = t->Pw ? 4 * (size_t)s->NL * Np : 0; return t->Pw;
    }
    *nbytes = 0;
    return NULL;
}

const int* osc_event_list(const osc_scene* s, int pair, int kind, int* n) {
    int idx = pair * (1 + s->NL) + kind;
    *n = s->nev[idx];
    return s->ev[idx];
}

/* ------------------------------------------------------------------ geometry */
/* poc_gpu.cu:137-142 */
static inline int vox_of(const osc_scene* s, v3 p) {
    int i = imin(imax((int)((p.x - s->lo[0]) / s->ext[0] * (float)s->VX), 0), s->VX - 1);
    int j = imin(imax((int)((p.y - s->lo[1]) / s->ext[1] * (float)s->VY), 0), s->VY - 1);
    int k = imin(imax((int)((p.z - s->lo[2]) / s->ext[2] * (float)s->VZ), 0), s->VZ - 1);
    return (k * s->VY + j) * s->VX + i;
}
/* poc_gpu.cu:171-190 Amanatides-Woo walk of segment a->b, bits into m[NW] */
static void dda(const osc_scene* s, v3 a, v3 b, uint32_t* m) {
    const int VX = s->VX, VY = s->VY, VZ = s->VZ;
    const float sx = (float)VX / s->ext[0], sy = (float)VY / s->ext[1], sz = (float)VZ / s->ext[2];
    float ax = (a.x - s->lo[0]) * sx, ay = (a.y - s->lo[1]) * sy, az = (a.z - s->lo[2]) * sz;
    float bx = (b.x - s->lo[0]) * sx, by = (b.y - s->lo[1]) * sy, bz = (b.z - s->lo[2]) * sz;
    int ix = imin(imax((int)ax, 0), VX - 1), iy = imin(imax((int)ay, 0), VY - 1), iz = imin(imax((int)az, 0), VZ - 1);
    int ex = imin(imax((int)bx, 0), VX - 1), ey = imin(imax((int)by, 0), VY - 1), ez = imin(imax((int)bz, 0), VZ - 1);
    float dx = bx - ax, dy = by - ay, dz = bz - az;
    int stx = dx > 0 ? 1 : -1, sty = dy > 0 ? 1 : -1, stz = dz > 0 ? 1 : -1;
    float tdx = dx != 0 ? fabsf(1.f / dx) : 1e30f, tdy = dy != 0 ? fabsf(1.f / dy) : 1e30f, tdz = dz != 0 ? fabsf(1.f / dz) : 1e30f;
    float tmx = dx != 0 ? ((dx > 0 ? ((float)(ix + 1) - ax) : (ax - (float)ix)) * tdx) : 1e30f;
    float tmy = dy != 0 ? ((dy > 0 ? ((float)(iy + 1) - ay) : (ay - (float)iy)) * tdy) : 1e30f;
    float tmz = dz != 0 ? ((dz > 0 ? ((float)(iz + 1) - az) : (az - (float)iz)) * tdz) : 1e30f;
    for (int g = 0; g < VX + VY + VZ; ++g) {
        int v = (iz * VY + iy) * VX + ix;
        m[v >> 5] |= 1u << (v & 31);
        if (ix == ex && iy == ey && iz == ez) break;
        if (tmx < tmy && tmx < tmz) { ix += stx; tmx += tdx; if (ix < 0 || ix >= VX) break; }
        else if (tmy < tmz) { iy += sty; tmy += tdy; if (iy < 0 || iy >= VY) break; }
        else { iz += stz; tmz += tdz; if (iz < 0 || iz >= VZ) break; }
    }
}
/* poc_gpu.cu:192-197 */
static void rast_seg(const osc_scene* s, v3 a, v3 b, uint32_t* m) {
    for (int k = 0; k < 20; ++k) {
        int v = vox_of(s, vadd(a, vmul(vsub(b, a), (float)k / 19.f)));
        m[v >> 5] |= 1u << (v & 31);
    }
}
/* poc_gpu.cu:199-220 brute-force closest hit over the dynamic triangles */
static int trace_dyn(v3 o, v3 d, const float* T, const int* TQ, int nt, float* tmin, int* q) {
    *tmin = INFINITY; *q = -1;
    for (int j = 0; j < nt; ++j) {
        v3 v0 = vld(T, 3 * j), e1 = vld(T, 3 * j + 1), e2 = vld(T, 3 * j + 2);
        v3 p = vcross(d, e2);
        float det = vdot(e1, p);
        if (fabsf(det) <= 1e-9f) continue;
        float inv = 1.f / det;
        v3 tv = vsub(o, v0);
        float u = vdot(tv, p) * inv;
        if (u < 0.f) continue;
        v3 qv = vcross(tv, e1);
        float v = vdot(d, qv) * inv;
        if (v < 0.f || u + v > 1.f) continue;
        float t = vdot(e2, qv) * inv;
        if (t > 1e-4f && t < *tmin) { *tmin = t; *q = TQ[j]; }
    }
    return *q >= 0;
}
/* poc_gpu.cu:288-295; fs scales the exit distance (1 = the reference; the watertight mode
 * uses 1 + 4 ulp, Ize's conservative slab test, JCGT 2(2), 2013) */
static inline float aabb_enter(const float* a, const float* b, v3 o, v3 inv, float tmax, float fs) {
    float tx1 = (a[0] - o.x) * inv.x, tx2 = (b[0] - o.x) * inv.x;
    float ty1 = (a[1] - o.y) * inv.y, ty2 = (b[1] - o.y) * inv.y;
    float tz1 = (a[2] - o.z) * inv.z, tz2 = (b[2] - o.z) * inv.z;
    float tn = fmaxf(fmaxf(fminf(tx1, tx2), fminf(ty1, ty2)), fmaxf(fminf(tz1, tz2), 0.f));
    float tf = fminf(fminf(fmaxf(tx1, tx2), fmaxf(ty1, ty2)), fminf(fmaxf(tz1, tz2), tmax));
    return tn <= tf * fs ? tn : 1e30f;
}
/* Watertight ray/triangle test (Woop, Benthin and Wald, JCGT 2(1), 2013), the
 * RC_FLAG_WATERTIGHT alternative of the GPU traversal: permute the ray's largest direction
 * component to z, shear the triangle into the ray frame, 2-D edge functions U, V, W (each
 * product and difference rounded on its own: this file is built without contraction), all
 * three recomputed in double when one is exactly zero; hit when they share a sign; t = T / det.
 * Vertices: v0, v0 + e1, v0 + e2.  Returns the hit distance or +inf. */
typedef struct { int kx, ky, kz; float sx, sy, sz; } wt_ray_t;
static inline float sel3(v3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
static wt_ray_t wt_ray(v3 d) {
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    wt_ray_t r;
    r.kz = ax >= ay ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
    r.kx = r.kz == 2 ? 0 : r.kz + 1;
    r.ky = r.kx == 2 ? 0 : r.kx + 1;
    float dz = sel3(d, r.kz);
    if (dz < 0.f) { int x = r.kx; r.kx = r.ky; r.ky = x; }
    r.sx = sel3(d, r.kx) / dz;
    r.sy = sel3(d, r.ky) / dz;
    r.sz = 1.f / dz;
    return r;
}
static inline float edge64(float ax, float by, float ay, float bx) { return (float)((double)ax * (double)by - (double)ay * (double)bx); }
static float wt_tri(const wt_ray_t* r, v3 o, v3 v0, v3 e1, v3 e2) {
    v3 A = vsub(v0, o), B = vsub(vadd(v0, e1), o), C = vsub(vadd(v0, e2), o);
    float az = sel3(A, r->kz), bz = sel3(B, r->kz), cz = sel3(C, r->kz);
    float Ax = sel3(A, r->kx) - r->sx * az, Ay = sel3(A, r->ky) - r->sy * az;
    float Bx = sel3(B, r->kx) - r->sx * bz, By = sel3(B, r->ky) - r->sy * bz;
    float Cx = sel3(C, r->kx) - r->sx * cz, Cy = sel3(C, r->ky) - r->sy * cz;
    float U = Cx * By - Cy * Bx, Vv = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.f || Vv == 0.f || W == 0.f) {
        U = edge64(Cx, By, Cy, Bx);
        Vv = edge64(Ax, Cy, Ay, Cx);
        W = edge64(Bx, Ay, By, Ax);
    }
    if ((U < 0.f || Vv < 0.f || W < 0.f) && (U > 0.f || Vv > 0.f || W > 0.f)) return INFINITY;
    float det = (U + Vv) + W;
    if (det == 0.f) return INFINITY;
    float T = (U * (r->sz * az) + Vv * (r->sz * bz)) + W * (r->sz * cz);
    return T / det;
}
/* poc_gpu.cu:297-338 stack BVH traversal over the static mesh; q = -2 - triangle.  With
 * watertight set, leaves use wt_tri instead of the reference's Moller-Trumbore. */
static void trace_bvh_m(const osc_scene* s, v3 o, v3 d, float* tmin, int* q, int watertight);
static void trace_bvh(const osc_scene* s, v3 o, v3 d, float* tmin, int* q) { trace_bvh_m(s, o, d, tmin, q, 0); }
static void trace_bvh_m(const osc_scene* s, v3 o, v3 d, float* tmin, int* q, int watertight) {
    v3 inv = V(fabsf(d.x) > 1e-12f ? 1.f / d.x : copysignf(1e30f, d.x),
               fabsf(d.y) > 1e-12f ? 1.f / d.y : copysignf(1e30f, d.y),
               fabsf(d.z) > 1e-12f ? 1.f / d.z : copysignf(1e30f, d.z));
    int stack[64], sp = 0, node = 0;
    for (;;) {
        const float* a = s->BN + 8 * (size_t)node;
        const float* b = a + 4;
        int lf = f2i(a[3]), cnt = f2i(b[3]);
        if (cnt > 0 && watertight) {
            wt_ray_t wr = wt_ray(d);
            for (int j = lf; j < lf + cnt; ++j) {
                const float* T = s->ST + 9 * (size_t)j;
                float t = wt_tri(&wr, o, V(T[0], T[1], T[2]), V(T[3], T[4], T[5]), V(T[6], T[7], T[8]));
                if (t > 1e-4f && t < *tmin) { *tmin = t; *q = -2 - j; }
            }
        } else if (cnt > 0) {
            for (int j = lf; j < lf + cnt; ++j) {
                const float* T = s->ST + 9 * (size_t)j;
                v3 v0 = V(T[0], T[1], T[2]), e1 = V(T[3], T[4], T[5]), e2 = V(T[6], T[7], T[8]);
                v3 p = vcross(d, e2);
                float det = vdot(e1, p);
                if (fabsf(det) <= 1e-12f) continue;
                float iv = 1.f / det;
                v3 tv = vsub(o, v0);
                float u = vdot(tv, p) * iv;
                if (u < 0.f || u > 1.f) continue;
                v3 qv = vcross(tv, e1);
                float v = vdot(d, qv) * iv;
                if (v < 0.f || u + v > 1.f) continue;
                float t = vdot(e2, qv) * iv;
                if (t > 1e-4f && t < *tmin) { *tmin = t; *q = -2 - j; }
            }
        } else {
            const float* la = s->BN + 8 * (size_t)lf;
            const float fs = watertight ? 1.00000048f : 1.f;
            float tl = aabb_enter(la, la + 4, o, inv, *tmin, fs), tr = aabb_enter(la + 8, la + 12, o, inv, *tmin, fs);
            int first = lf, second = lf + 1;
            if (tr < tl) { float x = tl; tl = tr; tr = x; first = lf + 1; second = lf; }
            if (tl < 1e30f) {
                if (tr < 1e30f && sp < 64) stack[sp++] = second;
                node = first;
                continue;
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
}
/* poc_gpu.cu:340-344 */
static int trace_full(const osc_scene* s, const ostate* st, v3 o, v3 d, float* t, int* q) {
    int h = trace_dyn(o, d, st->T, st->TQ, s->Nt, t, q);
    if (s->BN) { trace_bvh(s, o, d, t, q); h = *q != -1; }
    return h;
}
/* Caller-given rays (origin, direction) through trace_full of state si; prim = quad id,
 * -2 - static triangle, or -1; t = +inf when no hit (rc_trace_rays of the library). */
int osc_trace_rays(const osc_scene* s, int si, const float* rays, int n, int watertight, int* prim, float* t) {
    if (si < 0 || si >= s->NS) return -1;
    const ostate* st = &s->st[si];
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
        const float* r = rays + 6 * (size_t)i;
        v3 o = V(r[0], r[1], r[2]), d = V(r[3], r[4], r[5]);
        float tt;
        int q;
        trace_dyn(o, d, st->T, st->TQ, s->Nt, &tt, &q);
        if (s->BN) trace_bvh_m(s, o, d, &tt, &q, watertight);
        prim[i] = q;
        t[i] = q != -1 ? tt : INFINITY;
    }
    return 0;
}
/* poc_gpu.cu:239-246 */
static int point_index(const ostate* st, v3 H, int q) {
    const float* Q = st->Q + 12 * (size_t)q;
    v3 o = V(Q[0], Q[1], Q[2]), u = V(Q[3], Q[4], Q[5]), v = V(Q[6], Q[7], Q[8]);
    v3 d = vsub(H, o);
    float a = vdot(d, u) / vdot(u, u), b = vdot(d, v) / vdot(v, v);
    int nu = st->dims[2 * q], nv = st->dims[2 * q + 1];
    int iu = imin(imax((int)(a * (float)nu), 0), nu - 1), iv = imin(imax((int)(b * (float)nv), 0), nv - 1);
    return st->off[q] + iv * nu + iu;
}
/* poc_gpu.cu:263-272 */
static int hash_find(const osc_scene* s, uint64_t key) {
    unsigned mask = (unsigned)s->hsize - 1u;
    unsigned h = (unsigned)mix64(key) & mask;
    for (int probe = 0; probe < 64; ++probe) {
        uint64_t k = s->HK[h];
        if (k == key) return s->HV[h];
        if (k == 0ull) return -1;
        h = (h + 1) & mask;
    }
    return -1;
}
/* poc_gpu.cu:274-287 */
static int hash_point(const osc_scene* s, v3 H, v3 n) {
    int b = normal_bucket(n.x, n.y, n.z);
    float ih = 1.f / s->hcell;
    int cx = (int)floorf((H.x - s->lo[0]) * ih), cy = (int)floorf((H.y - s->lo[1]) * ih), cz = (int)floorf((H.z - s->lo[2]) * ih);
    int p = hash_find(s, cell_key(cx, cy, cz, b));
    if (p >= 0) return p;
    for (int d = 0; d < 27; ++d) {
        int dz = d / 9 - 1, dy = (d / 3) % 3 - 1, dx = d % 3 - 1;
        if (dx == 0 && dy == 0 && dz == 0) continue;
        p = hash_find(s, cell_key(cx + dx, cy + dy, cz + dz, b));
        if (p >= 0) return p;
    }
    return -1;
}
/* poc_gpu.cu:346-358: cache point of a hit; returns 1 when the hit does not count */
static int resolve_hit(const osc_scene* s, const ostate* st, int hit, v3 H, v3 D, int q, int i, int* pi) {
    if (!hit) { *pi = i; return 1; }
    if (q >= 0) {
        *pi = point_index(st, H, q);
        const float* Q = st->Q + 12 * (size_t)q;
        return vdot(V(Q[9], Q[10], Q[11]), D) > 0.f;
    }
    const float* n4 = s->STN + 4 * (size_t)(-2 - q);
    v3 n = V(n4[0], n4[1], n4[2]);
    if (vdot(n, D) > 0.f) {
        if (!(f2i(n4[3]) & 1)) { *pi = i; return 1; }
        n = vmul(n, -1.f);
    }
    *pi = hash_point(s, H, n);
    if (*pi < 0) { *pi = i; return 1; }
    return 0;
}
/* poc_gpu.cu:360-366; rsqrtf(x) restated as 1/sqrtf(x) */
static v3 cosine_dir(v3 N, float u1, float u2) {
    float r = sqrtf(u1), phi = 6.28318530718f * u2;
    v3 a = fabsf(N.x) > 0.9f ? V(0, 1, 0) : V(1, 0, 0);
    v3 T = vcross(N, a);
    T = vmul(T, 1.f / sqrtf(vdot(T, T)));
    v3 B = vcross(N, T);
    return vadd(vadd(vmul(T, r * cosf(phi)), vmul(B, r * sinf(phi))), vmul(N, sqrtf(fmaxf(0.f, 1.f - u1))));
}

/* poc_gpu.cu:369-391: direct light and static shadow-voxel mask per point */
void osc_build(osc_scene* s) {
    const int NL = s->NL, NW = s->NW;
    for (int k = 0; k < s->NS; ++k) {
        ostate* st = &s->st[k];
#pragma omp parallel for schedule(static)
        for (int i = 0; i < s->Np; ++i) {
            v3 P = vld(st->P, i), N = vld(st->N, i), O = vadd(P, vmul(N, 1e-3f));
            uint32_t m[64];
            memset(m, 0, sizeof(uint32_t) * (size_t)NW);
            for (int l = 0; l < NL; ++l) {
                v3 d = vsub(vld(s->L, l), P);
                float r = sqrtf(vdot(d, d));
                v3 D = vmul(d, 1.f / r);
                float c = vdot(N, D), t;
                int q;
                trace_full(s, st, O, D, &t, &q);
                int vis = t >= r - 1e-3f;
                float rr = fmaxf(r, 0.05f);
                st->Edir[(size_t)NL * i + l] = st->inten[l] * fmaxf(c, 0.f) / (rr * rr) * (vis ? 1.f : 0.f);
                rast_seg(s, O, vadd(O, vmul(D, fminf(t, r))), m);
            }
            for (int w = 0; w < NW; ++w) st->SV[(size_t)NW * i + w] = m[w];
        }
    }
}

/* ------------------------------------------------------------------ run state */
struct osc_run {
    osc_scene* S;
    osc_method M;
    float *Lc, *Lc2, *m, *n, *c0, *age, *snap, *neq, *coef, *rstat, *dstat;
    int* kk; uint8_t* pending; uint32_t *cur, *prev, *stale;
    float sumpr[2]; int npend[2];
    /* per-point scratch for ordered region sums */
    float *rs_part, *neq_part, *ds_part; int* pr_flag;
    /* Params + Runner locals (poc_gpu.cu:411-422, 839-850) */
    int mode, pend_left, dormant, proj_left, projK, slot[KSNAP], ramp, deps_param;
    float budget, nmax, nmax_resp, rays;
    uint32_t seed, frame;
    float ilearn[32];
    int nslots, slot_state[KSNAP], slot_next, last_event_f, prev_state, f;
};

static int g_threads = 0;
void osc_set_threads(int n) { g_threads = n; }

osc_run* osc_run_new(osc_scene* s) {
    osc_run* r = (osc_run*)calloc(1, sizeof(osc_run));
    size_t Np = (size_t)s->Np, NL = (size_t)s->NL, NW = (size_t)s->NW;
    r->S = s;
    r->Lc = calloc(NL * Np, 4); r->Lc2 = calloc(NL * Np, 4); r->m = calloc(NL * Np, 4);
    r->n = calloc(Np, 4); r->c0 = calloc(Np, 4); r->age = calloc(Np, 4); r->kk = calloc(Np, 4);
    r->pending = calloc(Np, 1); r->cur = calloc(NW * Np, 4); r->prev = calloc(NW * Np, 4); r->stale = calloc(Np, 4);
    r->snap = calloc((size_t)KSNAP * Np * NL, 4); r->neq = calloc((size_t)s->NR * NEQ, 4); r->coef = calloc((size_t)s->NR * KSNAP, 4);
    r->rstat = calloc(4 * (size_t)s->NR, 4); r->dstat = calloc(3 * (size_t)s->NR, 4);
    r->rs_part = calloc(4 * Np, 4); r->neq_part = NULL; r->ds_part = calloc(3 * Np, 4); r->pr_flag = calloc(Np, 4);
    return r;
}

void osc_run_free(osc_run* r) {
    if (!r) return;
    free(r->Lc); free(r->Lc2); free(r->m); free(r->n); free(r->c0); free(r->age); free(r->kk); free(r->pending);
    free(r->cur); free(r->prev); free(r->stale); free(r->snap); free(r->neq); free(r->coef); free(r->rstat); free(r->dstat);
    free(r->rs_part); free(r->neq_part); free(r->ds_part); free(r->pr_flag);
    free(r);
}

void* osc_run_array(osc_run* r, int which, size_t* nb) {
    const osc_scene* s = r->S;
    size_t Np = (size_t)s->Np, NL = (size_t)s->NL, NW = (size_t)s->NW;
    switch (which) {
        case OSC_A_LC: *nb = 4 * NL * Np; return r->Lc;
        case OSC_A_LC2: *nb = 4 * NL * Np; return r->Lc2;
        case OSC_A_M: *nb = 4 * NL * Np; return r->m;
        case OSC_A_N: *nb = 4 * Np; return r->n;
        case OSC_A_C0: *nb = 4 * Np; return r->c0;
        case OSC_A_KK: *nb = 4 * Np; return r->kk;
        case OSC_A_PENDING: *nb = Np; return r->pending;
        case OSC_A_CUR: *nb = 4 * NW * Np; return r->cur;
        case OSC_A_PREV: *nb = 4 * NW * Np; return r->prev;
        case OSC_A_STALE: *nb = 4 * Np; return r->stale;
        case OSC_A_AGE: *nb = 4 * Np; return r->age;
        case OSC_A_SNAP: *nb = 4 * (size_t)KSNAP * Np * NL; return r->snap;
        case OSC_A_NEQ: *nb = 4 * (size_t)s->NR * NEQ; return r->neq;
        case OSC_A_COEF: *nb = 4 * (size_t)s->NR * KSNAP; return r->coef;
        case OSC_A_RSTAT: *nb = 16 * (size_t)s->NR; return r->rstat;
        case OSC_A_DSTAT: *nb = 12 * (size_t)s->NR; return r->dstat;
        case OSC_A_SUMPR: *nb = 8; return r->sumpr;
        case OSC_A_NPEND: *nb = 8; return r->npend;
    }
    *nb = 0;
    return NULL;
}

void osc_run_set_scalar(osc_run* r, int which, int v) {
    switch (which) {
        case 0: r->pend_left = v; break;
        case 1: r->dormant = v; break;
        case 2: r->proj_left = v; break;
        case 3: r->f = v; break;
        case 4: r->nslots = v; break;
        case 5: r->last_event_f = v; break;
        case 6: r->projK = v; break;
    }
}

int osc_run_scalar(osc_run* r, int which) {
    switch (which) {
        case 0: return r->pend_left;
        case 1: return r->dormant;
        case 2: return r->proj_left;
        case 3: return r->f;
        case 4: return r->nslots;
        case 5: return r->last_event_f;
        case 6: return r->projK;
    }
    return 0;
}

/* Fixed reduction tree shared with the product kernels.  Level 1, per block of 256 values:
 * a butterfly over each warp of 32 (lane l += lane l+off, off = 16..1), then the 8 warp sums
 * in order.  Level 2, over the G block partials: slot t (0..255) sums partials t, t+256, ...
 * in order, then the 256 slots go through the same block tree.  Values past the end are 0. */
#define TREE_BLOCK(T, get)                                                             \
    {                                                                                  \
        T blk = 0;                                                                     \
        for (int w = 0; w < BLK / 32; ++w) {                                           \
            T lane[32];                                                                \
            for (int l = 0; l < 32; ++l) lane[l] = get(32 * w + l);                    \
            for (int off = 16; off > 0; off >>= 1)                                     \
                for (int l = 0; l < off; ++l) lane[l] = lane[l] + lane[l + off];       \
            blk = w == 0 ? lane[0] : blk + lane[0];                                    \
        }                                                                              \
        out = blk;                                                                     \
    }
static double tree_sum_d(const double* v, long n) {
    long G = (n + BLK - 1) / BLK;
    double* part = (double*)malloc(sizeof(double) * (size_t)(G ? G : 1));
    for (long b = 0; b < G; ++b) {
        double out;
#define GETD(k) ((b * BLK + (k)) < n ? v[b * BLK + (k)] : 0.0)
        TREE_BLOCK(double, GETD)
#undef GETD
        part[b] = out;
    }
    double slot[BLK];
    for (long t = 0; t < BLK; ++t) {
        double x = t < G ? part[t] : 0.0;
        for (long b = t + BLK; b < G; b += BLK) x = x + part[b];
        slot[t] = x;
    }
    free(part);
    double out;
#define GETS(k) (slot[(k)])
    TREE_BLOCK(double, GETS)
#undef GETS
    return out;
}

/* poc_gpu.cu:427-431 */
static inline float est_of(const osc_run* r, int i, int dormant) {
    float e = 0.f;
    for (int l = 0; l < r->S->NL; ++l) if (!((dormant >> l) & 1)) e += r->Lc[(size_t)r->S->NL * i + l];
    return e;
}

/* poc_gpu.cu:604-609.  The sum is exact: each 1/(n+1) is an integer number of 2^-40 units
 * (exact for terms >= 2^-16), the integers are added, and the total is rounded once to float,
 * as the product kernels do. */
static void sumpr_into(osc_run* r, int slot) {
    long Np = r->S->Np;
    uint64_t tot = 0;
    for (long i = 0; i < Np; ++i) {
        float pr = 1.f / (r->n[i] + 1.f);
        tot += (uint64_t)llrintf(pr * 1099511627776.0f);
    }
    r->sumpr[slot] = (float)tot * (1.0f / 1099511627776.0f);
}

void osc_run_begin(osc_run* r, const osc_method* m, int s0, uint32_t seed) {
    osc_scene* S = r->S;
    size_t Np = (size_t)S->Np, NL = (size_t)S->NL, NW = (size_t)S->NW;
    r->M = *m;
    /* poc_gpu.cu:830-850 */
    if (S->has_ref) memcpy(r->Lc, S->st[s0].Pw, 4 * NL * Np);
    else memset(r->Lc, 0, 4 * NL * Np);
    const float nmax = m->nmax * m->rays;
    for (size_t i = 0; i < Np; ++i) { r->n[i] = nmax; r->age[i] = 1e4f; }
    memset(r->pending, 0, Np); memset(r->cur, 0, 4 * NW * Np); memset(r->prev, 0, 4 * NW * Np);
    memset(r->stale, 0, 4 * Np);
    r->dormant = 0;
    for (int l = 0; l < 32; ++l) r->ilearn[l] = 0.f;
    r->sumpr[0] = (float)S->Np / (nmax + 1.f); r->sumpr[1] = 0.f;
    r->npend[0] = r->npend[1] = 0;
    r->mode = m->mode; r->seed = seed; r->frame = 0; r->pend_left = 0; r->deps_param = m->deps;
    r->ramp = m->ramp ? 1 : 0;
    r->proj_left = 0; r->projK = 0;
    for (int a = 0; a < KSNAP; ++a) r->slot[a] = 0;
    r->rays = m->rays; r->budget = m->budget * m->rays; r->nmax = nmax; r->nmax_resp = m->nmax_resp * m->rays;
    r->nslots = 0; r->slot_next = 0; r->last_event_f = 0;
    for (int k = 0; k < KSNAP; ++k) r->slot_state[k] = -1;
    r->prev_state = s0; r->f = 0;
}

/* ---------------------------------------------------------- per-frame point kernels */
/* poc_gpu.cu:433-530 for one point; region contributions go to per-point scratch */
static void trace_point(osc_run* r, const ostate* st, int i, int deps, osc_ray_rec* rec, int* nrec, int maxrec) {
    const osc_scene* s = r->S;
    const int NL = s->NL, NW = s->NW;
    const size_t Np = (size_t)s->Np;
    uint32_t rs = hash32(r->seed * 0x9E3779B9u ^ hash32(r->frame * 0x85EBCA6Bu ^ hash32((uint32_t)i + 1u)));
    int k;
    int pend = r->pend_left > 0 && r->pending[i];
    if (r->mode == 0) {
        float kb = floorf(r->budget);
        k = (int)kb + (rnd(&rs) < r->budget - kb ? 1 : 0);
    } else {
        float pr = 1.f / (r->n[i] + 1.f);
        float rrest = (float)(s->Np - r->npend[0]);
        float e = rrest * (0.5f / (float)s->Np + 0.5f * pr / r->sumpr[0]) * r->rays;
        float eb = floorf(e);
        k = (pend ? 1 : 0) + (int)eb + (rnd(&rs) < e - eb ? 1 : 0);
    }
    v3 P = vld(st->P, i), N = vld(st->N, i), O = vadd(P, vmul(N, 1e-3f));
    float acc[32];
    for (int l = 0; l < NL; ++l) acc[l] = 0.f;
    uint32_t m[64];
    memset(m, 0, sizeof(uint32_t) * (size_t)NW);
    float c0 = pend ? r->c0[i] : 0.f;
    float sd = 0.f, sq = 0.f;
    for (int ray = 0; ray < k; ++ray) {
        float u1 = rnd(&rs);
        float u2 = rnd(&rs);
        v3 D = cosine_dir(N, u1, u2);
        float t;
        int q;
        int hit = trace_full(s, st, O, D, &t, &q);
        v3 H = hit ? vadd(O, vmul(D, t)) : O;
        int pi;
        int back = resolve_hit(s, st, hit, H, D, q, i, &pi);
        if (rec && *nrec < maxrec) {
            osc_ray_rec* x = &rec[(*nrec)++];
            x->point = i; x->ray = ray; x->q = hit ? q : -1; x->pi = pi; x->back = back; x->t = hit ? t : INFINITY;
        }
        float val = 0.f;
        if (!back) {
            float A = s->A[pi];
            for (int l = 0; l < NL; ++l) {
                float lc = ((r->dormant >> l) & 1) ? 0.f : r->Lc[(size_t)NL * pi + l];
                float v = A * (st->Edir[(size_t)NL * pi + l] + lc);
                acc[l] += v;
                val += v;
            }
        }
        if (deps) {
            int src = back ? i : pi;
            for (int w = 0; w < NW; ++w) m[w] |= st->SV[(size_t)NW * src + w];
            dda(s, O, H, m);
        }
        if (pend) { float dv = val - c0; sd += dv; sq += dv * dv; }
    }
    if (rec) return;
    float* rp = r->rs_part + 4 * (size_t)i;
    if (pend && k > 0) { rp[0] = sd; rp[1] = sq; rp[2] = c0 * (float)k; rp[3] = (float)k; r->pr_flag[i] = 1; }
    else r->pr_flag[i] = 0;
    if (r->proj_left > 0 && k > 0) {
        float T[KSNAP];
        for (int a = 0; a < r->projK; ++a) {
            const float* sp = r->snap + ((size_t)r->slot[a] * Np + i) * NL;
            float tt = 0.f;
            for (int l = 0; l < NL; ++l) if (!((r->dormant >> l) & 1)) tt += sp[l];
            T[a] = tt;
        }
        float sv = 0.f;
        for (int l = 0; l < NL; ++l) sv += acc[l];
        float* qn = r->neq_part + (size_t)NEQ * i;
        memset(qn, 0, sizeof(float) * NEQ);
        int ix = 0;
        for (int a = 0; a < r->projK; ++a)
            for (int b = a; b < r->projK; ++b) qn[ix++] = (float)k * T[a] * T[b];
        for (int a = 0; a < r->projK; ++a) qn[21 + a] = sv * T[a];
        qn[27] = (float)k;
    }
    r->kk[i] = k;
    float ik = k > 0 ? 1.f / (float)k : 0.f;
    for (int l = 0; l < NL; ++l) r->m[(size_t)NL * i + l] = acc[l] * ik;
    if (r->M.ddgi && k > 0) {
        float sa = 0.f;
        for (int l = 0; l < NL; ++l) sa += acc[l];
        float* dp = r->ds_part + 3 * (size_t)i;
        dp[0] = sa * ik; dp[1] = est_of(r, i, r->dormant); dp[2] = 1.f;
    } else if (r->M.ddgi) {
        float* dp = r->ds_part + 3 * (size_t)i;
        dp[0] = dp[1] = dp[2] = -0.f;
    }
    if (deps && k > 0)
        for (int w = 0; w < NW; ++w) r->cur[(size_t)w * Np + i] |= m[w];
}

static void trace_all(osc_run* r, const ostate* st, int deps) {
    const osc_scene* s = r->S;
    const long Np = s->Np;
    if (r->proj_left > 0 && !r->neq_part) r->neq_part = (float*)calloc((size_t)NEQ * (size_t)Np, 4);
#pragma omp parallel for schedule(dynamic, 1024)
    for (long i = 0; i < Np; ++i) trace_point(r, st, (int)i, deps, NULL, NULL, 0);
    /* region sums in point order */
    for (long i = 0; i < Np; ++i) {
        if (r->pr_flag[i]) {
            float* d = r->rstat + 4 * (size_t)s->region[i];
            const float* p = r->rs_part + 4 * (size_t)i;
            d[0] += p[0]; d[1] += p[1]; d[2] += p[2]; d[3] += p[3];
        }
        if (r->proj_left > 0 && r->kk[i] > 0) {
            float* qd = r->neq + (size_t)NEQ * s->region[i];
            const float* qp = r->neq_part + (size_t)NEQ * i;
            int ix = 0;
            for (int a = 0; a < r->projK; ++a) for (int b = a; b < r->projK; ++b, ++ix) qd[ix] += qp[ix];
            for (int a = 0; a < r->projK; ++a) qd[21 + a] += qp[21 + a];
            qd[27] += qp[27];
        }
        if (r->M.ddgi && r->kk[i] > 0) {
            float* dd = r->dstat + 3 * (size_t)s->region[i];
            const float* dp = r->ds_part + 3 * (size_t)i;
            dd[0] += dp[0]; dd[1] += dp[1]; dd[2] += dp[2];
        }
    }
}

/* poc_gpu.cu:532-555 */
static void decide_all(osc_run* r) {
    const osc_scene* s = r->S;
    int cnt_pend = 0;
    for (long i = 0; i < s->Np; ++i) {
        if (!r->pending[i]) continue;
        const float* r4 = r->rstat + 4 * (size_t)s->region[i];
        float cnt = r4[3];
        int done = 0;
        if (cnt >= 8.f) {
            float mean = r4[0] / cnt;
            float se = sqrtf(fmaxf(r4[1] / cnt - mean * mean, 0.f) / cnt);
            float base = r4[2] / cnt;
            float rel = mean / base;
            if (fabsf(mean) > 2.f * se && fabsf(rel) > 0.03f) {
                float tgt = fminf(fmaxf(0.5f / fabsf(rel), 1.f) * r->rays, r->nmax);
                r->n[i] = fminf(r->n[i], tgt);
                r->pending[i] = 0;
                done = 1;
            }
        }
        if (!done) {
            if (r->pend_left <= 1) r->pending[i] = 0;
            else cnt_pend++;
        }
    }
    r->npend[1] += cnt_pend;
}

/* poc_gpu.cu:562-602 */
static void update_all(osc_run* r) {
    const osc_scene* s = r->S;
    const int NL = s->NL;
    const long Np = s->Np;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < Np; ++i) {
        int k = r->kk[i];
        float n = r->n[i], nn = n + (float)k;
        float nmx = r->nmax;
        if (r->ramp) { float a = r->age[i]; nmx = fminf(r->nmax, (4.f + 0.5f * a) * r->rays); r->age[i] = fminf(a + 1.f, 1e4f); }
        float alpha = k > 0 ? fminf((float)k / fminf(fmaxf(nn, 1.f), nmx), 1.f) : 0.f;
        if (r->M.ddgi) {
            const float* d3 = r->dstat + 3 * (size_t)s->region[i];
            float scale = 1.f, h = r->M.ddgi_h;
            if (d3[2] > 0.f) {
                float mn = d3[0] / d3[2], mc = d3[1] / d3[2];
                float rel = fabsf(mn - mc) / fmaxf(mc, 1e-3f);
                if (rel > r->M.ddgi_thr) h = fmaxf(0.f, h - 0.75f);
                if (r->M.ddgi_clamp && rel > 0.10f) scale = 0.25f;
            }
            float w = k > 0 ? (1.f - h) * scale : 0.f;
            for (int l = 0; l < NL; ++l) {
                float a = r->Lc[(size_t)NL * i + l];
                r->Lc2[(size_t)NL * i + l] = ((r->dormant >> l) & 1) ? a : a + w * (r->m[(size_t)NL * i + l] - a);
            }
        } else {
            float alpha_r = k > 0 ? fminf((float)k / fminf(fmaxf(nn, 1.f), r->nmax_resp), 1.f) : 0.f;
            for (int l = 0; l < NL; ++l) {
                float a = r->Lc[(size_t)NL * i + l];
                float al = ((r->M.resp_mask >> l) & 1) ? alpha_r : alpha;
                if ((r->dormant >> l) & 1) al = 0.f;
                r->Lc2[(size_t)NL * i + l] = a + al * (r->m[(size_t)NL * i + l] - a);
            }
        }
        n = fminf(nn, nmx);
        r->n[i] = n;
    }
    sumpr_into(r, 1);
}

/* poc_gpu.cu:612-617 */
static void restored_all(osc_run* r, int verify) {
    for (long i = 0; i < r->S->Np; ++i) {
        r->n[i] = r->nmax; r->age[i] = 1e4f; r->pending[i] = 0;
        if (verify) { r->pending[i] = 1; r->c0[i] = est_of(r, (int)i, r->dormant); r->npend[1]++; }
    }
}
/* poc_gpu.cu:620-635 */
static void proj_apply_all(osc_run* r) {
    const osc_scene* s = r->S;
    const int NL = s->NL;
    const size_t Np = (size_t)s->Np;
    for (size_t i = 0; i < Np; ++i) {
        if (r->n[i] >= 16.f) continue;
        const float* cf = r->coef + (size_t)s->region[i] * KSNAP;
        if (isnan(cf[0])) continue;
        for (int l = 0; l < NL; ++l) {
            if ((r->dormant >> l) & 1) continue;
            float v = 0.f;
            for (int a = 0; a < r->projK; ++a) v += cf[a] * r->snap[((size_t)r->slot[a] * Np + i) * NL + l];
            r->Lc[NL * i + l] = fmaxf(v, 0.f);
        }
        r->n[i] = 8.f * r->rays; r->age[i] = 8.f;
        r->pending[i] = 1; r->c0[i] = est_of(r, (int)i, r->dormant);
        r->npend[1]++;
    }
}
/* poc_gpu.cu:637-640 */
static void rescale_all(osc_run* r, int l, float ratio) {
    for (long i = 0; i < r->S->Np; ++i) r->Lc[(size_t)r->S->NL * i + l] *= ratio;
}
/* poc_gpu.cu:642-660 */
static void touched_all(osc_run* r, const int* Vl, int nv, int kind) {
    const osc_scene* s = r->S;
    const size_t Np = (size_t)s->Np;
    for (size_t i = 0; i < Np; ++i) {
        int t = 0;
        for (int j = 0; j < nv && !t; ++j) {
            int v = Vl[j];
            size_t o = (size_t)(v >> 5) * Np + i;
            t = ((r->cur[o] | r->prev[o]) >> (v & 31)) & 1u;
        }
        if (!t) continue;
        if (kind == 0) { r->n[i] = 0.f; r->age[i] = 0.f; }
        else if (kind == 1) { r->pending[i] = 1; r->c0[i] = est_of(r, (int)i, r->dormant); r->npend[1]++; }
        if (kind >= 1 && r->dormant) r->stale[i] |= (uint32_t)r->dormant;
    }
}
/* poc_gpu.cu:663-674 */
static void wake_all(osc_run* r, int l, int verify) {
    for (long i = 0; i < r->S->Np; ++i) {
        if ((r->stale[i] >> l) & 1) {
            if (verify) { r->pending[i] = 1; r->c0[i] = est_of(r, (int)i, r->dormant); r->npend[1]++; }
            else { r->Lc[(size_t)r->S->NL * i + l] = 0.f; r->n[i] = 0.f; r->age[i] = 0.f; }
            r->stale[i] &= ~(1u << l);
        }
    }
}
/* poc_gpu.cu:676-681 */
static void oracle_all(osc_run* r, const float* rold, const float* rnew) {
    for (long i = 0; i < r->S->Np; ++i) {
        float rel = fabsf(rnew[i] - rold[i]) / (rold[i] + 1e-2f);
        r->n[i] *= 1.f - fminf(fmaxf(4.f * rel, 0.f), 1.f);
    }
}

/* poc_gpu.cu:966-995: per-region FP64 least squares for the snapshot projection */
static void proj_solve(osc_run* r) {
    const osc_scene* s = r->S;
    const int K = r->projK;
    for (size_t x = 0; x < (size_t)s->NR * KSNAP; ++x) r->coef[x] = NAN;
    for (int rg = 0; rg < s->NR; ++rg) {
        const float* Q = r->neq + (size_t)rg * NEQ;
        if (Q[27] < 24.f) continue;
        double A[KSNAP][KSNAP + 1];
        int ix = 0;
        double tr = 0;
        for (int a = 0; a < K; ++a) for (int b = a; b < K; ++b) { A[a][b] = A[b][a] = Q[ix++]; }
        for (int a = 0; a < K; ++a) { A[a][K] = Q[21 + a]; tr += A[a][a]; }
        for (int a = 0; a < K; ++a) A[a][a] += 1e-3 * tr / K + 1e-9;
        int ok = 1;
        for (int a = 0; a < K && ok; ++a) {
            int pv = a;
            for (int b = a + 1; b < K; ++b) if (fabs(A[b][a]) > fabs(A[pv][a])) pv = b;
            if (fabs(A[pv][a]) < 1e-12) { ok = 0; break; }
            for (int t = 0; t <= K; ++t) { double x = A[a][t]; A[a][t] = A[pv][t]; A[pv][t] = x; }
            for (int b = 0; b < K; ++b)
                if (b != a) { double mm = A[b][a] / A[a][a]; for (int t = a; t <= K; ++t) A[b][t] -= mm * A[a][t]; }
        }
        if (!ok) continue;
        int sane = 1;
        double xs[KSNAP];
        for (int a = 0; a < K; ++a) { xs[a] = A[a][K] / A[a][a]; if (!isfinite(xs[a]) || fabs(xs[a]) > 4.0) sane = 0; }
        if (sane) for (int a = 0; a < K; ++a) r->coef[(size_t)rg * KSNAP + a] = (float)xs[a];
    }
}

/* poc_gpu.cu:851-1011: one frame of Runner::run */
int osc_frame(osc_run* r, int si, int want_err, double err3[3], float* errv) {
    osc_scene* S = r->S;
    const osc_method* M = &r->M;
    const int NL = S->NL;
    const size_t Np = (size_t)S->Np;
    if (si < 0 || si >= S->NS) return -1;
#ifdef _OPENMP
    if (g_threads > 0) omp_set_num_threads(g_threads);
#endif
    const ostate* st = &S->st[si];
    const int f = r->f;
    r->frame = (uint32_t)f;
    if (f > 0 && r->prev_state != si) {
        const int e = r->prev_state;
        const int pe = e * S->NS + si;
        if (M->snaps && f - r->last_event_f >= 20) {
            int k = -1;
            for (int a = 0; a < r->nslots; ++a) if (r->slot_state[a] == e) k = a;
            if (k < 0) { if (r->nslots < KSNAP) k = r->nslots++; else { k = r->slot_next; r->slot_next = (r->slot_next + 1) % KSNAP; } }
            r->slot_state[k] = e;
            memcpy(r->snap + (size_t)k * Np * NL, r->Lc, 4 * Np * (size_t)NL);
        }
        if (M->oracle && S->has_ref) oracle_all(r, S->st[e].ref, st->ref);
        if (M->rescale && !M->deps) {
            for (int l = 0; l < NL; ++l) {
                float a = S->st[e].inten[l], b = S->st[si].inten[l];
                if (a == b) continue;
                if (M->memory && a > 0 && b == 0) { r->dormant |= 1 << l; r->ilearn[l] = a; }
                else if (M->memory && a == 0 && b > 0 && ((r->dormant >> l) & 1)) { rescale_all(r, l, b / r->ilearn[l]); r->dormant &= ~(1 << l); }
                else if (a > 0) rescale_all(r, l, b / a);
            }
        }
        if (M->deps) {
            int woke = 0;
            for (int l = 0; l < NL; ++l) {
                float a = S->st[e].inten[l], b = S->st[si].inten[l];
                if (a == b) continue;
                if (M->memory && a > 0 && b == 0) { r->dormant |= 1 << l; r->ilearn[l] = a; }
                else if (M->memory && a == 0 && b > 0 && ((r->dormant >> l) & 1)) {
                    rescale_all(r, l, b / r->ilearn[l]);
                    r->dormant &= ~(1 << l);
                    woke |= 1 << l;
                    if (M->wake_verify) {
                        r->npend[0] = r->npend[1] = 0;
                        memset(r->rstat, 0, 16 * (size_t)S->NR);
                        wake_all(r, l, 1);
                        r->npend[0] = r->npend[1];
                        r->pend_left = VERIF_FRAMES;
                    } else wake_all(r, l, 0);
                } else if (a > 0) rescale_all(r, l, b / a);
            }
            for (int l = 0; l < NL; ++l) {
                int nv;
                const int* Vl = osc_event_list(S, pe, 1 + l, &nv);
                if (nv > 0 && !((woke >> l) & 1)) touched_all(r, Vl, nv, 0);
            }
            int no;
            const int* occ = osc_event_list(S, pe, 0, &no);
            if (no > 0) {
                if (M->verify) {
                    r->npend[0] = r->npend[1] = 0;
                    memset(r->rstat, 0, 16 * (size_t)S->NR);
                    touched_all(r, occ, no, 1);
                    r->npend[0] = r->npend[1];
                    r->pend_left = VERIF_FRAMES;
                } else if (r->dormant) touched_all(r, occ, no, 2);
            }
        }
        if (M->snaps) {
            int hit = -1;
            for (int a = 0; a < r->nslots; ++a) if (r->slot_state[a] == si) hit = a;
            if (hit >= 0) {
                memcpy(r->Lc, r->snap + (size_t)hit * Np * NL, 4 * Np * (size_t)NL);
                if (M->snap_verify) {
                    r->npend[0] = r->npend[1] = 0;
                    memset(r->rstat, 0, 16 * (size_t)S->NR);
                    restored_all(r, 1);
                    r->npend[0] = r->npend[1];
                    r->pend_left = VERIF_FRAMES;
                } else {
                    restored_all(r, 0);
                    r->npend[0] = r->npend[1] = 0;
                    r->pend_left = 0;
                }
                r->proj_left = 0;
            } else if (M->proj && r->nslots >= 2) {
                r->projK = r->nslots;
                for (int a = 0; a < r->nslots; ++a) r->slot[a] = a;
                memset(r->neq, 0, 4 * (size_t)S->NR * NEQ);
                r->proj_left = PROJ_FRAMES;
            }
        }
        r->last_event_f = f;
        if (r->mode == 1) sumpr_into(r, 0);
    }
    r->prev_state = si;
    if (M->ddgi) memset(r->dstat, 0, 12 * (size_t)S->NR);
    if (M->deps && f % 32 == 0) {
        uint32_t* t = r->cur; r->cur = r->prev; r->prev = t;
        memset(r->cur, 0, 4 * (size_t)S->NW * Np);
    }
    int track = M->deps && (f % (M->track_every > 0 ? M->track_every : 1) == 0);
    trace_all(r, st, track);
    if (r->pend_left > 0) {
        r->npend[1] = 0;
        decide_all(r);
        r->npend[0] = r->npend[1];
        r->pend_left--;
    }
    update_all(r);
    r->sumpr[0] = r->sumpr[1];
    { float* t = r->Lc; r->Lc = r->Lc2; r->Lc2 = t; }
    if (r->proj_left > 0 && --r->proj_left == 0) {
        proj_solve(r);
        r->npend[0] = r->npend[1] = 0;
        memset(r->rstat, 0, 16 * (size_t)S->NR);
        proj_apply_all(r);
        r->npend[0] = r->npend[1];
        r->pend_left = VERIF_FRAMES;
    }
    int have = 0;
    if (want_err && S->has_ref) {
        /* poc_gpu.cu:683-696 + 1005-1010 */
        double* d2 = (double*)malloc(sizeof(double) * Np);
        double* rsv = (double*)malloc(sizeof(double) * Np);
        double* cn = (double*)malloc(sizeof(double) * Np);
        for (size_t i = 0; i < Np; ++i) {
            if (st->valid[i]) {
                float e = est_of(r, (int)i, r->dormant) - st->ref[i];
                d2[i] = (double)e * e; rsv[i] = st->ref[i]; cn[i] = 1.0;
            } else d2[i] = rsv[i] = cn[i] = 0.0;
        }
        double h0 = tree_sum_d(d2, (long)Np), h1 = tree_sum_d(rsv, (long)Np), h2 = tree_sum_d(cn, (long)Np);
        free(d2); free(rsv); free(cn);
        if (err3) { err3[0] = h0; err3[1] = h1; err3[2] = h2; }
        if (errv) *errv = (float)(sqrt(h0 / h2) / (h1 / h2));
        have = 1;
    }
    r->f = f + 1;
    return have;
}

int osc_probe_rays(osc_run* r, int si, const int* pts, int npts, osc_ray_rec* out, int maxrec) {
    const osc_scene* S = r->S;
    if (si < 0 || si >= S->NS) return -1;
    r->frame = (uint32_t)r->f;
    int n = 0;
    for (int k = 0; k < npts; ++k) {
        if (pts[k] < 0 || pts[k] >= S->Np) continue;
        trace_point(r, &S->st[si], pts[k], 0, out, &n, maxrec);
    }
    return n;
}

/* Image pass of the product (no reference counterpart): pinhole camera, closest hit, cache
 * point, A * sum over lights of (direct + cached indirect, dormant lights without cache). */
int osc_render(osc_run* r, int si, const float* eye, const float* fwd, const float* right, const float* up, float tx, float ty,
               int w, int h, float* out) {
    const osc_scene* S = r->S;
    if (si < 0 || si >= S->NS || w <= 0 || h <= 0) return -1;
    const ostate* st = &S->st[si];
    const int NL = S->NL;
#pragma omp parallel for schedule(dynamic, 16)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            float sx = (((float)x + 0.5f) / (float)w * 2.f - 1.f) * tx, sy = (1.f - ((float)y + 0.5f) / (float)h * 2.f) * ty;
            v3 D = V(fwd[0] + right[0] * sx + up[0] * sy, fwd[1] + right[1] * sx + up[1] * sy, fwd[2] + right[2] * sx + up[2] * sy);
            D = vmul(D, 1.f / sqrtf(vdot(D, D)));
            v3 O = V(eye[0], eye[1], eye[2]);
            float t;
            int q, pi;
            int hit = trace_full(S, st, O, D, &t, &q);
            v3 H = hit ? vadd(O, vmul(D, t)) : O;
            int back = resolve_hit(S, st, hit, H, D, q, 0, &pi);
            float val = 0.f;
            if (hit && !back) {
                float A = S->A[pi];
                for (int l = 0; l < NL; ++l) {
                    float lc = ((r->dormant >> l) & 1) ? 0.f : r->Lc[(size_t)NL * pi + l];
                    val += A * (st->Edir[(size_t)NL * pi + l] + lc);
                }
            }
            out[(size_t)y * w + x] = val;
        }
    return 0;
}

/* ------------------------------------------------------------------ adjoint support */

/* The K rays of one reference iteration with `seed` (prep_mesh.cuh:182-200: per-point seed
 * hash32(seed ^ hash32(i + 1)), cosine directions, trace and hit resolution of the frame),
 * kept: hits[i * K + r] = the cache point reached, -1 when the ray does not count. */
void osc_frozen_hits(const osc_scene* S, int si, uint32_t seed, int K, int* hits) {
    const ostate* st = &S->st[si];
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < S->Np; ++i) {
        uint32_t rs = hash32(seed ^ hash32((uint32_t)i + 1u));
        v3 P = vld(st->P, i), N = vld(st->N, i), O = vadd(P, vmul(N, 1e-3f));
        for (int r = 0; r < K; ++r) {
            float u1 = rnd(&rs);
            float u2 = rnd(&rs);
            v3 D = cosine_dir(N, u1, u2);
            float t;
            int q, pi;
            int hit = trace_full(S, st, O, D, &t, &q);
            v3 H = hit ? vadd(O, vmul(D, t)) : O;
            int back = resolve_hit(S, st, hit, H, D, q, i, &pi);
            hits[(size_t)i * K + r] = back ? -1 : pi;
        }
    }
}

/* Direct light of every light at unit emission (k_build's formula, poc_gpu.cu:369-391, with
 * inten = 1): out[i * NL + l]. */
void osc_direct_unit(const osc_scene* S, int si, float* out) {
    const ostate* st = &S->st[si];
    const int NL = S->NL;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < S->Np; ++i) {
        v3 P = vld(st->P, i), N = vld(st->N, i), O = vadd(P, vmul(N, 1e-3f));
        for (int l = 0; l < NL; ++l) {
            v3 d = vsub(vld(S->L, l), P);
            float r = sqrtf(vdot(d, d));
            v3 D = vmul(d, 1.f / r);
            float c = vdot(N, D), t;
            int q;
            trace_full(S, st, O, D, &t, &q);
            int vis = t >= r - 1e-3f;
            float rr = fmaxf(r, 0.05f);
            out[(size_t)NL * i + l] = 1.f * fmaxf(c, 0.f) / (rr * rr) * (vis ? 1.f : 0.f);
        }
    }
}

/* ------------------------------------------------------------------ FP64 path tracer
 * An independent estimate of the converged cache (the fixed point the reference's scene
 * preparation iterates to, prep_mesh.cuh:182-213 and :459-518): random walks over the cache
 * points, everything in double -- directions, ray-triangle and ray-box tests, hit resolution,
 * direct light with its shadow ray (the formula of k_build, poc_gpu.cu:369-391) and the path
 * throughput.  A walk from point i takes a cosine ray from P_i + 1e-3 N_i, resolves the hit to
 * its cache point j as every frame does (poc_gpu.cu:339-358), adds throughput x A_j x direct_j
 * and continues from point j; it ends on a ray that does not count, or by Russian roulette
 * (survival probability A_j) after `min_bounces`.  Random numbers: splitmix64 streams. */
typedef struct { double x, y, z; } d3;
static inline d3 D3(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static inline d3 dadd(d3 a, d3 b) { return D3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline d3 dsub(d3 a, d3 b) { return D3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline d3 dmul(d3 a, double s) { return D3(a.x * s, a.y * s, a.z * s); }
static inline double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline d3 dcross(d3 a, d3 b) { return D3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline d3 dld(const float* p, long i) { return D3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

static inline double urand(uint64_t* s) {
    *s += 0x9E3779B97F4A7C15ull;
    return (double)(mix64(*s) >> 11) * (1.0 / 9007199254740992.0);
}

/* Moller-Trumbore in double; single triangle (v0, e1, e2), closest t > 1e-4 */
static inline int tri_d(d3 o, d3 d, const float* T, double eps, int clamp_u, double* t_out) {
    d3 v0 = D3(T[0], T[1], T[2]), e1 = D3(T[3], T[4], T[5]), e2 = D3(T[6], T[7], T[8]);
    d3 p = dcross(d, e2);
    double det = ddot(e1, p);
    if (fabs(det) <= eps) return 0;
    double inv = 1.0 / det;
    d3 tv = dsub(o, v0);
    double u = ddot(tv, p) * inv;
    if (u < 0.0 || (clamp_u && u > 1.0)) return 0;
    d3 qv = dcross(tv, e1);
    double v = ddot(d, qv) * inv;
    if (v < 0.0 || u + v > 1.0) return 0;
    *t_out = ddot(e2, qv) * inv;
    return 1;
}

static inline double box_d(const float* a, const float* b, d3 o, d3 inv, double tmax) {
    double tx1 = (a[0] - o.x) * inv.x, tx2 = (b[0] - o.x) * inv.x;
    double ty1 = (a[1] - o.y) * inv.y, ty2 = (b[1] - o.y) * inv.y;
    double tz1 = (a[2] - o.z) * inv.z, tz2 = (b[2] - o.z) * inv.z;
    double tn = fmax(fmax(fmin(tx1, tx2), fmin(ty1, ty2)), fmax(fmin(tz1, tz2), 0.0));
    double tf = fmin(fmin(fmax(tx1, tx2), fmax(ty1, ty2)), fmin(fmax(tz1, tz2), tmax));
    return tn <= tf ? tn : 1e300;
}

/* closest hit: dynamic triangles (q = quad id) then the static BVH (q = -2 - triangle) */
static int trace_d(const osc_scene* s, const ostate* st, d3 o, d3 d, double* tmin, int* q) {
    *tmin = INFINITY;
    *q = -1;
    double t;
    for (int j = 0; j < s->Nt; ++j)
        if (tri_d(o, d, st->T + 9 * (size_t)j, 1e-15, 0, &t) && t > 1e-4 && t < *tmin) { *tmin = t; *q = st->TQ[j]; }
    if (!s->BN) return *q != -1;
    d3 inv = D3(d.x != 0.0 ? 1.0 / d.x : copysign(1e300, d.x), d.y != 0.0 ? 1.0 / d.y : copysign(1e300, d.y),
                d.z != 0.0 ? 1.0 / d.z : copysign(1e300, d.z));
    int stack[128], sp = 0, node = 0;
    for (;;) {
        const float* a = s->BN + 8 * (size_t)node;
        const float* b = a + 4;
        int lf = f2i(a[3]), cnt = f2i(b[3]);
        if (cnt > 0) {
            for (int j = lf; j < lf + cnt; ++j)
                if (tri_d(o, d, s->ST + 9 * (size_t)j, 1e-18, 1, &t) && t > 1e-4 && t < *tmin) { *tmin = t; *q = -2 - j; }
        } else {
            const float* la = s->BN + 8 * (size_t)lf;
            double tl = box_d(la, la + 4, o, inv, *tmin), tr = box_d(la + 8, la + 12, o, inv, *tmin);
            int first = lf, second = lf + 1;
            if (tr < tl) { double x = tl; tl = tr; tr = x; first = lf + 1; second = lf; }
            if (tl < 1e300) {
                if (tr < 1e300 && sp < 128) stack[sp++] = second;
                node = first;
                continue;
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    return *q != -1;
}

/* cache point of a hit in double (poc_gpu.cu:239-287, 346-358); -1 when it does not count */
static int resolve_d(const osc_scene* s, const ostate* st, d3 H, d3 D, int q) {
    if (q >= 0) {
        const float* Q = st->Q + 12 * (size_t)q;
        if (ddot(D3(Q[9], Q[10], Q[11]), D) > 0.0) return -1;
        d3 o = D3(Q[0], Q[1], Q[2]), u = D3(Q[3], Q[4], Q[5]), v = D3(Q[6], Q[7], Q[8]);
        d3 dd = dsub(H, o);
        double a = ddot(dd, u) / ddot(u, u), b = ddot(dd, v) / ddot(v, v);
        int nu = st->dims[2 * q], nv = st->dims[2 * q + 1];
        int iu = imin(imax((int)(a * nu), 0), nu - 1), iv = imin(imax((int)(b * nv), 0), nv - 1);
        return st->off[q] + iv * nu + iu;
    }
    const float* n4 = s->STN + 4 * (size_t)(-2 - q);
    d3 n = D3(n4[0], n4[1], n4[2]);
    if (ddot(n, D) > 0.0) {
        if (!(f2i(n4[3]) & 1)) return -1;
        n = dmul(n, -1.0);
    }
    int bk = normal_bucket((float)n.x, (float)n.y, (float)n.z);
    double ih = 1.0 / s->hcell;
    int cx = (int)floor((H.x - s->lo[0]) * ih), cy = (int)floor((H.y - s->lo[1]) * ih), cz = (int)floor((H.z - s->lo[2]) * ih);
    int p = hash_find(s, cell_key(cx, cy, cz, bk));   /* own cell, then the 26 neighbours */
    if (p >= 0) return p;
    for (int k = 0; k < 27; ++k) {
        int dz = k / 9 - 1, dy = (k / 3) % 3 - 1, dx = k % 3 - 1;
        if (dx == 0 && dy == 0 && dz == 0) continue;
        p = hash_find(s, cell_key(cx + dx, cy + dy, cz + dz, bk));
        if (p >= 0) return p;
    }
    return -1;
}

static d3 cosine_d(d3 N, double u1, double u2) {
    double r = sqrt(u1), phi = 6.283185307179586 * u2;
    d3 a = fabs(N.x) > 0.9 ? D3(0, 1, 0) : D3(1, 0, 0);
    d3 T = dcross(N, a);
    T = dmul(T, 1.0 / sqrt(ddot(T, T)));
    d3 B = dcross(N, T);
    return dadd(dadd(dmul(T, r * cos(phi)), dmul(B, r * sin(phi))), dmul(N, sqrt(fmax(0.0, 1.0 - u1))));
}

/* direct light summed over the lights, per point, in double (k_build's formula) */
static void direct_d(const osc_scene* S, const ostate* st, double* out) {
    const int NL = S->NL;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < S->Np; ++i) {
        d3 P = dld(st->P, i), N = dld(st->N, i), O = dadd(P, dmul(N, 1e-3));
        double e = 0.0;
        for (int l = 0; l < NL; ++l) {
            d3 d = dsub(dld(S->L, l), P);
            double r = sqrt(ddot(d, d));
            d3 D = dmul(d, 1.0 / r);
            double c = ddot(N, D), t;
            int q;
            trace_d(S, st, O, D, &t, &q);
            if (!(t >= r - 1e-3)) continue;
            double rr = fmax(r, 0.05);
            e += (double)st->inten[l] * fmax(c, 0.0) / (rr * rr);
        }
        out[i] = e;
    }
}

int osc_path_trace(const osc_scene* S, int si, const int* pts, int npts, int paths, int min_bounces, uint64_t seed, double* mean,
                   double* sem) {
    if (si < 0 || si >= S->NS || paths < 2) return -1;
    const ostate* st = &S->st[si];
    double* dir = (double*)malloc(sizeof(double) * (size_t)S->Np);
    if (!dir) return -1;
    direct_d(S, st, dir);
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < npts; ++k) {
        const int i0 = pts[k];
        double s1 = 0.0, s2 = 0.0;
        for (int p = 0; p < paths; ++p) {
            uint64_t rs = mix64(seed ^ mix64(((uint64_t)(uint32_t)i0 << 32) | (uint32_t)p));
            int cur = i0;
            double beta = 1.0, val = 0.0;
            for (int b = 1; b <= 4096; ++b) {
                d3 P = dld(st->P, cur), N = dld(st->N, cur), O = dadd(P, dmul(N, 1e-3));
                double u1 = urand(&rs), u2 = urand(&rs);
                d3 D = cosine_d(N, u1, u2);
                double t;
                int q;
                if (!trace_d(S, st, O, D, &t, &q)) break;
                int j = resolve_d(S, st, dadd(O, dmul(D, t)), D, q);
                if (j < 0) break;
                const double A = S->A[j];
                beta *= A;
                val += beta * dir[j];
                if (b >= min_bounces) {
                    if (urand(&rs) >= A) break;
                    beta /= A;
                }
                cur = j;
            }
            s1 += val;
            s2 += val * val;
        }
        const double m = s1 / paths;
        mean[k] = m;
        sem[k] = sqrt(fmax(0.0, s2 / paths - m * m) / (paths - 1));
    }
    free(dir);
    return 0;
}

/* ------------------------------------------------------------------ taa mode
 * run_taa_mode (poc_gpu.cu:1175-1282) and its kernels k_taa_* (:1062-1166), sequentially:
 * region sums in point order, FP64 error sums in point order. */
struct osc_taa {
    osc_scene* S;
    float *x, *H, *H2, *mu, *sg, *rs, *cnt;
    int *nb, *react;
    uint8_t* pend;
    uint32_t *cur, *prev;
    int** V; int* nV;       /* event voxels per state pair */
    float alpha, gamma;
    int mask, f, prev_state, verify_left;
    uint32_t seed;
};

osc_taa* osc_taa_new(osc_scene* S) {
    if (S->fmt != 2 || !S->has_ref) return NULL;   /* the scene must have been built (osc_build) */
    osc_taa* t = (osc_taa*)calloc(1, sizeof(osc_taa));
    const size_t Np = (size_t)S->Np, NW = (size_t)S->NW;
    t->S = S;
    t->x = (float*)calloc(Np, 4); t->H = (float*)calloc(Np, 4); t->H2 = (float*)calloc(Np, 4);
    t->mu = (float*)calloc(Np, 4); t->sg = (float*)calloc(Np, 4);
    t->rs = (float*)calloc(3 * (size_t)S->NR, 4); t->cnt = (float*)calloc((size_t)S->NR, 4);
    t->nb = (int*)malloc(9 * Np * 4); t->react = (int*)calloc(Np, 4); t->pend = (uint8_t*)calloc(Np, 1);
    t->cur = (uint32_t*)calloc(NW * Np, 4); t->prev = (uint32_t*)calloc(NW * Np, 4);
    /* 3x3 neighbourhood on each quad's grid (poc_gpu.cu:1192-1203), state 0's grids */
    for (size_t k = 0; k < 9 * Np; ++k) t->nb[k] = -1;
    const ostate* s0 = &S->st[0];
    for (int q = 0; q < S->Nq; ++q) {
        int nu = s0->dims[2 * q], nv = s0->dims[2 * q + 1], o = s0->off[q];
        for (int iv = 0; iv < nv; ++iv)
            for (int iu = 0; iu < nu; ++iu) {
                size_t i = (size_t)o + (size_t)iv * nu + iu;
                int k = 0;
                for (int dv = -1; dv <= 1; ++dv)
                    for (int du = -1; du <= 1; ++du) {
                        int a = iu + du, b = iv + dv;
                        t->nb[9 * i + k++] = (a >= 0 && a < nu && b >= 0 && b < nv) ? o + b * nu + a : -1;
                    }
            }
    }
    /* event voxels: light voxels of changed intensities + occluders (poc_gpu.cu:1210-1219) */
    const int NS = S->NS, NL = S->NL;
    t->V = (int**)calloc((size_t)NS * NS, sizeof(int*));
    t->nV = (int*)calloc((size_t)NS * NS, sizeof(int));
    for (int a = 0; a < NS; ++a)
        for (int b = 0; b < NS; ++b) {
            if (a == b) continue;
            int fine[64], nf = 0;
            for (int l = 0; l < NL && nf < 64; ++l)
                if (S->st[a].inten[l] != S->st[b].inten[l]) {
                    const float* p = S->L + 3 * (size_t)l;
                    int i = imin(imax((int)(p[0] / 8.f * 16), 0), 15), j = imin(imax((int)(p[1] / 4.f * 8), 0), 7),
                        k = imin(imax((int)(p[2] / 3.f * 6), 0), 5);
                    fine[nf++] = (k * 8 + j) * 16 + i;
                }
            int ng = 0;
            int* g = to_grid(S, fine, nf, &ng);
            const int pe = a * NS + b, no = S->nev[pe * (1 + NL)];
            const int* occ = S->ev[pe * (1 + NL)];
            char* mark = (char*)calloc((size_t)S->NV, 1);
            for (int k = 0; k < ng; ++k) mark[g[k]] = 1;
            for (int k = 0; k < no; ++k) mark[occ[k]] = 1;
            free(g);
            int n = 0;
            for (int v = 0; v < S->NV; ++v) n += mark[v];
            t->V[pe] = (int*)malloc(sizeof(int) * (size_t)(n ? n : 1));
            n = 0;
            for (int v = 0; v < S->NV; ++v) if (mark[v]) t->V[pe][n++] = v;
            t->nV[pe] = n;
            free(mark);
        }
    return t;
}

void osc_taa_free(osc_taa* t) {
    if (!t) return;
    for (int e = 0; e < t->S->NS * t->S->NS; ++e) free(t->V[e]);
    free(t->V); free(t->nV);
    free(t->x); free(t->H); free(t->H2); free(t->mu); free(t->sg); free(t->rs); free(t->cnt);
    free(t->nb); free(t->react); free(t->pend); free(t->cur); free(t->prev);
    free(t);
}

void osc_taa_begin(osc_taa* t, float alpha, float gamma, int mask, int s0, uint32_t seed) {
    const size_t Np = (size_t)t->S->Np, NW = (size_t)t->S->NW;
    memcpy(t->H, t->S->st[s0].ref, Np * 4);
    memset(t->react, 0, Np * 4);
    memset(t->pend, 0, Np);
    memset(t->cur, 0, NW * Np * 4);
    memset(t->prev, 0, NW * Np * 4);
    t->alpha = alpha; t->gamma = gamma; t->mask = mask; t->seed = seed;
    t->f = 0; t->prev_state = s0; t->verify_left = 0;
}

/* k_taa_zone_acc + k_count_zone (poc_gpu.cu:1111-1118, 1129-1134) */
static void taa_zone_acc(osc_taa* t, int only_pending) {
    const osc_scene* S = t->S;
    for (int i = 0; i < S->Np; ++i) {
        if (only_pending && !t->pend[i]) continue;
        float d = t->x[i] - t->H[i];
        int r = S->region[i];
        t->rs[3 * r] += d; t->rs[3 * r + 1] += d * d; t->rs[3 * r + 2] += t->H[i];
        t->cnt[r] += 1.f;
    }
}
/* k_taa_zone_decide (poc_gpu.cu:1119-1128) */
static void taa_zone_decide(osc_taa* t, int only_pending, int rf, int clear_pending) {
    const osc_scene* S = t->S;
    for (int i = 0; i < S->Np; ++i) {
        if (only_pending && !t->pend[i]) continue;
        int r = S->region[i];
        float n = t->cnt[r];
        if (n >= 8.f) {
            float m = t->rs[3 * r] / n, se = sqrtf(fmaxf(t->rs[3 * r + 1] / n - m * m, 0.f) / n), base = t->rs[3 * r + 2] / n;
            if (fabsf(m) > 2.f * se && fabsf(m) > 0.05f * fmaxf(base, 1e-3f)) t->react[i] = rf;
        }
        if (clear_pending) t->pend[i] = 0;
    }
}

/* One frame of the loop of run_taa_mode (poc_gpu.cu:1246-1274). */
int osc_taa_frame(osc_taa* t, int si, double err3[3], float* err) {
    osc_scene* S = t->S;
    if (si < 0 || si >= S->NS) return -1;
    const int Np = S->Np, NW = S->NW, NL = S->NL, f = t->f, mask = t->mask, RF = 4;
    const float ALPHA_R = 0.5f;
    const ostate* st = &S->st[si];
    const int deps = mask == 2 || mask == 3;
    if (deps && f % 32 == 0) {
        uint32_t* x = t->cur; t->cur = t->prev; t->prev = x;
        memset(t->cur, 0, (size_t)NW * Np * 4);
    }
    /* k_taa_pt (poc_gpu.cu:1062-1098) */
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < Np; ++i) {
        uint32_t rs = hash32(t->seed * 0x9E3779B9u ^ hash32((uint32_t)f * 0x85EBCA6Bu ^ hash32((uint32_t)i + 7u)));
        v3 P = vld(st->P, i), N = vld(st->N, i), O = vadd(P, vmul(N, 1e-3f));
        float u1 = rnd(&rs);
        float u2 = rnd(&rs);
        v3 D = cosine_dir(N, u1, u2);
        float tt;
        int q, pi;
        int hit = trace_full(S, st, O, D, &tt, &q);
        v3 H = hit ? vadd(O, vmul(D, tt)) : O;
        int back = resolve_hit(S, st, hit, H, D, q, i, &pi);
        float v = 0.f;
        if (!back) {
            float ed = 0.f;
            for (int l = 0; l < NL; ++l) ed += st->Edir[(size_t)NL * pi + l];
            v = S->A[pi] * (ed + st->ref[pi]);
        }
        t->x[i] = v;
        if (deps) {
            uint32_t m[64];
            const uint32_t* sv = st->SV + (size_t)NW * (back ? i : pi);
            for (int w = 0; w < NW; ++w) m[w] = sv[w];
            dda(S, O, H, m);
            for (int w = 0; w < NW; ++w) t->cur[(size_t)w * Np + i] |= m[w];
        }
    }
    if (f > 0 && t->prev_state != si) {
        const int pe = t->prev_state * S->NS + si;
        if (mask == 2 || mask == 3) {   /* k_taa_touch (poc_gpu.cu:1136-1145) */
            for (int i = 0; i < Np; ++i) {
                int hitv = 0;
                for (int j = 0; j < t->nV[pe] && !hitv; ++j) {
                    int v = t->V[pe][j];
                    size_t o = (size_t)(v >> 5) * Np + i;
                    hitv = ((t->cur[o] | t->prev[o]) >> (v & 31)) & 1u;
                }
                if (!hitv) continue;
                if (mask == 3) t->pend[i] = 1;
                else t->react[i] = RF;
            }
            if (mask == 3) {
                t->verify_left = 2;
                memset(t->rs, 0, 12 * (size_t)S->NR);
                memset(t->cnt, 0, 4 * (size_t)S->NR);
            }
        }
        if (mask == 4) {   /* k_taa_oracle (poc_gpu.cu:1146-1150) */
            const float* ro = S->st[t->prev_state].ref;
            for (int i = 0; i < Np; ++i)
                if (fabsf(st->ref[i] - ro[i]) / (ro[i] + 1e-2f) > 0.10f) t->react[i] = RF;
        }
    }
    if (mask == 1) {
        memset(t->rs, 0, 12 * (size_t)S->NR);
        memset(t->cnt, 0, 4 * (size_t)S->NR);
        taa_zone_acc(t, 0);
        taa_zone_decide(t, 0, RF, 0);
    }
    if (mask == 3 && t->verify_left > 0) {
        taa_zone_acc(t, 1);
        if (--t->verify_left == 0) taa_zone_decide(t, 1, RF, 1);
    }
    /* k_taa_stats + k_taa_update (poc_gpu.cu:1100-1108, 1152-1159) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < Np; ++i) {
        float s1 = 0.f, s2 = 0.f;
        int n = 0;
        for (int k = 0; k < 9; ++k) {
            int j = t->nb[9 * (size_t)i + k];
            if (j < 0) continue;
            float v = t->x[j];
            s1 += v;
            s2 += v * v;
            n++;
        }
        float mu = s1 / (float)n;
        float sg = sqrtf(fmaxf(s2 / (float)n - mu * mu, 0.f));
        t->mu[i] = mu; t->sg[i] = sg;
        float h = t->H[i];
        if (t->gamma > 0.f) { float lo = mu - t->gamma * sg, hi = mu + t->gamma * sg; h = fminf(fmaxf(h, lo), hi); }
        float a = t->alpha, target = t->x[i];
        if (t->react[i] > 0) { a = ALPHA_R; t->react[i]--; target = mu; }
        t->H2[i] = h + a * (target - h);
    }
    { float* x = t->H; t->H = t->H2; t->H2 = x; }
    /* k_taa_err (poc_gpu.cu:1160-1166) */
    double d2 = 0, rsum = 0, c = 0;
    for (int i = 0; i < Np; ++i)
        if (st->valid[i]) { double e = t->H[i] - st->ref[i]; d2 += e * e; rsum += st->ref[i]; c += 1; }
    if (err3) { err3[0] = d2; err3[1] = rsum; err3[2] = c; }
    if (err) *err = (float)(sqrt(d2 / c) / (rsum / c));
    t->prev_state = si;
    t->f = f + 1;
    return 0;
}

/* 0 x, 1 H, 2 mu, 3 sg, 4 react, 5 pend, 6 cur, 7 prev */
void* osc_taa_array(osc_taa* t, int which, size_t* nbytes) {
    const size_t Np = (size_t)t->S->Np, NW = (size_t)t->S->NW;
    switch (which) {
        case 0: *nbytes = 4 * Np; return t->x;
        case 1: *nbytes = 4 * Np; return t->H;
        case 2: *nbytes = 4 * Np; return t->mu;
        case 3: *nbytes = 4 * Np; return t->sg;
        case 4: *nbytes = 4 * Np; return t->react;
        case 5: *nbytes = Np; return t->pend;
        case 6: *nbytes = 4 * NW * Np; return t->cur;
        case 7: *nbytes = 4 * NW * Np; return t->prev;
    }
    *nbytes = 0;
    return NULL;
}

/* ------------------------------------------------------------------ camera paths
 * The camera-path pass feeding the hash-grid cache (rc_hg_camera_paths; new, no reference),
 * in FP32 with this file's trace and hit resolution.  Per pixel: the primary ray through the
 * pixel centre, then `bounces` cosine bounces; one light sampled per vertex among the point
 * lights, the rectangle and the sun in proportion to its unshadowed contribution (the
 * rectangle's estimated at its centre with both cosines at least 0.1), its shadow ray traced;
 * radiance L_k = A_k (E_k + L_{k+1}) from the last surface vertex back.  Random numbers: the
 * frames' generator seeded per pixel. */
static inline float lumf(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

static float shadow_tf(const osc_scene* S, const ostate* st, v3 O, v3 D) {
    float t;
    int q;
    trace_full(S, st, O, D, &t, &q);
    return q == -1 ? INFINITY : t;
}

void osc_camera_paths(const osc_scene* S, int si, const osc_path_params* P, osc_path_vertex* vtx, float* pos, float* nrm, float* rgb,
                      int* len, float* img) {
    const ostate* st = &S->st[si];
    const int W = P->w, Hh = P->h, SL = P->bounces + 1, NL = S->NL;
    float an[3] = {0, 0, 0}, aarea = 0.f;
    const int area_on = P->area_rgb[0] > 0.f || P->area_rgb[1] > 0.f || P->area_rgb[2] > 0.f;
    const int sun_on = P->sun_rgb[0] > 0.f || P->sun_rgb[1] > 0.f || P->sun_rgb[2] > 0.f;
    if (area_on) {
        double n[3] = {(double)P->area_u[1] * P->area_v[2] - (double)P->area_u[2] * P->area_v[1],
                       (double)P->area_u[2] * P->area_v[0] - (double)P->area_u[0] * P->area_v[2],
                       (double)P->area_u[0] * P->area_v[1] - (double)P->area_u[1] * P->area_v[0]};
        double a = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int k = 0; k < 3; ++k) an[k] = (float)(n[k] / a);
        aarea = (float)a;
    }
    float sdir[3] = {0, 0, 0};
    if (sun_on) {
        double d[3] = {P->sun_dir[0], P->sun_dir[1], P->sun_dir[2]};
        double l = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int k = 0; k < 3; ++k) sdir[k] = (float)(d[k] / l);
    }
#pragma omp parallel for schedule(dynamic, 16)
    for (int y = 0; y < Hh; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t pix = (size_t)y * W + x, base = pix * SL;
            uint32_t rs = hash32(P->seed * 0x9E3779B9u ^ hash32(P->frame * 0x85EBCA6Bu ^ hash32((uint32_t)pix + 1u)));
            float sx = (((float)x + 0.5f) / (float)W * 2.f - 1.f) * P->tx, sy = (1.f - ((float)y + 0.5f) / (float)Hh * 2.f) * P->ty;
            v3 D = V(P->fwd[0] + P->right[0] * sx + P->up[0] * sy, P->fwd[1] + P->right[1] * sx + P->up[1] * sy,
                     P->fwd[2] + P->right[2] * sx + P->up[2] * sy);
            D = vmul(D, 1.f / sqrtf(vdot(D, D)));
            v3 O = V(P->eye[0], P->eye[1], P->eye[2]);
            float A[8], E[8][3];
            int n = 0, escaped = 0;
            for (int k = 0; k < SL; ++k) {
                float t;
                int q, pi;
                int hit = trace_full(S, st, O, D, &t, &q);
                v3 Hp = hit ? vadd(O, vmul(D, t)) : O;
                osc_path_vertex vx;
                memset(&vx, 0, sizeof vx);
                vx.origin[0] = O.x; vx.origin[1] = O.y; vx.origin[2] = O.z;
                vx.dir[0] = D.x; vx.dir[1] = D.y; vx.dir[2] = D.z;
                vx.light_index = -1;
                vx.entry = 0xFFFFFFFFu;
                if (!hit) {
                    vx.hit[0] = O.x; vx.hit[1] = O.y; vx.hit[2] = O.z;
                    vx.flags = 1u;
                    vtx[base + k] = vx;
                    escaped = 1;
                    n = k + 1;
                    break;
                }
                if (resolve_hit(S, st, hit, Hp, D, q, 0, &pi)) break;
                v3 nn;
                if (q >= 0) {
                    const float* Q = st->Q + 12 * (size_t)q;
                    nn = V(Q[9], Q[10], Q[11]);
                } else {
                    const float* n4 = S->STN + 4 * (size_t)(-2 - q);
                    nn = V(n4[0], n4[1], n4[2]);
                    if (vdot(nn, D) > 0.f) nn = vmul(nn, -1.f);
                }
                const float alb = S->A[pi];
                const v3 Os = vadd(Hp, vmul(nn, 1e-3f));
                float Wp = 0.f, wa = 0.f, ws = 0.f;
                for (int l = 0; l < NL; ++l) {
                    v3 d = vsub(V(P->lpos[l][0], P->lpos[l][1], P->lpos[l][2]), Hp);
                    float r = sqrtf(vdot(d, d)), rr = fmaxf(r, 0.05f);
                    Wp += P->lint[l] * lumf(P->lrgb[l][0], P->lrgb[l][1], P->lrgb[l][2]) * fmaxf(vdot(nn, d) / r, 0.f) / (rr * rr);
                }
                if (area_on) {
                    v3 C = V(P->area_corner[0] + 0.5f * (P->area_u[0] + P->area_v[0]), P->area_corner[1] + 0.5f * (P->area_u[1] + P->area_v[1]),
                             P->area_corner[2] + 0.5f * (P->area_u[2] + P->area_v[2]));
                    v3 d = vsub(C, Hp);
                    float r = sqrtf(vdot(d, d)), rr = fmaxf(r, 0.05f);
                    v3 w = vmul(d, 1.f / r);
                    wa = lumf(P->area_rgb[0], P->area_rgb[1], P->area_rgb[2]) * aarea * fmaxf(vdot(nn, w), 0.1f) *
                         fmaxf(-(an[0] * w.x + an[1] * w.y + an[2] * w.z), 0.1f) / (rr * rr);
                }
                if (sun_on) ws = lumf(P->sun_rgb[0], P->sun_rgb[1], P->sun_rgb[2]) * fmaxf(nn.x * sdir[0] + nn.y * sdir[1] + nn.z * sdir[2], 0.f);
                const float Wt = Wp + wa + ws;
                float e3[3] = {0.f, 0.f, 0.f};
                if (Wt > 0.f) {
                    const float u = rnd(&rs) * Wt;
                    if (u < Wp) {
                        int l;
                        float acc = 0.f, wl = 0.f, r = 0.f;
                        v3 d = V(0, 0, 0);
                        for (l = 0; l < NL; ++l) {
                            d = vsub(V(P->lpos[l][0], P->lpos[l][1], P->lpos[l][2]), Hp);
                            r = sqrtf(vdot(d, d));
                            float rr = fmaxf(r, 0.05f), cs = fmaxf(vdot(nn, d) / r, 0.f);
                            wl = P->lint[l] * lumf(P->lrgb[l][0], P->lrgb[l][1], P->lrgb[l][2]) * cs / (rr * rr);
                            acc += wl;
                            if (u < acc && wl > 0.f) break;
                        }
                        if (l > NL - 1) l = NL - 1;
                        v3 w = vmul(d, 1.f / r);
                        int vis = shadow_tf(S, st, Os, w) >= r - 1e-3f;
                        vx.to_light[0] = w.x; vx.to_light[1] = w.y; vx.to_light[2] = w.z;
                        vx.light_dist = r;
                        vx.light_index = l;
                        if (vis && wl > 0.f) {
                            vx.flags |= 2u;
                            float ln = lumf(P->lrgb[l][0], P->lrgb[l][1], P->lrgb[l][2]);
                            for (int ch = 0; ch < 3; ++ch) e3[ch] = Wt * P->lrgb[l][ch] / ln;
                        }
                    } else if (u < Wp + wa) {
                        float u1 = rnd(&rs);
                        float u2 = rnd(&rs);
                        v3 Y = V(P->area_corner[0] + u1 * P->area_u[0] + u2 * P->area_v[0], P->area_corner[1] + u1 * P->area_u[1] + u2 * P->area_v[1],
                                 P->area_corner[2] + u1 * P->area_u[2] + u2 * P->area_v[2]);
                        v3 d = vsub(Y, Hp);
                        float r = sqrtf(vdot(d, d)), rr = fmaxf(r, 0.05f);
                        v3 w = vmul(d, 1.f / r);
                        float cs = fmaxf(vdot(nn, w), 0.f), ca = fmaxf(-(an[0] * w.x + an[1] * w.y + an[2] * w.z), 0.f);
                        int vis = cs > 0.f && ca > 0.f && shadow_tf(S, st, Os, w) >= r - 1e-3f;
                        vx.to_light[0] = w.x; vx.to_light[1] = w.y; vx.to_light[2] = w.z;
                        vx.light_dist = r;
                        vx.light_index = NL;
                        if (vis) {
                            vx.flags |= 2u;
                            float geo = aarea * cs * ca / (rr * rr) * (Wt / wa);
                            for (int ch = 0; ch < 3; ++ch) e3[ch] = P->area_rgb[ch] * geo;
                        }
                    } else {
                        v3 w = V(sdir[0], sdir[1], sdir[2]);
                        int vis = shadow_tf(S, st, Os, w) == INFINITY;
                        vx.to_light[0] = w.x; vx.to_light[1] = w.y; vx.to_light[2] = w.z;
                        vx.light_dist = P->td;
                        vx.light_index = NL + 1;
                        if (vis) {
                            vx.flags |= 2u;
                            float ln = lumf(P->sun_rgb[0], P->sun_rgb[1], P->sun_rgb[2]);
                            for (int ch = 0; ch < 3; ++ch) e3[ch] = Wt * P->sun_rgb[ch] / ln;
                        }
                    }
                }
                vx.hit[0] = Hp.x; vx.hit[1] = Hp.y; vx.hit[2] = Hp.z;
                vtx[base + k] = vx;
                pos[3 * (base + k)] = Hp.x; pos[3 * (base + k) + 1] = Hp.y; pos[3 * (base + k) + 2] = Hp.z;
                nrm[3 * (base + k)] = nn.x; nrm[3 * (base + k) + 1] = nn.y; nrm[3 * (base + k) + 2] = nn.z;
                A[k] = alb;
                E[k][0] = e3[0]; E[k][1] = e3[1]; E[k][2] = e3[2];
                n = k + 1;
                float u1 = rnd(&rs);
                float u2 = rnd(&rs);
                O = Os;
                D = cosine_dir(nn, u1, u2);
            }
            const int nsurf = n - (escaped ? 1 : 0);
            for (int k = nsurf; k < SL; ++k)
                for (int ch = 0; ch < 3; ++ch) { rgb[3 * (base + k) + ch] = 0.f; nrm[3 * (base + k) + ch] = 0.f; pos[3 * (base + k) + ch] = 0.f; }
            float L[3] = {0.f, 0.f, 0.f};
            if (escaped) { L[0] = P->sky_rgb[0]; L[1] = P->sky_rgb[1]; L[2] = P->sky_rgb[2]; }
            for (int k = nsurf - 1; k >= 0; --k)
                for (int ch = 0; ch < 3; ++ch) { L[ch] = A[k] * (E[k][ch] + L[ch]); rgb[3 * (base + k) + ch] = L[ch]; }
            len[pix] = n;
            if (img)
                for (int ch = 0; ch < 3; ++ch) img[3 * pix + ch] = nsurf > 0 || escaped ? L[ch] : 0.f;
        }
}
