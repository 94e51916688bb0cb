/*
 * CPU oracle of the hash-grid cache with dependency masks — TEST INFRASTRUCTURE ONLY.
 * See hg_oracle.h for what each function restates.
 */
#include "hg_oracle.h"

#include <math.h>
#include <string.h>

#define ZX 6
#define ZY 4
#define ZZ 4
#define SKY 0x80000000u
#define INVALID 0xFFFFFFFFu
#define MAXD 8
#define TOMB 0xFFFFFFFFFFFFFFFFull /* evicted entry: probing goes on past it */

static inline float fminf_(float a, float b) { return a < b ? a : b; }
static inline float fmaxf_(float a, float b) { return a > b ? a : b; }

/* rtxgi_bench.patch:825-837 DepMarkPoint */
void hgo_mark_point(const hgo_config* c, uint32_t m[3], const float p[3]) {
    const float G[3] = {ZX, ZY, ZZ};
    float cc[3];
    for (int k = 0; k < 3; ++k) cc[k] = (p[k] - c->zone_lo[k]) / (c->zone_hi[k] - c->zone_lo[k]) * G[k];
    for (int k = 0; k < 3; ++k)
        if (cc[k] < 0.0f || cc[k] >= G[k]) return;
    uint32_t v[3];
    for (int k = 0; k < 3; ++k) v[k] = (uint32_t)cc[k];
    const uint32_t b = v[0] + ZX * (v[1] + ZY * v[2]);
    const uint32_t bit = 1u << (b & 31u);
    if (b < 32u) m[0] |= bit;
    else if (b < 64u) m[1] |= bit;
    else m[2] |= bit;
}

/* rtxgi_bench.patch:839-858 DepMarkSegment: the segment clipped to the zone box, sampled every
 * half of the smallest zone edge (at most 49 points). */
void hgo_mark_segment(const hgo_config* c, uint32_t m[3], const float a[3], const float b[3]) {
    const float* lo = c->zone_lo;
    const float* hi = c->zone_hi;
    float d[3], sd[3], tn[3], tf[3];
    for (int k = 0; k < 3; ++k) {
        d[k] = b[k] - a[k];
        sd[k] = fabsf(d[k]) > 1e-7f ? d[k] : 1e-7f;
        const float t0 = (lo[k] - a[k]) / sd[k];
        const float t1 = (hi[k] - a[k]) / sd[k];
        tn[k] = fminf_(t0, t1);
        tf[k] = fmaxf_(t0, t1);
    }
    const float tmin = fmaxf_(fmaxf_(tn[0], tn[1]), fmaxf_(tn[2], 0.0f));
    const float tmax = fminf_(fminf_(tf[0], tf[1]), fminf_(tf[2], 1.0f));
    if (tmin > tmax) return;
    float cell[3];
    const float G[3] = {ZX, ZY, ZZ};
    for (int k = 0; k < 3; ++k) cell[k] = (hi[k] - lo[k]) / G[k];
    const float dd = d[0] * d[0] + d[1] * d[1];
    const float len = sqrtf(dd + d[2] * d[2]) * (tmax - tmin);
    const float q = ceilf(len / (0.5f * fminf_(cell[0], fminf_(cell[1], cell[2]))));
    /* min(uint(q) + 1, 48), with the conversion saturating */
    const uint32_t n = q >= 47.0f ? 48u : (uint32_t)q + 1u;
    for (uint32_t i = 0; i <= n; ++i) {
        const float s = (float)i / (float)n;
        const float t = tmin + s * (tmax - tmin);
        float p[3];
        for (int k = 0; k < 3; ++k) p[k] = a[k] + d[k] * t;
        hgo_mark_point(c, m, p);
    }
}

static uint32_t* bank_of(hgo_state* s, int b) { return b == 0 ? s->bank0 : s->bank1; }

/* rtxgi_bench.patch:860-880 DepOr */
void hgo_dep_or(hgo_state* s, uint32_t entry, const uint32_t m[4]) {
    if (entry == INVALID || (m[0] | m[1] | m[2] | m[3]) == 0) return;
    uint32_t* bk = bank_of(s, s->bank) + 4 * (size_t)entry;
    for (int k = 0; k < 4; ++k) bk[k] |= m[k];
}

/* rtxgi_bench.patch:904-1006: the dependency part of the path loop, one path after another. */
void hgo_mark_paths(const hgo_config* c, hgo_state* s, const hgo_vertex* v, const int* path_start, int npaths) {
    const int D = c->max_depth < 1 ? 1 : (c->max_depth > MAXD ? MAXD : c->max_depth);
    for (int p = 0; p < npaths; ++p) {
        uint32_t idx[MAXD];
        int len = 0;
        for (int j = path_start[p]; j < path_start[p + 1]; ++j) {
            const hgo_vertex* x = &v[j];
            if (x->flags & 1u) {
                uint32_t sm[3] = {0, 0, 0};
                float e[3];
                for (int k = 0; k < 3; ++k) e[k] = x->origin[k] + x->dir[k] * c->tracing_distance;
                hgo_mark_segment(c, sm, x->origin, e);
                const uint32_t dm[4] = {sm[0], sm[1], sm[2], SKY};
                for (int di = 0; di < len; ++di) hgo_dep_or(s, idx[di], dm);
                break;
            }
            uint32_t din[3] = {0, 0, 0}, dloc[3] = {0, 0, 0}, lights = 0;
            hgo_mark_segment(c, din, x->origin, x->hit);
            hgo_mark_point(c, dloc, x->hit);
            if (x->light_index >= 0) {
                const float r = fminf_(x->light_dist, c->tracing_distance);
                float e[3];
                for (int k = 0; k < 3; ++k) e[k] = x->hit[k] + x->to_light[k] * r;
                hgo_mark_segment(c, dloc, x->hit, e);
                if (x->flags & 2u) lights |= 1u << (x->light_index < 30 ? x->light_index : 30);
            }
            const int prev = len;
            for (int k = (len < D ? len : D - 1); k > 0; --k) idx[k] = idx[k - 1];
            idx[0] = x->entry;
            len = len + 1 < D ? len + 1 : D;
            const uint32_t cur[4] = {dloc[0], dloc[1], dloc[2], lights};
            uint32_t prv[4] = {dloc[0] | din[0], dloc[1] | din[1], dloc[2] | din[2], lights};
            const int stop = (x->flags & 4u) != 0;
            if (stop && x->entry != INVALID)
                for (int k = 0; k < 4; ++k) prv[k] |= s->bank0[4 * (size_t)x->entry + k] | s->bank1[4 * (size_t)x->entry + k];
            hgo_dep_or(s, idx[0], cur);
            const int last = prev < D - 1 ? prev : D - 1;
            for (int di = 1; di <= last; ++di) hgo_dep_or(s, idx[di], prv);
            if (stop) break;
        }
    }
}

/* rtxgi_bench.patch:205-216 */
void hgo_begin_frame(const hgo_config* c, hgo_state* s, uint32_t dep_frame, uint32_t period) {
    const uint32_t P = period > 0 ? period : 16u;
    if (dep_frame % P == 0) {
        s->bank = (int)((dep_frame / P) % 2);
        memset(bank_of(s, s->bank), 0, 16 * (size_t)c->capacity);
    }
}

uint16_t hgo_f2h(float f) {
    uint32_t x;
    memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7FFFFFFFu;
    if (ax > 0x7F800000u) return (uint16_t)(sign | 0x7FFFu);
    if (ax >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u); /* rounds to infinity */
    uint32_t v, sh;
    if (ax >= 0x38800000u) { /* normal half: 13 mantissa bits dropped */
        v = ((ax >> 23) - 112u) << 23 | (ax & 0x7FFFFFu);
        sh = 13;
    } else {
        if (ax < 0x33000000u) return (uint16_t)sign; /* at most half the smallest subnormal */
        const uint32_t e = ax >> 23;
        v = (ax & 0x7FFFFFu) | 0x800000u;
        sh = 126u - e;
    }
    uint32_t r = v >> sh;
    const uint32_t rem = v & ((1u << sh) - 1u), halfu = 1u << (sh - 1u);
    if (rem > halfu || (rem == halfu && (r & 1u))) ++r;
    return (uint16_t)(sign | r);
}

float hgo_h2f(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 31u, m = h & 1023u;
    uint32_t x;
    if (e == 0) {
        if (m == 0) x = sign;
        else {
            float f = (float)m * 5.9604644775390625e-8f; /* 2^-24 */
            memcpy(&x, &f, 4);
            x |= sign;
        }
    } else if (e == 31) x = sign | 0x7F800000u | (m << 13);
    else x = sign | ((e + 112u) << 23) | (m << 13);
    float f;
    memcpy(&f, &x, 4);
    return f;
}

/* rtxgi_bench.patch:1028-1050 (invalidation, eviction clears the masks) around the cache's own
 * resolve (no reference; see hg_oracle.h). */
void hgo_resolve(const hgo_config* c, hgo_state* s, const uint32_t inv[4], uint32_t counts[3]) {
    const int any_inv = (inv[0] | inv[1] | inv[2] | inv[3]) != 0;
    counts[0] = counts[1] = counts[2] = 0;
    for (uint32_t e = 0; e < c->capacity; ++e) {
        if (s->keys[e] == 0 || s->keys[e] == TOMB) continue;   /* empty or evicted: holds no data */
        uint32_t* a = s->accum + 4 * (size_t)e;
        uint32_t* r = s->resolved + 4 * (size_t)e;
        uint32_t* b0 = s->bank0 + 4 * (size_t)e;
        uint32_t* b1 = s->bank1 + 4 * (size_t)e;
        uint32_t dep[4], meet = 0, all0 = 1;
        for (int k = 0; k < 4; ++k) {
            dep[k] = b0[k] | b1[k];
            meet |= dep[k] & inv[k];
            if (dep[k]) all0 = 0;
        }
        if (any_inv && (all0 || meet)) {
            memset(a, 0, 16);
            memset(r, 0, 16);
            if (s->keys[e] != 0 && s->keys[e] != TOMB) counts[0]++;
        }
        if (s->keys[e] != 0 && s->keys[e] != TOMB) {
            const uint32_t nold = r[2] & 0xFFFFu;
            uint32_t stale = r[2] >> 16;
            if (a[3] > 0) {
                const float sc = 0.0009765625f;
                float mean[3];
                const uint32_t n = nold + a[3];
                for (int k = 0; k < 3; ++k) {
                    const uint16_t h = (uint16_t)(k == 0 ? (r[0] & 0xFFFFu) : (k == 1 ? (r[0] >> 16) : (r[1] & 0xFFFFu)));
                    float sum = hgo_h2f(h) * (float)nold;
                    sum = sum + (float)a[k] * sc;
                    mean[k] = sum / (float)n;
                }
                const uint32_t nn = n < (uint32_t)c->acc_frames ? n : (uint32_t)c->acc_frames;
                r[0] = (uint32_t)hgo_f2h(mean[0]) | (uint32_t)hgo_f2h(mean[1]) << 16;
                r[1] = (uint32_t)hgo_f2h(mean[2]) | (uint32_t)hgo_f2h((float)nn) << 16;
                r[2] = nn;
                r[3] = 0;
            } else {
                stale++;
                if (stale > (uint32_t)c->stale_frames) {
                    s->keys[e] = TOMB;
                    memset(r, 0, 16);
                    counts[1]++;
                } else {
                    r[2] = nold | stale << 16;
                }
            }
            memset(a, 0, 16);
        }
        if (s->keys[e] == 0 || s->keys[e] == TOMB) {
            memset(b0, 0, 16);
            memset(b1, 0, 16);
        } else if ((r[1] >> 16) != 0) {
            counts[2]++;
        }
    }
}

/* rtxgi_bench.patch:592-615 BenchObjVoxels: zones overlapped by an object grown by 0.25 */
static void obj_zones(const hgo_config* c, const float* obj, uint32_t inv[4]) {
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
                int overlap = 1;
                for (int k = 0; k < 3; ++k) {
                    const float cs = (c->zone_hi[k] - c->zone_lo[k]) / (float)G[k];
                    const float c0 = c->zone_lo[k] + cs * (float)v[k], c1 = c0 + cs;
                    if (hi[k] < c0 || lo[k] > c1) overlap = 0;
                }
                if (overlap) {
                    const int b = x + G[0] * (y + G[1] * z);
                    inv[b / 32] |= 1u << (b % 32);
                }
            }
}

/* rtxgi_bench.patch:370-383 */
void hgo_event_mask(const hgo_config* c, const float* la, const float* lb, int nlights, int sky_a, int sky_b,
                    const float* obj_a, const float* obj_b, uint32_t inv[4]) {
    inv[0] = inv[1] = inv[2] = inv[3] = 0;
    for (int i = 0; i < nlights && i < 31; ++i)
        if (la[i] != lb[i]) inv[3] |= 1u << i;
    if (sky_a != sky_b) inv[3] |= SKY;
    int moved = 0;
    if ((obj_a == NULL) != (obj_b == NULL)) moved = 1;
    else if (obj_a && obj_b)
        for (int k = 0; k < 6; ++k)
            if (obj_a[k] != obj_b[k]) moved = 1;
    if (moved) {
        if (obj_a) obj_zones(c, obj_a, inv);
        if (obj_b) obj_zones(c, obj_b, inv);
    }
}

/* The reference's own cache-point hash (poc_gpu.cu:251-262), reused for the entries. */
static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull; x ^= x >> 27; x *= 0x94d049bb133111ebull; x ^= x >> 31;
    return x;
}
static inline int normal_bucket(float nx, float ny, float nz) {
    float ax = fabsf(nx), ay = fabsf(ny), az = fabsf(nz);
    if (ax >= ay && ax >= az) return nx > 0.f ? 0 : 1;
    if (ay >= az) return ny > 0.f ? 2 : 3;
    return nz > 0.f ? 4 : 5;
}
static inline uint64_t cell_key(int cx, int cy, int cz, int b) {
    uint64_t k = (uint64_t)(cx & 0xFFFFF);
    k = (k << 20) | (uint64_t)(cy & 0xFFFFF);
    k = (k << 20) | (uint64_t)(cz & 0xFFFFF);
    return ((k << 3) | (uint64_t)b) + 1ull;
}

uint64_t hgo_key(const hgo_config* c, const float p[3], const float n[3]) {
    const float ih = 1.f / c->cell;
    const int cx = (int)floorf((p[0] - c->origin[0]) * ih);
    const int cy = (int)floorf((p[1] - c->origin[1]) * ih);
    const int cz = (int)floorf((p[2] - c->origin[2]) * ih);
    return cell_key(cx, cy, cz, normal_bucket(n[0], n[1], n[2]));
}

/* Insertion in point order: linear probing from mix64(key) over at most 64 slots; an evicted
 * slot (TOMB) does not end the probe, and a missing key takes the first evicted slot seen, else
 * the empty slot that ended the probe. */
void hgo_insert(const hgo_config* c, hgo_state* s, const float* pos, const float* nrm, int n, uint32_t* entry) {
    const uint32_t mask = c->capacity - 1u;
    for (int i = 0; i < n; ++i) {
        entry[i] = INVALID;
        const float* nn = nrm + 3 * (size_t)i;
        if (nn[0] == 0.f && nn[1] == 0.f && nn[2] == 0.f) continue;   /* no surface point: no entry */
        const uint64_t key = hgo_key(c, pos + 3 * (size_t)i, nn);
        uint32_t h = (uint32_t)mix64(key) & mask, tomb = INVALID;
        for (int probe = 0; probe < 64; ++probe) {
            const uint64_t k = s->keys[h];
            if (k == key) { entry[i] = h; break; }
            if (k == TOMB) {
                if (tomb == INVALID) tomb = h;
            } else if (k == 0) {
                const uint32_t slot = tomb != INVALID ? tomb : h;
                s->keys[slot] = key;
                entry[i] = slot;
                break;
            }
            h = (h + 1u) & mask;
        }
        if (entry[i] == INVALID && tomb != INVALID) { s->keys[tomb] = key; entry[i] = tomb; }
    }
}

static uint32_t to_fixed(float x) {
    float y = x * 1024.f;
    if (!(y > 0.f)) return 0u;
    if (y > 2147483648.f) y = 2147483648.f;
    return (uint32_t)nearbyintf(y);
}

void hgo_accumulate(hgo_state* s, const uint32_t* entry, const float* rgb, int n) {
    for (int i = 0; i < n; ++i) {
        if (entry[i] == INVALID) continue;
        uint32_t* a = s->accum + 4 * (size_t)entry[i];
        for (int k = 0; k < 3; ++k) a[k] += to_fixed(rgb[3 * (size_t)i + k]);
        a[3] += 1u;
    }
}

/* BenchSnap.hlsl (rtxgi_bench.patch:1283-1345): valid = key set and a nonzero fp16 count */
uint32_t hgo_snapshot(const hgo_config* c, const hgo_state* s, hgo_snap_rec* recs, uint32_t cap) {
    uint32_t n = 0;
    for (uint32_t e = 0; e < c->capacity; ++e) {
        const uint32_t* r = s->resolved + 4 * (size_t)e;
        if (s->keys[e] == 0 || s->keys[e] == TOMB || (r[1] >> 16) == 0) continue;
        if (n < cap) {
            recs[n].index = e;
            recs[n].sample_data = r[2];
            recs[n].key[0] = (uint32_t)s->keys[e];
            recs[n].key[1] = (uint32_t)(s->keys[e] >> 32);
            recs[n].radiance[0] = r[0];
            recs[n].radiance[1] = r[1];
        }
        ++n;
    }
    return n;
}

void hgo_restore(hgo_state* s, const hgo_snap_rec* recs, uint32_t count) {
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t e = recs[i].index;
        s->keys[e] = (uint64_t)recs[i].key[0] | (uint64_t)recs[i].key[1] << 32;
        uint32_t* r = s->resolved + 4 * (size_t)e;
        r[0] = recs[i].radiance[0];
        r[1] = recs[i].radiance[1];
        r[2] = recs[i].sample_data & 0xFFFFu;
        r[3] = 0;
    }
}

/* Per-voxel light masks (rc_hg_voxels_mark): voxel of a point per axis
 * min(max(int((x - lo) * scale), 0), res - 1) with scale = res / (hi - lo) in float; for each
 * vertex whose sampled light l < 64 was visible, bit l in the voxels of 20 samples
 * h + (to_light * min(dist, td)) * k / 19. */
static int hgo_vox_axis(float x, float lo, float scale, int res) {
    int i = (int)((x - lo) * scale);
    return i < 0 ? 0 : (i > res - 1 ? res - 1 : i);
}
void hgo_voxels_mark(const hgo_config* c, int res, uint64_t* vox, const hgo_vertex* v, const int* len, int stride, int npaths) {
    for (int p = 0; p < npaths; ++p)
        for (int j = 0; j < len[p]; ++j) {
            const hgo_vertex* x = &v[(size_t)p * stride + j];
            if ((x->flags & 1u) || x->light_index < 0 || x->light_index >= 64 || !(x->flags & 2u)) continue;
            const uint64_t bit = 1ull << x->light_index;
            const float r = x->light_dist < c->tracing_distance ? x->light_dist : c->tracing_distance;
            float d[3];
            for (int k = 0; k < 3; ++k) d[k] = x->to_light[k] * r;
            float sc[3];
            for (int k = 0; k < 3; ++k) sc[k] = (float)res / (c->zone_hi[k] - c->zone_lo[k]);
            for (int k = 0; k < 20; ++k) {
                const float t = (float)k / 19.f;
                const int ix = hgo_vox_axis(x->hit[0] + d[0] * t, c->zone_lo[0], sc[0], res);
                const int iy = hgo_vox_axis(x->hit[1] + d[1] * t, c->zone_lo[1], sc[1], res);
                const int iz = hgo_vox_axis(x->hit[2] + d[2] * t, c->zone_lo[2], sc[2], res);
                vox[((size_t)iz * res + iy) * res + ix] |= bit;
            }
        }
}
