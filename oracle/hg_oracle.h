/*
 * CPU oracle of the hash-grid cache with dependency masks (include/rc_hashgrid.h) — TEST
 * INFRASTRUCTURE ONLY.
 *
 * The dependency part restates falcon123212/render_engine's windows/patch/rtxgi_bench.patch
 * (the HLSL of bench A): DepMarkPoint :825-837, DepMarkSegment :839-858, DepOr :860-880,
 * the path loop's propagation :904-1006, the resolve-time invalidation :1028-1050, the bank
 * rotation :205-216, BenchObjVoxels :592-615 with the event mask of :370-383, and
 * BenchSnap.hlsl :1283-1345.  HLSL float expressions are evaluated in the order they are
 * written, without fused multiply-adds (the library is built with -ffp-contract=off), and
 * lerp(a, b, s) is a + s * (b - a), the HLSL definition.  The HLSL itself cannot run here
 * (it needs a D3D12 device), so parity with it is unpinned; the GPU kernels are checked
 * against this restatement bit for bit.
 *
 * The hash-grid part (insert, accumulate, resolve, eviction) has no reference (the patch
 * calls the SHaRC SDK, which is not in the reference checkout); this file states the
 * semantics the GPU kernels implement.  Only tests use this file.
 */
#ifndef HG_ORACLE_H
#define HG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    float zone_lo[3], zone_hi[3];
    float origin[3];
    float cell;
    uint32_t capacity;
    int max_depth;
    int acc_frames;
    int stale_frames;
    float tracing_distance;
} hgo_config;

typedef struct {
    float origin[3], dir[3], hit[3], to_light[3];
    float light_dist;
    int32_t light_index;
    uint32_t entry;
    uint32_t flags;
} hgo_vertex;

typedef struct {
    uint32_t index, sample_data, key[2], radiance[2];
} hgo_snap_rec;

/* Cache state: arrays of `capacity` entries, laid out as on the device. */
typedef struct {
    uint64_t* keys;
    uint32_t* accum;     /* 4 per entry */
    uint32_t* resolved;  /* 4 per entry */
    uint32_t* bank0;     /* 4 per entry */
    uint32_t* bank1;
    int bank;            /* bank being filled */
} hgo_state;

void hgo_mark_point(const hgo_config* c, uint32_t m[3], const float p[3]);
void hgo_mark_segment(const hgo_config* c, uint32_t m[3], const float a[3], const float b[3]);
void hgo_dep_or(hgo_state* s, uint32_t entry, const uint32_t m[4]);
void hgo_mark_paths(const hgo_config* c, hgo_state* s, const hgo_vertex* v, const int* path_start, int npaths);
void hgo_begin_frame(const hgo_config* c, hgo_state* s, uint32_t dep_frame, uint32_t period);
void hgo_resolve(const hgo_config* c, hgo_state* s, const uint32_t inv[4], uint32_t counts[3]);
void hgo_event_mask(const hgo_config* c, const float* la, const float* lb, int nlights, int sky_a, int sky_b,
                    const float* obj_a, const float* obj_b, uint32_t inv[4]);
uint64_t hgo_key(const hgo_config* c, const float p[3], const float n[3]);
void hgo_insert(const hgo_config* c, hgo_state* s, const float* pos, const float* nrm, int n, uint32_t* entry);
void hgo_accumulate(hgo_state* s, const uint32_t* entry, const float* rgb, int n);
uint32_t hgo_snapshot(const hgo_config* c, const hgo_state* s, hgo_snap_rec* recs, uint32_t cap);
void hgo_restore(hgo_state* s, const hgo_snap_rec* recs, uint32_t count);
void hgo_voxels_mark(const hgo_config* c, int res, uint64_t* vox, const hgo_vertex* v, const int* len, int stride, int npaths);
uint16_t hgo_f2h(float f);
float hgo_h2f(uint16_t h);

#ifdef __cplusplus
}
#endif
#endif
