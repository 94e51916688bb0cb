/*
 * rc_hashgrid.h -- GPU hash-grid radiance cache with per-entry dependency masks.
 *
 * Two parts of falcon123212/render_engine's bench A (the SHaRC path tracer patched by
 * windows/patch/rtxgi_bench.patch) on CUDA, behind a plain C ABI (no CUDA or torch types):
 *
 *  1. Dependency tracking and targeted invalidation, restated from the patch's HLSL:
 *     - zone marking of points and segments on a 6 x 4 x 4 grid over a box (96 bits) plus 32
 *       light bits, bit 31 = sky (DepMarkPoint / DepMarkSegment, rtxgi_bench.patch:825-859);
 *     - OR of a vertex's mask into the entries of its path, in the bank being filled
 *       (DepOr, :861-880), with the propagation rules of the path loop (:904-1006):
 *       a miss marks the escaping segment and the sky, a hit marks its incoming segment, its
 *       point, its shadow segment and its visible light, earlier vertices inherit, and a
 *       vertex answered from the cache passes on that entry's masks;
 *     - two banks of masks, the one being filled cleared every `period` frames
 *       (:205-216);
 *     - invalidation at resolve: an entry whose masks are empty or meet the event's mask is
 *       zeroed, an evicted entry's masks are cleared (SharcResolve.hlsl part, :1028-1050);
 *     - the event mask: changed lights, sky, and the zones a moved object overlaps with a
 *       0.25 margin (BenchObjVoxels, :592-615 and :370-383);
 *     - compact snapshots of the valid entries, 24-byte records, and their restore
 *       (BenchSnap.hlsl, :1283-1345).
 *  2. The hash-grid cache those masks belong to.  The reference calls the SHaRC SDK (v1.6.5,
 *     not part of the reference checkout) for it, so this part has no reference to follow:
 *     entries are keyed like the reference's own cache-point hash (cell of size `cell` from
 *     `origin`, normal bucket; poc_gpu.cu:251-287), inserted by atomic compare-and-swap with
 *     linear probing, fed by integer atomics (order-free, so reproducible), and resolved
 *     into 4 x fp16 radiance + sample count with an accumulation cap and eviction by age.
 *
 * Every call returns rc_status (include/rc_api.h).  Pointers named d_* are device pointers;
 * everything runs on the stream given in rc_hg_config and returns without synchronising
 * unless stated.
 */
#ifndef RC_HASHGRID_H
#define RC_HASHGRID_H

#include <stddef.h>
#include <stdint.h>

#include "rc_api.h"

#ifdef __cplusplus
extern "C" {
#endif

#define RC_HG_INVALID 0xFFFFFFFFu      /* no entry (HASH_GRID_INVALID_CACHE_INDEX) */
#define RC_HG_ZONES_X 6                /* DEP_GX, DEP_GY, DEP_GZ of the patch */
#define RC_HG_ZONES_Y 4
#define RC_HG_ZONES_Z 4
#define RC_HG_SKY_BIT 0x80000000u      /* bit 31 of the light word */
#define RC_HG_MAX_DEPTH 8              /* longest path suffix a vertex propagates to */
#define RC_HG_EVICTED 0xFFFFFFFFFFFFFFFFull /* key of an evicted entry: probes go on past it */

typedef struct rc_hg rc_hg;

typedef struct {
    float zone_lo[3], zone_hi[3]; /* box of the dependency zones (benchGridMin / benchGridMax) */
    float origin[3];              /* hash grid origin */
    float cell;                   /* hash cell edge */
    uint32_t capacity;            /* entries, a power of two */
    int max_depth;                /* path vertices kept for propagation, 1..RC_HG_MAX_DEPTH */
    int acc_frames;               /* sample count cap of a resolved entry */
    int stale_frames;             /* frames without samples before an entry is evicted */
    float tracing_distance;       /* TRACING_DISTANCE: length of escaping and shadow segments */
    int device;
    void* stream;                 /* cudaStream_t, NULL = a stream of the context */
} rc_hg_config;

/* One bounce of a path, as the path loop sees it (rtxgi_bench.patch:540-750). */
typedef struct {
    float origin[3];       /* ray origin of this bounce */
    float dir[3];          /* ray direction (a miss marks origin -> origin + dir * tracing_distance) */
    float hit[3];          /* hit position */
    float to_light[3];     /* direction to the sampled light */
    float light_dist;      /* distance to the sampled light */
    int32_t light_index;   /* sampled light (SampleLightRIS), -1 = none */
    uint32_t entry;        /* cache entry of the hit, RC_HG_INVALID = none */
    uint32_t flags;        /* RC_HG_MISS, RC_HG_LIGHT_VISIBLE, RC_HG_STOP */
} rc_hg_vertex;
#define RC_HG_MISS 1u          /* the ray escaped: sky */
#define RC_HG_LIGHT_VISIBLE 2u /* the shadow ray reached the sampled light */
#define RC_HG_STOP 4u          /* the path ends here on a cached answer (SharcUpdateHit false) */

/* Snapshot record (BenchSnap.hlsl SnapRec, 24 bytes). */
typedef struct {
    uint32_t index;        /* entry */
    uint32_t sample_data;  /* resolved word z: sample count (low 16), frames since update (high 16) */
    uint32_t key[2];       /* hash key */
    uint32_t radiance[2];  /* 4 x fp16: r, g, b, sample count */
} rc_hg_snap_rec;

/* Device arrays of the cache, for rc_hg_array. */
enum {
    RC_HG_A_KEYS = 0,  /* uint64 per entry, 0 = empty, RC_HG_EVICTED = evicted */
    RC_HG_A_ACCUM,     /* uint32 x 4: r, g, b in 1/1024 units, sample count */
    RC_HG_A_RESOLVED,  /* uint32 x 4: half2(r, g), half2(b, count), sample data, 0 */
    RC_HG_A_BANK0,     /* uint32 x 4 dependency masks */
    RC_HG_A_BANK1,
    RC_HG_A_COUNT
};

rc_status rc_hg_create(const rc_hg_config* cfg, rc_hg** out);
void rc_hg_destroy(rc_hg* hg);
const char* rc_hg_last_error(const rc_hg* hg);

/* Device pointer and size in bytes of one array (RC_HG_A_*). */
rc_status rc_hg_array(rc_hg* hg, int which, void** d_ptr, size_t* bytes);

/* Copy one whole array between the device and host memory (to_device = 1: host -> device);
 * synchronises the stream.  For harnesses and tests. */
rc_status rc_hg_array_copy(rc_hg* hg, int which, void* host, size_t bytes, int to_device);

/* Empty the cache: keys, accumulation, resolved radiance and both banks (sharcEnableClear). */
rc_status rc_hg_clear(rc_hg* hg);

/* Entries of n surface points (d_pos, d_nrm: 3 floats each), inserted when missing (linear
 * probing over at most 64 slots; a missing key takes the first evicted slot it passed, else
 * the empty slot that ended the probe); d_entry[i] = RC_HG_INVALID when there was none, and
 * for a point whose normal is (0, 0, 0) (no surface: nothing is inserted). */
rc_status rc_hg_insert(rc_hg* hg, const float* d_pos, const float* d_nrm, int n, uint32_t* d_entry);

/* Add n radiance samples (d_rgb: 3 floats each) to their entries. */
rc_status rc_hg_accumulate(rc_hg* hg, const uint32_t* d_entry, const float* d_rgb, int n);

/* Frame start of the dependency banks (rtxgi_bench.patch:205-216): every `period` frames
 * (0 = 16) the bank (dep_frame / period) % 2 becomes the one filled and is cleared. */
rc_status rc_hg_begin_frame(rc_hg* hg, uint32_t dep_frame, uint32_t period);

/* Dependency marking of npaths paths; path p is d_vertices[d_path_start[p] ..
 * d_path_start[p + 1]) (npaths + 1 offsets). */
rc_status rc_hg_mark_paths(rc_hg* hg, const rc_hg_vertex* d_vertices, const int* d_path_start, int npaths);

/* The same for paths in fixed slots: path p is d_vertices[p * stride .. p * stride + d_len[p]). */
rc_status rc_hg_mark_paths_strided(rc_hg* hg, const rc_hg_vertex* d_vertices, const int* d_len, int stride, int npaths);

/* Per-voxel light masks (new, no reference): a res^3 grid (res <= 256) over the zone box,
 * 64 bits per voxel; bit l of a voxel is set when a shadow ray toward light l crossed it.  Where
 * the 96 zones of the entry masks say which region a path crossed, these say which lights'
 * visibility a change in a region can alter, at up to 256^3 resolution: an occluder event's
 * light bits are the OR of the voxel masks under the object (rc_hg_voxels_box_lights).
 * init (re)allocates and clears; clear empties the masks (e.g. every bank period). */
rc_status rc_hg_voxels_init(rc_hg* hg, int res);
rc_status rc_hg_voxels_clear(rc_hg* hg);
/* For every vertex whose sampled light l < 64 was visible: bit l in the voxels of 20 evenly
 * spaced samples of its shadow segment (the hit to the light, at most tracing_distance), as
 * k_build rasterises its shadow rays (poc_gpu.cu:192-197).  Voxel of a point per axis:
 * min(max(int((x - zone_lo) * scale), 0), res - 1), scale = res / (zone_hi - zone_lo) in float. */
rc_status rc_hg_voxels_mark(rc_hg* hg, const rc_hg_vertex* d_vertices, const int* d_len, int stride, int npaths);
/* OR of the masks of the voxels a box [lo, hi] overlaps (host arrays; synchronises). */
rc_status rc_hg_voxels_box_lights(rc_hg* hg, const float lo[3], const float hi[3], uint64_t* lights);
/* All res^3 masks to host memory, voxel (x, y, z) at (z * res + y) * res + x (synchronises). */
rc_status rc_hg_voxels_copy(rc_hg* hg, uint64_t* host, size_t count);

/* Camera paths over a loaded scene feeding the cache (new, no reference: bench B has no
 * camera, bench A's path tracer is HLSL).  One path per pixel of `cam` through the geometry
 * of `state` of the context's scene: a primary ray and `bounces` cosine-sampled bounces; a
 * back face, a surface without cache point or an escaping ray ends the path.  At every vertex
 * one light is sampled among the scene's point lights (intensity of the state x light_rgb),
 * the rectangle light and the sun, with probability proportional to its unshadowed
 * contribution, and its shadow ray traced; the vertex's radiance sample is
 * L_k = A_k (E_k + L_{k+1}) in RGB (A: the albedo of the hit's cache point, E: the sampled
 * direct light over its probability, L after the last vertex: sky_rgb for an escaping ray,
 * 0 otherwise), the convention of the reference's gather A (Edir + Lc), poc_gpu.cu:472-478.
 * Every vertex is inserted and its sample accumulated; the paths' dependency masks are marked
 * (rc_hg_mark_paths_strided: light index NL = the rectangle, NL + 1 = the sun) and, after
 * rc_hg_voxels_init, the per-voxel light masks.  d_image (may be NULL): width x height RGB
 * floats, the primary vertices' L_0.  Runs on the cache's stream after the context's work. */
typedef struct {
    rc_camera cam;
    int bounces;               /* 0 .. RC_HG_MAX_DEPTH - 1 */
    uint32_t seed, frame;
    float light_rgb[32][3];    /* colour of each point light (all zero = white) */
    float area_corner[3], area_u[3], area_v[3], area_rgb[3];   /* one-sided rectangle light facing u x v; rgb 0 = none */
    float sun_dir[3], sun_rgb[3];  /* direction towards the sun, irradiance; rgb 0 = none */
    float sky_rgb[3];          /* radiance of escaping rays */
} rc_hg_path_params;
rc_status rc_hg_camera_paths(rc_hg* hg, rc_ctx* ctx, int state, const rc_hg_path_params* prm, float* d_image);
/* Device arrays of the last camera pass, per slot (pixel p, vertex k at p * (bounces + 1) + k):
 * vertices (rc_hg_vertex), radiance samples (3 floats), entries (uint32) and per pixel the
 * path length (int); for harnesses.  Pointers stay valid until the next pass. */
rc_status rc_hg_camera_arrays(rc_ctx* ctx, const rc_hg_vertex** d_vertices, const float** d_rgb, const uint32_t** d_entry,
                              const int** d_len, int* stride, int* npaths);

/* Resolve every entry: invalidation by inv[4] (zones x, y, z, lights; all zero = none),
 * accumulation into the resolved radiance, eviction of entries stale for more than
 * stale_frames, and clearing of the masks of empty entries.  d_counts (may be NULL):
 * uint32 x 3 = keyed entries invalidated, entries evicted, valid entries after. */
rc_status rc_hg_resolve(rc_hg* hg, const uint32_t inv[4], uint32_t* d_counts);

/* The event mask between two bench states (host only, no device work):
 * lights whose intensity differs (bit i, i < 31), the sky, and the zones overlapped by a
 * moved object in either state (obj_*: centre xyz + full size xyz; NULL = no object). */
void rc_hg_event_mask(const rc_hg_config* cfg, const float* lights_a, const float* lights_b, int nlights, int sky_a,
                      int sky_b, const float* obj_a, const float* obj_b, uint32_t inv[4]);

/* Compact the valid entries (key set and a nonzero fp16 sample count) into d_recs, in entry
 * order; *count (host) receives how many there are, records past `cap` are not written.
 * Synchronises the stream. */
rc_status rc_hg_snapshot(rc_hg* hg, rc_hg_snap_rec* d_recs, uint32_t cap, uint32_t* count);

/* Write count snapshot records back (keys and resolved radiance; frames since update reset). */
rc_status rc_hg_restore(rc_hg* hg, const rc_hg_snap_rec* d_recs, uint32_t count);

#ifdef __cplusplus
}
#endif
#endif /* RC_HASHGRID_H */
