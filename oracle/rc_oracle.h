/*
 * CPU oracle for the radiance-cache frame loop — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's bench-B hot path (cuda/poc_gpu.cu of
 * falcon123212/render_engine): scene loading (formats 2 and 3), the per-state build
 * of direct light and shadow-voxel masks, the per-frame trace / decide / update
 * kernels, the event handling of Runner::run and the error metric.  Every function
 * cites the reference file:line it follows.  Floating-point work is FP32 in the same
 * operation order as the reference; FP64 only where the reference uses double
 * (k_error sums, the projection solve).
 *
 * Only the test suite, the smoke check and the CPU-baseline leg of the benchmark use
 * this library.  It is never linked into the product library.
 */
#ifndef RC_ORACLE_H
#define RC_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct osc_scene osc_scene;
typedef struct osc_run osc_run;

/* Same field list as rc_method in include/rc_api.h (reference Method, poc_gpu.cu:803-805). */
typedef struct {
    int mode;          /* 0 = fixed budget, 1 = adaptive allocation */
    float nmax;        /* history cap in frames (scaled by rays) */
    float budget;      /* rays per point per frame in mode 0 */
    int deps;          /* dependency tracking */
    int verify;        /* occluder events -> verification */
    int oracle;        /* reference-driven invalidation (upper bound) */
    int track_every;   /* track dependencies one frame in N */
    int rescale;       /* per-light storage + linear rescale on intensity change */
    int resp_mask;     /* SHaRC responsive lights (bit l) */
    float nmax_resp;
    int ddgi;
    float ddgi_h, ddgi_thr;
    int ddgi_clamp;
    int memory, ramp, wake_verify, snaps, proj, snap_verify;
    float rays;        /* BENCH_RAYONS multiplier */
} osc_method;

/* Load a scene file (formats 2 and 3), transit grid vx*vy*vz (multiple of 128 voxels). */
osc_scene* osc_load_file(const char* path, int vx, int vy, int vz, char* err, int errlen);
osc_scene* osc_load_mem(const void* buf, size_t n, int vx, int vy, int vz, char* err, int errlen);
void osc_free(osc_scene* s);
/* Np, Nq, Nt, NS, NL, NR, has_ref, fmt, NW, nst */
void osc_info(const osc_scene* s, int out[10]);
/* k_build for every state (direct light + static shadow-voxel masks). */
void osc_build(osc_scene* s);
/* Host arrays of a state: 0 Edir (float NL*Np), 1 SV (u32 NW*Np), 2 ref, 3 valid, 4 Pw. */
void* osc_state_array(osc_scene* s, int state, int which, size_t* nbytes);
/* Transit-grid voxel list of an event (pair e -> s): kind 0 = occluder list, 1.. = light l-1. */
const int* osc_event_list(const osc_scene* s, int pair, int kind, int* n);

osc_run* osc_run_new(osc_scene* s);
void osc_run_free(osc_run* r);
void osc_run_begin(osc_run* r, const osc_method* m, int s0, uint32_t seed);
/* One frame in state si (events handled when si differs from the previous frame's state).
 * When want_err and the scene has references, err3 receives the three FP64 sums. */
int osc_frame(osc_run* r, int si, int want_err, double err3[3], float* err);
/* Run arrays (see OSC_A_*). */
void* osc_run_array(osc_run* r, int which, size_t* nbytes);
/* Scalars: 0 pend_left, 1 dormant, 2 proj_left, 3 frame, 4 nslots, 5 last_event_f, 6 projK */
int osc_run_scalar(osc_run* r, int which);
void osc_run_set_scalar(osc_run* r, int which, int value);
void osc_set_threads(int n);

/* One-frame trace probe: rays of the listed points for (state, seed, frame) with the
 * current run state, writing per ray {point, ray, q, pi, back, t} records. */
typedef struct { int point, ray, q, pi, back; float t; } osc_ray_rec;
int osc_probe_rays(osc_run* r, int si, const int* pts, int npts, osc_ray_rec* out, int maxrec);

/* Closest hit of caller-given rays (6 floats each: origin, direction) against state si:
 * dynamic triangles, then the static mesh (Moller-Trumbore as the reference, or the watertight
 * test when watertight != 0).  prim = quad id, -2 - static triangle or -1; t = +inf when none. */
int osc_trace_rays(const osc_scene* s, int si, const float* rays, int n, int watertight, int* prim, float* t);

/* Image pass (pinhole camera, one ray per pixel), see rc_render in include/rc_api.h. */
int osc_render(osc_run* r, int si, const float* eye, const float* fwd, const float* right, const float* up, float tx, float ty,
               int w, int h, float* out);

/* Adjoint support: the K rays of one reference iteration with `seed` (prep_mesh.cuh:182-200)
 * kept per point, hits[i * K + r] = cache point reached or -1 (the FP32 trace of the frames). */
void osc_frozen_hits(const osc_scene* s, int si, uint32_t seed, int K, int* hits);
/* Direct light of every light at unit emission, out[i * NL + l] (FP32, k_build's formula). */
void osc_direct_unit(const osc_scene* s, int si, float* out);
/* FP64 path tracer: per listed point, the mean over `paths` random walks of the cache transport
 * (summed over lights) and its standard error; 0 = ok. */
int osc_path_trace(const osc_scene* s, int si, const int* pts, int npts, int paths, int min_bounces, uint64_t seed, double* mean,
                   double* sem);

/* Camera paths feeding the hash-grid cache (rc_hg_camera_paths in include/rc_hashgrid.h). */
typedef struct {
    float eye[3], fwd[3], right[3], up[3], tx, ty;   /* camera frame as rc_render derives it */
    int w, h, bounces;
    uint32_t seed, frame;
    float td;                                        /* tracing distance (sun shadow segments) */
    float lpos[32][3], lrgb[32][3], lint[32];        /* point lights: position, colour, intensity */
    float area_corner[3], area_u[3], area_v[3], area_rgb[3];
    float sun_dir[3], sun_rgb[3], sky_rgb[3];
} osc_path_params;
typedef struct {   /* the layout of rc_hg_vertex */
    float origin[3], dir[3], hit[3], to_light[3];
    float light_dist;
    int32_t light_index;
    uint32_t entry, flags;
} osc_path_vertex;
void osc_camera_paths(const osc_scene* s, int si, const osc_path_params* p, osc_path_vertex* vtx, float* pos, float* nrm, float* rgb,
                      int* len, float* img);

/* taa mode (run_taa_mode, poc_gpu.cu:1175-1282): format-2 scenes with references. */
typedef struct osc_taa osc_taa;
osc_taa* osc_taa_new(osc_scene* s);
void osc_taa_free(osc_taa* t);
void osc_taa_begin(osc_taa* t, float alpha, float gamma, int mask, int s0, uint32_t seed);
int osc_taa_frame(osc_taa* t, int si, double err3[3], float* err);
/* 0 x, 1 H, 2 mu, 3 sg, 4 react, 5 pend, 6 cur, 7 prev (host memory of the oracle) */
void* osc_taa_array(osc_taa* t, int which, size_t* nbytes);

enum {
    OSC_A_LC = 0, OSC_A_LC2, OSC_A_M, OSC_A_N, OSC_A_C0, OSC_A_KK, OSC_A_PENDING, OSC_A_CUR, OSC_A_PREV,
    OSC_A_STALE, OSC_A_AGE, OSC_A_SNAP, OSC_A_NEQ, OSC_A_COEF, OSC_A_RSTAT, OSC_A_DSTAT, OSC_A_SUMPR,
    OSC_A_NPEND, OSC_A_COUNT
};

#ifdef __cplusplus
}
#endif
#endif
