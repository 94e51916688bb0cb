/*
 * rc_api.h -- C ABI of the GB300 radiance-cache frame loop.
 *
 * The reference (falcon123212/render_engine, bench B) is a single CUDA program,
 * cuda/poc_gpu.cu, with no library boundary: its "operators" are the structs DevState /
 * Cache / Params handed by value to the kernels (poc_gpu.cu:222-237, 394-422), the
 * scene loader load() (poc_gpu.cu:751-801), the frame driver Runner::run
 * (poc_gpu.cu:809-1017) and the method record Method (poc_gpu.cu:803-805).  Each entry
 * point below names the piece of that program it replaces.  Plain C types only: no CUDA
 * or torch types appear in a signature (a stream is passed as void*).
 *
 * Conventions
 *  - Every call returns RC_OK or an error status and never exits the process; the
 *    reference exits on any error (CK macro, poc_gpu.cu:44-45).  rc_last_error() gives
 *    the message of the last failing call on a context.
 *  - The context owns every device buffer.  One context is used by one host thread at a
 *    time.  Work is issued on the context's stream; calls that return data to the host
 *    synchronise that stream.
 *  - There is no CPU fallback: rc_create fails with RC_ERR_CUDA when no usable GPU is
 *    present.
 */
#ifndef RC_API_H
#define RC_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RC_ABI_VERSION 1

typedef struct rc_ctx rc_ctx;

typedef enum rc_status {
    RC_OK = 0,
    RC_ERR_ARG = 1,         /* bad argument (null pointer, index out of range, ...) */
    RC_ERR_IO = 2,          /* file cannot be read */
    RC_ERR_FORMAT = 3,      /* scene file malformed or truncated */
    RC_ERR_CUDA = 4,        /* CUDA runtime error (message in rc_last_error) */
    RC_ERR_NOMEM = 5,       /* device or host allocation failed */
    RC_ERR_STATE = 6,       /* call out of order (no scene, no run begun, ...) */
    RC_ERR_DEVICE = 7,      /* a device-side bound check or iteration limit tripped */
    RC_ERR_UNSUPPORTED = 8, /* configuration outside what this build supports */
    RC_ERR_LIGHTS = 9       /* scene light count differs from the expected count */
} rc_status;

/* Context configuration.  Zero-initialised fields take the defaults noted. */
typedef struct rc_config {
    int grid[3];        /* transit voxel grid VX,VY,VZ (product a multiple of 128);
                           default 8,4,4 = the -DGX=8 -DGY=4 -DGZ=4 of cuda/build.sh:12 */
    int device;         /* CUDA device ordinal (default 0) */
    void* stream;       /* cudaStream_t to issue on; NULL = the context creates its own */
    unsigned flags;     /* RC_FLAG_* */
    int expect_lights;  /* >0: scenes must have exactly this many lights, as the reference
                           binaries compiled with -DNLIGHTS=3/8 require (poc_gpu.cu:755) */
} rc_config;

#define RC_FLAG_BRUTE_FORCE 1u  /* test every dynamic triangle (no plane culling) */
#define RC_FLAG_CHECK_TRACE 2u  /* trace both ways and count disagreements (slow; tests) */
#define RC_FLAG_RAY_QUEUE 8u    /* static-mesh scenes: trace the rays traced ahead of the frame through a
                                   compacted ray queue served to persistent warps instead of one
                                   thread per point (same hits; slower at a few rays per point) */
#define RC_FLAG_LOAD_ASYNC 16u  /* rc_scene_load_memory returns once the scene's global arrays and
                                   state 0 are on the device and checked; the other states' arrays
                                   keep streaming from the caller's buffer on the context's second
                                   stream, so the buffer must stay valid and unchanged until
                                   rc_sync, the next load or rc_destroy */
#define RC_FLAG_WATERTIGHT 4u   /* static-mesh triangles by the watertight test (Woop, Benthin,
                                   Wald 2013) instead of the reference's Moller-Trumbore
                                   (poc_gpu.cu:318-331); hits differ from the reference's at
                                   edges.  Format 3 stores each triangle as v0 and two edge
                                   vectors, and the test rebuilds v1 = v0 + e1, v2 = v0 + e2 in
                                   FP32: no ray leaks through an edge when both triangles
                                   rebuild its endpoints to the same floats (meshes whose
                                   edge vectors are exact differences, e.g. on a lattice);
                                   elsewhere a leak through a gap of one rounding is possible */

/* Reference Method (poc_gpu.cu:803-805) plus the BENCH_RAYONS multiplier (poc_gpu.cu:69). */
typedef struct rc_method {
    int mode;           /* 0 fixed budget, 1 adaptive allocation */
    float nmax;
    float budget;
    int deps, verify, oracle, track_every, rescale, resp_mask;
    float nmax_resp;
    int ddgi;
    float ddgi_h, ddgi_thr;
    int ddgi_clamp;
    int memory, ramp, wake_verify, snaps, proj, snap_verify;
    float rays;         /* rays per point and frame (BENCH_RAYONS, default 1) */
} rc_method;

/* Reference Timers (poc_gpu.cu:807): milliseconds summed over frames / events. */
typedef struct rc_timers {
    double trace, decide, update, swap, event;
    int frames, events;
} rc_timers;

typedef struct rc_scene_info {
    int np, nq, nt, ns, nl, nr, has_ref, fmt, nw, nst, nnodes, hsize;
    double scene_bytes;  /* device bytes held by the scene */
    double cache_bytes;  /* device bytes held by the cache buffers */
} rc_scene_info;

typedef struct rc_device_info {
    char name[256];
    int sm_count, cc_major, cc_minor;
    double mem_used_mb, mem_total_mb;
} rc_device_info;

/* Counters of the current run (rc_run_stats_get). */
typedef struct rc_run_stats {
    long long frames;        /* frames run since rc_run_begin */
    long long rays;          /* rays traced since rc_run_begin (sum of per-point ray counts) */
    long long launches;      /* kernels launched by the context since it was created */
    int last_frame_kernels;  /* kernels launched by the last frame, event included */
    int last_frame_fused;    /* 1 when the last frame was the single fused trace+update kernel */
    int last_frame_event;    /* 1 when the last frame started with an event */
} rc_run_stats;

/* Pinhole camera of the image pass. */
typedef struct rc_camera {
    float eye[3], at[3], up[3];
    float fov_y_deg;     /* vertical field of view */
    int width, height;   /* pixels, e.g. 1920 x 1080 */
} rc_camera;

/* Per-ray record of rc_probe_rays. */
typedef struct rc_ray_rec {
    int point, ray;
    int q;       /* quad id (>=0), -2-j for static triangle j, -1 no hit */
    int pi;      /* cache point of the hit (the tracing point when the hit does not count) */
    int back;    /* 1 when the hit does not count (no hit, back face, cell absent) */
    float t;     /* hit distance (+inf when no hit) */
    float dir[3];  /* ray direction */
    float hit[3];  /* the end of the ray's dependency walk: origin + dir * t, the origin when no hit */
} rc_ray_rec;

/* Arrays of the run state (rc_array_*).  Layouts follow the reference Cache
 * (poc_gpu.cu:394-409): per-light arrays are point-major NL floats per point; masks are
 * word-major (word w of point i at w*Np+i). */
enum {
    RC_A_LC = 0, RC_A_LC2, RC_A_M, RC_A_N, RC_A_C0, RC_A_KK, RC_A_PENDING, RC_A_CUR, RC_A_PREV,
    RC_A_STALE, RC_A_AGE, RC_A_SNAP, RC_A_NEQ, RC_A_COEF, RC_A_RSTAT, RC_A_DSTAT, RC_A_SUMPR,
    RC_A_NPEND, RC_A_COUNT
};
/* Host scalars of the run (rc_scalar_*): Runner::run locals, poc_gpu.cu:839-850. */
enum { RC_S_PEND_LEFT = 0, RC_S_DORMANT, RC_S_PROJ_LEFT, RC_S_FRAME, RC_S_NSLOTS, RC_S_LAST_EVENT, RC_S_PROJK,
       RC_S_LAST_FRAME_KERNELS, RC_S_LAST_FRAME_FUSED, RC_S_COUNT };   /* the last two are read-only */
/* Per-state scene arrays (rc_state_array_copy): the k_build outputs and the references. */
enum { RC_SA_EDIR = 0, RC_SA_SV, RC_SA_REF, RC_SA_VALID, RC_SA_PW };

int rc_abi_version(void);
const char* rc_status_string(rc_status s);

/* Create / destroy a context (replaces the process-level setup of main(),
 * poc_gpu.cu:1286-1313).  Fails with RC_ERR_CUDA when no GPU is usable. */
rc_status rc_create(const rc_config* cfg, rc_ctx** out);
void rc_destroy(rc_ctx* ctx);
const char* rc_last_error(const rc_ctx* ctx);
/* GPU name and memory in use (the reference prints the name and cudaMemGetInfo deltas,
 * poc_gpu.cu:42, 1315-1323). */
rc_status rc_device_info_get(rc_ctx* ctx, rc_device_info* out);

/* Load a scene, formats 2 and 3, and build every state's direct light and shadow-voxel
 * masks on the GPU.  Replaces load() + k_build (poc_gpu.cu:751-801, 369-391).  The memory
 * variant takes the same bytes from a host buffer (page-locked memory is copied by DMA).
 * The call returns once the bytes are on the device and checked.  The states' builds run on a
 * second stream of the context: state 0's is issued by the load, and the first use of a state
 * issues the next state's, so a run moving through the states finds each one built; the
 * context's stream waits for a state's build where it first uses the state (no host
 * synchronisation), and builds the state itself if it was not issued.  rc_sync waits for
 * them too. */
rc_status rc_scene_load(rc_ctx* ctx, const char* path);
rc_status rc_scene_load_memory(rc_ctx* ctx, const void* data, size_t nbytes);
rc_status rc_scene_info_get(const rc_ctx* ctx, rc_scene_info* out);
/* Light intensities of a state (the per-state `in` block of the scene file, poc_gpu.cu:774). */
rc_status rc_state_lights(const rc_ctx* ctx, int state, float* inten, int nl);

/* Start a run: warm start and cache reset of Runner::run (poc_gpu.cu:826-850). */
rc_status rc_run_begin(rc_ctx* ctx, const rc_method* m, int first_state, uint32_t seed);
/* One frame in `state`: event handling when the state changed, then the frame kernels
 * (poc_gpu.cu:851-1011).  Asynchronous unless the method's projection solve falls on this
 * frame.  With want_err and a scene with references, the frame's error is recorded. */
rc_status rc_frame(rc_ctx* ctx, int state, int want_err);
/* Errors recorded so far in this run (synchronises). */
rc_status rc_errors(rc_ctx* ctx, float* out, int max, int* n);
/* Whole run over a state sequence (Runner::run, poc_gpu.cu:826-1016).  errs may be NULL;
 * when tm is given each frame is timed with events like the reference's timing mode
 * (one synchronisation per frame). */
rc_status rc_run(rc_ctx* ctx, const rc_method* m, const int* seq, int nframes, uint32_t seed,
                 int want_err, float* errs, rc_timers* tm);
rc_status rc_sync(rc_ctx* ctx);
/* Issue the build of every state of the loaded scene that is not built or issued yet, on the
 * context's second stream (the context's stream waits for each where it first uses the state).
 * No counterpart in the reference, whose load builds every state before returning: for a caller
 * that wants every state ready before a section whose frames must not share the GPU with a
 * build (rc_sync then waits for them). */
rc_status rc_scene_build_states(rc_ctx* ctx);

/* Image pass (no counterpart in the reference, whose bench B has no camera): one primary ray
 * per pixel through the geometry of `state`, shaded from the current cache with the light
 * every cache ray gathers, A * (direct + cached indirect).  Asynchronous when `image` is NULL
 * (the image stays in a buffer of the context); otherwise the image (width * height floats,
 * row-major, top row first) is copied to `image`. */
rc_status rc_render(rc_ctx* ctx, int state, const rc_camera* cam, float* image, size_t image_floats);

/* Run-state access for parity harnesses: size and device pointer of an array, and a copy
 * between the array and a host buffer of exactly `nbytes` (to_device=0: device to host,
 * to_device=1: host to device).  Arrays use the reference layouts listed above. */
rc_status rc_array_info(rc_ctx* ctx, int which, size_t* nbytes, void** dev_ptr);
rc_status rc_array_copy(rc_ctx* ctx, int which, void* host, size_t nbytes, int to_device);
rc_status rc_scalar_get(rc_ctx* ctx, int which, int* value);
rc_status rc_scalar_set(rc_ctx* ctx, int which, int value);
rc_status rc_state_array_copy(rc_ctx* ctx, int state, int which, void* host, size_t nbytes);

/* Trace the rays that the next frame would trace for the listed points, without changing
 * the run, and return one record per ray. */
rc_status rc_probe_rays(rc_ctx* ctx, int state, const int* points, int npoints,
                        rc_ray_rec* out, int maxrec, int* nrec);
/* Closest hit of caller-given rays against the geometry of state `state`: its dynamic
 * triangles first, then the static mesh, as the reference's trace_full (poc_gpu.cu:340-344).
 * rays: 6 floats per ray in host memory (origin, direction; the direction need not be unit
 * length).  prim[i] = quad id (>= 0), -2 - j for static triangle j, -1 for no hit; t[i] =
 * hit distance in units of the direction (+inf when no hit).  Follows the context's
 * RC_FLAG_WATERTIGHT and RC_FLAG_BRUTE_FORCE.  Synchronous; needs a scene, not a run. */
rc_status rc_trace_rays(rc_ctx* ctx, int state, const float* rays, int nrays, int* prim, float* t);
/* Disagreements counted by RC_FLAG_CHECK_TRACE since the last call (then reset). */
rc_status rc_trace_check_count(rc_ctx* ctx, long long* mismatches, long long* rays);
/* Run counters (synchronises to read the ray count). */
rc_status rc_run_stats_get(rc_ctx* ctx, rc_run_stats* out);
/* Device-side guard flags raised since the last call (then reset); 0 = none. */
rc_status rc_device_flags(rc_ctx* ctx, unsigned* flags);

/* Converged references of every state of the loaded scene, computed on the GPU the way the
 * reference's scene preparation does (prep_mesh.cuh:459-518, kernel k_ref :182-213): two
 * chains of stochastic Jacobi iterations of K rays per point, `warmup` iterations, then blocks
 * of `block` iterations averaged until the chains' relative difference is below noise_target
 * or max_iter iterations are averaged.  ref = the mean over lights of the chains' mean, Pw =
 * the per-light warm start, valid = fewer than 30 % of the rays hit within 0.02.  The scene
 * then has references (error sums, warm starts).  noise / iters (NS entries each, may be NULL)
 * receive the final noise and iteration count per state.  Synchronises. */
typedef struct {
    int K;               /* rays per point and iteration (32) */
    int warmup;          /* iterations before averaging (16) */
    int block;           /* iterations per block (64) */
    int max_iter;        /* most averaged iterations (2048) */
    double noise_target; /* relative noise between the two chains (0.03) */
} rc_ref_params;
rc_status rc_reference_build(rc_ctx* ctx, const rc_ref_params* prm, double* noise, int* iters);

/* Adjoint of the cache transport with respect to the lights' emission.  No counterpart in the
 * reference.  For state `state`, K rays per point are traced once and kept -- the rays of one
 * reference iteration with `seed` (prep_mesh.cuh:182-200) -- which fixes the linear transport
 * every frame and every reference iteration samples:
 *     L_l = T (E_l G_l + L_l),  T[i, j] = A_j / K x (rays of point i reaching point j),
 * G_l = the direct light of light l at unit emission (k_build, poc_gpu.cu:369-391).  For the
 * objective J = sum_i w_i sum_l L_l[i] (e.g. w = 1 / n on n sampled points), one adjoint solve
 * u = w + T^T u gives every light's derivative:  dJ/dE_l = sum_j (u_j - w_j) G_l[j].
 * Both solves run `iterations` Jacobi sweeps from zero (from w for u); sums over points are
 * FP64 in a fixed order, so results are reproducible.  `weights` (Np floats) and `dJ_dE`
 * (NL floats) are host buffers.  Synchronises. */
typedef struct {
    int state;          /* scene state whose transport is differentiated */
    int K;              /* frozen rays per point (1..1024, Np * K < 2^31) */
    uint32_t seed;      /* seed of the frozen rays */
    int iterations;     /* Jacobi sweeps of each solve (0 = 64) */
    const float* emission;  /* NL light emissions of the forward solve (host; NULL = the state's
                               intensities): its direct light is sum_l emission_l G_l.  The
                               derivatives do not depend on it (L is linear in E); J and L do */
} rc_adjoint_params;
typedef struct {
    double J;           /* w . L from the forward solve (L summed over lights) */
    double J_grad;      /* sum_l E_l dJ/dE_l: equal to J up to rounding, L being linear in E */
    double fwd_change;  /* last forward sweep: max |L_t - L_{t-1}| / max |L_t| */
    double adj_change;  /* last adjoint sweep: max |u_t - u_{t-1}| / max |u_t| */
    long long rays;     /* frozen rays, K * Np */
    long long back;     /* frozen rays that do not count (no hit, back face, cell absent) */
    int max_incoming;   /* most rays reaching one point */
} rc_adjoint_result;
rc_status rc_adjoint(rc_ctx* ctx, const rc_adjoint_params* prm, const float* weights, float* dJ_dE, rc_adjoint_result* res);
/* Arrays of the last rc_adjoint call (host buffers, any may be NULL): the forward solution L
 * (Np floats, summed over lights), the adjoint importance u (Np floats) and the frozen rays'
 * hit points (Np * K ints, ray r of point i at i * K + r, -1 = not counted).  Synchronises. */
rc_status rc_adjoint_arrays(rc_ctx* ctx, float* L, float* u, int* hits);

/* Screen-space temporal accumulator of the reference's `taa` mode (poc_gpu.cu:1047-1282): every
 * cache point is a pixel that gets one unbiased sample per frame (one cosine ray; radiance at
 * the hit = A x (direct + converged reference)), blended into a history with a 3x3
 * neighbourhood clamp; a reactive mask (history rejected for 4 frames, replaced by the
 * neighbourhood mean) comes from none, a blind per-zone test, the dependency masks, the
 * dependency masks verified over two frames, or the references (oracle).  Format-2 scenes with
 * references only, as in the reference.  The state is separate from rc_run_begin's. */
typedef struct {
    float alpha;        /* history blend (0.05 .. 0.2) */
    float gamma;        /* neighbourhood clamp in standard deviations (0 = none) */
    int mask;           /* 0 none, 1 blind zones, 2 dependencies, 3 dependencies verified, 4 oracle */
} rc_taa_method;
/* Start: history = the converged reference of first_state, masks and counters cleared;
 * `seed` is the per-run seed of the samples (the reference uses 5000 + seed index). */
rc_status rc_taa_begin(rc_ctx* ctx, const rc_taa_method* m, int first_state, uint32_t seed);
/* One frame in `state` (event handling when the state changed).  With err != NULL the frame's
 * error sqrt(sum (H - ref)^2 / n) / (sum ref / n) over valid points is returned (synchronises). */
rc_status rc_taa_frame(rc_ctx* ctx, int state, float* err);
/* TAA arrays (host copies, `nbytes` exactly the array's size; to_device = 1 writes the array):
 * per point x (float), H (float), mu, sg (float), react (int32), pend (uint8), and the
 * word-major dependency masks cur, prev (NW uint32 words per point, word w of point i at w*Np+i). */
enum { RC_T_X = 0, RC_T_H, RC_T_MU, RC_T_SG, RC_T_REACT, RC_T_PEND, RC_T_CUR, RC_T_PREV, RC_T_COUNT };
rc_status rc_taa_array_copy(rc_ctx* ctx, int which, void* host, size_t nbytes, int to_device);

/* Scene preparation on the GPU, in place of the reference's `prep` mode
 * (prep_mesh.cuh:303-531): an MSH1 mesh (triangles in metres, z up, albedo and a double-sided
 * flag per triangle) becomes a format-3 scene with converged references, written to
 * scene_path.  The static BVH is a linear BVH over Morton codes with SAH leaf collapse (leaves
 * of at most four triangles); cache points are cells of side h and one normal bucket, sampled
 * on the triangles, h scaled towards target_points; `lamps` point lights and a movable cube are
 * placed in free space found by probe rays; the five states follow the reference's state table
 * for mesh scenes (cuda/scenes/scenarios_publiques.txt: 0 lamps 0-1 on, cube at A; 1 lamp 0
 * off; 2 cube at B; 3 lamp 2 on too; 4 lamp 0 off, cube at B; lamps beyond the third always
 * on); each lamp's intensity gives it a mean direct light of 1 / lamps over the points of state
 * 0; references by rc_reference_build (environment variables PREP_BRUIT_CIBLE and
 * PREP_ITER_MAX as the reference reads them).  The context ends with the prepared scene loaded.
 * The report holds what the reference prints in its `{"type":"prep",...}` line. */
typedef struct {
    int target_points;   /* cache points aimed at (the cell count lands within 5 %) */
    int lamps;           /* point lights, 1..32 (the reference places 3) */
    uint32_t seed;       /* sampling and placement seed */
    int ref_iterations;  /* most reference iterations per state: 0 = the preparation's default
                            (2048, or PREP_ITER_MAX), < 0 = no references (a scene without them,
                            for timing) */
} rc_prep_params;
typedef struct {
    int triangles, np, zones, bvh_nodes, ns;
    float cell_m, diag_m, cube_m;
    double valid_fraction;   /* mean over states of the valid points' fraction */
    double noise[8];
    int iterations[8];
    int nl, bvh_depth;
    float lights[32][3];
    double seconds;
} rc_prep_report;
rc_status rc_prep_mesh_params(rc_ctx* ctx, const char* mesh_path, const char* scene_path, const rc_prep_params* params,
                              rc_prep_report* out);
/* The reference's `prep <mesh> <scene> [points]`: three lamps, seed 1. */
rc_status rc_prep_mesh(rc_ctx* ctx, const char* mesh_path, const char* scene_path, int target_points, rc_prep_report* out);

/* Error sums without any device allocation.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory themselves -- a renderer whose per-frame path
 * runs under a budget fixed at start-up (cudaMalloc / cudaFree synchronise the device and can
 * fail mid-frame), or a process whose own memory manager owns all device memory and passes
 * this library only buffers it already holds.  All pointers are device pointers owned by the
 * caller: the cache `lc` (`lc_stride` floats per point, the first `nl` used; lights whose bit
 * is set in `dormant` are left out, as in rc_frame's error), the reference `ref` and the
 * valid flags `valid` of `np` points.  Writes to `out3` (3 doubles, device memory) the FP64
 * sum of squared errors, the sum of the reference and the count of valid points -- the sums
 * rc_frame records when asked for the error -- on `stream` (NULL = the legacy default
 * stream), asynchronously.  Scratch space is a fixed array in the library (393,224 bytes on
 * every GPU that loads it, held until the process exits), so np may not exceed
 * RC_NOALLOC_MAX_POINTS (RC_ERR_ARG otherwise).  The first call on a device looks up that
 * array's address for the device and keeps it for the life of the process; make that first
 * call before any stream capture.  A cudaDeviceReset (or any teardown of the device's primary
 * context) unloads the array, and the kept address then points at freed memory: do not call
 * this entry point on a device after resetting it.  Every
 * call uses the same array: calls whose work overlaps on the GPU (on different streams, or
 * from different threads) race and give wrong sums.  Allocates nothing: no cudaMalloc,
 * no cudaFree, no allocating library routine. */
#define RC_NOALLOC_MAX_POINTS 4194304
rc_status rc_error_sums_noalloc(const float* lc, int lc_stride, int nl, int dormant, const float* ref,
                                const uint8_t* valid, int np, double* out3, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RC_API_H */
