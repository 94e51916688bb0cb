/*
 * rc_mlp.h -- learned radiance cache on the fifth-generation tensor cores (sm_103a).
 *
 * New, no reference: falcon123212/render_engine's bench A calls the closed NRC library for
 * its learned cache; this is this repository's own network, trained online on the cache
 * points' radiance and queried like the hash-grid cache.  Every layer product is a tcgen05
 * MMA (bf16 operands in shared memory, FP32 accumulation in tensor memory).
 *
 * Device pointers are named d_*; calls run on the given stream and do not synchronise.
 */
#ifndef RC_MLP_H
#define RC_MLP_H

#include <stdint.h>

#include "rc_api.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One tensor-core tile product, the building block of every layer:
 * d_d[128 x N] (FP32, row-major) = d_a[128 x K] d_b[N x K]^T (bf16 bits, row-major),
 * K and N multiples of 16 in [16, 256].  *d_err |= 1 if the completion wait gave up. */
rc_status rc_mlp_tile_product(const uint16_t* d_a, const uint16_t* d_b, float* d_d, int K, int N, unsigned* d_err,
                              void* stream);

/* Health check of the bounded completion waits every kernel of this library uses (an mbarrier
 * polled at most a fixed number of times, then the error flag instead of a hang): one warp
 * waits on an mbarrier for at most `polls` polls; `arrive` = 1 makes one thread arrive on it
 * first (the wait must succeed), 0 leaves it without an arrival (the wait must give up).
 * *d_err |= 1 when the wait gave up.  polls in [1, 2^24]. */
rc_status rc_mlp_wait_check(uint32_t polls, int arrive, unsigned* d_err, void* stream);

/* The network: 168 input features -> 64 -> 64 -> 64 -> 64 -> n_out (<= 16), ReLU between
 * layers, no biases, bf16 weights and activations, FP32 accumulation, Adam (beta 0.9 / 0.99).
 * Inputs per point (float4 each): position (xyz), normal (xyz), and (albedo, direct light of
 * lights 0, 1, 2); the features are frequency and one-blob encodings of the position in the
 * box and of the normal, plus the raw values. */
typedef struct rc_mlp rc_mlp;

typedef struct {
    float box_lo[3], box_hi[3]; /* encoding box of the positions */
    int n_out;                  /* outputs, 1..16 */
    float lr;                   /* Adam learning rate */
    uint32_t seed;              /* initial weights */
    int max_batch;              /* largest training batch (samples) */
    int device;
    void* stream;               /* cudaStream_t, NULL = a stream of the network */
    float loss_scale;           /* initial loss scale, rounded down to a power of two; 0 = 1024 */
} rc_mlp_config;

rc_status rc_mlp_create(const rc_mlp_config* cfg, rc_mlp** out);
void rc_mlp_destroy(rc_mlp* m);
const char* rc_mlp_last_error(const rc_mlp* m);

/* One training step on n samples (a multiple of 128, at most max_batch): sample s is point
 * p = d_idx[s] (or s when d_idx is NULL) of d_pos4 / d_nrm4 / d_aux4, its target the first
 * n_out of the tstride floats at d_target + p * tstride (per-point arrays throughout).  Loss: relative L2,
 * (y - t)^2 / (y^2 + 0.01) averaged over samples and outputs; its sum is added to *d_loss
 * (when not NULL).  Gradients are summed over the batch in a fixed order.  A call whose
 * arguments (pointers, tstride, n) equal the previous call's is captured as a CUDA graph on the
 * network's stream and later calls with those arguments replay it (at most 16 graphs; none while
 * the stream is being captured by the caller): the same launches, fewer launch gaps. */
rc_status rc_mlp_train(rc_mlp* m, const float* d_pos4, const float* d_nrm4, const float* d_aux4, const float* d_target, int tstride,
                       const int* d_idx, int n, float* d_loss);

/* Loss scaling of the training steps: the output gradient is multiplied by a power-of-two
 * scale before the bf16 backward pass and divided out of the summed weight gradient before
 * Adam; a step whose gradient is not finite is skipped and the scale halved, and the scale
 * doubles after 1000 finite steps in a row (at most 65536).  The current scale, the steps
 * applied and the steps skipped (synchronises). */
rc_status rc_mlp_loss_scale(rc_mlp* m, float* scale, long long* steps, long long* skipped);

/* The network's n_out outputs for n points into d_out (ostride floats per point). */
rc_status rc_mlp_infer(rc_mlp* m, const float* d_pos4, const float* d_nrm4, const float* d_aux4, int n, float* d_out, int ostride);

/* FP32 master weights, 24,576 floats: per layer [out][in] row-major (176, 64, 64, 64, 64
 * inputs; 64, 64, 64, 64, 16 outputs); to_device = 1 sets them (and their bf16 copies).
 * Synchronises the stream. */
rc_status rc_mlp_weights(rc_mlp* m, float* host, size_t n, int to_device);

/* The summed gradient of the last training step, same layout.  Synchronises the stream. */
rc_status rc_mlp_gradients(rc_mlp* m, float* host, size_t n);

/* Bit 0: a completion wait gave up.  Synchronises the stream. */
rc_status rc_mlp_error_flags(rc_mlp* m, unsigned* flags);

#ifdef __cplusplus
}
#endif
#endif /* RC_MLP_H */
