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

#ifdef __cplusplus
}
#endif
#endif /* RC_MLP_H */
