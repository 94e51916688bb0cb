// Device side of the taa mode (kernels in rc_taa.cu; the per-point sample is Ops<NL>::taa_sample).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace rc {
namespace taa {

int post_blocks(int Np);
cudaError_t touch(const uint32_t* cur, const uint32_t* prev, int Np, const int* V, int nv, int* react, uint8_t* pend, int rf, int to_pending,
                  cudaStream_t st);
cudaError_t oracle(const float* rold, const float* rnew, int Np, int* react, int rf, cudaStream_t st);
cudaError_t zone_acc(const float* x, const float* H, const uint8_t* pend, const int* region, int Np, float* rs, float* cnt, int only_pending,
                     cudaStream_t st);
cudaError_t zone_decide(const float* rs, const float* cnt, uint8_t* pend, const int* region, int Np, int* react, int only_pending, int rf,
                        int clear_pending, cudaStream_t st);
// statistics, update into H2 and (part != NULL) the error sums of H2 into out[3]; qid = the
// quad of each point (-1: none), quad[q] = (first point, nu, nv, 0)
cudaError_t post(const float* x, const int* qid, const int4* quad, const float* H, float* H2, float* mu, float* sg, int* react, int Np,
                 float alpha, float alpha_r, float gamma, const float* ref, const uint8_t* valid, double* part, double* out, cudaStream_t st);
// out[1] = the sum of the references over the valid points, out[2] = their count, in post's
// fixed order (out[0], the squared error, is post's).  They depend only on the state.
cudaError_t ref_sums(const float* ref, const uint8_t* valid, int Np, double* part, double* out, cudaStream_t st);

}  // namespace taa
}  // namespace rc
