// Device side of rc_adjoint (kernels in rc_adjoint.cu): buffers and launch sequence.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace rc {
namespace adj {

constexpr int GRAD_BLOCKS = 512;   // fixed partial-sum count of the gradient reduction
constexpr int MAX_COLS = 40;       // lights + 1 reduced columns

struct Stats {
    double out[MAX_COLS];          // dJ/dE_l for l < NL, then J = w . L
    unsigned long long back;       // frozen rays that do not count
    unsigned chg[4];               // last sweep: max |dL|, max |L|, max |du|, max |u| (float bits)
    int max_incoming;              // most rays reaching one point
    int pad;
};

struct Bufs {
    int* hits;        // Np * K: hit point of ray r of point i at i * K + r, -1 = not counted
    int* cnt;         // Np + 1 (the last stays 0)
    int* off;         // Np + 1: start of each point's incoming rays, off[Np] = counted rays
    int* fill;        // Np
    int* unordered;   // Np * K
    int* src;         // Np * K: source point of each incoming ray, rays of a point in ray order
    int* scratch;     // scan_scratch_ints(Np + 1)
    float2* da;       // Np: (direct light summed over lights, albedo)
    float* L[2];      // forward iterates (total radiance per point)
    float* g[2];      // gathered values A_j (d_j + L_j) of the forward iterates
    float* u[2];      // adjoint iterates (importance per point)
    const float* L_final;   // the iterate holding the forward solution (set by solve)
    const float* u_final;   // the iterate holding the adjoint solution (set by solve)
    float* w;         // Np weights
    double* part;     // GRAD_BLOCKS * (NL + 1)
    Stats* stats;
};

size_t scan_scratch_ints(long long n);
// transposed ray lists from b.hits (also clears b.stats)
cudaError_t build_transpose(const Bufs& b, int Np, int K, cudaStream_t st);
// `iters` forward and adjoint Jacobi sweeps from L = 0, u = w, then the gradient against the
// unit-emission direct light AEu (same gather-record layout as AE, `aes` floats per point)
cudaError_t solve(Bufs* b, int Np, int K, int NL, int aes, const float* AE, const float* AEu, const float* em, int iters,
                  cudaStream_t st);

}  // namespace adj
}  // namespace rc
