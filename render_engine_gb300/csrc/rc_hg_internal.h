// Library-internal access to a hash-grid cache (for passes of the frame runtime that feed it).
#pragma once

#include <cuda_runtime.h>

#include "../../include/rc_hashgrid.h"

namespace rc {
cudaStream_t hg_stream(rc_hg* hg);   // the stream the cache's work is issued on
const rc_hg_config& hg_config(const rc_hg* hg);
bool hg_has_voxels(const rc_hg* hg);
// v[i].entry = entry[i], on the cache's stream
cudaError_t hg_set_entries(rc_hg* hg, rc_hg_vertex* v, const uint32_t* entry, long long n);
}  // namespace rc
