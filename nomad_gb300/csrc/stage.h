// stage.h -- host-to-device copies of the caller's pageable arrays through pinned
// staging buffers (host_stage.cpp).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace nomad {

// Host-to-device copy of pageable memory through two pinned staging buffers kept for the
// life of the process (32 MB each, allocated on first use; uploads are serialised by a
// lock): host threads fill one while the copy engine drains the other.  Returns when the
// copies are done.  Copies straight from pageable memory ran ~30x slower when the host
// had been under heavy allocation beforehand.
cudaError_t upload_staged(void* dst, const void* src, size_t bytes, cudaStream_t s);
// The same for `count` host arrays copied one after another into dst.
cudaError_t upload_staged_many(void* dst, const void* const* srcs, const size_t* bytes, size_t count,
                               cudaStream_t s);
// The same for `count` arrays of doubles (counts[i] values each), narrowed to floats (round
// to nearest, as a static_cast) while they are staged: half the bytes cross to the device.
cudaError_t upload_staged_narrow(float* dst, const double* const* srcs, const size_t* counts, size_t count,
                                 cudaStream_t s);

}  // namespace nomad
