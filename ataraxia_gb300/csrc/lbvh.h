// Device LBVH construction (lbvh.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "wavefront.h"

namespace atx {

// Device bytes lbvh_build needs for n spheres (tree, sorted leaves and sort scratch).
uint64_t lbvh_bytes(uint32_t n);

// Builds the tree over sph (cx, cy, cz, r*r) with radii radius[] into scratch
// (lbvh_bytes(n) bytes of device memory) on stream and fills *out with views
// into scratch.  n must be >= 1.
cudaError_t lbvh_build(const float4* sph, const float* radius, uint32_t n, uint32_t leaf_size, void* scratch,
                       uint64_t scratch_bytes, BvhView* out, cudaStream_t stream);

}  // namespace atx
