// Light buffer construction (light_buffer.cu): per point light, the spheres
// that can block a shadow ray in each direction cell around the light.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "wavefront.h"

namespace atx {

// Device bytes lb_build needs for nl lights.
uint64_t lb_bytes(uint32_t nl);

// Builds the light buffer of the n spheres sph (cx, cy, cz, r*r) with radii
// radius[] and the nl lights (1 <= nl <= kLbMaxLights, n <= kLbMaxSpheres)
// into buf (lb_bytes(nl) bytes of device memory) on stream; *out views buf.
cudaError_t lb_build(const float4* sph, const float* radius, uint32_t n, const DevLight* lights, uint32_t nl,
                     void* buf, uint64_t bytes, LightBufferView* out, cudaStream_t stream);

}  // namespace atx
