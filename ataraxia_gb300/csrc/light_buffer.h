// Light buffer and direction buffer construction (light_buffer.cu): per point
// light, the spheres that can block a shadow ray in each direction cell
// around the light; per sphere, the spheres a ray leaving it can hit in each
// direction cell.
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

// Device bytes db_build needs for n spheres.
uint64_t db_bytes(uint32_t n);

// Builds the direction buffer of the n spheres sph (cx, cy, cz, r*r) with
// radii radius[] (1 <= n <= kDbMaxSpheres) into buf (db_bytes(n) bytes of
// device memory) on stream; *out views buf.
cudaError_t db_build(const float4* sph, const float* radius, uint32_t n, void* buf, uint64_t bytes,
                     DirBufferView* out, cudaStream_t stream);

}  // namespace atx
