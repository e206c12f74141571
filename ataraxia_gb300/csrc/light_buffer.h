// Light buffer and direction buffer construction (light_buffer.cu): per point
// light, the spheres that can block a shadow ray in each direction cell
// around the light; per sphere, the spheres a ray leaving it can hit in each
// direction cell.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "wavefront.h"

namespace atx {

// Device bytes lb_build needs for nl lights at res cells along a face's edge.
uint64_t lb_bytes(uint32_t nl, uint32_t res);

// Builds the light buffer of the n spheres sph (cx, cy, cz, r*r) with radii
// radius[] and the nl lights (1 <= nl <= kLbMaxLights, n <= kLbMaxSpheres),
// res cells along a face's edge (kCellResMin..kCellResMax), into buf
// (lb_bytes(nl, res) bytes of device memory) on stream; *out views buf.
cudaError_t lb_build(const float4* sph, const float* radius, uint32_t n, const DevLight* lights, uint32_t nl,
                     uint32_t res, void* buf, uint64_t bytes, LightBufferView* out, cudaStream_t stream);

// Device bytes db_build needs for n spheres at res cells along a face's edge.
uint64_t db_bytes(uint32_t n, uint32_t res);

// Builds the direction buffer of the n spheres sph (cx, cy, cz, r*r) with
// radii radius[] (1 <= n <= kDbMaxSpheres), res cells along a face's edge,
// into buf (db_bytes(n, res) bytes of device memory) on stream; *out views
// buf.
cudaError_t db_build(const float4* sph, const float* radius, uint32_t n, uint32_t res, void* buf, uint64_t bytes,
                     DirBufferView* out, cudaStream_t stream);

}  // namespace atx
