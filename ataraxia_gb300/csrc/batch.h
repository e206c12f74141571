// Batched persistent rendering of many scenes in one launch (batch.cu).  No
// counterpart in the reference, which renders one scene per kernelRender
// launch (Renderer.cu:223).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "wavefront.h"

namespace atx {

// One scene's pass, as the persistent kernel reads it (device memory).
struct BatchSceneDev {
    SceneView sc;
    CameraView cam;
    float4* accum;          // W*H float4 of this scene
    uint32_t* image;        // W*H RGBA8 (packed at the pass's last frame)
    int32_t max_bounces;
    int32_t sky;
    uint32_t frame0;        // first frame of this pass; 1 = start from a cleared accumulator
    uint32_t spp;           // frames in this pass (0: scene idle this pass)
    uint32_t tile_w, tile_h, tiles_x;
    int32_t mode;           // 0 brute force from global, 1 from shared memory, 2 LBVH
};

// The pass: scenes, and the work items (scene, tile) in the order CTAs pull them.
struct BatchDev {
    const BatchSceneDev* scenes;
    const uint32_t* item_scene;
    const uint32_t* item_tile;
    uint32_t n_items;
    uint32_t* next_item;        // pulled with atomicAdd; reset before every pass
    unsigned long long* rays;   // [0] nearest-hit queries, [1] shadow rays (running sums)
    uint32_t smem_cap;          // spheres a CTA can stage
};

struct BatchShape {
    int blocks;
    int threads;
    size_t smem;
};

cudaError_t batch_plan(int device, int threads, uint32_t smem_spheres, BatchShape* out);
cudaError_t enqueue_batch(const BatchDev& b, const BatchShape& shape, cudaStream_t stream);

}  // namespace atx
