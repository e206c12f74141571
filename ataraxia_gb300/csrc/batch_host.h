// Batched persistent renderer: many resident scenes, one persistent launch per
// pass (batch.cu), the pass replayed from a captured CUDA graph.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "atx.h"
#include "batch.h"
#include "host_common.h"
#include "renderer.h"

namespace atx {

class Batch {
public:
    explicit Batch(const atx_config& cfg);
    ~Batch();
    atx_status init();

    atx_status add_scene(const atx_batch_scene& d, uint32_t* id);
    atx_status remove_scene(uint32_t id);
    atx_status set_spp(uint32_t id, uint32_t spp);
    atx_status reset(uint32_t id);
    atx_status frame_index(uint32_t id, uint32_t* f);
    atx_status run();
    atx_status synchronize();
    atx_status read_accumulation(uint32_t id, float* host, uint64_t n);
    atx_status read_image(uint32_t id, uint32_t* host, uint64_t n);
    atx_status stats(atx_batch_stats* out);
    atx_status set_tuning(const atx_batch_tuning& t);
    atx_batch_tuning tuning() const { return tuning_; }
    Budget& budget() { return budget_; }
    cudaStream_t stream() const { return stream_; }

private:
    struct Slot {
        SceneStore scene;
        DeviceBuffer accum, image;
        CameraView cam{};
        atx_settings settings{1, 0, {0, 0}, 15};
        uint32_t w = 0, h = 0;
        uint32_t frame = 1;
        uint32_t spp_next = 0;
        int mode = 0;
    };
    Slot* slot(uint32_t id);
    cudaError_t enqueue_pass(const BatchDev& b, uint32_t n_sc, uint64_t n_items);
    void invalidate_graph();

    atx_config cfg_;
    Budget budget_;
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    bool timed_ = false;
    std::vector<std::unique_ptr<Slot>> slots_;
    atx_batch_tuning tuning_{};

    BatchSceneDev* h_scenes_ = nullptr;   // pinned staging
    void* h_items_ = nullptr;             // pinned: item_scene[cap], item_tile[cap]
    uint32_t cap_scenes_ = 0;
    uint64_t cap_items_ = 0;
    DeviceBuffer d_scenes_, d_items_, counters_;

    BatchShape shape_{};
    bool shape_valid_ = false;
    uint32_t shape_smem_ = 0;

    cudaGraphExec_t graph_ = nullptr;
    uint32_t graph_scenes_ = 0;
    uint64_t graph_items_ = 0;

    atx_batch_stats st_{};
};

}  // namespace atx
