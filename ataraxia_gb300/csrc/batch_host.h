// Batched renderer: many resident scenes rendered together, one pass at a
// time.  No counterpart in the reference, which renders one scene per
// kernelRender launch (Renderer.cu:223) and synchronises after each frame.
//
// Each scene keeps its device state between passes (scene tables, LBVH,
// float4 accumulator, RGBA8 image, frame index).  A pass renders every scene
// with pending frames through the same wavefront kernels as the single-scene
// renderer (enqueue_frames), so a scene's results are bit-identical to
// rendering it alone.  Scenes are spread over `lanes` CUDA streams, each with
// its own path-state buffer: a lane renders its scenes one after another while
// the lanes run concurrently, so small scenes, the last bounces of a wave and
// the tails of big launches overlap with other scenes' work instead of leaving
// SMs idle.  Scenes are assigned to lanes longest-first by a cost model (LPT).
// A pass with the same shape as the previous one (same scenes on the same
// lanes, same waves) is captured as one CUDA graph (fork, every lane's
// kernels, join) and replayed, the instantiated graph's kernel arguments
// updated in place.  A pass of a new shape is launched directly and without
// the fork: each lane continues with its part as soon as it has finished its
// part of the previous pass (a scene that changes lanes waits for its old
// lane), so passes overlap instead of meeting at a barrier.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "atx.h"
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
    atx_status set_camera(uint32_t id, const atx_camera& c);
    // One pass; `done`, if given, is recorded on the batch stream after it.
    atx_status run(cudaEvent_t done = nullptr);
    atx_status synchronize();
    atx_status read_accumulation(uint32_t id, float* host, uint64_t n);
    atx_status read_image(uint32_t id, uint32_t* host, uint64_t n);
    // Queues copies of a scene's image and accumulator (either may be null)
    // after the passes already queued; complete when a later `done` event is.
    // Host buffers should be page-locked for the copies to be asynchronous.
    atx_status read_async(uint32_t id, uint32_t* image, float* accum, uint64_t n);
    atx_status stats(atx_batch_stats* out);
    atx_status set_tuning(const atx_batch_tuning& t);
    atx_status autotune(uint32_t passes, atx_batch_tuning* chosen);
    atx_batch_tuning tuning() const { return tuning_; }
    // Device bytes held by resident scenes (charged to the configured budget).
    uint64_t scene_bytes() const { return budget_.used(); }
    // Device bytes of the lanes' path state (not charged to the budget).
    uint64_t scratch_bytes() const { return scratch_.used(); }
    cudaStream_t stream() const { return stream_; }
    // Cells along a face's edge of the light and direction buffers of scenes
    // added from now on (0: default_cell_res by sphere count; the server's
    // per-job scenes use kCellResJobs, which are cheaper to build).
    void set_cell_res(uint32_t res) { cell_res_ = res; }

private:
    struct Slot {
        SceneStore scene;
        DeviceBuffer accum, image;
        DeviceBuffer prim;          // per-pixel primary hits, traced once per camera (8 B/pixel)
        DeviceBuffer dirs;          // per-pixel primary directions of the camera it was added with (16 B/pixel)
        bool prim_valid = false;
        atx_camera desc{};
        CameraView cam{};
        LaunchShape shape{};
        atx_settings settings{1, 0, {0, 0}, 15};
        uint32_t w = 0, h = 0;
        uint32_t frame = 1;
        uint32_t spp_next = 0;
        uint64_t lanes = 0;         // lanes its parts ran on in its last pass (bit l = lane l)
    };
    struct Lane {
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;   // after the lane's part of a pass
        cudaEvent_t mark = nullptr;   // everything queued on the lane before a pass (scenes moving off it)
        WaveStore wave;
    };
    Slot* slot(uint32_t id);
    atx_status ensure_lanes(uint32_t n);
    void drop_graph();
    void release_scratch();

    atx_config cfg_;
    uint32_t cell_res_ = 0;
    Budget budget_;      // resident scenes
    Budget scratch_;     // lanes' path state
    cudaStream_t stream_ = nullptr;      // passes, read-backs, frees
    cudaStream_t up_stream_ = nullptr;   // scene uploads and LBVH builds
    cudaEvent_t uploaded_ = nullptr;     // after the last upload
    cudaMemPool_t pool_ = nullptr;       // per-scene device memory, stream-ordered
    StreamOrder order_{};
    cudaEvent_t fork_ = nullptr, ev0_ = nullptr, ev1_ = nullptr;
    bool timed_ = false;
    std::vector<std::unique_ptr<Slot>> slots_;
    std::vector<Lane> lanes_;
    DeviceBuffer totals_;
    atx_batch_tuning tuning_{};

    cudaGraphExec_t graph_ = nullptr;
    std::vector<uint64_t> last_sig_;   // shape of the last pass
    bool last_graph_ = false;           // the last pass ran as a graph on the batch stream

    atx_batch_stats st_{};
    uint64_t primary_rays_ = 0;
};

}  // namespace atx
