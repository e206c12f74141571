// Host orchestration of one progressive render target: the GB300 counterpart
// of the reference's Renderer (Engine/include/Renderer.h, Renderer.cu:13-249).
#pragma once

#include <cstdint>
#include <vector>

#include "atx.h"
#include "host_common.h"
#include "wavefront.h"

namespace atx {

// Device-resident scene: sphere table (float4 centre + radius^2), clamped
// material ids, radii (for BVH boxes), shading tables and the optional LBVH.
struct SceneStore {
    DeviceBuffer sph, sph_mat, sph_rad, mat, lights, bvh, lbuf, dbuf;
    SceneView view{};
    uint32_t bvh_threshold = 0;
    uint32_t bvh_leaf = 0;
    uint32_t cell_res = 0;   // cells along a face's edge of the light and direction buffers (0: default_cell_res)
    const StreamOrder* order = nullptr;   // stream-ordered allocation (batches); nullptr: cudaMalloc

    // Validates, converts and uploads on stream (Renderer.cu:25-57).
    atx_status upload(const atx_sphere* s, uint32_t n, const atx_material* m, uint32_t nm, const atx_light* l,
                      uint32_t nl, Budget* budget, cudaStream_t stream);
    // Rebuilds the LBVH (when the scene uses one) with another leaf size from
    // the resident sphere table; results are unchanged (the walk is exact).
    atx_status rebuild_bvh(uint32_t leaf, cudaStream_t stream);
    uint32_t leaf_size() const;
    // Rebuilds the light and direction buffers (when the scene has them) with
    // res cells along a face's edge (0: default_cell_res); results are
    // unchanged (every cell's list holds whatever a ray in it can meet).
    atx_status rebuild_cells(uint32_t res, Budget* budget, cudaStream_t stream);
    // The buffers' cells along a face's edge (0: the scene has neither).
    uint32_t cells() const;
    // Builds the light and direction buffers of the uploaded tables at cell_res.
    atx_status build_cells(Budget* budget, cudaStream_t stream);
    uint64_t device_bytes() const
    {
        return sph.bytes() + sph_mat.bytes() + sph_rad.bytes() + mat.bytes() + lights.bytes() + bvh.bytes() +
               lbuf.bytes() + dbuf.bytes();
    }
};

// Path state for up to `capacity` paths (wavefront.h WaveState) in one block.
struct WaveStore {
    DeviceBuffer buf;
    WaveState view{};
    uint32_t bounces = 0;
    atx_status ensure(uint32_t capacity, uint32_t max_bounces, Budget* budget);
    static uint64_t bytes_for(uint32_t capacity, uint32_t max_bounces);
};

// Splits pixels x samples into waves of at most `capacity` paths: pixel-major
// ranges, each covering a chunk of consecutive samples; chunks of one pixel
// range are issued in frame order so the accumulator adds frames in order.
struct WavePlan {
    uint32_t pixels_per_wave;
    uint32_t spp_per_wave;
};
// max_spp (0: no cap) bounds the samples per wave: the wave's tile shape
// (pixels x samples) for a fixed capacity.
WavePlan plan_waves(uint64_t pixels, uint32_t spp, uint32_t capacity, uint32_t max_spp = 0);

// Enqueues frames [frame0, frame0 + spp) for pixels [pix_begin, pix_end) of
// the view (default: all of them).  prim_cache (W*H entries, optional) keeps
// the primary hits across calls: traced into it unless prim_cached says it
// already holds them for this scene and camera.
atx_status enqueue_frames(const SceneView& sc, const CameraView& cam, WaveStore& ws, const LaunchShape& shape,
                          uint32_t frame0, uint32_t spp, int32_t max_bounces, int32_t sky, float4* accum,
                          uint32_t* image, uint32_t capacity, cudaStream_t stream, uint32_t* launches,
                          KernelTimer* timer = nullptr, uint64_t* primary_rays = nullptr, uint64_t pix_begin = 0,
                          uint64_t pix_end = ~uint64_t(0), uint2* prim_cache = nullptr, bool prim_cached = false,
                          uint32_t wave_spp = 0);

// Records a pair of CUDA events around each kernel and sums their durations
// per kernel family when collected.
class EventTimer : public KernelTimer {
public:
    ~EventTimer() override;
    void begin(int family, cudaStream_t stream) override;
    void end(int family, cudaStream_t stream) override;
    // Synchronises the recorded events and adds their durations to times.
    atx_status collect(atx_kernel_times* times);

private:
    cudaEvent_t take();
    struct Rec { int family; cudaEvent_t a, b; };
    std::vector<Rec> recs_;
    std::vector<cudaEvent_t> pool_;
    cudaEvent_t open_ = nullptr;
};

class Renderer {
public:
    explicit Renderer(const atx_config& cfg);
    ~Renderer();
    atx_status init();

    atx_status resize(uint32_t w, uint32_t h);
    atx_status set_scene(const atx_sphere* s, uint32_t n, const atx_material* m, uint32_t nm, const atx_light* l,
                         uint32_t nl);
    atx_status set_settings(const atx_settings& s);
    atx_settings settings() const { return settings_; }
    void reset_frame_index() { frame_ = 1; }
    uint32_t frame_index() const { return frame_; }
    atx_status set_camera(const atx_camera& c);
    atx_status set_camera_matrices(const float inv_view[16], const float inv_proj[16], const float pos[3]);
    atx_status render(uint32_t spp);
    atx_status synchronize();
    // Makes the renderer's stream wait for every render enqueued so far (with
    // ATX_FLAG_OVERLAP_RENDERS the lanes of a render are not joined into it
    // until then; otherwise a no-op).
    atx_status join();
    atx_status read_accumulation(float* host, uint64_t n);
    atx_status read_image(uint32_t* host, uint64_t n);
    // Starts copying the last render's RGBA8 image into host memory on a copy
    // stream and returns at once; wait_read(ticket) blocks until it landed.
    atx_status read_image_async(uint32_t* host, uint64_t n, uint64_t* ticket);
    atx_status wait_read(uint64_t ticket);
    atx_status device_buffers(void** accum, void** image);
    atx_status stats(atx_stats* out);
    atx_status trace_nearest(const float* o, const float* d, uint64_t n, float* t, int32_t* id);
    atx_status primary_directions(float* host, uint64_t n);
    atx_status kernel_times(atx_kernel_times* out);
    void reset_kernel_times() { ktimes_ = atx_kernel_times{}; }
    // Launch tuning (atx_tuning): the fields in use, and the autotuner that
    // times candidates on the current scene, camera and viewport.
    atx_status set_tuning(const atx_tuning& t);
    atx_status tuning(atx_tuning* out);
    atx_status autotune(uint32_t spp, uint32_t passes, bool use_cache, atx_tuning* out);
    cudaStream_t stream() const { return stream_; }
    uint32_t width() const { return width_; }
    uint32_t height() const { return height_; }

private:
    atx_status activate() const;
    atx_status refresh_camera();
    atx_status refresh_dirs();
    atx_status refresh_masks();   // the primary-direction table for camv_
    atx_status ensure_shape();

    atx_config cfg_;
    Budget budget_;
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev_start_ = nullptr, ev_stop_ = nullptr;
    bool timed_ = false;

    uint32_t width_ = 0, height_ = 0;
    uint32_t frame_ = 1;
    atx_settings settings_{1, 0, {0, 0}, 15};

    bool cam_from_desc_ = true;
    atx_camera cam_desc_{{0.0f, 0.0f, 3.0f}, {0.0f, 0.0f, -1.0f}, 45.0f, 0.1f, 100.0f};
    CameraView camv_{};
    uint32_t cam_w_ = 0, cam_h_ = 0;
    bool cam_dirty_ = true;

    SceneStore scene_;
    // Lanes: a launch's pixels are split into kLanes ranges rendered on as
    // many streams with their own path state, so one range's last, sparse
    // bounces overlap the others' work instead of leaving SMs idle.  Lane 0
    // is the renderer's stream.
    static constexpr int kLanes = 8;
    static constexpr int kDefaultLanes = 4;    // LBVH scenes, and any scene with overlapped renders
    static constexpr int kBufferedLanes = 2;   // scenes with light and direction buffers, renders joined
    WaveStore wave_[kLanes];
    cudaStream_t lane_stream_[kLanes] = {};
    cudaEvent_t fork_ = nullptr, join_[kLanes] = {};
    // ATX_FLAG_OVERLAP_RENDERS: lane 0 is a stream of its own too, and a
    // render's lanes are joined into stream_ only by join(); the next render's
    // lanes then continue on their own streams (same pixel range per lane, so
    // each pixel's frames stay in order) and wait for stream_ only after work
    // was put on it (stream_dirty_) or the lane split changed.
    bool overlap_ = false;
    bool joins_pending_ = false;
    bool stream_dirty_ = true;
    uint32_t pending_lanes_ = 0;
    uint32_t last_lanes_ = 0;
    uint64_t last_lane_px_ = 0;
    cudaStream_t time_stream_ = nullptr;   // records the end of a render after all its lanes
    bool tables_current() const;
    DeviceBuffer accum_, image_, totals_;
    // With overlapped renders, renders alternate between image_ and
    // image_alt_, so an asynchronous read of one render's image runs while
    // the next render packs the other; a render waits only for the last read
    // of the buffer it is about to overwrite.
    DeviceBuffer image_alt_;
    int img_last_ = 0, img_next_ = 0;
    cudaStream_t copy_stream_ = nullptr;
    cudaEvent_t read_done_[2] = {};
    bool read_pending_[2] = {false, false};
    cudaEvent_t src_ready_ = nullptr;
    static constexpr int kTickets = 8;
    cudaEvent_t ticket_ev_[kTickets] = {};
    uint64_t tickets_ = 0;
    uint32_t* image_buf(int i) { return (i ? image_alt_ : image_).as<uint32_t>(); }
    // Primary directions for the camera they were computed for (dirs_cam_):
    // rebuilt when the camera's matrices or the viewport change.
    DeviceBuffer dirs_;
    CameraView dirs_cam_{};
    bool dirs_valid_ = false;
    // Primary tile masks for the camera, eye and scene they were built for
    // (masks_cam_; scenes on the brute-force tables up to 1,024 spheres):
    // rebuilt when any of them changes.
    DeviceBuffer masks_;
    CameraView masks_cam_{};
    bool masks_valid_ = false;
    // The same for LBVH scenes: per-tile candidate lists (tile_info_: offset
    // and length per tile, then the total; tile_lists_: sorted sphere indices).
    DeviceBuffer tile_info_, tile_lists_;
    // The camera of the previous render (prev_cam_valid_: since the last
    // scene change): masks and lists are built only for a camera that stayed
    // put since then, so a camera that moves every frame never pays the build.
    CameraView prev_cam_{};
    bool prev_cam_valid_ = false;
    LaunchShape shape_{};
    bool shape_valid_ = false;
    // 0 fields: the defaults (lanes by scene kind, path state sized to the
    // launch, the config's threads, as many samples per wave as fit)
    atx_tuning tune_{};
    atx_status time_renders(uint32_t spp, uint32_t passes, double* ms);

    atx_stats st_{};
    uint64_t totals_host_[2] = {0, 0};
    EventTimer timer_;
    atx_kernel_times ktimes_{};
};

}  // namespace atx
