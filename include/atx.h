/*
 * atx.h - C ABI of the GB300 path tracer (libatx.so).
 *
 * Drop-in boundary for the render call of 1neskk/Ataraxia.  Each entry point
 * names the reference interface it replaces (paths relative to the Ataraxia
 * tree).  Plain pointers and sizes only; every call returns an atx_status and
 * never exits the process (the reference's CUDA_CHECK calls exit(),
 * Engine/include/DeviceMemory.h:7-16).
 *
 * Threading: calls on one atx_renderer must be serialised by the caller;
 * different renderers may be used from different threads.  Work is enqueued on
 * the renderer's own CUDA stream; functions that return data to the host
 * synchronise that stream first.
 */
#ifndef ATX_H
#define ATX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define ATX_API __declspec(dllexport)
#else
#define ATX_API __attribute__((visibility("default")))
#endif

#define ATX_ABI_VERSION 1

typedef enum atx_status {
    ATX_OK = 0,
    ATX_ERR_INVALID_ARG = 1,   /* bad pointer, size, index or state */
    ATX_ERR_OUT_OF_MEMORY = 2, /* device allocation failed or the HBM budget is exceeded */
    ATX_ERR_CUDA = 3,          /* a CUDA runtime call failed; see atx_last_error() */
    ATX_ERR_TIMEOUT = 4,       /* a bounded wait ran out */
    ATX_ERR_BUSY = 5,          /* admission refused for now (queue full) */
    ATX_ERR_NOT_FOUND = 6,     /* unknown job id */
    ATX_ERR_CANCELLED = 7,     /* the job was cancelled */
    ATX_ERR_NO_DEVICE = 8,     /* no CUDA device is visible */
    ATX_ERR_PARSE = 9          /* malformed scene file */
} atx_status;

/* ------------------------------------------------------------------ scene */

/* Sphere: Engine/include/SceneNode.h:11-21 (glm::vec3 center; float radius;
 * int id), 20 bytes.  material indexes the material array; out-of-range
 * values render with material 0 (Renderer.cu:30-37). */
typedef struct atx_sphere {
    float center[3];
    float radius;
    int32_t material;
} atx_sphere;

/* Material: Engine/include/Scene.h:28-47, 52 bytes.  id is carried but unused. */
typedef struct atx_material {
    float albedo[3];
    float roughness;
    float metallic;
    float f0[3];
    float emission_color[3];
    float emission_intensity;
    int32_t id;
} atx_material;

/* Point light: Engine/include/Scene.h:17-26, 28 bytes. */
typedef struct atx_light {
    float position[3];
    float color[3];
    float intensity;
} atx_light;

/* Settings: Engine/include/Scene.h:49-56, same 8-byte layout (two bools and
 * an int).  Defaults: accumulation = 1, sky_light = 0, max_bounces = 15. */
typedef struct atx_settings {
    uint8_t accumulation;
    uint8_t sky_light;
    uint8_t reserved[2];
    int32_t max_bounces;
} atx_settings;

/* Camera parameters: Engine/include/Camera.h:63-75 (position, direction, fov
 * in degrees, near and far clip).  The reference's default camera is
 * fov 45, near 0.1, far 100, position (0, 0, 3), direction (0, 0, -1)
 * (Engine/src/Camera.cpp:14-21). */
typedef struct atx_camera {
    float position[3];
    float direction[3];
    float fov_deg;
    float near_clip;
    float far_clip;
} atx_camera;

/* --------------------------------------------------------------- renderer */

typedef struct atx_config {
    int32_t device;            /* CUDA device ordinal */
    uint32_t wave_paths;       /* paths in flight per wave; 0 = autotuned default */
    uint32_t threads;          /* threads per block; 0 = default */
    uint32_t bvh_threshold;    /* sphere count at which the LBVH replaces the brute-force tables; 0 = 1025 */
    uint32_t bvh_leaf_size;    /* spheres per BVH leaf; 0 = 16, or what atx_autotune picks */
    uint32_t flags;            /* ATX_FLAG_* */
    uint64_t hbm_budget_bytes; /* device bytes this renderer may hold; 0 = unlimited */
} atx_config;

#define ATX_FLAG_NO_GRAPHS 1u       /* launch kernels directly instead of replaying a CUDA graph */
#define ATX_FLAG_PROFILE_KERNELS 2u /* record CUDA events around every kernel (atx_get_kernel_times) */
#define ATX_FLAG_HOST_EXECUTOR 4u   /* server only: simulate the GPU on the host (scheduling tests, no device) */
/* Consecutive atx_render calls may overlap on the GPU: a render's lanes are
 * not joined into the renderer's stream at its end, so the next render's
 * lanes start while the last, sparse bounces of the previous one finish
 * (each lane keeps its pixel range, so every pixel's frames stay in order).
 * The library's own calls (reads, atx_synchronize, stats, scene, camera-table
 * and size changes) join first; a caller that orders its own work on
 * atx_get_stream's stream, or uses atx_device_buffers' pointers, calls
 * atx_join (or atx_synchronize) first.  Results are unchanged. */
#define ATX_FLAG_OVERLAP_RENDERS 8u

typedef struct atx_stats {
    uint64_t frames;           /* reference frames rendered (samples per pixel) since creation */
    uint64_t paths;            /* pixel-samples traced */
    uint64_t extension_rays;   /* nearest-hit queries traced (a primary ray shared by a pixel's samples counts once) */
    uint64_t shadow_rays;      /* shadow rays traced */
    uint64_t kernel_launches;  /* kernels this renderer launched */
    uint64_t device_bytes;     /* device memory currently held */
    double last_render_ms;     /* device time of the last atx_render (CUDA events) */
    uint32_t bvh_in_use;       /* 1 if the current scene uses the LBVH */
    uint32_t reserved;
    uint64_t shaded_first;     /* pixel-samples whose primary ray hits (the paths shaded at the first bounce) */
} atx_stats;

typedef struct atx_renderer atx_renderer;

ATX_API int atx_abi_version(void);
ATX_API const char* atx_status_string(atx_status status);
/* Message of the last failure on the calling thread (empty if none). */
ATX_API const char* atx_last_error(void);
ATX_API atx_status atx_device_count(int32_t* count);

/* Renderer::Renderer (Engine/src/Renderer.cu:13-15).  config may be NULL. */
ATX_API atx_status atx_renderer_create(const atx_config* config, atx_renderer** out);
/* Renderer::~Renderer (Engine/src/Renderer.cu:17-23). */
ATX_API atx_status atx_renderer_destroy(atx_renderer* r);

/* Renderer::onResize (Engine/include/Renderer.h:23, Renderer.cu:98-146):
 * reallocates the float4 accumulator and the RGBA8 image when the size
 * changes and resets the frame index to 1. */
ATX_API atx_status atx_resize(atx_renderer* r, uint32_t width, uint32_t height);

/* Scene upload (Renderer::allocateDeviceMemory, Renderer.cu:25-57).  The
 * scene graph is flattened by the caller (Renderer.cu:67-96); arrays are
 * copied, so the caller may free them on return.  Spheres with a material
 * index outside [0, n_materials) use material 0.  n_materials may be 0 only
 * when n_spheres is 0.  Does not reset the frame index (the reference's UI
 * resets it explicitly). */
ATX_API atx_status atx_set_scene(atx_renderer* r, const atx_sphere* spheres, uint32_t n_spheres,
                                 const atx_material* materials, uint32_t n_materials,
                                 const atx_light* lights, uint32_t n_lights);

/* Renderer::setSettings / getSettings (Engine/include/Renderer.h:28-29). */
ATX_API atx_status atx_set_settings(atx_renderer* r, const atx_settings* settings);
ATX_API atx_status atx_get_settings(const atx_renderer* r, atx_settings* settings);

/* Renderer::resetFrameIndex (Engine/include/Renderer.h:31). */
ATX_API atx_status atx_reset_frame_index(atx_renderer* r);
ATX_API atx_status atx_get_frame_index(const atx_renderer* r, uint32_t* frame_index);

/* Camera (Engine/src/Camera.cpp:134-195): the projection and view matrices
 * are computed as the reference does for the current viewport and recomputed
 * after a resize; primary rays are generated on the device. */
ATX_API atx_status atx_set_camera(atx_renderer* r, const atx_camera* camera);
/* Camera given directly by its inverse matrices (column-major, as glm) and
 * position, the inputs of Camera::UpdateRayDirection (Camera.cpp:161-195). */
ATX_API atx_status atx_set_camera_matrices(atx_renderer* r, const float inv_view[16], const float inv_proj[16],
                                           const float position[3]);

/* Renderer::Render (Engine/include/Renderer.h:24, Renderer.cu:173-249) for spp
 * consecutive frames.  Frame f of the reference (seed = pixel * f) is sample
 * f - frame_index of this call: with accumulation on, the accumulator after
 * this call equals the reference's after the same frames and the frame index
 * advances by spp; with accumulation off the accumulator is cleared, frames
 * 1..spp are accumulated and the frame index stays 1.  A frame index of 1
 * clears the accumulator first (Renderer.cu:181-182).  The RGBA8 image is
 * packed for the last frame (Renderer.cu:166-168).  Asynchronous. */
ATX_API atx_status atx_render(atx_renderer* r, uint32_t spp);
ATX_API atx_status atx_synchronize(atx_renderer* r);
/* Makes the renderer's stream wait for every render enqueued so far, without
 * blocking the host (needed only with ATX_FLAG_OVERLAP_RENDERS; otherwise a
 * no-op).  No counterpart in the reference, whose Render() synchronises the
 * device every frame (Renderer.cu:233). */
ATX_API atx_status atx_join(atx_renderer* r);

/* Reads n_pixels float4 of the accumulator (sum of (r, g, b, 1) per frame). */
ATX_API atx_status atx_read_accumulation(atx_renderer* r, float* host_rgba, uint64_t n_pixels);
/* Reads the RGBA8 image (Renderer::getImage, Renderer.h:26; the reference
 * copies it to the host every frame, Renderer.cu:240). */
ATX_API atx_status atx_read_image(atx_renderer* r, uint32_t* host_rgba8, uint64_t n_pixels);
/* Starts reading the last render's RGBA8 image into host memory (best
 * page-locked: atx_host_alloc) on the renderer's copy stream and returns at
 * once with a ticket; atx_wait_read(r, ticket) blocks until the pixels have
 * landed, and the host buffer must not be used before.  With
 * ATX_FLAG_OVERLAP_RENDERS, renders alternate between two device images, so
 * the next render runs while the read is in flight (a render waits only for
 * the last read of the image it is about to overwrite).  No counterpart in
 * the reference, whose Render() copies the image synchronously every frame
 * (Renderer.cu:240). */
ATX_API atx_status atx_read_image_async(atx_renderer* r, uint32_t* host_rgba8, uint64_t n_pixels, uint64_t* ticket);
ATX_API atx_status atx_wait_read(atx_renderer* r, uint64_t ticket);
/* Device pointers of the accumulator (float4) and of the last render's image
 * (uint32) for zero-copy consumers. */
ATX_API atx_status atx_device_buffers(atx_renderer* r, void** accumulation, void** image);

ATX_API atx_status atx_get_stats(const atx_renderer* r, atx_stats* stats);

/* Device time per kernel family, summed over launches since the last reset,
 * from CUDA events recorded on the renderer's stream when the renderer was
 * created with ATX_FLAG_PROFILE_KERNELS (all zero otherwise).  No counterpart
 * in the reference, which only times Render() on the host (main.cpp:213-219). */
typedef struct atx_kernel_times {
    double extend_ms;          /* nearest hit + shading + next ray, all bounces */
    double shadow_ms;          /* shadow-ray any-hit */
    double accumulate_ms;      /* accumulator update + RGBA8 pack */
    double other_ms;           /* clears, BVH build */
    uint64_t extend_launches;
    uint64_t shadow_launches;
    uint64_t accumulate_launches;
    uint64_t other_launches;
} atx_kernel_times;
ATX_API atx_status atx_get_kernel_times(atx_renderer* r, atx_kernel_times* times);
ATX_API atx_status atx_reset_kernel_times(atx_renderer* r);

/* The renderer's CUDA stream (a cudaStream_t), so callers can order their own
 * work and timing events after the renderer's. */
ATX_API atx_status atx_get_stream(atx_renderer* r, void** stream);

/* Launch tuning of one renderer.  No counterpart in the reference, which
 * launches one fixed (opt/32 x opt/32) grid per frame (Renderer.cu:190-207).
 * Every setting renders the same frames bit for bit; only speed changes.  A
 * zero field means the default. */
typedef struct atx_tuning {
    uint32_t bvh_leaf_size;    /* spheres per LBVH leaf cluster (LBVH scenes; default 16) */
    uint32_t lanes;            /* concurrent lanes (streams with their own path state) a launch is split over */
    uint32_t wave_paths;       /* path state per lane, paths (default: sized to the launch, up to 64 Mi) */
    uint32_t threads;          /* threads per block of the primary and shadow kernels (multiple of 32, <= 256) */
    uint32_t wave_spp;         /* samples per wave at most: the wave's tile shape of pixels x samples */
    uint32_t path_kernel;      /* 0: by scene size (whole paths in one thread up to 24 spheres), 1: the wavefront
                                  stages, 2: whole paths in one thread (brute-force tables; LBVH scenes keep the
                                  wavefront) */
    uint32_t from_cache;       /* atx_autotune: 1 when the setting came from the process-wide cache */
    uint32_t cell_res;         /* direction cells along a cube face's edge of the light and direction buffers
                                  (scenes on the brute-force tables; 8..32, 0 = 16 up to 64 spheres, else 32):
                                  finer cells list fewer spheres per shadow and extension ray and take longer to
                                  build */
    double ms;                 /* atx_autotune: device time of one render with the chosen setting */
} atx_tuning;

/* Times candidate settings on the renderer's current scene, camera,
 * viewport and bounce depth, rendering spp frames per trial (passes timed
 * renders each, after two untimed ones), by coordinate descent over the leaf
 * size, lanes, path state, block size and wave shape, and keeps the fastest.
 * Results are cached per process, keyed by the GPU (SM count, compute
 * capability) and the workload's bucket (log2 spheres, nearest-hit structure,
 * log2 paths per launch, bounces); use_cache = 1 takes a cached result
 * without timing.  The renderer is left at frame 1 (its accumulator holds
 * tuning frames until the next render clears it). */
ATX_API atx_status atx_autotune(atx_renderer* r, uint32_t spp, uint32_t passes, int32_t use_cache,
                                atx_tuning* out);
ATX_API atx_status atx_get_tuning(atx_renderer* r, atx_tuning* out);
ATX_API atx_status atx_set_tuning(atx_renderer* r, const atx_tuning* t);

/* Page-locked host memory for fast copies in and out. */
ATX_API atx_status atx_host_alloc(uint64_t bytes, void** out);
ATX_API atx_status atx_host_free(void* p);

/* ---------------------------------------------------------------- batches */

/* Many resident scenes rendered together, one pass at a time.  No
 * counterpart in the reference, which renders one scene per kernelRender
 * launch (Renderer.cu:223).  A pass runs every scene with pending frames
 * through the single-scene wavefront kernels, spread over concurrent lanes
 * (CUDA streams with their own path state) and captured as one CUDA graph;
 * each scene keeps the reference's per-scene semantics (frame index,
 * accumulate/reset, seed = pixel * frame), so a scene's images are
 * bit-identical to rendering it alone with atx_render. */
typedef struct atx_batch atx_batch;

typedef struct atx_batch_scene {
    const atx_sphere* spheres;
    uint32_t n_spheres;
    const atx_material* materials;
    uint32_t n_materials;
    const atx_light* lights;
    uint32_t n_lights;
    atx_camera camera;          /* matrices computed as Camera.cpp:134-159 for width x height */
    uint32_t width, height;
    atx_settings settings;      /* Scene.h:49-56 */
} atx_batch_scene;

typedef struct atx_batch_stats {
    uint64_t passes;            /* atx_batch_run calls */
    uint64_t paths;             /* pixel-samples traced */
    uint64_t extension_rays;    /* nearest-hit queries */
    uint64_t shadow_rays;
    uint64_t kernel_launches;
    uint64_t graph_launches;    /* passes replayed from a captured CUDA graph */
    uint64_t device_bytes;
    double last_pass_ms;        /* device time of the last pass */
    uint32_t scenes;            /* scenes held */
    uint32_t waves_last_pass;   /* path waves (each up to lane_wave_paths) of the last pass */
} atx_batch_stats;

/* Tuning knobs (0 = keep the current value). */
typedef struct atx_batch_tuning {
    uint32_t lanes;             /* concurrent streams, each with its own path state (default 8) */
    uint32_t lane_wave_paths;   /* path-state capacity of one lane, paths (default 16 Mi = 2.2 GB) */
    uint32_t threads;           /* threads per CTA of the wavefront kernels (0 = per-kernel default) */
    uint32_t bvh_threshold;     /* sphere count from which a scene uses its LBVH */
    uint32_t bvh_leaf_size;
    uint32_t primary_cache;     /* 1 (default): keep each scene's primary hits across passes; 2: trace them every pass */
    uint32_t reserved[2];
} atx_batch_tuning;

ATX_API atx_status atx_batch_create(const atx_config* config, atx_batch** out);
ATX_API atx_status atx_batch_destroy(atx_batch* b);
/* Uploads a scene (arrays copied) and allocates its accumulator and image;
 * its frame index starts at 1. */
ATX_API atx_status atx_batch_add_scene(atx_batch* b, const atx_batch_scene* scene, uint32_t* id);
ATX_API atx_status atx_batch_remove_scene(atx_batch* b, uint32_t id);
/* Frames of this scene in the next pass (0 = idle). */
ATX_API atx_status atx_batch_set_spp(atx_batch* b, uint32_t id, uint32_t spp);
ATX_API atx_status atx_batch_reset(atx_batch* b, uint32_t id);
ATX_API atx_status atx_batch_frame_index(atx_batch* b, uint32_t id, uint32_t* frame_index);
/* New camera for a scene (matrices as Camera.cpp:134-159); its accumulation
 * restarts at frame 1, as the reference resets on camera motion (main.cpp:24-29). */
ATX_API atx_status atx_batch_set_camera(atx_batch* b, uint32_t id, const atx_camera* camera);
/* One pass: every scene with spp > 0 renders its frames; asynchronous. */
ATX_API atx_status atx_batch_run(atx_batch* b);
ATX_API atx_status atx_batch_synchronize(atx_batch* b);
ATX_API atx_status atx_batch_read_accumulation(atx_batch* b, uint32_t id, float* host_rgba, uint64_t n_pixels);
ATX_API atx_status atx_batch_read_image(atx_batch* b, uint32_t id, uint32_t* host_rgba8, uint64_t n_pixels);
ATX_API atx_status atx_batch_get_stats(atx_batch* b, atx_batch_stats* stats);
ATX_API atx_status atx_batch_set_tuning(atx_batch* b, const atx_batch_tuning* tuning);
ATX_API atx_status atx_batch_get_tuning(atx_batch* b, atx_batch_tuning* tuning);
/* Times passes of the batch's current scenes (at their set spp) under lane
 * counts 2-16 and lane path state 8-64 Mi paths (at most ~37 GB of path
 * state) and keeps the fastest; `passes` timed passes per setting (0 = 2).
 * Every scene must be at frame 1 (nothing rendered yet) and is reset to frame
 * 1 afterwards, so the tuning passes leave no trace in the images. */
ATX_API atx_status atx_batch_autotune(atx_batch* b, uint32_t passes, atx_batch_tuning* chosen);

/* ---------------------------------------------------------------- serving */

/* A render server: jobs (a scene and a target sample count) are submitted
 * from any thread and rendered progressively by a worker thread that runs
 * batched passes (continuous batching).  A job is admitted (in arrival order,
 * or smallest first) when an active slot is free and its device memory (scene
 * tables, LBVH, accumulator, image, per-pixel primary hits) fits the HBM
 * budget; its scene, frame index, accumulator and primary hits (traced once
 * per camera) stay resident until it reaches its target, when its
 * image and accumulator are copied to host memory and its device memory is
 * released.  The worker queues the next pass, its uploads and read-backs
 * while the current one runs, so the GPU does not wait for the host.
 * No counterpart in the reference (an interactive single-scene viewer). */
typedef struct atx_server atx_server;

typedef struct atx_server_config {
    atx_config base;            /* device, hbm_budget_bytes (0 = unlimited), bvh settings, flags */
    uint32_t max_active_jobs;   /* jobs rendered together (0 = 16) */
    uint32_t pass_spp;          /* frames per job per pass (0 = 64, raised for small images to 16 Mi paths per slice) */
    uint64_t max_pass_paths;    /* bound on pixel-samples per pass, scaling slices down (0 = 2^30) */
    uint32_t max_pending;       /* queued jobs before submit returns ATX_ERR_BUSY (0 = unbounded) */
    uint32_t host_fail_pass;    /* with ATX_FLAG_HOST_EXECUTOR: pass number at which the simulated device
                                   reports an error (fault injection on the host; 0 = never) */
    uint32_t policy;            /* ATX_ADMIT_ARRIVAL or ATX_ADMIT_SMALLEST */
} atx_server_config;

#define ATX_ADMIT_ARRIVAL 0u    /* admit queued jobs in arrival order */
#define ATX_ADMIT_SMALLEST 1u   /* admit the queued job with the fewest pixel-samples first */

typedef enum atx_job_state {
    ATX_JOB_QUEUED = 0,
    ATX_JOB_ACTIVE = 1,
    ATX_JOB_DONE = 2,
    ATX_JOB_CANCELLED = 3,
    ATX_JOB_FAILED = 4
} atx_job_state;

typedef struct atx_job_info {
    int32_t state;              /* atx_job_state */
    uint32_t frames_done;
    uint32_t target_spp;
    uint32_t width, height;
    uint32_t reserved;
    double submit_s, admit_s, done_s;   /* server clock (atx_server_now) */
} atx_job_info;

typedef struct atx_server_stats {
    uint64_t submitted, admitted, completed, cancelled, failed, rejected;
    uint64_t passes, paths;
    double busy_s;              /* device time of the passes (with their read-backs) */
    uint64_t device_bytes;
    uint32_t active, queued;
} atx_server_stats;

ATX_API atx_status atx_server_create(const atx_server_config* config, atx_server** out);
/* Stops the worker (queued and active jobs are cancelled) and frees everything. */
ATX_API atx_status atx_server_destroy(atx_server* s);
/* Copies the scene; returns ATX_ERR_BUSY when max_pending jobs are queued and
 * ATX_ERR_INVALID_ARG for a malformed scene or a zero target. */
ATX_API atx_status atx_server_submit(atx_server* s, const atx_batch_scene* scene, uint32_t target_spp, uint32_t* job);
ATX_API atx_status atx_server_poll(atx_server* s, uint32_t job, atx_job_info* info);
/* Waits up to timeout_ms for the job to finish (ATX_ERR_TIMEOUT otherwise). */
ATX_API atx_status atx_server_wait(atx_server* s, uint32_t job, uint32_t timeout_ms);
ATX_API atx_status atx_server_read_image(atx_server* s, uint32_t job, uint32_t* host_rgba8, uint64_t n_pixels);
ATX_API atx_status atx_server_read_accumulation(atx_server* s, uint32_t job, float* host_rgba, uint64_t n_pixels);
ATX_API atx_status atx_server_cancel(atx_server* s, uint32_t job);
/* New camera for a queued or active job: its accumulation restarts from frame
 * 1 and it renders its full target again (main.cpp:24-29 resets the frame
 * index when the camera moves). */
ATX_API atx_status atx_server_set_camera(atx_server* s, uint32_t job, const atx_camera* camera);
/* Forgets a finished or cancelled job and its host copies. */
ATX_API atx_status atx_server_release(atx_server* s, uint32_t job);
ATX_API atx_status atx_server_get_stats(atx_server* s, atx_server_stats* stats);
ATX_API atx_status atx_server_now(atx_server* s, double* seconds);

/* ------------------------------------------------- allocation-free render */

/* Renders spp frames without allocating device memory.  No counterpart in
 * the reference (whose Renderer allocates with cudaMalloc on every frame).
 * For callers that cannot call cudaMalloc: code embedded in a runtime that
 * owns all device memory through its own pool, or code that must not
 * allocate because cudaMalloc/cudaFree synchronise the device or are not
 * allowed where it runs.  The scratch these kernels need (scene tables, path
 * state, queues) is a 64 MiB array compiled into libatx.so, held by every
 * device that loads the library until the process exits.
 *   - spheres/materials/lights, accumulation (width*height float4, read and
 *     updated) and image (width*height RGBA8, may be NULL) are DEVICE
 *     pointers; inv_view/inv_proj/position/settings are host pointers.
 *   - Frame semantics are atx_render's: frame frame_index (>= 1) onward,
 *     frame 1 clears the accumulator, accumulation off renders frames 1..spp.
 *     Frames past 2^32 - 1 return ATX_ERR_INVALID_ARG.
 *   - Limits: 16384 spheres, 4096 materials, 1024 lights, 1024 bounces;
 *     larger inputs return ATX_ERR_INVALID_ARG.  Always the brute-force
 *     nearest-hit loop (no BVH, which would need its own scratch).
 *   - Work is enqueued on stream (a cudaStream_t, NULL = default stream).
 *     All calls share the one scratch array, so calls that overlap on the GPU
 *     race: serialise them.
 *   - Every call looks up the array's device address on the current device
 *     (cudaGetSymbolAddress); the first call on a device also loads the
 *     library's device code there, so make that first call before any
 *     stream capture. */
ATX_API atx_status atx_render_noalloc(const atx_sphere* spheres, uint32_t n_spheres, const atx_material* materials,
                                      uint32_t n_materials, const atx_light* lights, uint32_t n_lights,
                                      const float inv_view[16], const float inv_proj[16], const float position[3],
                                      uint32_t width, uint32_t height, const atx_settings* settings,
                                      uint32_t frame_index, uint32_t spp, float* accumulation, uint32_t* image,
                                      void* stream);

/* ----------------------------------------------------- scene files, graph */

/* A scene as the reference stores it (Engine/include/Scene.h:58-75): a tree
 * of nodes with a translation / rotation / scale and their own spheres
 * (SceneNode.h:23-68), plus materials, lights, camera and settings.  Host
 * only; no GPU is needed.  Node 0 is the root, named "Scene". */
typedef struct atx_scene atx_scene;

typedef struct atx_scene_info {
    uint32_t n_spheres;      /* spheres of all nodes (the flattened count) */
    uint32_t n_materials;
    uint32_t n_lights;
    uint32_t n_nodes;
    atx_camera camera;       /* near/far are the Camera defaults 0.1 / 100 */
    atx_settings settings;
} atx_scene_info;

/* Scene() (Scene.h:66): an empty root node, default camera and settings. */
ATX_API atx_status atx_scene_create(atx_scene** out);
ATX_API atx_status atx_scene_destroy(atx_scene* s);
/* Utils::deserializeScene (Engine/src/Utils.cpp:97-173) of len bytes of JSON
 * text.  Malformed text or a missing required key returns ATX_ERR_PARSE with
 * the line, column or key in atx_last_error() (the reference throws). */
ATX_API atx_status atx_scene_parse_json(const char* text, uint64_t len, atx_scene** out);
/* Utils::importScene (Utils.cpp:175-187).  A file that cannot be opened
 * returns ATX_ERR_NOT_FOUND (the reference returns an empty Scene). */
ATX_API atx_status atx_scene_load(const char* path, atx_scene** out);
/* Utils::serializeScene + dump(4) (Utils.cpp:3-51): writes at most cap bytes
 * (no terminator) and the full length to *len; buf may be NULL to query. */
ATX_API atx_status atx_scene_to_json(const atx_scene* s, char* buf, uint64_t cap, uint64_t* len);
/* Utils::exportScene (Utils.cpp:53-62). */
ATX_API atx_status atx_scene_save(const atx_scene* s, const char* path);
ATX_API atx_status atx_scene_get_info(const atx_scene* s, atx_scene_info* info);
/* World-space spheres as Renderer::allocateDeviceMemory collects them
 * (Renderer.cu:25-37, 67-96): depth first, each node's centres through its
 * global transform, radii times the mean column length of that transform,
 * material indexes outside the material list set to 0.  cap >= n_spheres. */
ATX_API atx_status atx_scene_flatten(const atx_scene* s, atx_sphere* out, uint64_t cap);
ATX_API atx_status atx_scene_get_materials(const atx_scene* s, atx_material* out, uint64_t cap);
ATX_API atx_status atx_scene_get_lights(const atx_scene* s, atx_light* out, uint64_t cap);
/* Editing (SceneNode::addChild / setPosition / setRotation / setScale /
 * addSphere, SceneNode.h:30-41).  rotation is a quaternion x, y, z, w. */
ATX_API atx_status atx_scene_add_node(atx_scene* s, uint32_t parent, const char* name, uint32_t* node);
ATX_API atx_status atx_scene_set_transform(atx_scene* s, uint32_t node, const float position[3],
                                           const float rotation_xyzw[4], const float scale[3]);
ATX_API atx_status atx_scene_add_spheres(atx_scene* s, uint32_t node, const atx_sphere* spheres, uint32_t n);
ATX_API atx_status atx_scene_set_materials(atx_scene* s, const atx_material* materials, uint32_t n);
ATX_API atx_status atx_scene_set_lights(atx_scene* s, const atx_light* lights, uint32_t n);
ATX_API atx_status atx_scene_set_camera(atx_scene* s, const atx_camera* camera);
ATX_API atx_status atx_scene_set_settings(atx_scene* s, const atx_settings* settings);
/* Renderer::allocateDeviceMemory for a scene graph: flattens s and uploads it
 * as atx_set_scene does. */
ATX_API atx_status atx_set_scene_graph(atx_renderer* r, const atx_scene* s);

/* -------------------------------------------- interactive camera, files */

/* The window input Camera::onUpdate polls (Engine/src/Camera.cpp:31-108 via
 * Input::GetMousePosition / IsMouseButtonPressed / IsKeyPressed), passed in
 * by the caller: cursor position in window pixels, the right mouse button
 * (look / move mode) and the W S A D Q E keys, nonzero = held. */
typedef struct atx_camera_input {
    float mouse[2];
    uint8_t right_button;
    uint8_t key_w, key_s, key_a, key_d, key_q, key_e;
    uint8_t reserved;
} atx_camera_input;

/* Camera::onUpdate (Camera.cpp:31-108): moves camera->position at 5 units/s
 * along the direction, direction x up and up, and turns the direction by the
 * mouse delta (0.002 per pixel, 0.3 rotation speed), only while the right
 * button is held.  last_mouse is the caller-held previous cursor position
 * (Camera::m_lastMousePos), updated on every call.  *moved = 1 when the
 * camera changed. */
ATX_API atx_status atx_camera_on_update(atx_camera* camera, float last_mouse[2], const atx_camera_input* input,
                                        float dt, int32_t* moved);
/* Ataraxia::onUpdate (Engine/src/main.cpp:22-32): atx_camera_on_update, and
 * when the camera moved, atx_set_camera and atx_reset_frame_index on r so the
 * next render restarts the accumulation. */
ATX_API atx_status atx_update_camera(atx_renderer* r, atx_camera* camera, float last_mouse[2],
                                     const atx_camera_input* input, float dt, int32_t* moved);

#define ATX_IMAGE_PPM 1   /* binary PPM (P6), RGB, 8 bits */
#define ATX_IMAGE_PAM 2   /* PAM (P7) RGB_ALPHA, 8 bits */
#define ATX_IMAGE_PFM 3   /* PFM (PF), RGB float: accumulated colour / frames */

/* Headless stand-ins for the reference's Vulkan image upload
 * (Core/src/Image.cpp:183-271).  Buffer row 0 is the bottom of the picture
 * (Camera.cpp:180-182); PPM/PAM files store the top row first, as the
 * reference displays it (main.cpp:186-187), PFM the bottom row first.
 * rgba8: width*height pixels A<<24 | B<<16 | G<<8 | R (Renderer.h:70-78);
 * accum: width*height float4 sums with the frame count in w. */
ATX_API atx_status atx_write_rgba8(const char* path, const uint32_t* rgba8, uint32_t width, uint32_t height,
                                   int32_t format);
ATX_API atx_status atx_write_pfm(const char* path, const float* accum, uint32_t width, uint32_t height);
/* Reads the renderer's image (PPM, PAM) or accumulator (PFM) back and writes it. */
ATX_API atx_status atx_save_image(atx_renderer* r, const char* path, int32_t format);

/* --------------------------------------------------------- host helpers */

/* Camera.cpp:134-159 on the host for a width x height viewport: view, inverse
 * view, projection and inverse projection, column-major.  Needs no GPU. */
ATX_API atx_status atx_camera_matrices(const atx_camera* camera, uint32_t width, uint32_t height, float view[16],
                                       float inv_view[16], float proj[16], float inv_proj[16]);

/* --------------------------------------------------------- parity hooks */

/* Nearest hit of n rays against the renderer's current scene through the
 * device code the renderer traces with (brute force or LBVH).  origins and
 * dirs are host arrays of 3 floats per ray; t_out is -1 and id_out -1 on a
 * miss (Renderer.cu:251-285). */
ATX_API atx_status atx_trace_nearest(atx_renderer* r, const float* origins, const float* dirs, uint64_t n,
                                     float* t_out, int32_t* id_out);
/* W*H*3 primary ray directions for the current camera (Camera.cpp:161-195). */
ATX_API atx_status atx_primary_directions(atx_renderer* r, float* host_dirs, uint64_t n_pixels);

#ifdef __cplusplus
}
#endif
#endif
