// Shared host/device layout of the wavefront renderer: scene tables in HBM,
// per-wave path state and the launch entry points implemented in
// wavefront.cu.  Plain structs only, so host C++ compiled by the system
// compiler can include it.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace atx {

// Material as the shading code reads it: three float4 rows.  emission holds
// emissionColor * emissionIntensity (Scene.h:41, one IEEE product done on the
// host, the same bits the reference's getEmission() gives).
struct alignas(16) DevMaterial {
    float albedo[3];
    float roughness;
    float f0[3];
    float metallic;
    float emission[3];
    float emission_intensity;
};
static_assert(sizeof(DevMaterial) == 48, "DevMaterial is three float4 rows");

// Point light: position and color * intensity (Renderer.cu:362, one product).
struct alignas(16) DevLight {
    float pos[3];
    float pad0;
    float le[3];
    float pad1;
};
static_assert(sizeof(DevLight) == 32, "DevLight is two float4 rows");

// Linear BVH over the spheres (built on the device by lbvh.cu, Karras' binary
// radix tree over 30-bit Morton codes).  Nodes [0, n-1) are internal with
// node 0 the root; node n-1+k is the leaf holding sorted sphere k.  Boxes are
// stored as centre and half extent.  An internal node whose sorted range holds
// at most leaf_size spheres is treated as a leaf and its range tested
// directly.
struct BvhView {
    const float4* node_ctr;       // [2n-1] box centre xyz, w = bit-cast left child (internal nodes)
    const float4* node_half;      // [2n-1] half extent xyz, w = bit-cast right child (internal nodes)
    const uint2* node_range;      // [n-1] first, last sorted sphere under an internal node
    const float4* quad;           // [8(n-1)] 4-wide nodes (lbvh.cu k_pack_quads), used by the traversal
    const float4* leaf_sph;       // [n] spheres in Morton order (cx, cy, cz, r*r)
    const uint32_t* leaf_id;      // [n] original sphere index of each sorted slot
    uint32_t n_leaves;
    uint32_t leaf_size;
    uint32_t root;
};

// Light buffer (Haines and Greenberg's light buffer, 1986) for the
// brute-force sphere tables: for each point light a cube of directions around
// it, 6 faces of res x res cells, and for each cell the spheres that can
// block a shadow ray towards that light whose origin, seen from the light,
// lies in the cell (built by light_buffer.cu).  A shadow ray then tests the
// spheres of one cell instead of the whole table.
// Each cell is one 64-byte line of 16-bit words: word 0 the number of spheres
// listed (or kLbAll when they did not fit), words 1.. their indices in
// ascending order, so the count and the first seven indices arrive in one
// 16-byte load.
// res, the cells along a face's edge, is a property of each buffer: finer
// cells list fewer spheres (the 256-sphere scene: 2.9 per extension-ray
// lookup and 8.7 for a warp's longest list at 16; at 32 the longest about 30%
// shorter) and cost more to build and hold (four times the lines at 32).
constexpr uint32_t kCellResMin = 8;
constexpr uint32_t kCellResMax = 32;
constexpr uint32_t kCellResDefault = 32;   // a renderer's and a batch's resident scenes
constexpr uint32_t kCellResJobs = 16;      // the server's jobs (tables built per job)
// Up to this many spheres the lists are about one sphere already at 16, and
// finer cells only make the tables larger (the 9-sphere scene: -1% at 32).
constexpr uint32_t kCellResFewSpheres = 64;
__host__ __device__ constexpr uint32_t default_cell_res(uint32_t n_spheres)
{
    return n_spheres <= kCellResFewSpheres ? 16u : kCellResDefault;
}
__host__ __device__ constexpr uint32_t cells_for(uint32_t res) { return 6u * res * res; }
constexpr uint32_t kLbLine = 32;                 // 16-bit words per cell
constexpr uint32_t kLbMaxList = kLbLine - 1;     // spheres a cell can list
constexpr uint32_t kLbMaxLights = 64;
constexpr uint32_t kLbMaxSpheres = 65534;        // indices are 16-bit, 0xffff is kLbAll
constexpr uint32_t kLbAll = 0xffff;              // the cell's list overflowed: test every sphere
struct LightBufferView {
    const uint16_t* line;    // [n_lights * cells_for(res) * kLbLine] cell lines
    const float* dcap;       // [n_lights] the lists hold for shadow-ray origins within dcap of the light
    uint32_t n_lights;       // 0: no light buffer
    uint32_t res;            // cells along a face's edge
};

// Direction buffer for the extension rays of the brute-force tables (ray
// classification by origin sphere and direction, in the spirit of Arvo and
// Kirk's ray classification, 1987): for each sphere a cube of direction cells
// as the light buffer's, and for each cell the spheres a ray leaving that
// sphere in a direction of the cell can hit (built by light_buffer.cu).
// Every extension ray after the first bounce leaves the sphere its path last
// hit, so its nearest hit tests the spheres of one cell.
constexpr uint32_t kDbMaxSpheres = 1024;   // 393 KB of cells per sphere at res 32
struct DirBufferView {
    const uint16_t* line;    // [n * cells_for(res) * kLbLine] cell lines, as the light buffer's
    const float* reach;      // [n] the lists hold for ray origins within reach of the sphere's centre
    uint32_t n;              // spheres covered; 0: no direction buffer
    uint32_t res;            // cells along a face's edge
};

// Shadow-ray records carry the sphere the ray leaves from and the light it
// goes to in one word: sphere in the low 26 bits, light in the high 6 (only
// read when the light buffer, at most 64 lights, is in use).
constexpr uint32_t kShadowSphereMask = (1u << 26) - 1u;
__host__ __device__ inline uint32_t shadow_tag(uint32_t sphere, uint32_t light)
{
    return (sphere & kShadowSphereMask) | (light << 26);
}

// Scene tables, all in device memory.
struct SceneView {
    const float4* sph;        // (cx, cy, cz, radius*radius), n_sph entries
    const int32_t* sph_mat;   // material index, already clamped to [0, n_mat)
    const DevMaterial* mat;
    const DevLight* lights;
    uint32_t n_sph;
    uint32_t n_mat;
    uint32_t n_lights;
    uint32_t use_bvh;         // 1: traverse bvh instead of the brute-force loop
    BvhView bvh;
    LightBufferView lb;       // shadow-ray cells of the brute-force tables (lb.n_lights 0: none)
    DirBufferView db;         // extension-ray cells of the brute-force tables (db.n 0: none)
    uint64_t light_mod;       // fastmod_multiplier(n_lights): x % n_lights by multiplication
};

// x % d for d >= 1 by two multiplications (Lemire, Kaser and Kurz, "Faster
// remainder by direct computation", 2019): with M = floor((2^64 - 1) / d) + 1,
// x % d is the high 64 bits of (M * x mod 2^64) * d, for every 32-bit x
// (d = 1 gives M = 0 and the right answer, 0).
__host__ __device__ inline uint64_t fastmod_multiplier(uint32_t d)
{
    return d ? ~uint64_t(0) / d + 1u : 0u;
}

// Camera as the ray generator needs it (Camera.cpp:161-195): column-major
// inverse projection and inverse view, the eye position and the viewport.
struct CameraView {
    float inv_proj[16];
    float inv_view[16];
    float pos[3];
    uint32_t width;
    uint32_t height;
    // Optional per-pixel primary directions for this camera and viewport
    // (xyz, w unused), as the reference keeps them between camera changes
    // (Camera.cpp:161-195); nullptr: computed where needed.
    const float4* dirs;
    // Optional per-tile sphere masks for this camera, eye and scene
    // (k_tile_masks): for tile t, the 32 pixels 32t..32t+31, bit i % 32 of
    // word t * mask_words + i / 32 is set unless sphere i certainly misses
    // every one of their primary rays.  nullptr: culled per warp when needed.
    const uint32_t* masks;
    uint32_t mask_words;
    // Optional per-tile candidate lists for LBVH scenes (k_tile_lists), for
    // the same tiles: lists[info[t].x ...] holds info[t].y sorted sphere
    // indices (BvhView::leaf_sph) that may be hit by the tile's primary rays;
    // info[t].y = kNoTileList: none (the rays walk the LBVH).
    const uint2* tile_info;
    const uint32_t* tile_lists;
};

constexpr uint32_t kNoTileList = 0xffffffffu;
constexpr uint32_t kTileListMax = 1024;   // longer lists are not kept (the rays walk the LBVH)

// Per-wave path state, structure of arrays of float4 rows.
//   ray_o  (ox, oy, oz, seed bits)     ray_d (dx, dy, dz, -)
//   thr    (throughput rgb, -)         col   (path colour rgb, -)
//   q[2]   ping-pong extension queues of path ids
//   sh_o   (shadow origin xyz, distance^2)   sh_d (direction xyz, path id bits)
//   sh_c   (unoccluded contribution rgb, -)
//   counters[2*b] extension rays queued for bounce b, [2*b+1] shadow rays of bounce b
//   prim   one primary hit per pixel: the reference's primary ray depends on
//          the pixel only (Camera.cpp:161-195, no jitter), so every sample of a
//          pixel in one launch shares the same nearest hit
struct WaveState {
    float4* ray_o;
    float4* ray_d;
    float4* thr;
    float4* col;
    uint32_t* q[2];
    float4* sh_o;
    float4* sh_d;
    float4* sh_c;
    uint32_t* counters;
    unsigned long long* totals;   // running sums: [0] extension rays after bounce 0, [1] shadow rays,
                                  // [2] paths shaded at the first bounce
    uint2* prim;                  // per pixel of the wave: primary hit (t bits, sphere id), shared by its samples
    uint32_t* hitq;               // wave pixels whose primary ray hits (only those get first-bounce paths)
    uint32_t* vis;                // per pixel of the wave: bit l set when light l is visible from the primary hit
    uint32_t capacity;
};

// Path state per path slot: ray_o, ray_d, thr, col, sh_o, sh_d, sh_c (float4),
// q[0], q[1], hitq, vis (uint32) and prim (uint2); kWaveArrays arrays, each
// aligned to 256 bytes.
constexpr uint64_t kWaveBytesPerPath = 7 * 16 + 4 * 4 + 8;
constexpr uint64_t kWaveArrays = 12;

// Counter slots after the per-bounce pairs: [2*(max_bounces+1)] = hit pixels,
// [2*(max_bounces+1)+1] = paths shaded at the first bounce (counted only when
// the wave does not share primary hits; else it is hit pixels x spp),
// [2*(max_bounces+1)+2] = rays of k_paths' starting queue claimed so far,
// [2*(max_bounces+1)+3] = extension rays traced that no queue counts (with a
// light buffer a ray is traced where it is made and only hits are queued:
// the misses, and every ray k_paths traces).
inline size_t wave_counter_words(int max_bounces) { return 2 * ((size_t)(max_bounces > 0 ? max_bounces : 0) + 1) + 4; }

// One wave: pixels [pixel0, pixel0 + n_pixels) x samples [0, spp) with the
// sample s of pixel p at path id (p - pixel0) * spp + s, traced as the
// reference's frame frame0 + s.
struct WaveJob {
    uint32_t pixel0;
    uint32_t n_pixels;
    uint32_t spp;
    uint32_t frame0;
    int32_t max_bounces;
    int32_t sky;
    uint32_t pack_frame;      // when non-zero, pack the RGBA8 image at this frame index after accumulating
    // Per-pixel primary hits of the whole image (indexed by pixel), kept by the
    // caller across launches of the same scene and camera; nullptr: the wave's
    // own ws.prim (indexed by wave pixel).  prim_cached: prim_cache already
    // holds this view's hits, so they are not traced again.
    uint2* prim_cache;
    int32_t prim_cached;
};

// Whether a wave shares each pixel's primary hit among its samples (the hit is
// traced once, by k_primary, or comes from the cache).
__host__ __device__ inline bool wave_shares_primary(const WaveJob& j)
{
    return j.max_bounces > 0 && (j.spp > 1 || j.prim_cache != nullptr);
}

// Whether the first bounce's shadow rays are traced once per (pixel, light)
// instead of once per sample.  A pixel's samples share the primary hit, so
// samples that pick the same light (Renderer.cu:339, PcgHash(seed) % lights)
// cast the same shadow ray: k_primary queues one ray per distinct light the
// pixel's samples pick, k_shadow records the visible ones in ws.vis, and the
// first bounce adds the light of a sample whose light is visible.  Needs the
// light set to fit one 32-bit word (and a wave's hit slots 26 bits).
__host__ __device__ inline bool wave_light_vis(const WaveJob& j, uint32_t n_lights)
{
    return wave_shares_primary(j) && n_lights > 0u && n_lights <= 32u && j.n_pixels <= (1u << 26);
}

// Kernel families timed by KernelTimer.
enum KernelFamily { kFamExtend = 0, kFamShadow = 1, kFamAccumulate = 2, kFamOther = 3, kFamCount = 4 };

// Optional hook around each kernel launch (records CUDA events on the stream).
class KernelTimer {
public:
    virtual ~KernelTimer() = default;
    virtual void begin(int family, cudaStream_t stream) = 0;
    virtual void end(int family, cudaStream_t stream) = 0;
};

struct LaunchShape {
    int blocks_extend;
    int blocks_shadow;
    int blocks_primary;
    int threads;
    size_t smem_spheres;      // dynamic shared memory for the sphere table (0: read from global)
    int mode;                 // nearest-hit structure: 0 brute force from global, 1 from shared memory, 2 LBVH
    int fused;                // whole paths in one thread (k_fused): 0 never, 1 for waves of at most
                              // kFusedMaxSpp samples per pixel, 2 always (brute-force tables only)
};

// Scenes of at most this many spheres on the brute-force tables render waves
// of at most kFusedMaxSpp samples per pixel with whole paths in one thread
// unless told otherwise (small scene: 1 sample per call +38%, 8 about even,
// 64 -16% against the wavefront stages, whose shared first-bounce work pays
// with many samples).
constexpr uint32_t kFusedMaxSpheres = 24;
constexpr uint32_t kFusedMaxSpp = 8;

// Fills in grid sizes for this device and scene (occupancy-derived).
// path_kernel: 0 by scene size, 1 the wavefront stages, 2 whole paths in one
// thread (brute-force tables only; the wavefront for LBVH scenes).
cudaError_t plan_launch(const SceneView& sc, int device, int threads, LaunchShape* out, int path_kernel = 0);

// Enqueues one wave on stream: 2*max_bounces + 1 kernels plus a counter reset.
// accum is W*H float4, image W*H uint32 (may be null when pack_frame == 0).
// Returns the number of kernels launched through *launches.
cudaError_t enqueue_wave(const SceneView& sc, const CameraView& cam, const WaveState& ws, const WaveJob& job,
                         const LaunchShape& shape, float4* accum, uint32_t* image, cudaStream_t stream,
                         uint32_t* launches, KernelTimer* timer = nullptr);

// Zeroes n float4 on stream.
cudaError_t enqueue_clear_accum(float4* accum, uint64_t n, cudaStream_t stream);

// Debug / parity hook: nearest hit for n rays through the same device code the
// renderer uses.  origins/dirs are 3 floats per ray in device memory.
cudaError_t enqueue_trace_nearest(const SceneView& sc, const float* origins, const float* dirs, uint64_t n,
                                  float* t_out, int32_t* id_out, cudaStream_t stream);

// Writes W*H*3 primary directions (debug / parity hook).
cudaError_t enqueue_primary_dirs(const CameraView& cam, float* out, cudaStream_t stream);

// Fills the camera's per-pixel direction table (W*H float4, see CameraView::dirs).
cudaError_t enqueue_dir_table(const CameraView& cam, float4* out, cudaStream_t stream);

// Tile masks (see CameraView::masks) for scenes on the brute-force tables with
// at most kTileMaskMaxSpheres spheres: ceil(W*H/32) * ceil(n/32) words.
constexpr uint32_t kTileMaskMaxSpheres = 1024;
__host__ __device__ inline uint32_t tile_mask_words(uint32_t n_sph) { return (n_sph + 31u) / 32u; }
cudaError_t enqueue_tile_masks(const SceneView& sc, const CameraView& cam, uint32_t* masks, cudaStream_t stream);

// Tile candidate lists (see CameraView::tile_info) for an LBVH scene, in two
// steps: enqueue_tile_list_counts writes info[t].y (a length or kNoTileList),
// info[t].x (the exclusive sum of the lengths) and *total; after reading
// *total the caller provides lists of that many words to enqueue_tile_list_fill.
cudaError_t enqueue_tile_list_counts(const SceneView& sc, const CameraView& cam, uint2* info, uint32_t* total,
                                     cudaStream_t stream);
cudaError_t enqueue_tile_list_fill(const SceneView& sc, const CameraView& cam, const uint2* info, uint32_t* lists,
                                   cudaStream_t stream);

}  // namespace atx
