// atx_render_noalloc: the wavefront render for callers that cannot allocate
// device memory (an allocator-less embedding, a caller whose memory pool is
// owned by another runtime, code that must not call cudaMalloc/cudaFree
// because those synchronise the device or are forbidden in its context).
//
// All scratch the kernels need (the converted scene tables and the per-wave
// path state, queues and counters) lives in one file-scope __device__ array of
// kScratchBytes.  The caller passes its inputs and outputs as device pointers;
// nothing here calls cudaMalloc, cudaFree or an allocating library routine.
//
// The array is a module global: every device that loads the library holds it
// until the process exits, and every call on a device reuses it.  Calls whose
// work overlaps on the GPU (two streams, or two host threads) race on it and
// must be serialised by the caller.  In host code the array's name is only a
// host-side stand-in, so every call looks up its device address on the current
// device with cudaGetSymbolAddress.  The first call on a device also loads the
// module there (the set-up); make that first call before any stream capture.
// Looking the address up on every call (cheap once the module is loaded) keeps
// it right after the caller resets the device and the module loads again.
#include <algorithm>
#include <cstdint>
#include <cstring>

#include "atx.h"
#include "host_common.h"
#include "renderer.h"
#include "wavefront.h"

namespace atx {
namespace {

constexpr uint64_t kScratchBytes = 64ull << 20;   // 64 MiB
constexpr uint32_t kMaxSpheres = 16384;
constexpr uint32_t kMaxMaterials = 4096;
constexpr uint32_t kMaxLights = 1024;
constexpr int32_t kMaxBounces = 1024;

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Device address of g_scratch on the current device.
atx_status scratch_address(unsigned char** out)
{
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
    *out = static_cast<unsigned char*>(p);
    return ATX_OK;
}

// Converts the reference-layout arrays into the shading tables (the same
// conversion SceneStore::upload does on the host, done here on the device).
__global__ void k_convert(const atx_sphere* s, uint32_t n, const atx_material* m, uint32_t nm, const atx_light* l,
                          uint32_t nl, float4* sph, int32_t* smat, DevMaterial* mat, DevLight* lts)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float r = s[i].radius;
        sph[i] = make_float4(s[i].center[0], s[i].center[1], s[i].center[2], r * r);
        smat[i] = ((uint32_t)s[i].material >= nm) ? 0 : s[i].material;   // Renderer.cu:30-37
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nm; i += stride) {
        DevMaterial d;
        for (int k = 0; k < 3; ++k) {
            d.albedo[k] = m[i].albedo[k];
            d.f0[k] = m[i].f0[k];
            d.emission[k] = m[i].emission_color[k] * m[i].emission_intensity;
        }
        d.roughness = m[i].roughness;
        d.metallic = m[i].metallic;
        d.emission_intensity = m[i].emission_intensity;
        mat[i] = d;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nl; i += stride) {
        DevLight d;
        for (int k = 0; k < 3; ++k) {
            d.pos[k] = l[i].position[k];
            d.le[k] = l[i].color[k] * l[i].intensity;
        }
        d.pad0 = d.pad1 = 0.0f;
        lts[i] = d;
    }
}

uint64_t up(uint64_t x) { return (x + 255u) & ~uint64_t(255u); }

}  // namespace
}  // namespace atx

extern "C" ATX_API atx_status atx_render_noalloc(const atx_sphere* spheres, uint32_t n_spheres,
                                                 const atx_material* materials, uint32_t n_materials,
                                                 const atx_light* lights, uint32_t n_lights, const float inv_view[16],
                                                 const float inv_proj[16], const float position[3], uint32_t width,
                                                 uint32_t height, const atx_settings* settings, uint32_t frame_index,
                                                 uint32_t spp, float* accumulation, uint32_t* image, void* stream)
{
    using namespace atx;
    clear_error();
    if (!inv_view || !inv_proj || !position || !settings || !accumulation)
        return fail(ATX_ERR_INVALID_ARG, "render_noalloc: null argument");
    if ((n_spheres && !spheres) || (n_materials && !materials) || (n_lights && !lights))
        return fail(ATX_ERR_INVALID_ARG, "render_noalloc: null scene array");
    if (width == 0 || height == 0 || (uint64_t)width * height > 0xffffffffull)
        return fail(ATX_ERR_INVALID_ARG, "render_noalloc: bad viewport %ux%u", width, height);
    if (n_spheres > kMaxSpheres)
        return fail(ATX_ERR_INVALID_ARG, "render_noalloc: %u spheres exceed the limit of %u", n_spheres, kMaxSpheres);
    if (n_materials > kMaxMaterials)
        return fail(ATX_ERR_INVALID_ARG, "render_noalloc: %u materials exceed the limit of %u", n_materials,
                    kMaxMaterials);
    if (n_lights > kMaxLights)
        return fail(ATX_ERR_INVALID_ARG, "render_noalloc: %u lights exceed the limit of %u", n_lights, kMaxLights);
    if (settings->max_bounces > kMaxBounces)
        return fail(ATX_ERR_INVALID_ARG, "render_noalloc: max_bounces %d exceeds the limit of %d",
                    settings->max_bounces, kMaxBounces);
    if (n_spheres > 0 && n_materials == 0)
        return fail(ATX_ERR_INVALID_ARG, "render_noalloc: spheres need at least one material");
    if (frame_index == 0) return fail(ATX_ERR_INVALID_ARG, "render_noalloc: frame_index starts at 1");
    if (spp == 0) return ATX_OK;
    if ((uint64_t)(settings->accumulation ? frame_index : 1u) + spp - 1u > 0xffffffffull)
        return fail(ATX_ERR_INVALID_ARG, "render_noalloc: frames %u..%u+%u-1 pass the frame index range",
                    frame_index, frame_index, spp);

    int device = 0;
    ATX_CUDA(cudaGetDevice(&device));
    unsigned char* base = nullptr;
    ATX_TRY(scratch_address(&base));
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // carve the scratch: scene tables first, then the wave state
    unsigned char* p = base;
    auto take = [&](uint64_t bytes) { unsigned char* r = p; p += up(bytes); return r; };
    float4* sph = reinterpret_cast<float4*>(take((uint64_t)kMaxSpheres * sizeof(float4)));
    int32_t* smat = reinterpret_cast<int32_t*>(take((uint64_t)kMaxSpheres * sizeof(int32_t)));
    DevMaterial* mat = reinterpret_cast<DevMaterial*>(take((uint64_t)kMaxMaterials * sizeof(DevMaterial)));
    DevLight* lts = reinterpret_cast<DevLight*>(take((uint64_t)kMaxLights * sizeof(DevLight)));
    uint32_t* counters = reinterpret_cast<uint32_t*>(take(wave_counter_words(kMaxBounces) * sizeof(uint32_t)));
    const uint64_t used = (uint64_t)(p - base);
    const uint32_t capacity = (uint32_t)((kScratchBytes - used - (kWaveArrays + 1) * 256) / kWaveBytesPerPath);
    WaveState ws{};
    ws.ray_o = reinterpret_cast<float4*>(take((uint64_t)capacity * sizeof(float4)));
    ws.ray_d = reinterpret_cast<float4*>(take((uint64_t)capacity * sizeof(float4)));
    ws.thr = reinterpret_cast<float4*>(take((uint64_t)capacity * sizeof(float4)));
    ws.col = reinterpret_cast<float4*>(take((uint64_t)capacity * sizeof(float4)));
    ws.sh_o = reinterpret_cast<float4*>(take((uint64_t)capacity * sizeof(float4)));
    ws.sh_d = reinterpret_cast<float4*>(take((uint64_t)capacity * sizeof(float4)));
    ws.sh_c = reinterpret_cast<float4*>(take((uint64_t)capacity * sizeof(float4)));
    ws.q[0] = reinterpret_cast<uint32_t*>(take((uint64_t)capacity * sizeof(uint32_t)));
    ws.q[1] = reinterpret_cast<uint32_t*>(take((uint64_t)capacity * sizeof(uint32_t)));
    ws.prim = reinterpret_cast<uint2*>(take((uint64_t)capacity * sizeof(uint2)));
    ws.hitq = reinterpret_cast<uint32_t*>(take((uint64_t)capacity * sizeof(uint32_t)));
    ws.vis = reinterpret_cast<uint32_t*>(take((uint64_t)capacity * sizeof(uint32_t)));
    ws.counters = counters;
    ws.totals = nullptr;
    ws.capacity = capacity;
    if ((uint64_t)(p - base) > kScratchBytes) return fail(ATX_ERR_OUT_OF_MEMORY, "render_noalloc: scratch layout");

    if (n_spheres || n_materials || n_lights) {
        k_convert<<<64, 256, 0, st>>>(spheres, n_spheres, materials, n_materials, lights, n_lights, sph, smat, mat,
                                      lts);
        ATX_CUDA(cudaGetLastError());
    }
    SceneView sc{};
    sc.sph = n_spheres ? sph : nullptr;
    sc.sph_mat = n_spheres ? smat : nullptr;
    sc.mat = n_materials ? mat : nullptr;
    sc.lights = n_lights ? lts : nullptr;
    sc.n_sph = n_spheres;
    sc.n_mat = n_materials;
    sc.n_lights = n_lights;
    sc.light_mod = fastmod_multiplier(n_lights);
    sc.use_bvh = 0;

    CameraView cam{};
    std::memcpy(cam.inv_view, inv_view, sizeof(cam.inv_view));
    std::memcpy(cam.inv_proj, inv_proj, sizeof(cam.inv_proj));
    std::memcpy(cam.pos, position, sizeof(cam.pos));
    cam.width = width;
    cam.height = height;

    LaunchShape shape{};
    ATX_CUDA(plan_launch(sc, device, 0, &shape));

    // Renderer.cu:181-182 / :245-248: frame 1 starts from a cleared
    // accumulator; with accumulation off the frames are 1..spp
    const uint32_t f0 = settings->accumulation ? frame_index : 1u;
    float4* acc = reinterpret_cast<float4*>(accumulation);
    if (f0 == 1) ATX_CUDA(enqueue_clear_accum(acc, (uint64_t)width * height, st));

    const uint64_t pixels = (uint64_t)width * height;
    const WavePlan plan = plan_waves(pixels, spp, capacity);
    const uint32_t last_frame = f0 + spp - 1;
    uint32_t launches = 0;
    for (uint64_t p0 = 0; p0 < pixels; p0 += plan.pixels_per_wave) {
        const uint32_t np = (uint32_t)std::min<uint64_t>(plan.pixels_per_wave, pixels - p0);
        for (uint32_t s0 = 0; s0 < spp; s0 += plan.spp_per_wave) {
            WaveJob job;
            job.pixel0 = (uint32_t)p0;
            job.n_pixels = np;
            job.spp = std::min(plan.spp_per_wave, spp - s0);
            job.frame0 = f0 + s0;
            job.max_bounces = settings->max_bounces;
            job.sky = settings->sky_light ? 1 : 0;
            job.pack_frame = (s0 + job.spp >= spp && image) ? last_frame : 0u;
            job.prim_cache = nullptr;
            job.prim_cached = 0;
            ATX_CUDA(enqueue_wave(sc, cam, ws, job, shape, acc, image, st, &launches, nullptr));
        }
    }
    return ATX_OK;
}
