// GPU baseline: the reference's render kernel restated for sm_103a.
//
// Ataraxia's own render path cannot be compiled here (it needs glm, Vulkan and
// GLFW, none of which are present), so this file restates its CUDA kernel in
// the reference's own structure to time "the reference's kernel on the same
// GPU": one thread per pixel and one sample per launch (kernelRender,
// Engine/src/Renderer.cu:150-171), brute-force traceRay over the AoS Sphere
// array in global memory (:251-285), perPixel (:287-387), rayHit/rayMiss
// (:389-409), BRDF.cu:9-117 and the PCG helpers (Core/include/Random.h:59-70),
// a 2-D launch of (opt/32 x opt/32) blocks from cudaOccupancyMaxPotentialBlockSize
// (Renderer.cu:190-207), built with the reference's -use_fast_math
// (Engine/CMakeLists.txt:8).  It is a measuring stick, not part of the product:
// only bench.py loads it.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

namespace {

struct V3 {
    float x, y, z;
    __host__ __device__ V3() : x(0), y(0), z(0) {}
    __host__ __device__ V3(float a, float b, float c) : x(a), y(b), z(c) {}
    __host__ __device__ explicit V3(float a) : x(a), y(a), z(a) {}
};
__host__ __device__ inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
__host__ __device__ inline V3 operator*(V3 a, V3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ inline V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ inline V3 operator*(float s, V3 a) { return V3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ inline V3 operator/(V3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
__host__ __device__ inline V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
__host__ __device__ inline V3& operator*=(V3& a, V3 b) { a = a * b; return a; }
__host__ __device__ inline V3& operator/=(V3& a, float s) { a = a / s; return a; }
__host__ __device__ inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline V3 normalize(V3 v) { return v * (1.0f / sqrtf(dot(v, v))); }
__host__ __device__ inline float length(V3 v) { return sqrtf(dot(v, v)); }
__host__ __device__ inline V3 cross(V3 a, V3 b)
{
    return V3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

struct Sphere { V3 center; float radius; int id; };                       // 20 B
struct Material { V3 albedo; float roughness; float metallic; V3 F0; V3 emissionColor; float emissionIntensity; int id; };
struct Light { V3 position; V3 color; float intensity; };
struct Settings { bool accumulation; bool skyLight; int maxBounces; };
struct Ray { V3 origin, direction; };
struct HitRecord { float t; V3 worldPos; V3 worldNormal; uint32_t id; };
struct DeviceCamera { V3 position, direction; uint32_t width, height; V3* rayDirection; };
struct V4 { float x, y, z, w; };

constexpr float kPi = 3.14159265358979323846f;

__device__ uint32_t PcgHash(uint32_t& seed)
{
    uint32_t state = seed * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
__device__ float PcgFloat(uint32_t& seed)
{
    seed = PcgHash(seed);
    return static_cast<float>(seed) / static_cast<float>(UINT32_MAX);
}

__device__ V3 fresnelSchlick(V3 F0, float c)
{
    c = fminf(fmaxf(c, 0.0f), 1.0f);
    return F0 + (V3(1.0f) - F0) * powf(1.0f - c, 5.0f);
}
__device__ float distributionGGX(float NdotH, float r)
{
    const float a = r * r, a2 = a * a;
    float d = NdotH * NdotH * (a2 - 1.0f) + 1.0f;
    d = kPi * d * d;
    return a2 / d;
}
__device__ float geometrySchlickGGX(float NdotV, float r)
{
    const float rr = r + 1.0f, k = (rr * rr) / 8.0f;
    return NdotV / (NdotV * (1.0f - k) + k);
}
__device__ V3 cookTorrance(V3 albedo, V3 F0, float metallic, float roughness, V3 N, V3 V, V3 L)
{
    V3 H = normalize(V + L);
    float NdotL = fmaxf(dot(N, L), 0.0000001f), NdotV = fmaxf(dot(N, V), 0.0000001f);
    float NdotH = fmaxf(dot(N, H), 0.0f), VdotH = fmaxf(dot(V, H), 0.0f);
    V3 F = fresnelSchlick(F0, VdotH);
    float D = distributionGGX(NdotH, roughness);
    float G = geometrySchlickGGX(NdotV, roughness) * geometrySchlickGGX(NdotL, roughness);
    V3 kD = (V3(1.0f) - F) * (1.0f - metallic);
    V3 spec = (D * G * F) / (4.0f * NdotL * NdotV + 0.001f);
    V3 diffuse = (V3(1.0f) - F) * albedo / kPi;
    return (kD * diffuse + spec) * NdotL;
}
__device__ void frame(V3 N, V3& T, V3& B)
{
    if (fabsf(N.x) > fabsf(N.y)) T = V3(-N.z, 0, N.x) / sqrtf(N.x * N.x + N.z * N.z);
    else T = V3(0, -N.z, N.y) / sqrtf(N.y * N.y + N.z * N.z);
    B = cross(N, T);
}
__device__ V3 sampleHemisphereCosineWeighted(V3 N, uint32_t& seed)
{
    const float u1 = PcgFloat(seed), u2 = PcgFloat(seed);
    const float r = sqrtf(u1), theta = 2.0f * kPi * u2;
    const float x = r * cosf(theta), y = r * sinf(theta), z = sqrtf(1 - u1);
    V3 T, B;
    frame(N, T, B);
    return x * T + y * B + z * N;
}
__device__ V3 sampleGGX(V3 N, float roughness, uint32_t& seed)
{
    const float u1 = PcgFloat(seed), u2 = PcgFloat(seed);
    const float a = roughness * roughness;
    const float cosT = sqrtf((1.0f - u1) / (1.0f + (a * a - 1.0f) * u1));
    const float sinT = sqrtf(1 - cosT * cosT);
    const float phi = 2.0f * kPi * u2;
    V3 T, B;
    frame(N, T, B);
    return sinT * cosf(phi) * T + sinT * sinf(phi) * B + cosT * N;
}

__device__ HitRecord traceRay(const Ray& ray, const Sphere* spheres, size_t numSpheres)
{
    int closest = -1;
    float tmin = FLT_MAX;
    for (size_t i = 0; i < numSpheres; i++) {
        const Sphere& s = spheres[i];
        V3 oc = ray.origin - s.center;
        const float a = dot(ray.direction, ray.direction);
        const float b = 2.0f * dot(oc, ray.direction);
        const float c = dot(oc, oc) - s.radius * s.radius;
        const float disc = b * b - 4 * a * c;
        if (disc < 0.0f) continue;
        float t0 = (-b - sqrtf(disc)) / (2.0f * a);
        float t1 = (-b + sqrtf(disc)) / (2.0f * a);
        const float t = t0 < t1 ? t0 : t1;
        if (t > 0.0f && t < tmin) { tmin = t; closest = (int)i; }
    }
    HitRecord ht;
    if (closest < 0) { ht.t = -1.0f; return ht; }
    ht.t = tmin;
    ht.id = closest;
    const V3 origin = ray.origin - spheres[closest].center;
    ht.worldPos = origin + ray.direction * tmin;
    ht.worldNormal = normalize(ht.worldPos);
    ht.worldPos += spheres[closest].center;
    return ht;
}

__device__ V4 perPixel(uint32_t x, uint32_t y, uint32_t width, const Sphere* spheres, size_t numSpheres,
                       const DeviceCamera& cam, const Material* materials, size_t numMaterials, uint32_t frameIndex,
                       const Light* lights, size_t numLights, Settings settings)
{
    Ray ray;
    ray.origin = cam.position;
    ray.direction = cam.rayDirection[x + y * width];
    V3 color(0.0f), throughput(1.0f);
    uint32_t seed = x + y * width;
    seed *= frameIndex;
    for (int i = 0; i < settings.maxBounces; i++) {
        seed += i;
        HitRecord ht = traceRay(ray, spheres, numSpheres);
        if (ht.t < 0.0f) {
            if (settings.skyLight) color += V3(0.6f, 0.7f, 0.9f) * throughput;
            break;
        }
        const Material* mat = &materials[spheres[ht.id].id];
        if (mat->emissionIntensity > 0.0f) color += mat->emissionColor * mat->emissionIntensity * throughput;
        V3 base = mat->F0 * (1.0f - mat->metallic) + mat->albedo * mat->metallic;
        if (numLights > 0) {
            const Light& light = lights[PcgHash(seed) % numLights];
            V3 L = light.position - ht.worldPos;
            float d2 = dot(L, L);
            L = normalize(L);
            Ray sr;
            sr.origin = ht.worldPos + ht.worldNormal * 0.0001f;
            sr.direction = L;
            HitRecord sh = traceRay(sr, spheres, numSpheres);
            if (!(sh.t > 0.0f && sh.t * sh.t < d2)) {
                V3 f = cookTorrance(mat->albedo, base, mat->metallic, mat->roughness, ht.worldNormal, -ray.direction, L);
                color += light.color * light.intensity * f * throughput / 1.0f;
            }
        }
        throughput *= mat->albedo;
        ray.origin = ht.worldPos + ht.worldNormal * 0.0001f;
        float p = fmaxf(0.1f, fminf(1.0f, length(throughput)));
        if (PcgFloat(seed) > p) break;
        throughput /= p;
        ray.direction = mat->metallic > 0.0f ? sampleGGX(ht.worldNormal, mat->roughness, seed)
                                             : sampleHemisphereCosineWeighted(ht.worldNormal, seed);
    }
    return {color.x, color.y, color.z, 1.0f};
}

__device__ uint32_t vec4ToRGBA(V4 c)
{
    const uint8_t r = (uint8_t)(c.x * 255.0f), g = (uint8_t)(c.y * 255.0f), b = (uint8_t)(c.z * 255.0f),
                  a = (uint8_t)(c.w * 255.0f);
    return (a << 24) | (b << 16) | (g << 8) | r;
}

__global__ void kernelRender(uint32_t width, uint32_t height, uint32_t* imageData, const Sphere* spheres,
                             size_t numSpheres, const DeviceCamera cam, const Material* materials, size_t numMaterials,
                             V4* accumulation, uint32_t frameIndex, const Light* lights, size_t numLights,
                             Settings settings)
{
    if (width == 0 || height == 0 || cam.width == 0 || cam.height == 0) return;
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x < width && y < height) {
        const V4 c = perPixel(x, y, width, spheres, numSpheres, cam, materials, numMaterials, frameIndex, lights,
                              numLights, settings);
        const uint32_t p = x + y * width;
        V4 acc = accumulation[p];
        acc = {acc.x + c.x, acc.y + c.y, acc.z + c.z, acc.w + c.w};
        accumulation[p] = acc;
        const float f = (float)frameIndex;
        V4 fc = {fminf(fmaxf(acc.x / f, 0.f), 1.f), fminf(fmaxf(acc.y / f, 0.f), 1.f),
                 fminf(fmaxf(acc.z / f, 0.f), 1.f), fminf(fmaxf(acc.w / f, 0.f), 1.f)};
        imageData[p] = vec4ToRGBA(fc);
    }
}

struct Port {
    uint32_t w = 0, h = 0;
    Sphere* sph = nullptr;
    Material* mat = nullptr;
    Light* lts = nullptr;
    size_t ns = 0, nm = 0, nl = 0;
    V4* acc = nullptr;
    uint32_t* img = nullptr;
    V3* dirs = nullptr;                 // resident copy for kernel-only timing
    std::vector<V3> host_dirs;
    std::vector<uint32_t> host_img;
    V3 pos;
    Settings settings{true, false, 8};
    uint32_t frame = 1;
};

}  // namespace

extern "C" {

// Sets up the scene (arrays in the reference's AoS layout), the viewport, the
// camera position and precomputed primary directions (W*H*3 floats).
__attribute__((visibility("default"))) int refport_create(const void* spheres, uint32_t ns, const void* mats,
                                                          uint32_t nm, const void* lights, uint32_t nl,
                                                          uint32_t width, uint32_t height, const float* dirs,
                                                          const float* pos, int max_bounces, void** out)
{
    Port* p = new Port();
    p->w = width;
    p->h = height;
    p->ns = ns; p->nm = nm; p->nl = nl;
    p->settings.maxBounces = max_bounces;
    p->pos = V3(pos[0], pos[1], pos[2]);
    const size_t px = (size_t)width * height;
    if (cudaMalloc(&p->sph, sizeof(Sphere) * (ns ? ns : 1)) || cudaMalloc(&p->mat, sizeof(Material) * (nm ? nm : 1)) ||
        cudaMalloc(&p->lts, sizeof(Light) * (nl ? nl : 1)) || cudaMalloc(&p->acc, sizeof(V4) * px) ||
        cudaMalloc(&p->img, sizeof(uint32_t) * px) || cudaMalloc(&p->dirs, sizeof(V3) * px))
        return 1;
    // Renderer.cu:30-37: material ids outside the table become 0
    std::vector<Sphere> hs(ns);
    std::memcpy(hs.data(), spheres, sizeof(Sphere) * ns);
    for (auto& s : hs) if ((uint32_t)s.id >= nm) s.id = 0;
    cudaMemcpy(p->sph, hs.data(), sizeof(Sphere) * ns, cudaMemcpyHostToDevice);
    cudaMemcpy(p->mat, mats, sizeof(Material) * nm, cudaMemcpyHostToDevice);
    cudaMemcpy(p->lts, lights, sizeof(Light) * nl, cudaMemcpyHostToDevice);
    p->host_dirs.assign(reinterpret_cast<const V3*>(dirs), reinterpret_cast<const V3*>(dirs) + px);
    cudaMemcpy(p->dirs, p->host_dirs.data(), sizeof(V3) * px, cudaMemcpyHostToDevice);
    cudaMemset(p->acc, 0, sizeof(V4) * px);
    p->host_img.resize(px);
    *out = p;
    return cudaGetLastError() != cudaSuccess;
}

// One frame.  full = 0: the kernel alone with resident ray directions (times
// kernelRender).  full = 1: the reference's whole Renderer::Render sequence
// (Renderer.cu:173-249 with Camera::allocateDevice/freeDevice): device
// properties and occupancy query, cudaMalloc + copy of the W*H ray directions
// + device sync, the launch, sync, image copy to the host, free.
__attribute__((visibility("default"))) int refport_frame(void* handle, int full)
{
    Port* p = static_cast<Port*>(handle);
    DeviceCamera cam;
    cam.position = p->pos;
    cam.direction = V3(0, 0, -1);
    cam.width = p->w;
    cam.height = p->h;
    cam.rayDirection = p->dirs;
    const size_t px = (size_t)p->w * p->h;
    if (full) {
        if (cudaMalloc(&cam.rayDirection, sizeof(V3) * px)) return 1;
        cudaMemcpy(cam.rayDirection, p->host_dirs.data(), sizeof(V3) * px, cudaMemcpyHostToDevice);
        cudaDeviceSynchronize();
        cudaDeviceProp prop;
        cudaGetDeviceProperties(&prop, 0);
    }
    int min_grid = 0, opt = 0;
    cudaOccupancyMaxPotentialBlockSize(&min_grid, &opt, kernelRender, 0, 0);
    dim3 block(opt / 32, opt / 32);
    dim3 grid((p->w + block.x - 1) / block.x, (p->h + block.y - 1) / block.y);
    kernelRender<<<grid, block>>>(p->w, p->h, p->img, p->sph, p->ns, cam, p->mat, p->nm, p->acc, p->frame, p->lts,
                                  p->nl, p->settings);
    if (cudaGetLastError() != cudaSuccess) return 1;
    if (full) {
        if (cudaDeviceSynchronize() != cudaSuccess) return 1;
        cudaMemcpy(p->host_img.data(), p->img, sizeof(uint32_t) * px, cudaMemcpyDeviceToHost);
        cudaDeviceSynchronize();
        cudaFree(cam.rayDirection);
    }
    p->frame++;
    return 0;
}

__attribute__((visibility("default"))) int refport_sync(void) { return cudaDeviceSynchronize() != cudaSuccess; }

__attribute__((visibility("default"))) int refport_block(int* bx, int* by)
{
    int min_grid = 0, opt = 0;
    if (cudaOccupancyMaxPotentialBlockSize(&min_grid, &opt, kernelRender, 0, 0)) return 1;
    *bx = opt / 32;
    *by = opt / 32;
    return 0;
}

__attribute__((visibility("default"))) int refport_read_accum(void* handle, float* out)
{
    Port* p = static_cast<Port*>(handle);
    return cudaMemcpy(out, p->acc, sizeof(V4) * (size_t)p->w * p->h, cudaMemcpyDeviceToHost) != cudaSuccess;
}

__attribute__((visibility("default"))) void refport_destroy(void* handle)
{
    Port* p = static_cast<Port*>(handle);
    if (!p) return;
    cudaFree(p->sph); cudaFree(p->mat); cudaFree(p->lts); cudaFree(p->acc); cudaFree(p->img); cudaFree(p->dirs);
    delete p;
}

}  // extern "C"
