// Light buffer construction for the brute-force sphere tables (wavefront.h
// LightBufferView), after Haines and Greenberg's light buffer (1986): around
// each point light a cube of direction cells, and per cell the spheres a
// shadow ray towards the light can meet when its origin, seen from the light,
// lies in that cell.  Built once per scene, in double precision.
//
// Exactness.  A shadow ray (origin o = p + 1e-4 N on a sphere, direction
// L = normalize(light - p), occluded when some sphere has t > 0 and
// t^2 < |light - p|^2, Renderer.cu:348-352) runs the float test of
// trace.cuh.  A sphere that test accepts is passed by the exact ray within
// r + 4 sqrt(eps) D of its centre, D = |o - c| (the bound the LBVH walk uses,
// bvh_traverse.cuh), at a parameter between -4.5 sqrt(eps) D and the light.
// The ray stays within 2e-4 + kK |o - light| of the segment from the light to
// o (the 1e-4 offset and the float error of L), so that segment passes within
// R' = r + m + 2e-4 + kK dcap of the centre, m = kK (D + 1e-3) and
// D <= |c - light| + dcap, where dcap bounds |o - light| (every origin lies on
// a sphere; the lookup checks it).  Every point of the segment lies, seen from
// the light, in the origin's direction; so the sphere's cap of directions
// (half-angle asin(R' / |c - light|)) contains that direction, and the cell
// the lookup finds lists the sphere: a cell lists every sphere whose cap,
// widened by 1e-4 rad for the lookup's rounding, meets the cell's bounding
// cone.  A sphere whose centre lies within R' + m of the light (the segment
// could end inside it) is listed in every cell.
#include "light_buffer.h"

namespace atx {
namespace {

constexpr double kK = 1.2207031e-3;   // 5 sqrt(2^-24) per unit of distance, as kBvhK

uint64_t up(uint64_t x) { return (x + 255u) & ~uint64_t(255u); }

// Unit direction of face f (0..5: +x, -x, +y, -y, +z, -z) at in-face
// coordinates (u, v): the axes trace.cuh lb_cell divides by the face axis
// (face x: y, z; face y: x, z; face z: x, y).
__device__ void face_dir(uint32_t f, double u, double v, double out[3])
{
    const uint32_t ax = f >> 1;
    const uint32_t a = ax == 0 ? 1u : 0u, b = ax == 2 ? 1u : 2u;
    out[ax] = (f & 1u) ? -1.0 : 1.0;
    out[a] = u;
    out[b] = v;
    const double s = 1.0 / sqrt(out[0] * out[0] + out[1] * out[1] + out[2] * out[2]);
    out[0] *= s;
    out[1] *= s;
    out[2] *= s;
}

// dcap[l] = max over spheres of |c - light| + r, plus 1: every shadow-ray
// origin (a hit point lifted by 1e-4) lies within it.
__global__ void k_lb_dcap(const float4* __restrict__ sph, const float* __restrict__ rad, uint32_t n,
                          const DevLight* __restrict__ lights, float* dcap)
{
    __shared__ double red[256];
    const DevLight lt = lights[blockIdx.x];
    double mx = 0.0;
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
        const float4 s = sph[k];
        const double x = (double)s.x - lt.pos[0], y = (double)s.y - lt.pos[1], z = (double)s.z - lt.pos[2];
        mx = fmax(mx, sqrt(x * x + y * y + z * z) + (double)rad[k]);
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (uint32_t h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + h]);
        __syncthreads();
    }
    if (threadIdx.x == 0) dcap[blockIdx.x] = (float)(red[0] * (1.0 + 1e-6) + 1.0);
}

// One thread per (light, cell).
__global__ void k_lb_build(const float4* __restrict__ sph, const float* __restrict__ rad, uint32_t n,
                           const DevLight* __restrict__ lights, uint32_t nl, const float* __restrict__ dcap,
                           uint8_t* count, uint16_t* list)
{
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nl * kLbCells) return;
    const uint32_t l = id / kLbCells, cell = id % kLbCells;
    const uint32_t f = cell / (kLbRes * kLbRes), i = (cell / kLbRes) % kLbRes, j = cell % kLbRes;
    const double u0 = 2.0 * i / kLbRes - 1.0, u1 = 2.0 * (i + 1) / kLbRes - 1.0;
    const double v0 = 2.0 * j / kLbRes - 1.0, v1 = 2.0 * (j + 1) / kLbRes - 1.0;
    double ctr[3];
    face_dir(f, 0.5 * (u0 + u1), 0.5 * (v0 + v1), ctr);
    // bounding cone of the cell: its farthest points from the centre are corners
    double half = 0.0;
    for (int k = 0; k < 4; ++k) {
        double c[3];
        face_dir(f, (k & 1) ? u1 : u0, (k & 2) ? v1 : v0, c);
        const double dp = ctr[0] * c[0] + ctr[1] * c[1] + ctr[2] * c[2];
        half = fmax(half, acos(fmin(1.0, fmax(-1.0, dp))));
    }
    half += 1e-6;
    const DevLight lt = lights[l];
    const double dc = dcap[l];
    uint32_t cnt = 0;
    bool all = false;
    uint16_t* out = list + (size_t)id * kLbMaxList;
    for (uint32_t k = 0; k < n; ++k) {
        const float4 s = sph[k];
        const double vx = (double)s.x - lt.pos[0], vy = (double)s.y - lt.pos[1], vz = (double)s.z - lt.pos[2];
        const double dist = sqrt(vx * vx + vy * vy + vz * vz);
        const double m = kK * (dist + dc + 1e-3);
        const double rp = (double)rad[k] * (1.0 + 1e-5) + m + 2e-4 + kK * dc;
        bool listed = dist <= rp + m;
        if (!listed) {
            const double cosang = (ctr[0] * vx + ctr[1] * vy + ctr[2] * vz) / dist;
            listed = acos(fmin(1.0, fmax(-1.0, cosang))) <= half + asin(fmin(1.0, rp / dist)) + 1e-4;
        }
        if (!listed) continue;
        if (cnt < kLbMaxList) out[cnt] = (uint16_t)k;
        else all = true;
        ++cnt;
    }
    count[id] = all ? kLbAll : (uint8_t)cnt;
}

}  // namespace

uint64_t lb_bytes(uint32_t nl)
{
    const uint64_t cells = (uint64_t)nl * kLbCells;
    return up(cells) + up(cells * kLbMaxList * sizeof(uint16_t)) + up(nl * sizeof(float)) + 256;
}

cudaError_t lb_build(const float4* sph, const float* radius, uint32_t n, const DevLight* lights, uint32_t nl,
                     void* buf, uint64_t bytes, LightBufferView* out, cudaStream_t stream)
{
    if (nl == 0 || nl > kLbMaxLights || n == 0 || n > kLbMaxSpheres || bytes < lb_bytes(nl))
        return cudaErrorInvalidValue;
    const uint64_t cells = (uint64_t)nl * kLbCells;
    unsigned char* p = static_cast<unsigned char*>(buf);
    uint8_t* count = p;
    p += up(cells);
    uint16_t* list = reinterpret_cast<uint16_t*>(p);
    p += up(cells * kLbMaxList * sizeof(uint16_t));
    float* dcap = reinterpret_cast<float*>(p);
    k_lb_dcap<<<nl, 256, 0, stream>>>(sph, radius, n, lights, dcap);
    k_lb_build<<<(unsigned)((cells + 127) / 128), 128, 0, stream>>>(sph, radius, n, lights, nl, dcap, count, list);
    out->count = count;
    out->list = list;
    out->dcap = dcap;
    out->n_lights = nl;
    return cudaGetLastError();
}

}  // namespace atx
