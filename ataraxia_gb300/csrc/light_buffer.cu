// Light buffer construction for the brute-force sphere tables (wavefront.h
// LightBufferView), after Haines and Greenberg's light buffer (1986): around
// each point light a cube of direction cells, and per cell the spheres a
// shadow ray towards the light can meet when its origin, seen from the light,
// lies in that cell.  Built once per scene.
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

// Scratch for the cell cones (k_cell_cones) at the end of both buffers.
uint64_t cone_bytes(uint32_t res)
{
    return up(cells_for(res) * sizeof(float4)) + up(cells_for(res) * sizeof(float));
}

// Unit direction of face f (0..5: +x, -x, +y, -y, +z, -z) at in-face
// coordinates (u, v): the axes trace.cuh lb_cell divides by the face axis
// (face x: y, z; face y: x, z; face z: x, y).
__device__ float3 face_dir(uint32_t f, float u, float v)
{
    const uint32_t ax = f >> 1;
    float c[3];
    const uint32_t a = ax == 0 ? 1u : 0u, b = ax == 2 ? 1u : 2u;
    c[ax] = (f & 1u) ? -1.0f : 1.0f;
    c[a] = u;
    c[b] = v;
    const float s = 1.0f / sqrtf(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    return make_float3(c[0] * s, c[1] * s, c[2] * s);
}

__device__ float dotf3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Bounding cone of every direction cell, widened by 2e-4 rad (1e-4 for the
// lookup's rounding, the rest for the build's arithmetic): axis and the
// cosine of the half-angle in cone[cell], its sine in cone_sin[cell].  The
// farthest points of a cell from its centre are its corners.
__global__ void k_cell_cones(uint32_t res, float4* cone, float* cone_sin)
{
    const uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= cells_for(res)) return;
    const uint32_t f = cell / (res * res), i = (cell / res) % res, j = cell % res;
    const float fr = (float)res;
    const float u0 = 2.0f * i / fr - 1.0f, u1 = 2.0f * (i + 1) / fr - 1.0f;
    const float v0 = 2.0f * j / fr - 1.0f, v1 = 2.0f * (j + 1) / fr - 1.0f;
    const float3 ctr = face_dir(f, 0.5f * (u0 + u1), 0.5f * (v0 + v1));
    float cmin = 1.0f;
    for (int k = 0; k < 4; ++k) cmin = fminf(cmin, dotf3(ctr, face_dir(f, (k & 1) ? u1 : u0, (k & 2) ? v1 : v0)));
    const float hw = acosf(fminf(1.0f, cmin)) + 2e-4f;
    cone[cell] = make_float4(ctr.x, ctr.y, ctr.z, cosf(hw));
    cone_sin[cell] = sinf(hw);
}

// dcap[l] = max over spheres of |c - light| + r, plus 1: every shadow-ray
// origin (a hit point lifted by 1e-4) lies within it.
__global__ void k_lb_dcap(const float4* __restrict__ sph, const float* __restrict__ rad, uint32_t n,
                          const DevLight* __restrict__ lights, float* dcap)
{
    __shared__ float red[256];
    const DevLight lt = lights[blockIdx.x];
    float mx = 0.0f;
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
        const float4 s = sph[k];
        const float3 v = make_float3(s.x - lt.pos[0], s.y - lt.pos[1], s.z - lt.pos[2]);
        mx = fmaxf(mx, sqrtf(dotf3(v, v)) + rad[k]);
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (uint32_t h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + h]);
        __syncthreads();
    }
    if (threadIdx.x == 0) dcap[blockIdx.x] = red[0] * 1.0001f + 1.0f;
}

// One warp per (light, cell); the lanes test 32 spheres at a time and append
// the listed ones in index order.  Float arithmetic with every bound rounded
// towards listing: the widened cell cone, sin(beta) rounded up, cos(beta)
// taken from it, a 2e-5 slack on the final comparison.
__global__ void k_lb_build(const float4* __restrict__ sph, const float* __restrict__ rad, uint32_t n,
                           const DevLight* __restrict__ lights, uint32_t nl, const float* __restrict__ dcap,
                           uint32_t res, const float4* __restrict__ cone, const float* __restrict__ cone_sin,
                           uint16_t* line)
{
    const uint32_t cells = cells_for(res);
    const uint32_t id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (id >= nl * cells) return;   // whole warps: blockDim is a multiple of 32
    const uint32_t l = id / cells, cell = id % cells;
    const float4 cc = cone[cell];
    const float3 ctr = make_float3(cc.x, cc.y, cc.z);
    const float ch = cc.w, sh = cone_sin[cell];
    const DevLight lt = lights[l];
    const float dc = dcap[l];
    uint16_t* out = line + (size_t)id * kLbLine + 1;
    uint32_t cnt = 0;
    for (uint32_t base = 0; base < n && cnt <= kLbMaxList; base += 32u) {
        const uint32_t k = base + lane;
        bool listed = false;
        if (k < n) {
            const float4 s = sph[k];
            const float3 v = make_float3(s.x - lt.pos[0], s.y - lt.pos[1], s.z - lt.pos[2]);
            const float dist = sqrtf(dotf3(v, v));
            const float m = (float)kK * (dist + dc + 1e-3f);
            const float rp = rad[k] * 1.00001f + m + 2e-4f + (float)kK * dc;
            if (!(dist > (rp + m) * 1.0001f)) {
                listed = true;   // the light may sit in (or next to) the sphere
            } else {
                const float sb = fminf(1.0f, rp / dist * 1.0001f);
                const float cb = sqrtf(fmaxf(0.0f, 1.0f - sb * sb));
                listed = dotf3(ctr, v) >= dist * (ch * cb - sh * sb - 2e-5f);   // cos(angle) >= cos(hw + beta)
            }
        }
        const uint32_t mask = __ballot_sync(0xffffffffu, listed);
        const uint32_t pos = cnt + __popc(mask & ((1u << lane) - 1u));
        if (listed && pos < kLbMaxList) out[pos] = (uint16_t)k;
        cnt += __popc(mask);
    }
    if (lane == 0) out[-1] = (uint16_t)(cnt > kLbMaxList ? kLbAll : cnt);
}

// ---------------------------------------------------------- direction buffer
//
// Exactness.  An extension ray leaves the sphere its path last hit: origin
// o = p + 1e-4 N with p the float hit point, direction d.  The lookup uses the
// lists of that sphere i only when |o - c_i| <= reach_i (checked per ray;
// else the whole table), so o = c_i + e with |e| <= reach_i.  A sphere j the
// float test accepts has a ray point X = o + t d, t >= -4.5 sqrt(eps) D_j,
// within r_j + 4 sqrt(eps) D_j of c_j (D_j = |o - c_j| <= |c_j - c_i| +
// reach_i).  Then c_i + t d = X - e lies within R' = r_j + m + reach_i of c_j,
// m = kK (D_j + 1e-3): for t >= 0 the ball (c_j, R') meets the cone of
// directions of d's cell from apex c_i, and for t < 0 its centre lies within
// R' + m of c_i.  A cell lists every sphere passing one of those two tests
// (cell cone widened by 2e-4 rad, bounds rounded towards listing), sphere i
// itself included.

// E = max over spheres of |c|_1 + r, a bound on the coordinates the hit-point
// arithmetic sees (one block).
__global__ void k_db_extent(const float4* __restrict__ sph, const float* __restrict__ rad, uint32_t n, float* ext)
{
    __shared__ float red[256];
    float mx = 0.0f;
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
        const float4 s = sph[k];
        mx = fmaxf(mx, fabsf(s.x) + fabsf(s.y) + fabsf(s.z) + rad[k]);
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (uint32_t h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + h]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *ext = red[0];
}

// reach_i: the sphere's radius, its 1e-4 surface offset and a float hit
// point's typical error (a hit point farther off falls back to the whole table).
__global__ void k_db_reach(const float* __restrict__ rad, uint32_t n, const float* __restrict__ ext, float* reach)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) reach[i] = rad[i] * 1.001f + 2e-4f + (float)kK * *ext;
}

// Whether sphere (s, r) may be hit by a ray leaving within rho of o whose
// direction lies in the cone (axis ctr, half-angle with cosine ch and sine
// sh): see the exactness note above.  Bounds rounded towards listing.
__device__ bool db_listed(float3 ctr, float ch, float sh, float4 o, float rho, float4 s, float r)
{
    const float3 v = make_float3(s.x - o.x, s.y - o.y, s.z - o.z);
    const float dist = sqrtf(dotf3(v, v));
    const float m = (float)kK * (dist + rho + 1e-3f);
    const float rp = r * 1.00001f + m + rho;
    if (!(dist > (rp + m) * 1.0001f)) return true;   // overlaps the origin's neighbourhood (sphere i itself too)
    const float sb = fminf(1.0f, rp / dist * 1.0001f);
    const float cb = sqrtf(fmaxf(0.0f, 1.0f - sb * sb));
    return dotf3(ctr, v) >= dist * (ch * cb - sh * sb - 2e-5f);   // cos(angle) >= cos(half-angle + beta)
}

// One block of 256 threads per (sphere i, cube face): first the spheres whose
// caps meet the face's bounding cone (its corners lie acos(1/sqrt 3) from the
// face axis), kept in index order; then one warp per cell at a time tests only
// those and appends the listed ones in index order.
__global__ void __launch_bounds__(256) k_db_build(const float4* __restrict__ sph, const float* __restrict__ rad,
                                                  uint32_t n, const float* __restrict__ reach, uint32_t res,
                                                  const float4* __restrict__ cone, const float* __restrict__ cone_sin,
                                                  uint16_t* line)
{
    __shared__ uint16_t cand[kDbMaxSpheres];
    __shared__ uint32_t warp_n[8];
    const uint32_t i = blockIdx.x / 6u, f = blockIdx.x % 6u;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const float4 o = sph[i];
    const float rho = reach[i];

    // pass 1: candidates of the face, block-wide ordered compaction
    const float3 axis = face_dir(f, 0.0f, 0.0f);
    const float hf = 0.95531662f + 3e-4f;   // acos(1/sqrt(3)), widened
    const float chf = cosf(hf), shf = sinf(hf);
    uint32_t nc = 0;
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        const uint32_t k = base + threadIdx.x;
        const bool listed = k < n && db_listed(axis, chf, shf, o, rho, sph[k], rad[k]);
        const uint32_t mask = __ballot_sync(0xffffffffu, listed);
        if (lane == 0) warp_n[warp] = (uint32_t)__popc(mask);
        __syncthreads();
        uint32_t off = nc, tot = 0;
        for (uint32_t w = 0; w < 8u; ++w) {
            if (w < warp) off += warp_n[w];
            tot += warp_n[w];
        }
        if (listed) cand[off + __popc(mask & ((1u << lane) - 1u))] = (uint16_t)k;
        nc += tot;
        __syncthreads();
    }

    // pass 2: one warp per cell
    for (uint32_t c = warp; c < res * res; c += 8u) {
        const uint32_t cell = f * res * res + c;
        const float4 cc = cone[cell];
        const float3 ctr = make_float3(cc.x, cc.y, cc.z);
        const float ch = cc.w, sh = cone_sin[cell];
        const uint32_t id = i * cells_for(res) + cell;
        uint16_t* out = line + (size_t)id * kLbLine + 1;
        uint32_t cnt = 0;
        for (uint32_t base = 0; base < nc && cnt <= kLbMaxList; base += 32u) {
            const uint32_t q = base + lane;
            uint32_t k = 0;
            bool listed = false;
            if (q < nc) {
                k = cand[q];
                listed = db_listed(ctr, ch, sh, o, rho, sph[k], rad[k]);
            }
            const uint32_t mask = __ballot_sync(0xffffffffu, listed);
            const uint32_t pos = cnt + __popc(mask & ((1u << lane) - 1u));
            if (listed && pos < kLbMaxList) out[pos] = (uint16_t)k;
            cnt += __popc(mask);
        }
        if (lane == 0) out[-1] = (uint16_t)(cnt > kLbMaxList ? kLbAll : cnt);
    }
}

}  // namespace

uint64_t lb_bytes(uint32_t nl, uint32_t res)
{
    const uint64_t cells = (uint64_t)nl * cells_for(res);
    return up(cells * kLbLine * sizeof(uint16_t)) + up(nl * sizeof(float)) + cone_bytes(res) + 256;
}

cudaError_t lb_build(const float4* sph, const float* radius, uint32_t n, const DevLight* lights, uint32_t nl,
                     uint32_t res, void* buf, uint64_t bytes, LightBufferView* out, cudaStream_t stream)
{
    if (nl == 0 || nl > kLbMaxLights || n == 0 || n > kLbMaxSpheres || res < kCellResMin || res > kCellResMax ||
        bytes < lb_bytes(nl, res))
        return cudaErrorInvalidValue;
    const uint64_t cells = (uint64_t)nl * cells_for(res);
    unsigned char* p = static_cast<unsigned char*>(buf);
    uint16_t* line = reinterpret_cast<uint16_t*>(p);
    p += up(cells * kLbLine * sizeof(uint16_t));
    float* dcap = reinterpret_cast<float*>(p);
    p += up(nl * sizeof(float));
    float4* cone = reinterpret_cast<float4*>(p);
    float* cone_sin = reinterpret_cast<float*>(p + up(cells_for(res) * sizeof(float4)));
    k_cell_cones<<<(cells_for(res) + 255) / 256, 256, 0, stream>>>(res, cone, cone_sin);
    k_lb_dcap<<<nl, 256, 0, stream>>>(sph, radius, n, lights, dcap);
    k_lb_build<<<(unsigned)((cells * 32 + 255) / 256), 256, 0, stream>>>(sph, radius, n, lights, nl, dcap, res,
                                                                       cone, cone_sin, line);
    out->line = line;
    out->dcap = dcap;
    out->n_lights = nl;
    out->res = res;
    return cudaGetLastError();
}

uint64_t db_bytes(uint32_t n, uint32_t res)
{
    const uint64_t cells = (uint64_t)n * cells_for(res);
    return up(cells * kLbLine * sizeof(uint16_t)) + up(n * sizeof(float)) + up(sizeof(float)) + cone_bytes(res) +
           256;
}

cudaError_t db_build(const float4* sph, const float* radius, uint32_t n, uint32_t res, void* buf, uint64_t bytes,
                     DirBufferView* out, cudaStream_t stream)
{
    if (n == 0 || n > kDbMaxSpheres || res < kCellResMin || res > kCellResMax || bytes < db_bytes(n, res))
        return cudaErrorInvalidValue;
    const uint64_t cells = (uint64_t)n * cells_for(res);
    unsigned char* p = static_cast<unsigned char*>(buf);
    uint16_t* line = reinterpret_cast<uint16_t*>(p);
    p += up(cells * kLbLine * sizeof(uint16_t));
    float* reach = reinterpret_cast<float*>(p);
    p += up(n * sizeof(float));
    float* ext = reinterpret_cast<float*>(p);
    p += up(sizeof(float));
    float4* cone = reinterpret_cast<float4*>(p);
    float* cone_sin = reinterpret_cast<float*>(p + up(cells_for(res) * sizeof(float4)));
    k_cell_cones<<<(cells_for(res) + 255) / 256, 256, 0, stream>>>(res, cone, cone_sin);
    k_db_extent<<<1, 256, 0, stream>>>(sph, radius, n, ext);
    k_db_reach<<<(n + 255) / 256, 256, 0, stream>>>(radius, n, ext, reach);
    k_db_build<<<n * 6u, 256, 0, stream>>>(sph, radius, n, reach, res, cone, cone_sin, line);
    out->line = line;
    out->reach = reach;
    out->n = n;
    out->res = res;
    return cudaGetLastError();
}

}  // namespace atx
