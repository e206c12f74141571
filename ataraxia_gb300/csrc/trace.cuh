// Device-side tracing used by the wavefront kernels (wavefront.cu) and the
// allocation-free entry point (noalloc.cu): primary directions, the
// brute-force nearest / any hit over a sphere table and their dispatch to the
// LBVH.
#pragma once

#include <cstdint>

#include "bvh_traverse.cuh"
#include "device_math.cuh"
#include "wavefront.h"

namespace atx {

// Nearest-hit structure a kernel instantiation is compiled for.
enum : int { kIsGlobal = 0, kIsSmem = 1, kIsBvh = 2 };

// Camera.cpp:173-187 for pixel (x, y): NDC without a pixel-centre offset, y = 0
// the bottom row; target = invProj * (cx, cy, 1, 1); direction =
// normalize(invView * (normalize(target.xyz / target.w), 0)).  The reference
// computes these on the host in IEEE single precision without contraction
// (Camera::UpdateRayDirection), so this evaluates the same expressions in the
// same order with nothing fused: matrix-vector products as pairwise column
// sums, and the two normalisations with dot products (x*x + y*y) + z*z.  The
// directions are then the reference's host-computed ones bit for bit.
__device__ __forceinline__ float3 normalize3_host(float3 v)
{
    const float d = (v.x * v.x + v.y * v.y) + v.z * v.z;
    return muls3(v, 1.0f / sqrtf(d));
}

__device__ __forceinline__ float3 primary_dir(const CameraView& cam, uint32_t x, uint32_t y)
{
    const float qx = __uint2float_rn(x) / __uint2float_rn(cam.width);
    const float qy = __uint2float_rn(y) / __uint2float_rn(cam.height);
    const float cx = qx * 2.0f - 1.0f;
    const float cy = qy * 2.0f - 1.0f;
    float t[4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
        t[r] = (cam.inv_proj[r] * cx + cam.inv_proj[4 + r] * cy) + (cam.inv_proj[8 + r] + cam.inv_proj[12 + r]);
    const float3 tv = normalize3_host(mk3(t[0] / t[3], t[1] / t[3], t[2] / t[3]));
    float dv[3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
        dv[r] = (cam.inv_view[r] * tv.x + cam.inv_view[4 + r] * tv.y) +
                (cam.inv_view[8 + r] * tv.z + cam.inv_view[12 + r] * 0.0f);
    return normalize3_host(mk3(dv[0], dv[1], dv[2]));
}

// The shared-memory sphere table in pair layout: spheres 2j and 2j+1 share
// the float4s at 2j and 2j+1, {-x0, -x1, -y0, -y1} and {-z0, -z1, -w0, -w1}
// (w = r^2).  One packed f32x2 instruction then does an operation for both
// spheres, with the same IEEE rounding per component as the scalar one, and
// the negated centres let a packed add form o - c exactly (x + (-y) is x - y).
// For an odd count the last pair repeats its sphere; its second half is never
// a candidate (candidate_bits masks it).
__device__ __forceinline__ void stage_spheres(const SceneView& sc, float4* s)
{
    const uint32_t n = sc.n_sph, np = (n + 1u) >> 1;
    for (uint32_t j = threadIdx.x; j < np; j += blockDim.x) {
        const float4 p = __ldg(&sc.sph[2u * j]);
        const float4 q = 2u * j + 1u < n ? __ldg(&sc.sph[2u * j + 1u]) : p;
        s[2u * j] = make_float4(-p.x, -q.x, -p.y, -q.y);
        s[2u * j + 1u] = make_float4(-p.z, -q.z, -p.w, -q.w);
    }
    __syncthreads();
}

// Bytes of the pair-layout table for n spheres.
__host__ __device__ constexpr size_t smem_table_bytes(uint32_t n)
{
    return (size_t)((n + 1u) & ~1u) * 16u;
}

// Sphere i (x, y, z, r^2) of the pair-layout table.
__device__ __forceinline__ float4 smem_sphere(const float4* s, uint32_t i)
{
    const float4 p = s[i & ~1u], q = s[i | 1u];
    const bool odd = (i & 1u) != 0u;
    return make_float4(-(odd ? p.y : p.x), -(odd ? p.w : p.z), -(odd ? q.y : q.x), -(odd ? q.w : q.z));
}

// Sphere i of a kernel's table: the shared-memory pair layout or the plain
// global array.
template <bool SMEM>
__device__ __forceinline__ float4 table_sphere(const float4* __restrict__ sph, uint32_t i)
{
    return SMEM ? smem_sphere(sph, i) : __ldg(&sph[i]);
}

// Candidate bits of up to 32 spheres starting at base.  The exact test
// (sphere_t) accepts a sphere only when its discriminant disc = b*b - a*c is
// >= 0 and its half-b term b is < 0: with b >= 0 the root -(b + sqrt(disc))/a
// is <= 0 and fails t > 0.  The filter computes h = fma(b, -|b|, -(a*c)) and
// marks a sphere when h's sign bit is clear.  For b < 0, -|b| = b, so h is the
// exact test's discriminant (same operations, same rounding) and the sphere is
// marked exactly when disc >= 0, +0 included.  For b >= 0, h = -b*b - a*c,
// marked only when c <= 0 (origin inside or on the sphere): a few extra
// candidates, which the exact test then rejects.  So candidates are a
// superset of the accepted spheres and results equal the plain loop's.  The
// cheap pass has no branches, which keeps the square root and the IEEE
// division out of the inner loop.  Each sphere shifts h's sign bit in from the
// right (one funnel shift) and the word is inverted once at the end, so
// sphere base+k ends at bit 31-k: the highest set bit is the lowest index.
// CNT is 32 for a full chunk, 31 for a partial one of cnt spheres.  EXIT:
// a partial chunk leaves the unrolled loop after its last sphere instead of
// stepping over the rest (k_fused, whose small tables are one partial chunk;
// elsewhere the guarded form compiles to the better code for full chunks).
template <bool SMEM, int CNT, bool EXIT = false>
__device__ __forceinline__ uint32_t candidate_bits(const float4* __restrict__ sph, uint32_t base, float3 o, float3 d,
                                                   float a, uint32_t cnt)
{
    uint32_t mask = 0u;
    if (SMEM) {
        // pair layout, base even: b, c and h of two spheres per packed
        // instruction, in the order of the scalar branch below
        const float2 ox = make_float2(o.x, o.x), oy = make_float2(o.y, o.y), oz = make_float2(o.z, o.z);
        const float2 dx = make_float2(d.x, d.x), dy = make_float2(d.y, d.y), dz = make_float2(d.z, d.z);
        const float2 na = make_float2(-a, -a);
        const uint32_t np = CNT == 32 ? 16u : (cnt + 1u) >> 1;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            if (EXIT && CNT != 32 && (uint32_t)k >= np) break;
            if (CNT == 32 || (uint32_t)k < np) {
                const float4 p = sph[base + 2u * k], q = sph[base + 2u * k + 1u];
                const float2 vx = __fadd2_rn(ox, make_float2(p.x, p.y));
                const float2 vy = __fadd2_rn(oy, make_float2(p.z, p.w));
                const float2 vz = __fadd2_rn(oz, make_float2(q.x, q.y));
                const float2 b = __ffma2_rn(vz, dz, __ffma2_rn(vy, dy, __fmul2_rn(vx, dx)));
                const float2 cc = __ffma2_rn(vz, vz, __ffma2_rn(vy, vy, __ffma2_rn(vx, vx, make_float2(q.z, q.w))));
                const float2 h = __ffma2_rn(b, make_float2(-fabsf(b.x), -fabsf(b.y)), __fmul2_rn(na, cc));
                mask = __funnelshift_l(__float_as_uint(h.x), mask, 1);
                mask = __funnelshift_l(__float_as_uint(h.y), mask, 1);
            }
        }
        mask = ~mask;
        // align the first sphere to bit 31 and drop an odd count's repeat
        if (CNT != 32) mask = (mask << (32u - 2u * np)) & ~(0xffffffffu >> cnt);
        return mask;
    }
#pragma unroll
    for (int k = 0; k < CNT; ++k) {
        if (EXIT && CNT != 32 && (uint32_t)k >= cnt) break;
        if (CNT == 32 || (uint32_t)k < cnt) {
            const float4 s = __ldg(&sph[base + k]);
            const float ox = o.x - s.x, oy = o.y - s.y, oz = o.z - s.z;
            const float b = __fmaf_rn(oz, d.z, __fmaf_rn(oy, d.y, ox * d.x));
            const float cc = __fmaf_rn(oz, oz, __fmaf_rn(oy, oy, __fmaf_rn(ox, ox, -s.w)));
            const float h = __fmaf_rn(b, -fabsf(b), -(a * cc));
            mask = __funnelshift_l(__float_as_uint(h), mask, 1);
        }
    }
    mask = ~mask;
    if (CNT != 32) mask <<= (32u - cnt);   // align the first sphere to bit 31
    return mask;
}

// Renderer.cu:256-279: brute-force nearest hit, lowest index on equal t.
template <bool SMEM, bool EXIT = false>
__device__ __forceinline__ int32_t nearest_brute(const float4* __restrict__ sph, uint32_t n, float3 o, float3 d,
                                                 float& tmin)
{
    const float a = dot3(d, d);
    int32_t best = -1;
    float tm = kFltMax;
    for (uint32_t base = 0; base < n; base += 32u) {
        const uint32_t cnt = n - base;
        uint32_t mask = cnt >= 32u ? candidate_bits<SMEM, 32>(sph, base, o, d, a, 32u)
                                   : candidate_bits<SMEM, 31, EXIT>(sph, base, o, d, a, cnt);
        while (mask) {
            const uint32_t k = (uint32_t)__clz(mask);   // lowest sphere index first (ties keep it)
            mask &= ~(0x80000000u >> k);
            const uint32_t i = base + k;
            float t;
            if (sphere_t(table_sphere<SMEM>(sph, i), o, d, a, t) && t > 0.0f && t < tm) {
                tm = t;
                best = (int32_t)i;
            }
        }
    }
    tmin = tm;
    return best;
}

// Renderer.cu:351-352 as an any-hit query.  The reference takes the nearest
// hit and tests t > 0 && t*t < dist2; since the nearest accepted t is <= every
// accepted t and squaring is monotone, that equals "some sphere has t > 0 and
// t*t < dist2", so the loop can stop at the first such sphere.
template <bool SMEM, bool EXIT = false>
__device__ __forceinline__ bool occluded_brute(const float4* __restrict__ sph, uint32_t n, float3 o, float3 d,
                                               float dist2)
{
    const float a = dot3(d, d);
    for (uint32_t base = 0; base < n; base += 32u) {
        const uint32_t cnt = n - base;
        uint32_t mask = cnt >= 32u ? candidate_bits<SMEM, 32>(sph, base, o, d, a, 32u)
                                   : candidate_bits<SMEM, 31, EXIT>(sph, base, o, d, a, cnt);
        while (mask) {
            const uint32_t k = (uint32_t)__clz(mask);
            mask &= ~(0x80000000u >> k);
            const uint32_t i = base + k;
            float t;
            if (sphere_t(table_sphere<SMEM>(sph, i), o, d, a, t) && t > 0.0f && t * t < dist2) return true;
        }
    }
    return false;
}

// ------------------------------------------------------------- warp cones
//
// Rays of one warp that leave one apex in a narrow cone of directions: the
// primary rays of 32 neighbouring pixels (apex: the camera), and the
// first-bounce shadow rays of neighbouring hit points towards one light, seen
// from the light.  The warp tests every sphere once against the cone of its
// active lanes' directions and the lanes run the exact test only on the
// spheres that pass, in index order; results equal the brute-force loop's.
//
// Exactness.  A sphere the float test accepts for a ray from o is passed by
// the exact ray within r + 4 sqrt(eps) D of its centre, D = |o - c|, at a ray
// parameter above -4.5 sqrt(eps) D (the bound the LBVH walk uses, bvh_traverse
// .cuh).  The cone test inflates the radius by m = kBvhK (D + 1e-3) >=
// 5 sqrt(eps) (D + 1e-3), plus an absolute e for shadow rays (their 1e-4
// surface offset bends the segment from the light), and passes a sphere whose
// inflated ball meets the cone, or whose centre lies within R + m of the apex
// (an acceptance just behind the apex).  Every bound below errs towards
// passing: cos of the half-angle from below, sines from above, a relative
// 1e-5 slack on the final comparison.
struct WarpCone {
    float3 u;       // unit axis
    float cos_lo;   // <= cos(half-angle)
    float sin_hi;   // >= sin(half-angle)
};

// The cone of the unit directions w of the lanes with me set (at least one).
// All 32 lanes call it; the butterfly sums and minimum leave the same bits on
// every lane, so the result is warp-uniform.  False when the cone is too
// wide to pay (cos(half-angle) below 0.5) or a direction is not finite.
__device__ __forceinline__ bool warp_cone(bool me, float3 w, WarpCone& c)
{
    float sx = me ? w.x : 0.0f, sy = me ? w.y : 0.0f, sz = me ? w.z : 0.0f;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, off);
        sy += __shfl_xor_sync(0xffffffffu, sy, off);
        sz += __shfl_xor_sync(0xffffffffu, sz, off);
    }
    const float inv = rsqrtf(sx * sx + sy * sy + sz * sz);   // approximate: cos_lo is measured against this u
    c.u = mk3(sx * inv, sy * inv, sz * inv);
    float cmin = me ? dot3(w, c.u) : 2.0f;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) cmin = fminf(cmin, __shfl_xor_sync(0xffffffffu, cmin, off));
    c.cos_lo = cmin - 1e-5f;
    if (!(c.cos_lo > 0.5f)) return false;
    c.sin_hi = sqrtf(fmaxf(0.0f, 1.0f - c.cos_lo * c.cos_lo)) + 1e-6f;
    return true;
}

// Whether a sphere (centre at v from the apex, radius r) may be hit by a ray
// of the cone.  extra: added to |v| for the origin-to-centre distance D of the
// margin; e: absolute inflation.  Approximate reciprocal square roots (a few
// ulp) are covered by the relative slacks.
__device__ __forceinline__ bool cone_meets(const WarpCone& c, float3 v, float r, float extra, float e)
{
    const float d2 = dot3(v, v);
    const float inv = rsqrtf(d2);
    const float dist = d2 * inv;
    const float m = kBvhK * (dist + extra + 1e-3f);
    const float R = r * 1.00001f + m + e;
    if (!(dist > R + m)) return true;   // also a centre at the apex (dist NaN)
    const float sb = R * inv * 1.0001f;   // >= sin(beta), beta = asin(R / dist)
    // cos(theta + beta) >= cos(theta) (1 - sin^2 beta) - sin(theta) sin(beta),
    // since cos(beta) >= cos^2(beta) = 1 - sin^2(beta)
    const float rhs = c.cos_lo * (1.0f - sb * sb) - c.sin_hi * sb;
    return dot3(v, c.u) >= dist * (rhs - 1e-5f);
}

// Radius of a sphere from its r^2, rounded up by more than the error of the
// approximate square root (r^2 = 0 gives NaN, which passes every cone test).
__device__ __forceinline__ float cone_radius(float r2)
{
    return r2 * rsqrtf(r2) * 1.000001f;
}

// Nearest hit of the rays (o, d) of the lanes with me set, all leaving the
// apex o (the same on every lane) inside cone c.  All 32 lanes call it.
template <bool SMEM>
__device__ __forceinline__ int32_t nearest_cone(const float4* __restrict__ sph, uint32_t n, float3 o, float3 d, bool me,
                                                const WarpCone& c, float& tmin)
{
    const float a = dot3(d, d);
    const uint32_t lane = threadIdx.x & 31u;
    int32_t best = -1;
    float tm = kFltMax;
    for (uint32_t base = 0; base < n; base += 32u) {
        bool pass = false;
        if (base + lane < n) {
            const float4 s = table_sphere<SMEM>(sph, base + lane);
            pass = cone_meets(c, mk3(s.x - o.x, s.y - o.y, s.z - o.z), cone_radius(s.w), 0.0f, 0.0f);
        }
        uint32_t mask = __ballot_sync(0xffffffffu, pass);
        while (mask) {   // lowest index first: ties keep it, as in the brute-force loop
            const uint32_t i = base + (uint32_t)(__ffs(mask) - 1);
            mask &= mask - 1u;
            float t;
            if (me && sphere_t(table_sphere<SMEM>(sph, i), o, d, a, t) && t > 0.0f && t < tm) {
                tm = t;
                best = (int32_t)i;
            }
        }
    }
    tmin = tm;
    return best;
}

// nearest_cone with the candidates read from a tile mask row (words words,
// bit i % 32 of word i / 32 for sphere i) built with the same cone test for
// a cone that contains every lane's direction: the same candidates or more,
// each decided by the same exact test in the same index order.
template <bool SMEM>
__device__ __forceinline__ int32_t nearest_masked(const float4* __restrict__ sph, const uint32_t* __restrict__ row,
                                                  uint32_t words, float3 o, float3 d, bool me, float& tmin)
{
    const float a = dot3(d, d);
    int32_t best = -1;
    float tm = kFltMax;
    for (uint32_t w = 0; w < words; ++w) {
        uint32_t mask = __ldg(&row[w]);
        while (mask) {   // lowest index first: ties keep it, as in the brute-force loop
            const uint32_t i = 32u * w + (uint32_t)(__ffs(mask) - 1);
            mask &= mask - 1u;
            float t;
            if (me && sphere_t(table_sphere<SMEM>(sph, i), o, d, a, t) && t > 0.0f && t < tm) {
                tm = t;
                best = (int32_t)i;
            }
        }
    }
    tmin = tm;
    return best;
}

// Any hit for the shadow rays (o, d, dist2) of the lanes with me set, whose
// segments end near the light at apex; c is the cone of the directions from
// the apex to the origins and dmax the largest apex-to-origin distance.  All
// 32 lanes call it.
template <bool SMEM>
__device__ __forceinline__ bool occluded_cone(const float4* __restrict__ sph, uint32_t n, float3 o, float3 d,
                                              float dist2, bool me, float3 apex, const WarpCone& c, float dmax)
{
    const float a = dot3(d, d);
    const uint32_t lane = threadIdx.x & 31u;
    bool occ = false;
    for (uint32_t base = 0; base < n; base += 32u) {
        bool pass = false;
        if (base + lane < n) {
            const float4 s = table_sphere<SMEM>(sph, base + lane);
            // D <= |c - apex| + dmax; the segment's bend (1e-4 offset, float
            // error of the direction) stays within 2e-4 + kBvhK dmax
            pass = cone_meets(c, mk3(s.x - apex.x, s.y - apex.y, s.z - apex.z), cone_radius(s.w), 2.0f * dmax, 2e-4f);
        }
        uint32_t mask = __ballot_sync(0xffffffffu, pass);
        while (mask) {
            const uint32_t i = base + (uint32_t)(__ffs(mask) - 1);
            mask &= mask - 1u;
            float t;
            if (me && !occ && sphere_t(table_sphere<SMEM>(sph, i), o, d, a, t) && t > 0.0f && t * t < dist2)
                occ = true;
        }
        if (__all_sync(0xffffffffu, occ || !me)) break;
    }
    return occ;
}

// ------------------------------------------------------------ light buffer

// Cell of direction w around a light, as light_buffer.cu lays out the cube:
// the face of the largest |component| (+x, -x, +y, -y, +z, -z), then the other
// two components over it (in [-1, 1]) on a res x res grid.  -1 for a zero or
// non-finite w.
__device__ __forceinline__ int lb_cell(float3 w, uint32_t res)
{
    const float ax = fabsf(w.x), ay = fabsf(w.y), az = fabsf(w.z);
    uint32_t face;
    float m, a, b;
    if (ax >= ay && ax >= az) {
        face = w.x >= 0.0f ? 0u : 1u;
        m = ax, a = w.y, b = w.z;
    } else if (ay >= az) {
        face = w.y >= 0.0f ? 2u : 3u;
        m = ay, a = w.x, b = w.z;
    } else {
        face = w.z >= 0.0f ? 4u : 5u;
        m = az, a = w.x, b = w.y;
    }
    if (!(m > 0.0f && m < 3.0e38f) || !(fabsf(a) <= m && fabsf(b) <= m)) return -1;
    const float h = 0.5f * (float)res / m;
    const int i = min((int)((a + m) * h), (int)res - 1);
    const int j = min((int)((b + m) * h), (int)res - 1);
    return (int)((face * res + (uint32_t)i) * res + (uint32_t)j);
}

// The spheres of a cell line (words 1..count after the count in word 0):
// calls f(i) for each in ascending order until f returns true, and returns
// whether one did.  The count and the first seven indices come in one 16-byte
// load (h, already loaded); the rest, for longer lists, word by word.
template <class F>
__device__ __forceinline__ bool walk_line(const uint16_t* line, uint4 h, uint32_t cnt, F&& f)
{
    // words 1..7 of h as a 112-bit window, consumed 16 bits at a time
    uint64_t lo = (((uint64_t)h.y << 32) | h.x) >> 16 | ((uint64_t)h.z << 48);
    uint64_t hi = (((uint64_t)h.w << 32) | h.z) >> 16;
    const uint32_t first = cnt < 7u ? cnt : 7u;
    for (uint32_t k = 0; k < first; ++k) {
        if (f((uint32_t)(lo & 0xffffu))) return true;
        lo = (lo >> 16) | (hi << 48);
        hi >>= 16;
    }
    for (uint32_t k = 7; k < cnt; ++k)
        if (f((uint32_t)__ldg(&line[1 + k]))) return true;
    return false;
}

// Any hit for a shadow ray (o, d, dist2) towards light li: the spheres the
// light buffer lists for the cell of o seen from the light, or the whole table
// when that cell overflowed, o lies beyond the buffer's reach or the
// direction is degenerate.
template <bool SMEM>
__device__ __forceinline__ bool occluded_lb(const SceneView& sc, const float4* __restrict__ sph, uint32_t li, float3 o,
                                            float3 d, float dist2)
{
    const float4 l0 = __ldg(reinterpret_cast<const float4*>(sc.lights + li));
    const float3 w = mk3(o.x - l0.x, o.y - l0.y, o.z - l0.z);
    const float dc = __ldg(&sc.lb.dcap[li]);
    const int cell = dot3(w, w) <= dc * dc ? lb_cell(w, sc.lb.res) : -1;
    if (cell < 0) return occluded_brute<SMEM>(sph, sc.n_sph, o, d, dist2);
    const uint16_t* line = sc.lb.line + ((size_t)li * cells_for(sc.lb.res) + (uint32_t)cell) * kLbLine;
    const uint4 h = __ldg(reinterpret_cast<const uint4*>(line));
    const uint32_t cnt = h.x & 0xffffu;
    if (cnt == kLbAll) return occluded_brute<SMEM>(sph, sc.n_sph, o, d, dist2);
    const float a = dot3(d, d);
    return walk_line(line, h, cnt, [&](uint32_t i) {
        float t;
        return sphere_t(table_sphere<SMEM>(sph, i), o, d, a, t) && t > 0.0f && t * t < dist2;
    });
}

// Nearest hit of an extension ray leaving sphere own: the spheres the
// direction buffer lists for own and the cell of d, in index order (ties keep
// the lowest index, as in the brute-force loop), or the whole table when own
// is not covered (~0u: also when the ray's origin lay beyond own's reach,
// which the shading that made the ray checks), the cell overflowed or d is
// degenerate.
template <bool SMEM>
__device__ __forceinline__ int32_t nearest_db(const SceneView& sc, const float4* __restrict__ sph, uint32_t own,
                                              float3 o, float3 d, float& tmin)
{
    const int cell = own < sc.db.n ? lb_cell(d, sc.db.res) : -1;
    if (cell < 0) return nearest_brute<SMEM>(sph, sc.n_sph, o, d, tmin);
    const uint16_t* line = sc.db.line + ((size_t)own * cells_for(sc.db.res) + (uint32_t)cell) * kLbLine;
    const uint4 h = __ldg(reinterpret_cast<const uint4*>(line));
    const uint32_t cnt = h.x & 0xffffu;
    if (cnt == kLbAll) return nearest_brute<SMEM>(sph, sc.n_sph, o, d, tmin);
    const float a = dot3(d, d);
    int32_t best = -1;
    float tm = kFltMax;
    walk_line(line, h, cnt, [&](uint32_t i) {
        float t;
        if (sphere_t(table_sphere<SMEM>(sph, i), o, d, a, t) && t > 0.0f && t < tm) {
            tm = t;
            best = (int32_t)i;
        }
        return false;
    });
    tmin = tm;
    return best;
}

// Whether the direction buffer's lists of sphere own hold for a ray leaving
// from o (within reach of own's centre c).
__device__ __forceinline__ bool db_reaches(const SceneView& sc, uint32_t own, float4 c, float3 o)
{
    if (own >= sc.db.n) return false;
    const float3 e = mk3(o.x - c.x, o.y - c.y, o.z - c.z);
    const float reach = __ldg(&sc.db.reach[own]);
    return dot3(e, e) <= reach * reach;
}

template <int IS, bool EXIT = false>
__device__ __forceinline__ int32_t scene_nearest(const SceneView& sc, const float4* sph, float3 o, float3 d,
                                                 float& tmin)
{
    if (IS == kIsBvh) return bvh_nearest(sc, o, d, tmin);
    return nearest_brute<IS == kIsSmem, EXIT>(sph, sc.n_sph, o, d, tmin);
}

// Nearest hit of a ray leaving sphere own (~0u: from elsewhere).
template <int IS>
__device__ __forceinline__ int32_t scene_nearest_from(const SceneView& sc, const float4* sph, uint32_t own, float3 o,
                                                      float3 d, float& tmin)
{
    if (IS != kIsBvh && sc.db.n != 0u) return nearest_db<IS == kIsSmem>(sc, sph, own, o, d, tmin);
    return scene_nearest<IS>(sc, sph, o, d, tmin);
}

template <int IS, bool EXIT = false>
__device__ __forceinline__ bool scene_occluded(const SceneView& sc, const float4* sph, float3 o, float3 d,
                                               float dist2)
{
    if (IS == kIsBvh) return bvh_occluded(sc, o, d, dist2);
    return occluded_brute<IS == kIsSmem, EXIT>(sph, sc.n_sph, o, d, dist2);
}

}  // namespace atx
