// Device arithmetic of the path: vector helpers, the PCG stream, sin/cos of
// 2*pi*u, the ray-sphere test, Cook-Torrance and the two samplers.
//
// Numerics contract.  Every file that includes this header is compiled with
// -fmad=false and without fast math, so a*b+c rounds twice unless it is
// written __fmaf_rn(), division and sqrtf are IEEE round-to-nearest and there
// is no flush to zero.  Fused operations are used in exactly four places:
// vector dot products (z*z' + (y*y' + x*x')), the half-b ray-sphere quadratic,
// the sincos polynomial and the quarter-turn reduction.  Three quotients are
// regrouped: a vector divided by a scalar is multiplied by the scalar's IEEE
// reciprocal (the tangent frame, the roulette's throughput), the diffuse term
// multiplies by 1/pi rounded to float, and the specular term's D * G / denom
// is one quotient.  Everything else evaluates the reference's expressions as
// written (BRDF.cu, Renderer.cu), so a CPU evaluation in the same order gives
// the same bits.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace atx {

#define ATX_HD __host__ __device__ __forceinline__

ATX_HD float3 mk3(float x, float y, float z) { return make_float3(x, y, z); }
ATX_HD float3 add3(float3 a, float3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
ATX_HD float3 sub3(float3 a, float3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
ATX_HD float3 mul3(float3 a, float3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
ATX_HD float3 muls3(float3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
// a / s as a * (1 / s): one IEEE division for the three components
ATX_HD float3 mul_rcp3(float3 a, float s)
{
    const float r = 1.0f / s;
    return mk3(a.x * r, a.y * r, a.z * r);
}
ATX_HD float3 neg3(float3 a) { return mk3(-a.x, -a.y, -a.z); }

__device__ __forceinline__ float dot3(float3 a, float3 b)
{
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, a.x * b.x));
}
// glm::normalize: v * (1 / sqrt(dot(v, v)))
__device__ __forceinline__ float3 normalize3(float3 v) { return muls3(v, 1.0f / sqrtf(dot3(v, v))); }
__device__ __forceinline__ float length3(float3 v) { return sqrtf(dot3(v, v)); }
ATX_HD float3 cross3(float3 a, float3 b)
{
    return mk3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
// glm::max(a, b) = (a < b) ? b : a ; glm::min(a, b) = (b < a) ? b : a
ATX_HD float gmax(float a, float b) { return (a < b) ? b : a; }
ATX_HD float gmin(float a, float b) { return (b < a) ? b : a; }

// Random.h:59-64.  The PCG output permutation applied to one LCG step; it
// returns the hash and leaves its argument alone.
ATX_HD uint32_t pcg_hash(uint32_t seed)
{
    uint32_t state = seed * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

// Random.h:66-70.  float(UINT32_MAX) is 2^32, so the division is an exact
// scaling by 2^-32 of the round-to-nearest conversion.
__device__ __forceinline__ float pcg_float(uint32_t& seed)
{
    seed = pcg_hash(seed);
    return __uint2float_rn(seed) * 2.3283064365386963e-10f;
}

// cos(2*pi*u), sin(2*pi*u).  Exact reduction to w = u - rint(u) - q/4 with
// |w| <= 1/8, then the Maclaurin series of sin/cos(2*pi*w) with coefficients
// (2*pi)^k/k! rounded to float, by Horner's rule in fused multiply-adds, then
// a rotation by q quarter turns.
__device__ __forceinline__ void sincos_2pi(float u, float& c, float& s)
{
    float v = u - rintf(u);
    float q = rintf(v * 4.0f);
    float w = __fmaf_rn(q, -0.25f, v);
    float w2 = w * w;
    float ps = __fmaf_rn(w2, 0x1.507834p+5f, -0x1.32d2ccp+6f);
    ps = __fmaf_rn(w2, ps, 0x1.466bc6p+6f);
    ps = __fmaf_rn(w2, ps, -0x1.4abbcep+5f);
    ps = __fmaf_rn(w2, ps, 0x1.921fb6p+2f);
    float sn = w * ps;
    float pc = __fmaf_rn(w2, -0x1.a6d1f2p+4f, 0x1.e1f506p+5f);
    pc = __fmaf_rn(w2, pc, -0x1.55d3c8p+6f);
    pc = __fmaf_rn(w2, pc, 0x1.03c1f0p+6f);
    pc = __fmaf_rn(w2, pc, -0x1.3bd3ccp+4f);
    float cs = __fmaf_rn(w2, pc, 1.0f);
    int qi = ((int)q) & 3;
    float cc = (qi == 0) ? cs : (qi == 1) ? -sn : (qi == 2) ? -cs : sn;
    float ss = (qi == 0) ? sn : (qi == 1) ? cs : (qi == 2) ? -sn : -cs;
    c = cc;
    s = ss;
}

constexpr float kPi = 0x1.921fb6p+1f;   // glm::pi<float>()
constexpr float kInvPi = 1.0f / kPi;    // rounded to float
constexpr float kOffset = 0.0001f;      // Renderer.cu:348, :372
constexpr float kFltMax = 3.402823466e+38f;

// One ray-sphere test in half-b form.  The reference (Renderer.cu:260-272)
// solves a t^2 + b t + c = 0 with b = 2 dot(oc, d) and keeps the smaller root;
// dividing through by 2 gives t = (-b' - sqrt(b'^2 - a c)) / a with
// b' = dot(oc, d), the same root.  Returns false when the discriminant is
// negative.  sph = (cx, cy, cz, radius*radius).
__device__ __forceinline__ bool sphere_t(float4 sph, float3 o, float3 d, float a, float& t)
{
    float ox = o.x - sph.x, oy = o.y - sph.y, oz = o.z - sph.z;
    float b = __fmaf_rn(oz, d.z, __fmaf_rn(oy, d.y, ox * d.x));
    float cc = __fmaf_rn(oz, oz, __fmaf_rn(oy, oy, __fmaf_rn(ox, ox, -sph.w)));
    float disc = __fmaf_rn(b, b, -(a * cc));
    if (disc < 0.0f) return false;
    t = -(b + sqrtf(disc)) / a;
    return true;
}

// Renderer.cu:396-409: position and normalised normal at t.
__device__ __forceinline__ void ray_hit(float4 sph, float3 o, float3 d, float t, float3& pos, float3& nrm)
{
    float3 c = mk3(sph.x, sph.y, sph.z);
    float3 p = add3(sub3(o, c), muls3(d, t));
    nrm = normalize3(p);
    pos = add3(p, c);
}

// BRDF.cu:9-34 with fresnelSchlick (:36-40), distributionGGX (:42-53) and
// geometrySmith / geometrySchlickGGX (:55-70) inlined.  The specular term
// F * (D * G) / denom, D = a2 / den and G = ndotv / g_v * ndotl / g_l, is
// evaluated as F * X with X = (a2 * ndotv * ndotl) / (den * g_v * g_l * denom):
// one division for five.  The factors stay in range for roughness >= 1e-4
// (den >= pi a2^2, g >= 1/8, denom >= 0.001), so the regrouping changes X by
// a few units in the last place; the diffuse term's / pi is * (1 / pi).

__device__ __forceinline__ float3 cook_torrance(float3 albedo, float3 f0, float metallic, float rough, float3 n,
                                                float3 v, float3 l)
{
    float3 h = normalize3(add3(v, l));
    float ndotl = gmax(dot3(n, l), 1e-7f);
    float ndotv = gmax(dot3(n, v), 1e-7f);
    float ndoth = gmax(dot3(n, h), 0.0f);
    float vdoth = gmax(dot3(v, h), 0.0f);

    float ct = gmin(gmax(vdoth, 0.0f), 1.0f);
    float m = 1.0f - ct;
    float m2 = m * m;
    float m4 = m2 * m2;
    float p5 = m4 * m;
    float3 F = mk3(f0.x + (1.0f - f0.x) * p5, f0.y + (1.0f - f0.y) * p5, f0.z + (1.0f - f0.z) * p5);

    const float a = rough * rough;
    const float a2 = a * a;
    float nh2 = ndoth * ndoth;
    float den = nh2 * (a2 - 1.0f) + 1.0f;
    den = kPi * den * den;
    const float r = rough + 1.0f;
    const float k = (r * r) * 0.125f;
    const float gv = ndotv * (1.0f - k) + k;
    const float gl = ndotl * (1.0f - k) + k;
    float denom = 4.0f * ndotl * ndotv + 0.001f;
    const float X = ((a2 * ndotv) * ndotl) / (((den * gv) * gl) * denom);

    float3 one_f = sub3(mk3(1.0f, 1.0f, 1.0f), F);
    float3 kd = muls3(one_f, 1.0f - metallic);
    float3 spec = muls3(F, X);
    float3 diffuse = muls3(mul3(one_f, albedo), kInvPi);
    return muls3(add3(mul3(kd, diffuse), spec), ndotl);
}

// BRDF.cu:84-90 / :108-114
__device__ __forceinline__ void tangent_frame(float3 n, float3& t, float3& b)
{
    if (fabsf(n.x) > fabsf(n.y))
        t = mul_rcp3(mk3(-n.z, 0.0f, n.x), sqrtf(n.x * n.x + n.z * n.z));
    else
        t = mul_rcp3(mk3(0.0f, -n.z, n.y), sqrtf(n.y * n.y + n.z * n.z));
    b = cross3(n, t);
}

__device__ __forceinline__ float3 to_world(float x, float y, float z, float3 t, float3 b, float3 n)
{
    return add3(add3(muls3(t, x), muls3(b, y)), muls3(n, z));
}

// BRDF.cu:72-93
__device__ __forceinline__ float3 sample_cosine(float3 n, uint32_t& seed)
{
    const float u1 = pcg_float(seed);
    const float u2 = pcg_float(seed);
    const float r = sqrtf(u1);
    float c, s;
    sincos_2pi(u2, c, s);
    const float x = r * c;
    const float y = r * s;
    const float z = sqrtf(1.0f - u1);
    float3 t, b;
    tangent_frame(n, t, b);
    return to_world(x, y, z, t, b, n);
}

// BRDF.cu:95-117: the sampled half vector is returned as the new direction.
__device__ __forceinline__ float3 sample_ggx(float3 n, float rough, uint32_t& seed)
{
    const float u1 = pcg_float(seed);
    const float u2 = pcg_float(seed);
    const float a = rough * rough;
    const float cos_t = sqrtf((1.0f - u1) / (1.0f + (a * a - 1.0f) * u1));
    const float sin_t = sqrtf(1.0f - cos_t * cos_t);
    float c, s;
    sincos_2pi(u2, c, s);
    float3 t, b;
    tangent_frame(n, t, b);
    return to_world(sin_t * c, sin_t * s, cos_t, t, b, n);
}

// Renderer.cu:381-384: the next direction, sample_ggx for a metallic surface
// and sample_cosine otherwise, with their shared steps written once: only the
// polar terms differ (GGX: sin and cos of the sampled half-vector angle;
// cosine: sqrt(u1) and sqrt(1 - u1)), so a warp whose lanes take both kinds
// runs the random numbers, the sin/cos of 2*pi*u2, the tangent frame and the
// change of basis once.  Every value is computed as in the two functions.
__device__ __forceinline__ float3 sample_next(float3 n, float rough, float metallic, uint32_t& seed)
{
    const float u1 = pcg_float(seed);
    const float u2 = pcg_float(seed);
    float radial, z;
    if (metallic > 0.0f) {
        const float a = rough * rough;
        const float cos_t = sqrtf((1.0f - u1) / (1.0f + (a * a - 1.0f) * u1));
        radial = sqrtf(1.0f - cos_t * cos_t);
        z = cos_t;
    } else {
        radial = sqrtf(u1);
        z = sqrtf(1.0f - u1);
    }
    float c, s;
    sincos_2pi(u2, c, s);
    float3 t, b;
    tangent_frame(n, t, b);
    return to_world(radial * c, radial * s, z, t, b, n);
}

// Renderer.cu:166-168 + Renderer.h:70-78: accum / frame, clamp to [0, 1],
// truncating x*255 per channel, packed A<<24 | B<<16 | G<<8 | R.
__device__ __forceinline__ uint32_t pack_rgba8(float4 acc, float frame)
{
    float v[4] = { acc.x / frame, acc.y / frame, acc.z / frame, acc.w / frame };
    uint32_t ch[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float x = v[i] < 0.0f ? 0.0f : v[i];
        x = x > 1.0f ? 1.0f : x;
        float s = x * 255.0f;
        ch[i] = (s == s) ? (uint32_t)s : 0u;
    }
    return (ch[3] << 24) | (ch[2] << 16) | (ch[1] << 8) | ch[0];
}

}  // namespace atx
