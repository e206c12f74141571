// Nearest-hit and any-hit traversal of the linear BVH (built by lbvh.cu) that
// return exactly what the brute-force loop returns (Renderer.cu:251-285 and
// the shadow test at :351-352).
//
// Exactness argument.  Leaves run the same float test as the brute-force loop
// (sphere_t), so any sphere the traversal reaches yields the same t.  It
// remains to never cull a sphere whose float test would be accepted.  For a
// ray origin o and sphere centre c with |o - c| = D, the float half-b test
// (three roundings per fused term, a = |d|^2 within 1e-6 of 1) computes its
// discriminant within 16 eps D^2 of the exact one (eps = 2^-24), so an accepted
// sphere is passed by the exact ray within r + 4 sqrt(eps) D of its centre,
// and its float t is at least the exact entry distance minus 4.5 sqrt(eps) D.
// A node box is therefore inflated by M = K (D_max + 1e-3) with
// K = 5 sqrt(eps) = 1.2207e-3 and D_max bounded by the L1 distance from o to
// the box centre plus the L1 half extent, and a node is culled only when the
// ray misses the inflated box or enters it beyond tmin + M.  Ties on t are
// broken toward the lower original sphere index, as the strict '<' of the
// brute-force loop does.
#pragma once

#include "device_math.cuh"
#include "wavefront.h"

namespace atx {

constexpr float kBvhK = 1.2207031e-3f;
constexpr int kBvhStack = 64;

// Node box test against the box inflated by M.  Returns the entry distance
// (may be negative when the origin is inside) or +inf when culled.
__device__ __forceinline__ float bvh_box_enter(float4 ctr, float4 half, float3 o, float3 inv_d, float limit)
{
    const float dx = ctr.x - o.x, dy = ctr.y - o.y, dz = ctr.z - o.z;
    const float dmax = (fabsf(dx) + fabsf(dy) + fabsf(dz)) + (half.x + half.y + half.z);
    const float m = kBvhK * (dmax + 1e-3f);
    const float hx = half.x + m, hy = half.y + m, hz = half.z + m;
    // slab distances; inv_d may be +-inf for zero components, where the
    // products give +-inf or NaN; fminf/fmaxf drop NaN operands.
    const float tx0 = (dx - hx) * inv_d.x, tx1 = (dx + hx) * inv_d.x;
    const float ty0 = (dy - hy) * inv_d.y, ty1 = (dy + hy) * inv_d.y;
    const float tz0 = (dz - hz) * inv_d.z, tz1 = (dz + hz) * inv_d.z;
    const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
    const float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
    // slack on the slab distances themselves: relative 1e-5 of their size
    const float sl = 1e-5f * (fabsf(tn) + fabsf(tf)) + m;
    if (tf + sl < 0.0f || tn - sl > tf + sl || tn - sl > limit + m) return __int_as_float(0x7f800000);
    return tn;
}

__device__ __forceinline__ float3 safe_inv(float3 d)
{
    return mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
}

// Candidate bits of the leaf cluster [first, first + cnt) (1 <= cnt <= 32):
// bit k set unless sphere first + k certainly misses, with the brute-force
// loop's filter and arithmetic (trace.cuh candidate_bits: the sign of
// h = fma(b, -|b|, -(a*c)), clear for every sphere the exact test can
// accept), so candidates are decided by the same exact test.
__device__ __forceinline__ uint32_t leaf_candidates(const BvhView& b, uint32_t first, uint32_t cnt, float3 o,
                                                    float3 d, float a)
{
    uint32_t mask = 0u;
    for (uint32_t k = 0; k < cnt; ++k) {
        const float4 s = __ldg(&b.leaf_sph[first + k]);
        const float ox = o.x - s.x, oy = o.y - s.y, oz = o.z - s.z;
        const float bb = __fmaf_rn(oz, d.z, __fmaf_rn(oy, d.y, ox * d.x));
        const float cc = __fmaf_rn(oz, oz, __fmaf_rn(oy, oy, __fmaf_rn(ox, ox, -s.w)));
        const float h = __fmaf_rn(bb, -fabsf(bb), -(a * cc));
        mask = __funnelshift_l(__float_as_uint(h), mask, 1);   // sphere k at bit cnt-1-k
    }
    return __brev(~mask << (32u - cnt));   // sphere k at bit k
}

__device__ __forceinline__ void leaf_nearest(const BvhView& b, uint32_t first, uint32_t cnt, float3 o, float3 d,
                                             float a, float& tm, int32_t& best)
{
    uint32_t mask = leaf_candidates(b, first, cnt, o, d, a);
    while (mask) {
        const uint32_t k = (uint32_t)(__ffs(mask) - 1);
        mask &= mask - 1u;
        float t;
        if (sphere_t(__ldg(&b.leaf_sph[first + k]), o, d, a, t) && t > 0.0f) {
            const int32_t id = (int32_t)__ldg(&b.leaf_id[first + k]);
            if (t < tm || (t == tm && best >= 0 && id < best)) {
                tm = t;
                best = id;
            }
        }
    }
}

__device__ __forceinline__ bool leaf_occluded(const BvhView& b, uint32_t first, uint32_t cnt, float3 o, float3 d,
                                              float a, float dist2)
{
    uint32_t mask = leaf_candidates(b, first, cnt, o, d, a);
    while (mask) {
        const uint32_t k = (uint32_t)(__ffs(mask) - 1);
        mask &= mask - 1u;
        float t;
        if (sphere_t(__ldg(&b.leaf_sph[first + k]), o, d, a, t) && t > 0.0f && t * t < dist2) return true;
    }
    return false;
}

// A child of a child-pair node: (ref, count) decoded and bounds-checked.
// Returns 1 for a leaf cluster (first, cnt set), 2 for an internal node,
// 0 for a malformed reference (skipped).
__device__ __forceinline__ int bvh_child(const BvhView& b, uint32_t ref, uint32_t count, uint32_t& first,
                                         uint32_t& cnt)
{
    if (count) {
        if (ref >= b.n_leaves || count > 32u) return 0;
        first = ref;
        cnt = min(count, b.n_leaves - ref);
        return 1;
    }
    return ref < b.n_leaves - 1u ? 2 : 0;
}

__device__ __forceinline__ int32_t bvh_nearest(const SceneView& sc, float3 o, float3 d, float& tmin)
{
    const BvhView& b = sc.bvh;
    const float a = dot3(d, d);
    float tm = kFltMax;
    int32_t best = -1;
    if (b.n_leaves < 2 || b.n_leaves <= b.leaf_size) {   // the whole tree is one cluster
        leaf_nearest(b, 0u, min(b.n_leaves, 32u), o, d, a, tm, best);
        tmin = tm;
        return best;
    }
    const float3 inv_d = safe_inv(d);
    const float inf = __int_as_float(0x7f800000);
    uint32_t stack[kBvhStack];
    int sp = 0;
    stack[sp++] = b.root;
    // every internal node is pushed at most once; the cap only guards against
    // a malformed tree
    uint32_t budget = 2u * b.n_leaves + 8u;
    while (sp > 0 && budget-- > 0u) {
        const uint32_t node = stack[--sp];
        if (node >= b.n_leaves - 1u) continue;
        const float4* p = b.pair + 4 * (size_t)node;
        const float4 c0 = __ldg(p), h0 = __ldg(p + 1), c1 = __ldg(p + 2), h1 = __ldg(p + 3);
        const float t0 = bvh_box_enter(c0, h0, o, inv_d, tm);
        const float t1 = bvh_box_enter(c1, h1, o, inv_d, tm);
        uint32_t f0 = 0, n0 = 0, f1 = 0, n1 = 0;
        int k0 = t0 < inf ? bvh_child(b, __float_as_uint(c0.w), __float_as_uint(h0.w), f0, n0) : 0;
        int k1 = t1 < inf ? bvh_child(b, __float_as_uint(c1.w), __float_as_uint(h1.w), f1, n1) : 0;
        // leaf clusters at once, nearer first; internal children onto the stack
        if (k0 == 1 && k1 == 1 && t1 < t0) {
            leaf_nearest(b, f1, n1, o, d, a, tm, best);
            leaf_nearest(b, f0, n0, o, d, a, tm, best);
            k0 = k1 = 0;
        }
        if (k0 == 1) {
            leaf_nearest(b, f0, n0, o, d, a, tm, best);
            k0 = 0;
        }
        if (k1 == 1) {
            leaf_nearest(b, f1, n1, o, d, a, tm, best);
            k1 = 0;
        }
        const uint32_t r0 = __float_as_uint(c0.w), r1 = __float_as_uint(c1.w);
        if (k0 == 2 && k1 == 2) {
            // push the farther child first so the nearer one is popped next
            if (sp + 2 > kBvhStack) break;
            if (t0 <= t1) { stack[sp++] = r1; stack[sp++] = r0; }
            else          { stack[sp++] = r0; stack[sp++] = r1; }
        } else if (k0 == 2 || k1 == 2) {
            if (sp + 1 > kBvhStack) break;
            stack[sp++] = k0 == 2 ? r0 : r1;
        }
    }
    tmin = tm;
    return best;
}

__device__ __forceinline__ bool bvh_occluded(const SceneView& sc, float3 o, float3 d, float dist2)
{
    const BvhView& b = sc.bvh;
    const float a = dot3(d, d);
    if (b.n_leaves < 2 || b.n_leaves <= b.leaf_size) return leaf_occluded(b, 0u, min(b.n_leaves, 32u), o, d, a, dist2);
    const float3 inv_d = safe_inv(d);
    const float inf = __int_as_float(0x7f800000);
    // any accepted t has t*t < dist2, so t < sqrt(dist2) (1 + 2^-22)
    const float limit = sqrtf(dist2) * 1.0000003f;
    uint32_t stack[kBvhStack];
    int sp = 0;
    stack[sp++] = b.root;
    uint32_t budget = 2u * b.n_leaves + 8u;
    while (sp > 0 && budget-- > 0u) {
        const uint32_t node = stack[--sp];
        if (node >= b.n_leaves - 1u) continue;
        const float4* p = b.pair + 4 * (size_t)node;
        const float4 c0 = __ldg(p), h0 = __ldg(p + 1), c1 = __ldg(p + 2), h1 = __ldg(p + 3);
        uint32_t f0 = 0, n0 = 0, f1 = 0, n1 = 0;
        const int k0 = bvh_box_enter(c0, h0, o, inv_d, limit) < inf
                           ? bvh_child(b, __float_as_uint(c0.w), __float_as_uint(h0.w), f0, n0) : 0;
        const int k1 = bvh_box_enter(c1, h1, o, inv_d, limit) < inf
                           ? bvh_child(b, __float_as_uint(c1.w), __float_as_uint(h1.w), f1, n1) : 0;
        if (k0 == 1 && leaf_occluded(b, f0, n0, o, d, a, dist2)) return true;
        if (k1 == 1 && leaf_occluded(b, f1, n1, o, d, a, dist2)) return true;
        if (sp + 2 > kBvhStack) break;
        if (k0 == 2) stack[sp++] = __float_as_uint(c0.w);
        if (k1 == 2) stack[sp++] = __float_as_uint(c1.w);
    }
    return false;
}

}  // namespace atx
