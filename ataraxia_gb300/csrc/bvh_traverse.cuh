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

__device__ __forceinline__ int32_t bvh_nearest(const SceneView& sc, float3 o, float3 d, float& tmin)
{
    const BvhView& b = sc.bvh;
    const float a = dot3(d, d);
    const float3 inv_d = safe_inv(d);
    float tm = kFltMax;
    int32_t best = -1;
    const uint32_t n_int = b.n_leaves - 1u;
    uint32_t stack[kBvhStack];
    int sp = 0;
    stack[sp++] = b.root;
    // a tree visits each of its 2n-1 nodes at most once; the cap only guards
    // against a malformed tree
    uint32_t budget = 2u * b.n_leaves + 8u;
    while (sp > 0 && budget-- > 0u) {
        const uint32_t node = stack[--sp];
        if (node >= n_int + b.n_leaves) continue;
        uint32_t first, last;
        if (node >= n_int) {
            first = last = node - n_int;
        } else {
            const uint2 r = __ldg(&b.node_range[node]);
            first = r.x;
            last = r.y < b.n_leaves ? r.y : b.n_leaves - 1u;   // never read past the leaves
        }
        if (last - first + 1u <= b.leaf_size || node >= n_int) {
            for (uint32_t k = first; k <= last; ++k) {
                float t;
                if (sphere_t(__ldg(&b.leaf_sph[k]), o, d, a, t) && t > 0.0f) {
                    const int32_t id = (int32_t)__ldg(&b.leaf_id[k]);
                    if (t < tm || (t == tm && best >= 0 && id < best)) {
                        tm = t;
                        best = id;
                    }
                }
            }
            continue;
        }
        const float4 cl = __ldg(&b.node_ctr[node]);
        const float4 hl = __ldg(&b.node_half[node]);
        const uint32_t left = __float_as_uint(cl.w);
        const uint32_t right = __float_as_uint(hl.w);
        if (left >= n_int + b.n_leaves || right >= n_int + b.n_leaves) continue;   // malformed: skip
        const float4 c0 = __ldg(&b.node_ctr[left]), h0 = __ldg(&b.node_half[left]);
        const float4 c1 = __ldg(&b.node_ctr[right]), h1 = __ldg(&b.node_half[right]);
        const float t0 = bvh_box_enter(c0, h0, o, inv_d, tm);
        const float t1 = bvh_box_enter(c1, h1, o, inv_d, tm);
        const bool v0 = t0 < __int_as_float(0x7f800000);
        const bool v1 = t1 < __int_as_float(0x7f800000);
        if (v0 && v1) {
            // push the farther child first so the nearer one is popped next
            if (sp + 2 > kBvhStack) break;
            if (t0 <= t1) { stack[sp++] = right; stack[sp++] = left; }
            else          { stack[sp++] = left;  stack[sp++] = right; }
        } else if (v0 || v1) {
            if (sp + 1 > kBvhStack) break;
            stack[sp++] = v0 ? left : right;
        }
    }
    tmin = tm;
    return best;
}

__device__ __forceinline__ bool bvh_occluded(const SceneView& sc, float3 o, float3 d, float dist2)
{
    const BvhView& b = sc.bvh;
    const float a = dot3(d, d);
    const float3 inv_d = safe_inv(d);
    // any accepted t has t*t < dist2, so t < sqrt(dist2) (1 + 2^-22)
    const float limit = sqrtf(dist2) * 1.0000003f;
    const uint32_t n_int = b.n_leaves - 1u;
    uint32_t stack[kBvhStack];
    int sp = 0;
    stack[sp++] = b.root;
    // a tree visits each of its 2n-1 nodes at most once; the cap only guards
    // against a malformed tree
    uint32_t budget = 2u * b.n_leaves + 8u;
    while (sp > 0 && budget-- > 0u) {
        const uint32_t node = stack[--sp];
        if (node >= n_int + b.n_leaves) continue;
        uint32_t first, last;
        if (node >= n_int) {
            first = last = node - n_int;
        } else {
            const uint2 r = __ldg(&b.node_range[node]);
            first = r.x;
            last = r.y < b.n_leaves ? r.y : b.n_leaves - 1u;   // never read past the leaves
        }
        if (last - first + 1u <= b.leaf_size || node >= n_int) {
            for (uint32_t k = first; k <= last; ++k) {
                float t;
                if (sphere_t(__ldg(&b.leaf_sph[k]), o, d, a, t) && t > 0.0f && t * t < dist2) return true;
            }
            continue;
        }
        const float4 cl = __ldg(&b.node_ctr[node]);
        const float4 hl = __ldg(&b.node_half[node]);
        const uint32_t left = __float_as_uint(cl.w);
        const uint32_t right = __float_as_uint(hl.w);
        if (left >= n_int + b.n_leaves || right >= n_int + b.n_leaves) continue;   // malformed: skip
        const float4 c0 = __ldg(&b.node_ctr[left]), h0 = __ldg(&b.node_half[left]);
        const float4 c1 = __ldg(&b.node_ctr[right]), h1 = __ldg(&b.node_half[right]);
        const bool v0 = bvh_box_enter(c0, h0, o, inv_d, limit) < __int_as_float(0x7f800000);
        const bool v1 = bvh_box_enter(c1, h1, o, inv_d, limit) < __int_as_float(0x7f800000);
        if (sp + 2 > kBvhStack) break;
        if (v0) stack[sp++] = left;
        if (v1) stack[sp++] = right;
    }
    return false;
}

}  // namespace atx
