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

// Box tests of two slots of a 4-wide node (lbvh.cu k_pack_quads: rows r0..r2
// hold the two boxes interleaved) against the boxes inflated by M.
// Each packed f32x2 instruction rounds its two halves as the scalar
// instruction would, so the results are those of one scalar test per child.
// Sets t0/t1 to +inf when the slot is culled, else to its cull key
// w = ((tn - sl) - m) rounded down, tn the entry distance (may be negative
// when the origin is inside): w > limit' implies tn - sl > limit' + m, the
// test's own cull condition, for any later (smaller) limit', so a slot can be
// dropped by comparing its key with the nearest hit found since.  A slab the
// ray never enters (tn = +inf, where sl = +inf and tn - sl is NaN) is culled,
// so a key is finite or -inf.  no = -o; x - y is computed as x + (-y), or as
// fma(y, -1, x): both round the exact difference once.
__device__ __forceinline__ void bvh_boxes_enter(float4 r0, float4 r1, float4 r2, float3 no, float3 inv_d,
                                                float limit, float& t0, float& t1)
{
    const float2 dx = __fadd2_rn(make_float2(r0.x, r0.y), make_float2(no.x, no.x));
    const float2 dy = __fadd2_rn(make_float2(r0.z, r0.w), make_float2(no.y, no.y));
    const float2 dz = __fadd2_rn(make_float2(r1.x, r1.y), make_float2(no.z, no.z));
    const float2 hx = make_float2(r1.z, r1.w), hy = make_float2(r2.x, r2.y), hz = make_float2(r2.z, r2.w);
    const float2 ad = __fadd2_rn(__fadd2_rn(make_float2(fabsf(dx.x), fabsf(dx.y)), make_float2(fabsf(dy.x), fabsf(dy.y))),
                                 make_float2(fabsf(dz.x), fabsf(dz.y)));
    const float2 dmax = __fadd2_rn(ad, __fadd2_rn(__fadd2_rn(hx, hy), hz));
    const float2 m = __fmul2_rn(make_float2(kBvhK, kBvhK), __fadd2_rn(dmax, make_float2(1e-3f, 1e-3f)));
    const float2 ex = __fadd2_rn(hx, m), ey = __fadd2_rn(hy, m), ez = __fadd2_rn(hz, m);
    const float2 neg = make_float2(-1.0f, -1.0f);
    // slab distances; inv_d may be +-inf for zero components, where the
    // products give +-inf or NaN; fminf/fmaxf drop NaN operands.
    const float2 ix = make_float2(inv_d.x, inv_d.x), iy = make_float2(inv_d.y, inv_d.y),
                 iz = make_float2(inv_d.z, inv_d.z);
    const float2 tx0 = __fmul2_rn(__ffma2_rn(ex, neg, dx), ix), tx1 = __fmul2_rn(__fadd2_rn(dx, ex), ix);
    const float2 ty0 = __fmul2_rn(__ffma2_rn(ey, neg, dy), iy), ty1 = __fmul2_rn(__fadd2_rn(dy, ey), iy);
    const float2 tz0 = __fmul2_rn(__ffma2_rn(ez, neg, dz), iz), tz1 = __fmul2_rn(__fadd2_rn(dz, ez), iz);
    const float2 tn = make_float2(fmaxf(fmaxf(fminf(tx0.x, tx1.x), fminf(ty0.x, ty1.x)), fminf(tz0.x, tz1.x)),
                                  fmaxf(fmaxf(fminf(tx0.y, tx1.y), fminf(ty0.y, ty1.y)), fminf(tz0.y, tz1.y)));
    const float2 tf = make_float2(fminf(fminf(fmaxf(tx0.x, tx1.x), fmaxf(ty0.x, ty1.x)), fmaxf(tz0.x, tz1.x)),
                                  fminf(fminf(fmaxf(tx0.y, tx1.y), fmaxf(ty0.y, ty1.y)), fmaxf(tz0.y, tz1.y)));
    // slack on the slab distances themselves: relative 1e-5 of their size
    const float2 sl = __fadd2_rn(
        __fmul2_rn(make_float2(1e-5f, 1e-5f),
                   __fadd2_rn(make_float2(fabsf(tn.x), fabsf(tn.y)), make_float2(fabsf(tf.x), fabsf(tf.y)))),
        m);
    const float inf = __int_as_float(0x7f800000);
    const float e0 = tn.x - sl.x, e1 = tn.y - sl.y;
    const bool cull0 = !(tn.x < inf) || tf.x + sl.x < 0.0f || e0 > tf.x + sl.x || e0 > limit + m.x;
    const bool cull1 = !(tn.y < inf) || tf.y + sl.y < 0.0f || e1 > tf.y + sl.y || e1 > limit + m.y;
    t0 = cull0 ? inf : __fsub_rd(e0, m.x);
    t1 = cull1 ? inf : __fsub_rd(e1, m.y);
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

// A slot of a 4-wide node: true when its (ref, count) is well formed (a leaf
// cluster inside the sorted spheres, or an internal node index); empty slots
// (ref = ~0, count = 0) and malformed references are skipped.
__device__ __forceinline__ bool bvh_slot_ok(const BvhView& b, uint32_t ref, uint32_t count)
{
    return count ? (ref < b.n_leaves && count <= 32u) : ref < b.n_leaves - 1u;
}

// The four slot box tests of 4-wide node `node` (lbvh.cu k_pack_quads); a slot
// that is culled, empty or malformed gets t = +inf.
struct BvhSlots {
    float t0, t1, t2, t3;
    uint32_t r0, r1, r2, r3;
    uint32_t c0, c1, c2, c3;
};

__device__ __forceinline__ BvhSlots bvh_visit(const BvhView& b, uint32_t node, float3 no, float3 inv_d, float limit)
{
    const float4* p = b.quad + 8 * (size_t)node;
    const float4 q0 = __ldg(p), q1 = __ldg(p + 1), q2 = __ldg(p + 2), q3 = __ldg(p + 3);
    const float4 q4 = __ldg(p + 4), q5 = __ldg(p + 5), q6 = __ldg(p + 6), q7 = __ldg(p + 7);
    BvhSlots s;
    bvh_boxes_enter(q0, q1, q2, no, inv_d, limit, s.t0, s.t1);
    bvh_boxes_enter(q4, q5, q6, no, inv_d, limit, s.t2, s.t3);
    s.r0 = __float_as_uint(q3.x); s.r1 = __float_as_uint(q3.y);
    s.c0 = __float_as_uint(q3.z); s.c1 = __float_as_uint(q3.w);
    s.r2 = __float_as_uint(q7.x); s.r3 = __float_as_uint(q7.y);
    s.c2 = __float_as_uint(q7.z); s.c3 = __float_as_uint(q7.w);
    const float inf = __int_as_float(0x7f800000);
    if (!bvh_slot_ok(b, s.r0, s.c0)) s.t0 = inf;
    if (!bvh_slot_ok(b, s.r1, s.c1)) s.t1 = inf;
    if (!bvh_slot_ok(b, s.r2, s.c2)) s.t2 = inf;
    if (!bvh_slot_ok(b, s.r3, s.c3)) s.t3 = inf;
    return s;
}

__device__ __forceinline__ void bvh_order(float& ta, uint32_t& ra, uint32_t& ca, float& tb, uint32_t& rb,
                                          uint32_t& cb)
{
    if (tb < ta) {
        const float t = ta; ta = tb; tb = t;
        const uint32_t r = ra; ra = rb; rb = r;
        const uint32_t c = ca; ca = cb; cb = c;
    }
}

// Stack depth.  Each step pops one node and pushes at most four, all one
// 4-wide level down, so the stack holds at most three entries per level plus
// one.  A Karras tree over 30-bit codes made distinct by the sorted position
// is at most 30 + ceil(log2 n) binary levels deep, 62 for n = 2^32, so at most
// 31 4-wide levels: 94 entries.
constexpr int kBvhStack = 96;

__device__ __forceinline__ int32_t bvh_nearest(const SceneView& sc, float3 o, float3 d, float& tmin)
{
    const BvhView& b = sc.bvh;
    const float a = dot3(d, d);
    // tm must start finite: culled slots carry the key +inf, and the leaf loop
    // below ends at the first key beyond tm, so +inf here would run the leaf
    // test on culled clusters
    static_assert(kFltMax < __builtin_huge_valf(), "the nearest-hit walk's tm must start finite");
    float tm = kFltMax;
    int32_t best = -1;
    if (b.n_leaves < 2 || b.n_leaves <= b.leaf_size) {   // the whole tree is one cluster
        leaf_nearest(b, 0u, min(b.n_leaves, 32u), o, d, a, tm, best);
        tmin = tm;
        return best;
    }
    const float3 inv_d = safe_inv(d);
    const float3 no = mk3(-o.x, -o.y, -o.z);
    const float inf = __int_as_float(0x7f800000);
    uint32_t stack[kBvhStack];
    int sp = 0;
    stack[sp++] = b.root;
    // every internal node is visited at most once; the cap only guards
    // against a malformed tree
    uint32_t budget = 2u * b.n_leaves + 8u;
    while (sp > 0 && budget-- > 0u) {
        const uint32_t node = stack[--sp];
        if (node >= b.n_leaves - 1u) continue;
        BvhSlots s = bvh_visit(b, node, no, inv_d, tm);
        // slots in order of cull key (a sorting network), culled ones last
        bvh_order(s.t0, s.r0, s.c0, s.t1, s.r1, s.c1);
        bvh_order(s.t2, s.r2, s.c2, s.t3, s.r3, s.c3);
        bvh_order(s.t0, s.r0, s.c0, s.t2, s.r2, s.c2);
        bvh_order(s.t1, s.r1, s.c1, s.t3, s.r3, s.c3);
        bvh_order(s.t1, s.r1, s.c1, s.t2, s.r2, s.c2);
        // internal slots onto the stack, farthest first, so the nearest is popped next
        if (sp + 4 > kBvhStack) break;
        if (s.t3 < inf && s.c3 == 0u) stack[sp++] = s.r3;
        if (s.t2 < inf && s.c2 == 0u) stack[sp++] = s.r2;
        if (s.t1 < inf && s.c1 == 0u) stack[sp++] = s.r1;
        if (s.t0 < inf && s.c0 == 0u) stack[sp++] = s.r0;
        // leaf clusters, nearest first, until a hit found in an earlier one is
        // nearer than the next one's key (one copy of the leaf test, slots
        // shifted through it)
#pragma unroll 1
        for (int j = 0; j < 4 && s.t0 <= tm; ++j) {
            if (s.c0) leaf_nearest(b, s.r0, min(s.c0, b.n_leaves - s.r0), o, d, a, tm, best);
            s.t0 = s.t1; s.r0 = s.r1; s.c0 = s.c1;
            s.t1 = s.t2; s.r1 = s.r2; s.c1 = s.c2;
            s.t2 = s.t3; s.r2 = s.r3; s.c2 = s.c3;
            s.t3 = inf;
        }
    }
    tmin = tm;
    return best;
}

// Nearest hit among a tile's candidate list (sorted sphere indices, built by
// k_tile_lists for a cone that holds every lane's direction): the warp reads
// 32 entries at a time, one per lane, and hands each sphere to every lane by
// shuffle; the brute-force filter (leaf_candidates' arithmetic) and the exact
// test decide, and ties go to the lowest original index as in leaf_nearest,
// so the list's order does not matter.  All 32 lanes call it.
__device__ __forceinline__ int32_t nearest_listed(const BvhView& b, const uint32_t* __restrict__ list, uint32_t len,
                                                  float3 o, float3 d, bool me, float& tmin)
{
    const float a = dot3(d, d);
    const uint32_t lane = threadIdx.x & 31u;
    float tm = kFltMax;
    int32_t best = -1;
    for (uint32_t base = 0; base < len; base += 32u) {
        const uint32_t k = base + lane;
        const uint32_t s = k < len ? __ldg(&list[k]) : 0u;
        const float4 v = __ldg(&b.leaf_sph[s]);
        const uint32_t m = min(32u, len - base);
        for (uint32_t j = 0; j < m; ++j) {
            const float4 q = make_float4(__shfl_sync(0xffffffffu, v.x, j), __shfl_sync(0xffffffffu, v.y, j),
                                         __shfl_sync(0xffffffffu, v.z, j), __shfl_sync(0xffffffffu, v.w, j));
            const uint32_t sj = __shfl_sync(0xffffffffu, s, j);
            const float ox = o.x - q.x, oy = o.y - q.y, oz = o.z - q.z;
            const float bb = __fmaf_rn(oz, d.z, __fmaf_rn(oy, d.y, ox * d.x));
            const float cc = __fmaf_rn(oz, oz, __fmaf_rn(oy, oy, __fmaf_rn(ox, ox, -q.w)));
            const float h = __fmaf_rn(bb, -fabsf(bb), -(a * cc));
            float t;
            if (me && (__float_as_uint(h) >> 31) == 0u && sphere_t(q, o, d, a, t) && t > 0.0f) {
                const int32_t id = (int32_t)__ldg(&b.leaf_id[sj]);
                if (t < tm || (t == tm && best >= 0 && id < best)) {
                    tm = t;
                    best = id;
                }
            }
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
    const float3 no = mk3(-o.x, -o.y, -o.z);
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
        BvhSlots s = bvh_visit(b, node, no, inv_d, limit);
        // nearest slots first: a shadow ray leaves a surface, and its likeliest
        // occluders lie near its origin (any hit ends the query, so the order
        // changes only how soon)
        bvh_order(s.t0, s.r0, s.c0, s.t1, s.r1, s.c1);
        bvh_order(s.t2, s.r2, s.c2, s.t3, s.r3, s.c3);
        bvh_order(s.t0, s.r0, s.c0, s.t2, s.r2, s.c2);
        bvh_order(s.t1, s.r1, s.c1, s.t3, s.r3, s.c3);
        bvh_order(s.t1, s.r1, s.c1, s.t2, s.r2, s.c2);
        if (sp + 4 > kBvhStack) break;
        if (s.t3 < inf && s.c3 == 0u) stack[sp++] = s.r3;
        if (s.t2 < inf && s.c2 == 0u) stack[sp++] = s.r2;
        if (s.t1 < inf && s.c1 == 0u) stack[sp++] = s.r1;
        if (s.t0 < inf && s.c0 == 0u) stack[sp++] = s.r0;
#pragma unroll 1
        for (int j = 0; j < 4 && s.t0 < inf; ++j) {
            if (s.c0 && leaf_occluded(b, s.r0, min(s.c0, b.n_leaves - s.r0), o, d, a, dist2))
                return true;
            s.t0 = s.t1; s.r0 = s.r1; s.c0 = s.c1;
            s.t1 = s.t2; s.r1 = s.r2; s.c1 = s.c2;
            s.t2 = s.t3; s.r2 = s.r3; s.c2 = s.c3;
            s.t3 = inf;
        }
    }
    return false;
}

}  // namespace atx
