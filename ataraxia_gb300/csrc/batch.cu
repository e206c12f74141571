// Batched persistent path tracing: many scenes of uneven size, resolution and
// bounce depth in one launch.
//
// CTAs stay resident and pull work items (scene, tile of pixels) from a global
// counter; items are ordered by estimated cost, largest first.  A CTA that
// changes scene copies the scene descriptor to shared memory and, for scenes
// that fit, stages the sphere table there too; large scenes use their LBVH.
// Within an item each lane owns one pixel at a time and traces its samples in
// frame order, so the pixel's accumulator is updated in registers exactly as
// Renderer.cu:165 does frame after frame; a lane that finishes its pixel pulls
// the next pixel of the tile.  Every loop iteration is one bounce of the lane's
// current path (a finished path immediately starts the pixel's next sample),
// so lanes stay busy whatever their path lengths.  The nearest-hit and shadow
// queries of an iteration are shared by the whole warp (see the cooperative
// queries below), so a warp with few pending queries still uses all 32 lanes
// on them.  The primary hit of a pixel is traced once and reused by its samples
// (the primary ray depends on the pixel only).  Arithmetic and the random
// stream are those of the wavefront kernels, so results are bit-identical to
// rendering each scene alone.
#include <type_traits>

#include "batch.h"
#include "device_math.cuh"
#include "trace.cuh"

namespace atx {
namespace {

constexpr uint32_t kFull = 0xffffffffu;
constexpr int kThreads = 256;

// ------------------------------------------------ warp-cooperative queries
//
// In a loop iteration only some lanes of a warp need a nearest-hit (or shadow)
// query.  All 32 lanes share the work: with k queries pending, each query gets
// a group of g = 32/k lanes (rounded down to a power of two); lane r of a group
// tests spheres r, r+g, r+2g, ... of the scene, in increasing index order, and
// the group merges its partial results by (t, index).  Each sphere is tested
// once with the same float test as the brute-force loop, and the lexicographic
// (t, index) minimum is exactly the loop's answer (nearest t, lowest index on
// equal t), so results are bit-identical.  LBVH scenes keep one query per lane.

// Strided brute-force pieces over spheres first, first+stride, ...
template <bool SMEM>
__device__ __forceinline__ void strided_nearest(const float4* __restrict__ sph, uint32_t n, uint32_t first,
                                                uint32_t stride, float3 o, float3 d, float a, float& tm, int32_t& best)
{
    for (uint32_t i = first; i < n; i += stride) {
        const float4 s = SMEM ? sph[i] : __ldg(&sph[i]);
        const float ox = o.x - s.x, oy = o.y - s.y, oz = o.z - s.z;
        const float b = __fmaf_rn(oz, d.z, __fmaf_rn(oy, d.y, ox * d.x));
        const float cc = __fmaf_rn(oz, oz, __fmaf_rn(oy, oy, __fmaf_rn(ox, ox, -s.w)));
        const float disc = __fmaf_rn(b, b, -(a * cc));
        // candidate filter of candidate_bits (trace.cuh): sign of max(b, -disc)
        if ((int32_t)__float_as_uint(fmaxf(b, -disc)) < 0) {
            float t;
            if (sphere_t(s, o, d, a, t) && t > 0.0f && t < tm) {
                tm = t;
                best = (int32_t)i;
            }
        }
    }
}

template <bool SMEM>
__device__ __forceinline__ bool strided_occluded(const float4* __restrict__ sph, uint32_t n, uint32_t first,
                                                 uint32_t stride, float3 o, float3 d, float a, float dist2)
{
    for (uint32_t i = first; i < n; i += stride) {
        const float4 s = SMEM ? sph[i] : __ldg(&sph[i]);
        const float ox = o.x - s.x, oy = o.y - s.y, oz = o.z - s.z;
        const float b = __fmaf_rn(oz, d.z, __fmaf_rn(oy, d.y, ox * d.x));
        const float cc = __fmaf_rn(oz, oz, __fmaf_rn(oy, oy, __fmaf_rn(ox, ox, -s.w)));
        const float disc = __fmaf_rn(b, b, -(a * cc));
        if ((int32_t)__float_as_uint(fmaxf(b, -disc)) < 0) {
            float t;
            if (sphere_t(s, o, d, a, t) && t > 0.0f && t * t < dist2) return true;
        }
    }
    return false;
}

struct CoopGroup {
    unsigned mask;   // lanes with a query
    int g;           // lanes per query
    int q;           // query this lane helps with (>= k: idle)
    int owner;       // lane that owns query q
    bool work;
};

__device__ __forceinline__ CoopGroup coop_plan(bool need)
{
    CoopGroup c;
    c.mask = __ballot_sync(kFull, need);
    const int k = __popc(c.mask);
    int g = 32;
    while (g > 1 && g * k > 32) g >>= 1;
    c.g = g;
    const int lane = (int)(threadIdx.x & 31u);
    c.q = lane / g;
    c.work = k > 0 && c.q < k;
    c.owner = c.work ? (int)__fns(c.mask, 0, c.q + 1) : lane;
    return c;
}

template <int IS>
__device__ __forceinline__ void coop_nearest(const SceneView& sc, const float4* sph, bool need, float3 o, float3 d,
                                             float& t_out, int32_t& id_out)
{
    if (IS == kIsBvh) {
        if (need) id_out = bvh_nearest(sc, o, d, t_out);
        return;
    }
    const CoopGroup c = coop_plan(need);
    if (!c.mask) return;
    const float3 qo = mk3(__shfl_sync(kFull, o.x, c.owner), __shfl_sync(kFull, o.y, c.owner),
                          __shfl_sync(kFull, o.z, c.owner));
    const float3 qd = mk3(__shfl_sync(kFull, d.x, c.owner), __shfl_sync(kFull, d.y, c.owner),
                          __shfl_sync(kFull, d.z, c.owner));
    float tm = kFltMax;
    int32_t best = -1;
    if (c.work) {
        const uint32_t r = threadIdx.x & (uint32_t)(c.g - 1);
        strided_nearest<IS == kIsSmem>(sph, sc.n_sph, r, (uint32_t)c.g, qo, qd, dot3(qd, qd), tm, best);
    }
    for (int off = 1; off < c.g; off <<= 1) {
        const float t2 = __shfl_xor_sync(kFull, tm, off);
        const int32_t b2 = __shfl_xor_sync(kFull, best, off);
        if (b2 >= 0 && (best < 0 || t2 < tm || (t2 == tm && b2 < best))) {
            tm = t2;
            best = b2;
        }
    }
    const int lane = (int)(threadIdx.x & 31u);
    const int myq = __popc(c.mask & ((1u << lane) - 1u));
    const int leader = (myq * c.g) & 31;
    const float rt = __shfl_sync(kFull, tm, leader);
    const int32_t rb = __shfl_sync(kFull, best, leader);
    if (need) {
        t_out = rt;
        id_out = rb;
    }
}

template <int IS>
__device__ __forceinline__ bool coop_occluded(const SceneView& sc, const float4* sph, bool need, float3 o, float3 d,
                                              float dist2)
{
    if (IS == kIsBvh) return need && bvh_occluded(sc, o, d, dist2);
    const CoopGroup c = coop_plan(need);
    if (!c.mask) return false;
    const float3 qo = mk3(__shfl_sync(kFull, o.x, c.owner), __shfl_sync(kFull, o.y, c.owner),
                          __shfl_sync(kFull, o.z, c.owner));
    const float3 qd = mk3(__shfl_sync(kFull, d.x, c.owner), __shfl_sync(kFull, d.y, c.owner),
                          __shfl_sync(kFull, d.z, c.owner));
    const float qd2 = __shfl_sync(kFull, dist2, c.owner);
    bool hit = false;
    if (c.work) {
        const uint32_t r = threadIdx.x & (uint32_t)(c.g - 1);
        hit = strided_occluded<IS == kIsSmem>(sph, sc.n_sph, r, (uint32_t)c.g, qo, qd, dot3(qd, qd), qd2);
    }
    // OR within each group: a group's lanes are contiguous and aligned to g
    const unsigned hits = __ballot_sync(kFull, hit);
    const int lane = (int)(threadIdx.x & 31u);
    const int myq = __popc(c.mask & ((1u << lane) - 1u));
    const unsigned gmask = (c.g == 32) ? kFull : (((1u << c.g) - 1u) << ((myq * c.g) & 31));
    return need && (hits & gmask) != 0u;
}

// ---------------------------------------------------------------- one tile

template <int IS>
__device__ __forceinline__ void render_tile(const BatchSceneDev& S, const float4* s_sph, uint32_t tile,
                                            uint32_t* s_next_px, unsigned long long* rays)
{
    const SceneView& sc = S.sc;
    const float4* sph = (IS == kIsSmem) ? s_sph : sc.sph;
    const uint32_t W = S.cam.width, H = S.cam.height;
    const uint32_t tw = S.tile_w, th = S.tile_h;
    const uint32_t tx0 = (tile % S.tiles_x) * tw, ty0 = (tile / S.tiles_x) * th;
    const uint32_t tpx = tw * th;
    const uint32_t spp = S.spp;
    const int32_t B = S.max_bounces;
    const float3 cam_o = mk3(S.cam.pos[0], S.cam.pos[1], S.cam.pos[2]);
    const float fpack = __uint2float_rn(S.frame0 + spp - 1u);

    unsigned long long nq = 0, ns = 0;
    bool active = false;
    uint32_t p = 0, s = 0, seed = 0;
    int32_t bounce = 0, pid = -2;
    float pt = 0.0f;
    float3 o = cam_o, d = cam_o, dprim = cam_o, thr = cam_o, col = cam_o;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);

    // claims the next pixel of the tile; false when the tile is exhausted
    auto next_pixel = [&]() -> bool {
        for (;;) {
            const uint32_t l = atomicAdd(s_next_px, 1u);
            if (l >= tpx) return false;
            const uint32_t x = tx0 + l % tw, y = ty0 + l / tw;
            if (x >= W || y >= H) continue;
            p = x + y * W;
            acc = (S.frame0 == 1u) ? make_float4(0.f, 0.f, 0.f, 0.f) : S.accum[p];
            dprim = primary_dir(S.cam, x, y);
            s = 0;
            pid = -2;
            return true;
        }
    };
    auto start_sample = [&]() {
        o = cam_o;
        d = dprim;
        thr = mk3(1.f, 1.f, 1.f);
        col = mk3(0.f, 0.f, 0.f);
        bounce = 0;
        seed = p * (S.frame0 + s);
    };

    if (next_pixel()) {
        active = true;
        start_sample();
    }
    while (__any_sync(kFull, active)) {
        // phase 1: the nearest hit of every active path (cooperatively)
        bool traced = active && B > 0;
        if (traced) seed += (uint32_t)bounce;                        // Renderer.cu:306
        const bool need = traced && !(bounce == 0 && pid != -2);
        float tmin = pt;
        int32_t hit = pid;
        coop_nearest<IS>(sc, sph, need, o, d, tmin, hit);
        if (need) {
            ++nq;
            if (bounce == 0) {
                pt = tmin;
                pid = hit;
            }
        }
        // phase 2: shading and the shadow ray
        bool end_path = active && !traced;                           // max_bounces <= 0: empty path
        bool shadow = false;
        float3 pos = cam_o, nrm = cam_o, L = cam_o, le = cam_o, albedo = cam_o, base = cam_o;
        float dist2 = 0.0f, rough = 0.0f, metallic = 0.0f;
        if (traced) {
            if (hit < 0) {
                if (S.sky) col = add3(col, mul3(mk3(0.6f, 0.7f, 0.9f), thr));   // Renderer.cu:311-316
                end_path = true;
            } else {
                const float4 sv = (IS == kIsSmem) ? sph[hit] : __ldg(&sc.sph[hit]);
                ray_hit(sv, o, d, tmin, pos, nrm);
                const int32_t mi = __ldg(&sc.sph_mat[hit]);
                const float4* mrow = reinterpret_cast<const float4*>(sc.mat + mi);
                const float4 m0 = __ldg(mrow), m1 = __ldg(mrow + 1), m2 = __ldg(mrow + 2);
                albedo = mk3(m0.x, m0.y, m0.z);
                rough = m0.w;
                metallic = m1.w;
                if (m2.w > 0.0f) col = add3(col, mul3(mk3(m2.x, m2.y, m2.z), thr));   // Renderer.cu:329-333
                base = add3(muls3(mk3(m1.x, m1.y, m1.z), 1.0f - metallic), muls3(albedo, metallic));
                if (sc.n_lights > 0u) {                                  // Renderer.cu:338-352
                    const uint32_t li = pcg_hash(seed) % sc.n_lights;
                    const float4* lrow = reinterpret_cast<const float4*>(sc.lights + li);
                    const float4 l0 = __ldg(lrow), l1 = __ldg(lrow + 1);
                    L = sub3(mk3(l0.x, l0.y, l0.z), pos);
                    dist2 = dot3(L, L);
                    L = muls3(L, 1.0f / sqrtf(dist2));
                    le = mk3(l1.x, l1.y, l1.z);
                    shadow = true;
                    ++ns;
                }
            }
        }
        const float3 so = add3(pos, muls3(nrm, kOffset));
        const bool occluded = coop_occluded<IS>(sc, sph, shadow, so, L, dist2);
        // phase 3: light contribution, roulette, next direction
        if (traced && hit >= 0) {
            if (shadow && !occluded) {                                   // Renderer.cu:356-368
                const float3 f = cook_torrance(albedo, base, metallic, rough, nrm, neg3(d), L);
                col = add3(col, mul3(mul3(le, f), thr));
            }
            if (bounce + 1 >= B) {
                end_path = true;
            } else {                                                     // Renderer.cu:371-384
                thr = mul3(thr, albedo);
                o = so;
                const float prr = gmax(0.1f, gmin(1.0f, length3(thr)));
                if (pcg_float(seed) > prr) {
                    end_path = true;
                } else {
                    thr = divs3(thr, prr);
                    d = (metallic > 0.0f) ? sample_ggx(nrm, rough, seed) : sample_cosine(nrm, seed);
                    ++bounce;
                }
            }
        }
        if (end_path) {
            acc.x = acc.x + col.x;                                       // Renderer.cu:165
            acc.y = acc.y + col.y;
            acc.z = acc.z + col.z;
            acc.w = acc.w + 1.0f;
            ++s;
            if (pid == -1 || !traced) {
                // the pixel's primary ray missed (or no bounces): every remaining
                // sample has this same colour, 0 + sky * 1 or 0; add them in order
                const float3 m = (traced && S.sky) ? mk3(0.6f, 0.7f, 0.9f) : mk3(0.f, 0.f, 0.f);
                for (; s < spp; ++s) {
                    acc.x = acc.x + m.x;
                    acc.y = acc.y + m.y;
                    acc.z = acc.z + m.z;
                    acc.w = acc.w + 1.0f;
                }
            }
            if (s < spp) {
                start_sample();
            } else {
                S.accum[p] = acc;
                if (S.image) S.image[p] = pack_rgba8(acc, fpack);       // Renderer.cu:166-168
                if (next_pixel()) start_sample();
                else active = false;
            }
        }
    }
    // per-warp ray counts
    for (int off = 16; off > 0; off >>= 1) {
        nq += __shfl_xor_sync(kFull, nq, off);
        ns += __shfl_xor_sync(kFull, ns, off);
    }
    if ((threadIdx.x & 31u) == 0u && rays) {
        atomicAdd(&rays[0], nq);
        atomicAdd(&rays[1], ns);
    }
}

__global__ void __launch_bounds__(kThreads, 2) k_batch(BatchDev b)
{
    extern __shared__ float4 s_sph[];
    __shared__ BatchSceneDev s_scene;
    __shared__ uint32_t s_item, s_next_px;
    int32_t staged = -1;
    for (;;) {
        __syncthreads();   // everyone is done with the previous item and its shared state
        if (threadIdx.x == 0) {
            s_item = atomicAdd(b.next_item, 1u);
            s_next_px = 0u;
        }
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= b.n_items) return;
        const uint32_t si = __ldg(&b.item_scene[item]);
        if ((int32_t)si != staged) {
            if (threadIdx.x == 0) s_scene = b.scenes[si];
            __syncthreads();
            if (s_scene.mode == kIsSmem)
                for (uint32_t i = threadIdx.x; i < s_scene.sc.n_sph; i += blockDim.x) s_sph[i] = __ldg(&s_scene.sc.sph[i]);
            __syncthreads();
            staged = (int32_t)si;
        }
        const uint32_t tile = __ldg(&b.item_tile[item]);
        if (s_scene.mode == kIsSmem) render_tile<kIsSmem>(s_scene, s_sph, tile, &s_next_px, b.rays);
        else if (s_scene.mode == kIsBvh) render_tile<kIsBvh>(s_scene, s_sph, tile, &s_next_px, b.rays);
        else render_tile<kIsGlobal>(s_scene, s_sph, tile, &s_next_px, b.rays);
    }
}

}  // namespace

cudaError_t batch_plan(int device, int threads, uint32_t smem_spheres, BatchShape* out)
{
    if (threads <= 0 || threads > kThreads) threads = kThreads;
    int sms = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    const size_t bytes = (size_t)smem_spheres * sizeof(float4);
    if (bytes > 48 * 1024) {
        e = cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e != cudaSuccess) return e;
    }
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, threads, bytes);
    if (e != cudaSuccess) return e;
    out->blocks = sms * (per_sm > 0 ? per_sm : 1);
    out->threads = threads;
    out->smem = bytes;
    return cudaSuccess;
}

cudaError_t enqueue_batch(const BatchDev& b, const BatchShape& shape, cudaStream_t stream)
{
    if (b.n_items == 0) return cudaSuccess;
    k_batch<<<shape.blocks, shape.threads, shape.smem, stream>>>(b);
    return cudaGetLastError();
}

}  // namespace atx
