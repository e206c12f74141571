// Wavefront path tracer for sm_103a: the reference's per-pixel loop
// (Renderer.cu:287-387) split into queue-driven stages.
//
//   k_primary        primary nearest hit once per pixel (Camera.cpp:161-195
//                    for the ray), shared by the pixel's samples; queues the
//                    first bounce's (pixel, light) shadow rays.
//   k_first          bounce 0 over (hit pixel, sample): shading, light pick
//                    and the shadow ray, Russian roulette and the next
//                    direction.  Survivors go to the extension queue.
//   k_bounce         bounce b >= 1 (LBVH scenes): nearest hit, then the same
//                    shading, with the block's hits gathered in shared memory
//                    first.
//   With a light buffer and a direction buffer (scenes up to 1,024 spheres)
//   shadow rays are tested right after the shading and a continuation ray is
//   traced where it is made, so only rays that hit are queued:
//   k_shade          bounce 1: shades its queue of hits on full warps.
//   k_paths          bounces >= 2 in one persistent launch: each block
//                    carries a pool of paths to the end.
//   k_shadow         any-hit over a shadow queue: the first bounce's (pixel,
//                    light) rays, and per-sample shadow rays of LBVH scenes.
//   k_accumulate     adds the wave's per-sample colours to the float4
//                    accumulator in frame order (Renderer.cu:165) and packs
//                    the RGBA8 image (Renderer.cu:166-168).
//
// Queues are filled through warp-aggregated atomics.  Order of the colour
// sums is the reference's: emission of bounce b, light of bounce b, then
// bounce b+1.  Each path owns its colour row, so no float atomics are needed
// and results do not depend on queue order.  The random stream is consumed
// per path exactly as the reference does: seed += b at the top of the bounce,
// PcgHash(seed) (no advance) for the light, one PcgFloat for roulette and two
// for the new direction.
#include <type_traits>

#include "wavefront.h"
#include "device_math.cuh"
#include "trace.cuh"

namespace atx {
namespace {

constexpr uint32_t kFull = 0xffffffffu;
constexpr int kThreads = 256;
// k_first's and k_bounce's block: the shading code sets the register count.
// 4 blocks of 256 threads per SM (64 registers) beat 6 of 192 (56 registers)
// and 3 of 256 (80 registers) on the medium scene.
constexpr int kExtendThreads = 256;
constexpr int kExtendBlocksPerSm = 4;
// With a light buffer, bounces from this one on run in one persistent k_paths
// launch instead of a k_bounce launch each.
constexpr int kPathsFrom = 2;

// k_shadow's blocks per SM: the shared-memory variant fits 40 registers
// without spilling (6 blocks of 256 threads); the others take up to 64 (4).
// k_fused's blocks per SM (whole paths in one thread: 64 registers).
constexpr int kFusedBlocksPerSm = 4;

template <int IS>
constexpr int kShadowBlocksPerSm = IS == kIsSmem ? 6 : 4;

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// One atomicAdd per warp; pushing lanes receive consecutive slots in lane order.
// Must be reached by all 32 lanes of the warp.
__device__ __forceinline__ uint32_t warp_push(uint32_t* counter, bool pred)
{
    const unsigned mask = __ballot_sync(kFull, pred);
    if (mask == 0u) return 0u;
    const uint32_t lane = lane_id();
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0u;
    if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(kFull, base, leader);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

// Adds every lane's n to *counter with one atomicAdd per warp.  Must be
// reached by all 32 lanes of the warp.
__device__ __forceinline__ void warp_push_n(uint32_t* counter, uint32_t n)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) n += __shfl_xor_sync(kFull, n, off);
    if (lane_id() == 0u && n) atomicAdd(counter, n);
}

// The primary direction of wave pixel p: from the camera's per-pixel table
// when it has one (the same function filled it), else computed.
__device__ __forceinline__ float3 primary_ray(const CameraView& cam, uint32_t p)
{
    if (cam.dirs) {
        const float4 v = __ldg(&cam.dirs[p]);
        return mk3(v.x, v.y, v.z);
    }
    return primary_dir(cam, p % cam.width, p / cam.width);
}

// Renderer.cu:339: the light a shading point samples, PcgHash(seed) % lights
// (the seed is not advanced), the remainder by multiplication (fastmod).
__device__ __forceinline__ uint32_t light_pick(const SceneView& sc, uint32_t seed)
{
    const uint64_t low = sc.light_mod * (uint64_t)pcg_hash(seed);
    return (uint32_t)__umul64hi(low, (uint64_t)sc.n_lights);
}

// Renderer.cu:339-348: light li's parameter row, the unit direction L from pos
// to the light and the squared distance.  One function for the first bounce
// and the per-(pixel, light) shadow rays, so both compute the same floats.
__device__ __forceinline__ float4 light_dir(const SceneView& sc, uint32_t li, float3 pos, float3& L, float& dist2)
{
    const float4* lrow = reinterpret_cast<const float4*>(sc.lights + li);
    const float4 l0 = __ldg(lrow), l1 = __ldg(lrow + 1);
    L = sub3(mk3(l0.x, l0.y, l0.z), pos);
    dist2 = dot3(L, L);
    L = muls3(L, 1.0f / sqrtf(dist2));
    return l1;
}

// Primary nearest hit once per pixel of the wave (shared by its samples).
// With the brute-force tables a warp's 32 neighbouring primary rays share the
// camera as apex and a narrow cone of directions, so the warp culls the
// sphere table against the cone first (nearest_cone).
// With per-(pixel, light) shadow rays (wave_light_vis) it also clears the
// pixel's visibility word, stores at the pixel's hit slot the hit point with
// its sphere and the shadow-ray origin with the pixel, and queues in q[0], as
// bounce 0's shadow rays, one entry (hit slot, light) per distinct light the
// pixel's samples pick (q[0] is idle until the second bounce).
template <int IS>
__global__ void __launch_bounds__(kThreads) k_primary(SceneView sc, CameraView cam, WaveState ws, WaveJob job)
{
    constexpr bool SMEM = IS == kIsSmem;
    extern __shared__ float4 s_sph[];
    const uint32_t n = job.n_pixels;
    if (blockIdx.x * blockDim.x >= n) return;
    const bool cached = job.prim_cached != 0;   // uniform: only the hit queue is built
    if (SMEM && !cached) stage_spheres(sc, s_sph);
    const float4* sph = SMEM ? s_sph : sc.sph;
    const float3 o = mk3(cam.pos[0], cam.pos[1], cam.pos[2]);
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t* hits = &ws.counters[2 * ((uint32_t)job.max_bounces + 1u)];
    uint2* prim = job.prim_cache ? job.prim_cache + job.pixel0 : ws.prim;
    const bool vis = wave_light_vis(job, sc.n_lights);   // uniform
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {   // warp-uniform trip count
        const uint32_t j = base + threadIdx.x;
        const bool me = j < n;
        const uint32_t p = job.pixel0 + j;
        int32_t id = -1;
        float t = 0.0f;
        float3 d = o;
        if (cached) {
            if (me) {
                const uint2 pr = prim[j];
                id = (int32_t)pr.y;
                t = __uint_as_float(pr.x);
                if (vis && id >= 0) d = primary_ray(cam, p);
            }
        } else {
            if (me) d = primary_ray(cam, p);
            // a warp whose pixels are one aligned tile (its first pixel inside
            // the wave, so the tile is inside the image) takes the camera's
            // tile mask or candidate list
            const uint32_t warp_j = base + (threadIdx.x & ~31u);                  // warp-uniform
            const uint32_t tile_px = job.pixel0 + warp_j;
            const bool tiled = warp_j < n && (tile_px & 31u) == 0u;
            WarpCone cone;
            uint2 ti = make_uint2(0u, kNoTileList);
            if (IS == kIsBvh && cam.tile_info && tiled) ti = __ldg(&cam.tile_info[tile_px >> 5]);
            if (IS == kIsBvh && ti.y != kNoTileList)
                id = nearest_listed(sc.bvh, cam.tile_lists + ti.x, ti.y, o, d, me, t);
            else if (IS != kIsBvh && cam.masks && tiled)
                id = nearest_masked<SMEM>(sph, cam.masks + (size_t)(tile_px >> 5) * cam.mask_words, cam.mask_words,
                                          o, d, me, t);
            else if (IS != kIsBvh && warp_cone(me, d, cone)) id = nearest_cone<SMEM>(sph, sc.n_sph, o, d, me, cone, t);
            else if (me) id = scene_nearest<IS>(sc, sph, o, d, t);
            if (me) prim[j] = make_uint2(__float_as_uint(t), (uint32_t)id);
        }
        // pixels whose primary ray hits get first-bounce paths; the others'
        // samples are closed-form (accumulated by k_accumulate)
        const uint32_t slot = warp_push(hits, id >= 0);
        if (id >= 0) ws.hitq[slot] = j;
        if (!vis) continue;

        uint32_t lights = 0u;   // distinct lights the pixel's samples pick (Renderer.cu:339)
        float3 pos = o, nrm = o;
        if (id >= 0) {
            ray_hit(__ldg(&sc.sph[id]), o, d, t, pos, nrm);
            for (uint32_t s = 0; s < job.spp; ++s) lights |= 1u << light_pick(sc, p * (job.frame0 + s));
        }
        if (me) ws.vis[j] = 0u;
        if (id >= 0) {
            const float3 so = add3(pos, muls3(nrm, kOffset));
            ws.sh_o[slot] = make_float4(pos.x, pos.y, pos.z, __uint_as_float((uint32_t)id));
            ws.sh_d[slot] = make_float4(so.x, so.y, so.z, __uint_as_float(j));
        }
        // one slot range per warp, lane after lane: an inclusive scan of the
        // lanes' light counts and one atomicAdd
        const uint32_t cnt = (uint32_t)__popc(lights);
        uint32_t incl = cnt;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t v = __shfl_up_sync(kFull, incl, off);
            if ((int)lane_id() >= off) incl += v;
        }
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        uint32_t at = 0u;
        if (lane_id() == 31u && total) at = atomicAdd(&ws.counters[1], total);
        at = __shfl_sync(kFull, at, 31) + incl - cnt;
        while (lights) {
            const uint32_t li = (uint32_t)(__ffs(lights) - 1);
            lights &= lights - 1u;
            ws.q[0][at++] = shadow_tag(slot, li);
        }
    }
}

// What shading a hit leaves behind (Renderer.cu:318-384 for one bounce).
struct Shaded {
    float3 add;        // emission (Renderer.cu:329-333), when touch
    float3 lc;         // the light's contribution, when lit
    bool touch, lit;
    bool traced_sh;    // a shadow ray was tested here (light buffer)
    bool push_sh;      // a shadow ray goes to k_shadow: sho, shd, shc
    bool push_next;    // the path continues: o, d, thr, own, seed
    float4 sho, shd, shc;
};

// Shading of the hit (sphere hit at tmin) of path pid's ray (o, d) with
// throughput thr at bounce `bounce` (seed already advanced by it): emission,
// the light pick and its BRDF term, the shadow ray (visibility bit j for vis,
// tested here through the light buffer for INL, else a record for k_shadow),
// roulette and the next direction, which replace o, d, thr, own and advance
// seed.
template <bool SMEM, bool INL>
__device__ __forceinline__ void shade_hit(const SceneView& sc, const float4* sph, const WaveState& ws, uint32_t pid,
                                          int32_t hit, float tmin, float3& o, float3& d, float3& thr, uint32_t& own,
                                          uint32_t& seed, bool last, bool vis, uint32_t j, Shaded& r)
{
    const float4 s = table_sphere<SMEM>(sph, (uint32_t)hit);
    float3 pos, nrm;
    ray_hit(s, o, d, tmin, pos, nrm);
    const int32_t mi = __ldg(&sc.sph_mat[hit]);
    const float4* mrow = reinterpret_cast<const float4*>(sc.mat + mi);
    const float4 m0 = __ldg(mrow), m1 = __ldg(mrow + 1), m2 = __ldg(mrow + 2);
    const float3 albedo = mk3(m0.x, m0.y, m0.z);
    const float rough = m0.w;
    const float3 f0 = mk3(m1.x, m1.y, m1.z);
    const float metallic = m1.w;

    if (m2.w > 0.0f) {  // Renderer.cu:329-333
        r.add = mul3(mk3(m2.x, m2.y, m2.z), thr);
        r.touch = true;
    }
    // glm::mix(F0, albedo, metallic), Renderer.cu:335
    const float3 base = add3(muls3(f0, 1.0f - metallic), muls3(albedo, metallic));

    if (sc.n_lights > 0u) {  // Renderer.cu:338-369
        const uint32_t li = light_pick(sc, seed);
        float3 L;
        float dist2;
        const float4 l1 = light_dir(sc, li, pos, L, dist2);
        const float3 f = cook_torrance(albedo, base, metallic, rough, nrm, neg3(d), L);
        const float3 c = mul3(mul3(mk3(l1.x, l1.y, l1.z), f), thr);
        if (vis) {
            r.lit = ((ws.vis[j] >> li) & 1u) != 0u;
            r.lc = c;
        } else if (INL) {   // Renderer.cu:348-352
            const float3 so = add3(pos, muls3(nrm, kOffset));
            r.lit = sc.n_sph == 0u || !occluded_lb<SMEM>(sc, sph, li, so, L, dist2);
            r.lc = c;
            r.traced_sh = true;
        } else {
            const float3 so = add3(pos, muls3(nrm, kOffset));
            r.sho = make_float4(so.x, so.y, so.z, dist2);
            r.shd = make_float4(L.x, L.y, L.z, __uint_as_float(pid));
            // w: the sphere the shadow ray leaves from (tested first by the
            // LBVH walk) and the light (for the light buffer)
            r.shc = make_float4(c.x, c.y, c.z, __uint_as_float(shadow_tag((uint32_t)hit, li)));
            r.push_sh = true;
        }
    }

    if (!last) {  // Renderer.cu:371-384
        thr = mul3(thr, albedo);
        o = add3(pos, muls3(nrm, kOffset));
        const float p = gmax(0.1f, gmin(1.0f, length3(thr)));
        if (!(pcg_float(seed) > p)) {
            thr = mul_rcp3(thr, p);
            d = sample_next(nrm, rough, metallic, seed);
            // the next ray leaves this sphere (~0u: beyond the direction buffer's reach)
            own = db_reaches(sc, (uint32_t)hit, s, o) ? (uint32_t)hit : ~0u;
            r.push_next = true;
        }
    }
}

// Queue pushes after shading (all 32 lanes of the warp call it).
template <bool INL>
__device__ __forceinline__ void push_shaded(const WaveState& ws, uint32_t* qout, int bounce, uint32_t pid,
                                            const Shaded& r, float3 o, float3 d, float3 thr, uint32_t own,
                                            uint32_t seed)
{
    if (INL) {
        warp_push(&ws.counters[2 * bounce + 1], r.traced_sh);   // count the traced rays
    } else {
        const uint32_t ss = warp_push(&ws.counters[2 * bounce + 1], r.push_sh);
        if (r.push_sh) {
            ws.sh_o[ss] = r.sho;
            ws.sh_d[ss] = r.shd;
            ws.sh_c[ss] = r.shc;
        }
    }
    const uint32_t sn = warp_push(&ws.counters[2 * (bounce + 1)], r.push_next);
    if (r.push_next) {
        qout[sn] = pid;
        ws.ray_o[pid] = make_float4(o.x, o.y, o.z, __uint_as_float(seed));
        ws.ray_d[pid] = make_float4(d.x, d.y, d.z, __uint_as_float(own));
        ws.thr[pid] = make_float4(thr.x, thr.y, thr.z, 0.0f);
    }
}

// With a light buffer (INL) a continuation ray is traced where shading makes
// it, and only a ray that hits is queued: its record carries the hit (ray_o:
// origin, seed; ray_d: direction, t; thr: throughput, sphere).  A ray that
// misses ends its path there, and the sky term of the next bounce
// (Renderer.cu:311-316, sky_term) goes into the colour after this bounce's
// terms, as the reference's loop adds it.
__device__ __forceinline__ float3 sky_term(float3 c, float3 thr)
{
    return add3(c, mul3(mk3(0.6f, 0.7f, 0.9f), thr));
}

// Queues a traced continuation ray that hits (all 32 lanes of the warp call it).
__device__ __forceinline__ void push_hit(const WaveState& ws, uint32_t* qout, uint32_t* counter, bool push,
                                         uint32_t pid, float3 o, uint32_t seed, float3 d, float t, float3 thr,
                                         int32_t hit)
{
    const uint32_t sn = warp_push(counter, push);
    if (push) {
        qout[sn] = pid;
        ws.ray_o[pid] = make_float4(o.x, o.y, o.z, __uint_as_float(seed));
        ws.ray_d[pid] = make_float4(d.x, d.y, d.z, t);
        ws.thr[pid] = make_float4(thr.x, thr.y, thr.z, __uint_as_float((uint32_t)hit));
    }
}

// The first bounce over (pixel, sample) paths.  SHARED: the nearest hit comes
// from k_primary's per-pixel record instead of tracing the primary ray again,
// and idx enumerates (hit pixel, sample).
// INL: the scene has a light buffer and shadow rays are tested right after
// the shading (a lookup and a few spheres) instead of through k_shadow.
template <int IS, bool SHARED, bool INL>
__global__ void __launch_bounds__(kExtendThreads, kExtendBlocksPerSm)
    k_first(SceneView sc, CameraView cam, WaveState ws, WaveJob job)
{
    constexpr bool SMEM = IS == kIsSmem;
    extern __shared__ float4 s_sph[];
    const uint32_t n = SHARED ? ws.counters[2 * ((uint32_t)job.max_bounces + 1u)] * job.spp
                              : job.n_pixels * job.spp;
    if (blockIdx.x * blockDim.x >= n) return;
    if (SMEM) stage_spheres(sc, s_sph);
    const float4* sph = SMEM ? s_sph : sc.sph;
    const bool last = 1 >= job.max_bounces;
    const uint32_t stride = gridDim.x * blockDim.x;
    // per-(pixel, light) shadow rays: the light of a sample is added here when
    // k_shadow found it visible from the pixel's hit
    const bool vis = SHARED && wave_light_vis(job, sc.n_lights);
    uint32_t missed = 0u;   // INL: continuation rays traced here that missed

    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t idx = base + threadIdx.x;
        Shaded r{};
        uint32_t pid = 0u, seed = 0u, own = ~0u;
        bool shaded = false;
        float3 o = mk3(0.f, 0.f, 0.f), d = o, thr = o;
        int32_t nhit = -1;   // INL: the next ray's hit
        float nt = 0.0f;
        if (idx < n) {
            const uint32_t j = SHARED ? ws.hitq[idx / job.spp] : idx / job.spp;   // path ids stay pixel-major
            const uint32_t smp = idx % job.spp;
            pid = j * job.spp + smp;
            const uint32_t p = job.pixel0 + j;
            o = mk3(cam.pos[0], cam.pos[1], cam.pos[2]);
            d = primary_ray(cam, p);
            thr = mk3(1.f, 1.f, 1.f);
            seed = p * (job.frame0 + smp);   // bounce 0: seed += 0
            float tmin;
            int32_t hit;
            if (SHARED) {
                const uint2 pr = job.prim_cache ? job.prim_cache[job.pixel0 + j] : ws.prim[j];
                tmin = __uint_as_float(pr.x);
                hit = (int32_t)pr.y;
            } else {
                hit = scene_nearest<IS>(sc, sph, o, d, tmin);
            }
            if (hit < 0) {
                if (job.sky) {  // Renderer.cu:311-316
                    r.add = mul3(mk3(0.6f, 0.7f, 0.9f), thr);
                    r.touch = true;
                }
            } else {
                shade_hit<SMEM, INL>(sc, sph, ws, pid, hit, tmin, o, d, thr, own, seed, last, vis, j, r);
                shaded = true;
            }
            float3 c = add3(mk3(0.f, 0.f, 0.f), r.add);
            if (r.lit) c = add3(c, r.lc);   // as k_shadow adds it: after the emission
            if (INL && r.push_next) {
                nhit = scene_nearest_from<IS>(sc, sph, own, o, d, nt);
                r.push_next = nhit >= 0;
                if (!r.push_next) {
                    ++missed;
                    if (job.sky) c = sky_term(c, thr);
                }
            }
            ws.col[pid] = make_float4(c.x, c.y, c.z, 0.0f);
        }
        // count the shaded paths (SHARED: every path of the launch is one)
        if (!SHARED) warp_push(&ws.counters[2 * ((uint32_t)job.max_bounces + 1u) + 1u], shaded);
        if (INL) {
            warp_push(&ws.counters[1], r.traced_sh);   // count the shadow rays tested here
            push_hit(ws, ws.q[1], &ws.counters[2], r.push_next, pid, o, seed, d, nt, thr, nhit);
        } else {
            push_shaded<INL>(ws, ws.q[1], 0, pid, r, o, d, thr, own, seed);
        }
    }
    if (INL) warp_push_n(&ws.counters[2 * ((uint32_t)job.max_bounces + 1u) + 3u], missed);
}

// Bounce b >= 1 over the extension queue, in rounds of two phases per block.
// Intersect: each thread takes rays from its grid-stride share of the queue;
// a miss is finished at once (sky), a hit goes to the block's hit list in
// shared memory (path, sphere, t).  Shade: once the list holds a block's
// worth of hits, or the queue is done, every thread shades one.  Most rays
// after the first bounce leave the scene, so shading (the larger part of the
// work) then runs on full warps instead of on the few lanes that hit.
template <int IS>
__global__ void __launch_bounds__(kExtendThreads, kExtendBlocksPerSm)
    k_bounce(SceneView sc, WaveState ws, WaveJob job, int bounce)
{
    constexpr bool SMEM = IS == kIsSmem;
    constexpr uint32_t kCap = 2u * kExtendThreads;
    extern __shared__ float4 s_sph[];
    __shared__ uint32_t h_pid[kCap], h_id[kCap];
    __shared__ float h_t[kCap];
    __shared__ uint32_t h_n;
    const uint32_t n = ws.counters[2 * bounce];
    if (blockIdx.x * blockDim.x >= n) return;
    if (SMEM) stage_spheres(sc, s_sph);   // ends with a barrier
    const float4* sph = SMEM ? s_sph : sc.sph;
    if (threadIdx.x == 0) h_n = 0u;

    // select, not index: a runtime index into the parameter's array would
    // copy the whole WaveState to local memory
    const uint32_t* qin = (bounce & 1) ? ws.q[1] : ws.q[0];
    uint32_t* qout = (bounce & 1) ? ws.q[0] : ws.q[1];
    const bool last = bounce + 1 >= job.max_bounces;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t base = blockIdx.x * blockDim.x;
    __syncthreads();

    for (;;) {   // ends: every round takes rays off the queue or hits off the list
        while (base < n && h_n < blockDim.x) {   // block-uniform: base, h_n after the barrier
            const uint32_t idx = base + threadIdx.x;
            bool found = false;
            uint32_t pid = 0u;
            int32_t hit = -1;
            float tmin = 0.0f;
            if (idx < n) {
                pid = qin[idx];
                const float4 ro = ws.ray_o[pid];
                const float4 rd = ws.ray_d[pid];
                hit = scene_nearest_from<IS>(sc, sph, __float_as_uint(rd.w), mk3(ro.x, ro.y, ro.z),
                                             mk3(rd.x, rd.y, rd.z), tmin);
                found = hit >= 0;
                if (!found && job.sky) {   // Renderer.cu:311-316: the path ends in the sky
                    const float4 tt = ws.thr[pid];
                    const float3 add = mul3(mk3(0.6f, 0.7f, 0.9f), mk3(tt.x, tt.y, tt.z));
                    float4 c = ws.col[pid];
                    c.x = c.x + add.x;
                    c.y = c.y + add.y;
                    c.z = c.z + add.z;
                    ws.col[pid] = c;
                }
            }
            const uint32_t k = warp_push(&h_n, found);
            if (found) {
                h_pid[k] = pid;
                h_id[k] = (uint32_t)hit;
                h_t[k] = tmin;
            }
            base += stride;
            __syncthreads();
        }
        const uint32_t nh = h_n;
        if (nh == 0u) break;   // and the queue is done
        const uint32_t take = min(nh, blockDim.x);
        Shaded r{};
        uint32_t pid = 0u, seed = 0u, own = ~0u;
        float3 o = mk3(0.f, 0.f, 0.f), d = o, thr = o;
        if (threadIdx.x < take) {
            const uint32_t k = nh - take + threadIdx.x;
            pid = h_pid[k];
            const int32_t hit = (int32_t)h_id[k];
            const float tmin = h_t[k];
            const float4 ro = ws.ray_o[pid];
            const float4 rd = ws.ray_d[pid];
            const float4 tt = ws.thr[pid];
            o = mk3(ro.x, ro.y, ro.z);
            seed = __float_as_uint(ro.w) + (uint32_t)bounce;
            d = mk3(rd.x, rd.y, rd.z);
            thr = mk3(tt.x, tt.y, tt.z);
            shade_hit<SMEM, false>(sc, sph, ws, pid, hit, tmin, o, d, thr, own, seed, last, false, 0u, r);
            if (r.touch || r.lit) {
                // emission of bounce b, then its light (the order k_shadow adds it in)
                float4 c = ws.col[pid];
                if (r.touch) {
                    c.x = c.x + r.add.x;
                    c.y = c.y + r.add.y;
                    c.z = c.z + r.add.z;
                }
                if (r.lit) {
                    c.x = c.x + r.lc.x;
                    c.y = c.y + r.lc.y;
                    c.z = c.z + r.lc.z;
                }
                ws.col[pid] = c;
            }
        }
        push_shaded<false>(ws, qout, bounce, pid, r, o, d, thr, own, seed);
        __syncthreads();   // every thread has read its entry
        if (threadIdx.x == 0) h_n = nh - take;
        __syncthreads();
    }
}

// Adds the terms of one shaded bounce to a path's colour in the reference's
// order: emission, then the light (then, by the caller, the sky when the
// continuation missed).
__device__ __forceinline__ float3 bounce_terms(float3 c, const Shaded& r)
{
    if (r.touch) c = add3(c, r.add);
    if (r.lit) c = add3(c, r.lc);
    return c;
}

// Bounce b >= 1 of scenes with a light buffer: every queued ray hits (it was
// traced where it was made), so each thread shades one, on full warps, then
// traces its continuation and queues it if it hits.  Launched over the
// global sphere table (IS = kIsGlobal): the few spheres a list walk touches
// come faster from L1 than from the shared-memory pair layout, and no block
// stages the table.
template <int IS>
__global__ void __launch_bounds__(kExtendThreads, kExtendBlocksPerSm)
    k_shade(SceneView sc, WaveState ws, WaveJob job, int bounce)
{
    constexpr bool SMEM = IS == kIsSmem;
    extern __shared__ float4 s_sph[];
    const uint32_t n = ws.counters[2 * bounce];
    if (blockIdx.x * blockDim.x >= n) return;
    if (SMEM) stage_spheres(sc, s_sph);
    const float4* sph = SMEM ? s_sph : sc.sph;
    // select, not index: a runtime index into the parameter's array would
    // copy the whole WaveState to local memory
    const uint32_t* qin = (bounce & 1) ? ws.q[1] : ws.q[0];
    uint32_t* qout = (bounce & 1) ? ws.q[0] : ws.q[1];
    const bool last = bounce + 1 >= job.max_bounces;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t missed = 0u;   // continuation rays traced here that missed

    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t idx = base + threadIdx.x;
        Shaded r{};
        uint32_t pid = 0u, seed = 0u, own = ~0u;
        float3 o = mk3(0.f, 0.f, 0.f), d = o, thr = o;
        int32_t nhit = -1;
        float nt = 0.0f;
        if (idx < n) {
            pid = qin[idx];
            const float4 ro = ws.ray_o[pid];
            const float4 rd = ws.ray_d[pid];
            const float4 tt = ws.thr[pid];
            o = mk3(ro.x, ro.y, ro.z);
            seed = __float_as_uint(ro.w) + (uint32_t)bounce;
            d = mk3(rd.x, rd.y, rd.z);
            thr = mk3(tt.x, tt.y, tt.z);
            shade_hit<SMEM, true>(sc, sph, ws, pid, (int32_t)__float_as_uint(tt.w), rd.w, o, d, thr, own, seed, last,
                                  false, 0u, r);
            bool sky = false;
            if (r.push_next) {
                nhit = scene_nearest_from<IS>(sc, sph, own, o, d, nt);
                r.push_next = nhit >= 0;
                missed += r.push_next ? 0u : 1u;
                sky = !r.push_next && job.sky;
            }
            if (r.touch || r.lit || sky) {
                const float4 c0 = ws.col[pid];
                float3 c = bounce_terms(mk3(c0.x, c0.y, c0.z), r);
                if (sky) c = sky_term(c, thr);
                ws.col[pid] = make_float4(c.x, c.y, c.z, c0.w);
            }
        }
        warp_push(&ws.counters[2 * bounce + 1], r.traced_sh);   // count the shadow rays tested here
        push_hit(ws, qout, &ws.counters[2 * (bounce + 1)], r.push_next, pid, o, seed, d, nt, thr, nhit);
    }
    warp_push_n(&ws.counters[2 * ((uint32_t)job.max_bounces + 1u) + 3u], missed);
}

// The sparse late bounces (b >= b0) of scenes with a light buffer in one
// persistent launch: a block keeps a pool of paths (path id and bounce) whose
// next ray hits, in shared memory, refilled with chunks of bounce b0's queue
// (one atomic claim per chunk), and carries each path through all its
// remaining bounces: a round shades up to a block of pool paths on full
// warps, traces their continuations and puts those that hit back into the
// pool.  Late bounces hold few rays, so separate launches would be mostly
// launch latency and tails.  A path's bounces run in order in one block, so
// its colour sums are in the reference's order.
template <int IS>
__global__ void __launch_bounds__(kExtendThreads, kExtendBlocksPerSm)
    k_paths(SceneView sc, WaveState ws, WaveJob job, int b0)
{
    constexpr bool SMEM = IS == kIsSmem;
    constexpr uint32_t kPool = 2u * kExtendThreads;
    extern __shared__ float4 s_sph[];
    __shared__ uint32_t p_pid[kPool];
    __shared__ uint16_t p_bounce[kPool];   // bounces are at most 4096
    __shared__ uint32_t p_n, chunk;
    __shared__ bool dry;                      // bounce b0's queue is used up
    const uint32_t n0 = ws.counters[2 * b0];  // bounce b0's queue
    if (n0 == 0u) return;
    if (SMEM) stage_spheres(sc, s_sph);   // ends with a barrier
    const float4* sph = SMEM ? s_sph : sc.sph;
    const uint32_t* q0 = (b0 & 1) ? ws.q[1] : ws.q[0];
    uint32_t* claim = &ws.counters[2 * ((uint32_t)job.max_bounces + 1u) + 2u];
    uint32_t rays = 0u, traced = 0u;   // this thread's continuation rays, shadow rays
    if (threadIdx.x == 0) {
        p_n = 0u;
        dry = false;
    }
    __syncthreads();

    for (;;) {   // ends: every round takes paths off the pool, which only the queue refills
        if (!dry && p_n < blockDim.x) {   // block-uniform: refill from bounce b0's queue
            if (threadIdx.x == 0) {
                chunk = atomicAdd(claim, blockDim.x);
                dry = chunk >= n0;
            }
            __syncthreads();
            const uint32_t c0 = chunk;
            if (c0 < n0) {
                const uint32_t take = min(blockDim.x, n0 - c0), at = p_n;
                if (threadIdx.x < take) {
                    p_pid[at + threadIdx.x] = q0[c0 + threadIdx.x];
                    p_bounce[at + threadIdx.x] = (uint16_t)b0;
                }
                __syncthreads();
                if (threadIdx.x == 0) p_n = at + take;
            }
            __syncthreads();
        }
        const uint32_t np = p_n;
        if (np == 0u) break;

        // shade up to a block of pool paths (from the top of the pool)
        const uint32_t take = min(np, blockDim.x);
        uint32_t pid = 0u, b = 0u;
        if (threadIdx.x < take) {
            pid = p_pid[np - 1u - threadIdx.x];
            b = p_bounce[np - 1u - threadIdx.x];
        }
        __syncthreads();
        if (threadIdx.x == 0) p_n = np - take;
        __syncthreads();

        Shaded r{};
        uint32_t seed = 0u, own = ~0u;
        float3 o = mk3(0.f, 0.f, 0.f), d = o, thr = o;
        int32_t nhit = -1;
        float nt = 0.0f;
        if (threadIdx.x < take) {
            const float4 ro = ws.ray_o[pid];
            const float4 rd = ws.ray_d[pid];
            const float4 tt = ws.thr[pid];
            o = mk3(ro.x, ro.y, ro.z);
            seed = __float_as_uint(ro.w) + b;
            d = mk3(rd.x, rd.y, rd.z);
            thr = mk3(tt.x, tt.y, tt.z);
            const bool last = (int)b + 1 >= job.max_bounces;
            shade_hit<SMEM, true>(sc, sph, ws, pid, (int32_t)__float_as_uint(tt.w), rd.w, o, d, thr, own, seed, last,
                                  false, 0u, r);
            traced += r.traced_sh ? 1u : 0u;
            bool sky = false;
            if (r.push_next) {
                ++rays;
                nhit = scene_nearest_from<IS>(sc, sph, own, o, d, nt);
                r.push_next = nhit >= 0;
                sky = !r.push_next && job.sky;
            }
            if (r.touch || r.lit || sky) {
                const float4 c0 = ws.col[pid];
                float3 c = bounce_terms(mk3(c0.x, c0.y, c0.z), r);
                if (sky) c = sky_term(c, thr);
                ws.col[pid] = make_float4(c.x, c.y, c.z, c0.w);
            }
            if (r.push_next) {
                ws.ray_o[pid] = make_float4(o.x, o.y, o.z, __uint_as_float(seed));
                ws.ray_d[pid] = make_float4(d.x, d.y, d.z, nt);
                ws.thr[pid] = make_float4(thr.x, thr.y, thr.z, __uint_as_float((uint32_t)nhit));
            }
        }
        const uint32_t k = warp_push(&p_n, r.push_next);
        if (r.push_next) {
            p_pid[k] = pid;
            p_bounce[k] = (uint16_t)(b + 1u);
        }
        __syncthreads();
    }
    // statistics: every continuation ray traced here, shadow rays into bounce
    // b0's slot (only sums over bounces are read)
    warp_push_n(&ws.counters[2 * ((uint32_t)job.max_bounces + 1u) + 3u], rays);
    warp_push_n(&ws.counters[2 * b0 + 1], traced);
}

// Whether the sphere a shadow ray leaves from (own, an index into the table)
// occludes it, with the brute-force test.  Testing it first changes nothing
// but the time: "occluded" means some sphere has t > 0 and t*t < dist2, in any
// order (see occluded_brute).  A surface facing away from its light is
// shadowed by its own sphere; the LBVH walk tests it first and skips the walk
// (+5% on the 65,536-sphere scene).  The brute-force loop does not: there the
// extra divergent test cost more than the chunks it saves (-2% on 256 spheres).
__device__ __forceinline__ bool own_occludes(const SceneView& sc, const float4* sph, bool smem, uint32_t own,
                                             float3 o, float3 d, float dist2)
{
    if (own >= sc.n_sph) return false;
    const float4 s = smem ? smem_sphere(sph, own) : __ldg(&sc.sph[own]);
    float t;
    return sphere_t(s, o, d, dot3(d, d), t) && t > 0.0f && t * t < dist2;
}

// A shadow ray of one bounce's queue: origin, direction, squared distance to
// the light, tag (the sphere it leaves from and the light) and target (the
// path, or for VIS the wave pixel).  Per-sample rays are stored whole (sh_o:
// origin, dist^2; sh_d: direction, path; sh_c: light contribution, tag).
// First-bounce (pixel, light) entries (VIS) hold the hit slot and the light;
// the slot's record gives the hit point and sphere, the origin and the pixel,
// and the direction and distance are recomputed by light_dir exactly as the
// shading computes them.
struct ShadowRay {
    float3 o, d;
    float dist2;
    uint32_t tag;
    uint32_t target;
};

template <bool VIS>
__device__ __forceinline__ ShadowRay load_shadow(const SceneView& sc, const WaveState& ws, uint32_t idx)
{
    ShadowRay r;
    if (VIS) {
        const uint32_t e = ws.q[0][idx];
        const uint32_t slot = e & kShadowSphereMask, li = e >> 26;
        const float4 a = ws.sh_o[slot], b = ws.sh_d[slot];
        light_dir(sc, li, mk3(a.x, a.y, a.z), r.d, r.dist2);
        r.o = mk3(b.x, b.y, b.z);
        r.tag = shadow_tag(__float_as_uint(a.w), li);
        r.target = __float_as_uint(b.w);
    } else {
        const float4 so = ws.sh_o[idx], sd = ws.sh_d[idx];
        r.o = mk3(so.x, so.y, so.z);
        r.d = mk3(sd.x, sd.y, sd.z);
        r.dist2 = so.w;
        r.tag = __float_as_uint(ws.sh_c[idx].w);
        r.target = __float_as_uint(sd.w);
    }
    return r;
}

// Adds the light an unoccluded shadow ray carries to its path (Renderer.cu:
// 356-368), or, for a (pixel, light) ray (VIS), marks the light visible from
// the pixel.
template <bool VIS>
__device__ __forceinline__ void shadow_light(const WaveState& ws, uint32_t idx, const ShadowRay& r)
{
    if (VIS) {
        atomicOr(&ws.vis[r.target], 1u << (r.tag >> 26));
        return;
    }
    const float4 c = ws.sh_c[idx];
    float4 col = ws.col[r.target];
    col.x = col.x + c.x;
    col.y = col.y + c.y;
    col.z = col.z + c.z;
    ws.col[r.target] = col;
}

template <int IS, bool VIS>
__global__ void __launch_bounds__(kThreads, kShadowBlocksPerSm<IS>) k_shadow(SceneView sc, WaveState ws, int bounce)
{
    constexpr bool SMEM = IS == kIsSmem;
    extern __shared__ float4 s_sph[];
    const uint32_t n = ws.counters[2 * bounce + 1];
    if (blockIdx.x * blockDim.x >= n) return;
    if (SMEM) stage_spheres(sc, s_sph);
    const float4* sph = SMEM ? s_sph : sc.sph;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;

    if (IS == kIsBvh || sc.n_sph == 0u || sc.lb.n_lights != 0u) {
        for (uint32_t idx = first; idx < n; idx += stride) {
            const ShadowRay r = load_shadow<VIS>(sc, ws, idx);
            bool occ;
            if (IS == kIsBvh) occ = own_occludes(sc, sph, SMEM, r.tag & kShadowSphereMask, r.o, r.d, r.dist2) ||
                                    scene_occluded<IS>(sc, sph, r.o, r.d, r.dist2);
            else occ = sc.n_sph != 0u && occluded_lb<SMEM>(sc, sph, r.tag >> 26, r.o, r.d, r.dist2);
            if (!occ) shadow_light<VIS>(ws, idx, r);
        }
        return;
    }

    // Brute force, any hit.  Rays stop at their first occluder, so lanes of a
    // warp finish at different times; instead of idling until the slowest lane
    // is done, a lane that finishes loads its next ray at once and tests it
    // from the warp's current 32-sphere chunk on, wrapping around.  Every
    // iteration the whole warp tests the same chunk (one broadcast read per
    // sphere) and each lane counts the chunks its ray has left.  An any-hit
    // query does not depend on the order in which spheres are tested.
    // Each lane also holds its next ray, loaded when the current one starts,
    // so a lane that moves on does not stall the warp on a memory load.
    const uint32_t nchunks = (sc.n_sph + 31u) / 32u;
    const uint32_t tail = sc.n_sph - (nchunks - 1u) * 32u;   // spheres in the last chunk
    uint32_t idx = 0u, left = 0u, chunk = 0u;
    float a = 0.0f;
    ShadowRay cur{}, nxt{};
    bool live = false;   // lane holds a ray
    uint32_t nidx = first;
    if (nidx < n) nxt = load_shadow<VIS>(sc, ws, nidx);
    for (;;) {   // ends: every iteration retires a ray or takes a chunk off one
        if (!live && nidx < n) {
            idx = nidx;
            cur = nxt;
            a = dot3(cur.d, cur.d);
            left = nchunks;
            live = true;
            nidx += stride;
            if (nidx < n) nxt = load_shadow<VIS>(sc, ws, nidx);
        }
        const float3 o = cur.o, d = cur.d;
        const float dist2 = cur.dist2;
        if (!__any_sync(kFull, live)) break;
        if (live) {
            const uint32_t base = chunk * 32u;
            uint32_t mask = (chunk + 1u < nchunks || tail == 32u)
                                ? candidate_bits<SMEM, 32>(sph, base, o, d, a, 32u)
                                : candidate_bits<SMEM, 31>(sph, base, o, d, a, tail);
            bool hit = false;
            while (mask) {
                const uint32_t k = (uint32_t)__clz(mask);
                mask &= ~(0x80000000u >> k);
                float t;
                if (sphere_t(table_sphere<SMEM>(sph, base + k), o, d, a, t) && t > 0.0f &&
                    t * t < dist2) {
                    hit = true;
                    break;
                }
            }
            if (hit || --left == 0u) {
                if (!hit) shadow_light<VIS>(ws, idx, cur);   // Renderer.cu:353-369: unoccluded
                live = false;
            }
        }
        chunk = (chunk + 1u == nchunks) ? 0u : chunk + 1u;
    }
}

__global__ void __launch_bounds__(kThreads) k_accumulate(WaveState ws, WaveJob job, float4* accum, uint32_t* image)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    const float fpack = __uint2float_rn(job.pack_frame);
    if (blockIdx.x == 0 && threadIdx.x == 0 && ws.totals) {
        unsigned long long ext = 0, sh = 0;
        for (int b = 0; b < job.max_bounces; ++b) {
            if (b > 0) ext += ws.counters[2 * b];
            sh += ws.counters[2 * b + 1];
        }
        if (job.max_bounces > 0) ext += ws.counters[2 * ((uint32_t)job.max_bounces + 1u) + 3u];
        atomicAdd(&ws.totals[0], ext);
        atomicAdd(&ws.totals[1], sh);
        if (job.max_bounces > 0) {
            const uint32_t* hc = &ws.counters[2 * ((uint32_t)job.max_bounces + 1u)];   // hit pixels, shaded paths
            atomicAdd(&ws.totals[2], wave_shares_primary(job) ? (unsigned long long)hc[0] * job.spp
                                                              : (unsigned long long)hc[1]);
        }
    }
    // a sample whose shared primary ray missed has colour 0 + sky * 1 (Renderer.cu:311-316)
    const bool shared = wave_shares_primary(job);
    const uint2* prim = job.prim_cache ? job.prim_cache + job.pixel0 : ws.prim;
    const float4 miss = job.sky ? make_float4(0.6f, 0.7f, 0.9f, 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float fspp = __uint2float_rn(job.spp);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < job.n_pixels; j += stride) {
        const uint32_t p = job.pixel0 + j;
        float4 a = accum[p];
        const bool missed = shared && (int32_t)prim[j].y < 0;
        // Every sample adds (0, 0, 0) and a frame (a missed primary without
        // sky light, or no bounces): the spp additions of 0 leave x, y, z as
        // the first one does (-0 becomes +0), and spp additions of 1 to an
        // integer count stay exact up to 2^24, so one addition of spp equals
        // them.
        if ((missed ? !job.sky : job.max_bounces <= 0) && job.spp > 0u && a.w >= 0.0f &&
            a.w <= 16777216.0f - fspp && a.w == truncf(a.w)) {
            a.x = a.x + 0.0f;
            a.y = a.y + 0.0f;
            a.z = a.z + 0.0f;
            a.w = a.w + fspp;
            accum[p] = a;
            if (job.pack_frame) image[p] = pack_rgba8(a, fpack);
            continue;
        }
        for (uint32_t s = 0; s < job.spp; ++s) {
            float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
            if (missed) c = miss;
            else if (job.max_bounces > 0) c = ws.col[(uint64_t)j * job.spp + s];
            a.x = a.x + c.x;
            a.y = a.y + c.y;
            a.z = a.z + c.z;
            a.w = a.w + 1.0f;
        }
        accum[p] = a;
        if (job.pack_frame) image[p] = pack_rgba8(a, fpack);
    }
}

// Whole paths in one thread, for small scenes on the brute-force table
// (Renderer.cu:150-171 and :287-387 in their own structure): one thread per
// pixel of the wave traces the pixel's primary ray once (its samples share
// it), then each sample's path through all its bounces, and adds the
// samples to the accumulator in frame order.  A few spheres make every
// nearest-hit and shadow test cheap, and nothing goes through memory between
// bounces, where the wavefront kernels write and read the path state and pay
// a launch per stage: for one or a few samples per pixel and call (the
// reference's interactive loop renders one) this is faster; with many, the
// wavefront's shared first-bounce work wins.  The bounce-0 light visibility
// is kept per pixel (the samples share the primary hit, so a light's shadow
// ray is the same for all of them).  Every float is computed by the
// functions the wavefront kernels use, in the same order, so the results are
// theirs bit for bit.
template <int IS>
__global__ void __launch_bounds__(kThreads, kFusedBlocksPerSm) k_fused(SceneView sc, CameraView cam, WaveState ws,
                                                                        WaveJob job, float4* accum, uint32_t* image)
{
    constexpr bool SMEM = IS == kIsSmem;
    extern __shared__ float4 s_sph[];
    if (blockIdx.x * blockDim.x >= job.n_pixels) return;
    if (SMEM) stage_spheres(sc, s_sph);
    const float4* sph = SMEM ? s_sph : sc.sph;
    const uint32_t stride = gridDim.x * blockDim.x;
    const float fpack = __uint2float_rn(job.pack_frame);
    const float3 o0 = mk3(cam.pos[0], cam.pos[1], cam.pos[2]);
    const float3 sky = mk3(0.6f, 0.7f, 0.9f);
    const bool cache_vis = sc.n_lights <= 32u;
    uint32_t n_ext = 0u, n_sh = 0u, n_first = 0u;   // rays traced, for the renderer's statistics
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < job.n_pixels; j += stride) {
        const uint32_t p = job.pixel0 + j;
        const float3 d0 = primary_ray(cam, p);
        float t0 = 0.0f;
        int32_t h0 = -1;
        if (job.max_bounces > 0) {
            if (job.prim_cache && job.prim_cached) {
                const uint2 pr = job.prim_cache[p];
                t0 = __uint_as_float(pr.x);
                h0 = (int32_t)pr.y;
            } else {
                h0 = scene_nearest<IS, true>(sc, sph, o0, d0, t0);
                if (job.prim_cache) job.prim_cache[p] = make_uint2(__float_as_uint(t0), (uint32_t)h0);
            }
        }
        float4 a = accum[p];
        uint32_t known = 0u, seen = 0u;   // bounce-0 lights tested from this pixel's hit, and the visible ones
        for (uint32_t s = 0; s < job.spp; ++s) {
            float3 c = mk3(0.f, 0.f, 0.f);
            float3 o = o0, d = d0, thr = mk3(1.f, 1.f, 1.f);
            uint32_t seed = p * (job.frame0 + s);
            for (int32_t i = 0; i < job.max_bounces; ++i) {   // Renderer.cu:304-385
                seed += (uint32_t)i;
                float tmin = t0;
                int32_t hit = h0;
                if (i > 0) {
                    hit = scene_nearest<IS, true>(sc, sph, o, d, tmin);
                    ++n_ext;
                } else if (hit >= 0) {
                    ++n_first;
                }
                if (hit < 0) {   // Renderer.cu:309-318
                    if (job.sky) c = add3(c, mul3(sky, thr));
                    break;
                }
                const float4 sp = table_sphere<SMEM>(sph, (uint32_t)hit);
                float3 pos, nrm;
                ray_hit(sp, o, d, tmin, pos, nrm);
                const int32_t mi = __ldg(&sc.sph_mat[hit]);
                const float4* mrow = reinterpret_cast<const float4*>(sc.mat + mi);
                const float4 m0 = __ldg(mrow), m1 = __ldg(mrow + 1), m2 = __ldg(mrow + 2);
                const float3 albedo = mk3(m0.x, m0.y, m0.z);
                const float rough = m0.w;
                const float metallic = m1.w;
                if (m2.w > 0.0f) c = add3(c, mul3(mk3(m2.x, m2.y, m2.z), thr));   // Renderer.cu:329-333
                const float3 base = add3(muls3(mk3(m1.x, m1.y, m1.z), 1.0f - metallic), muls3(albedo, metallic));
                if (sc.n_lights > 0u) {   // Renderer.cu:338-369
                    const uint32_t li = light_pick(sc, seed);
                    float3 L;
                    float dist2;
                    const float4 l1 = light_dir(sc, li, pos, L, dist2);
                    const float3 f = cook_torrance(albedo, base, metallic, rough, nrm, neg3(d), L);
                    const float3 lc = mul3(mul3(mk3(l1.x, l1.y, l1.z), f), thr);
                    bool lit;
                    const uint32_t bit = 1u << (li & 31u);
                    if (i == 0 && cache_vis && (known & bit)) {
                        lit = (seen & bit) != 0u;
                    } else {
                        const float3 so = add3(pos, muls3(nrm, kOffset));
                        lit = sc.n_sph == 0u || !scene_occluded<IS, true>(sc, sph, so, L, dist2);
                        ++n_sh;
                        if (i == 0 && cache_vis) {
                            known |= bit;
                            if (lit) seen |= bit;
                        }
                    }
                    if (lit) c = add3(c, lc);
                }
                if (i + 1 >= job.max_bounces) break;   // Renderer.cu:371-384 change nothing after the last
                thr = mul3(thr, albedo);
                o = add3(pos, muls3(nrm, kOffset));
                const float pr = gmax(0.1f, gmin(1.0f, length3(thr)));
                if (pcg_float(seed) > pr) break;
                thr = mul_rcp3(thr, pr);
                d = sample_next(nrm, rough, metallic, seed);
            }
            a.x = a.x + c.x;
            a.y = a.y + c.y;
            a.z = a.z + c.z;
            a.w = a.w + 1.0f;
        }
        accum[p] = a;
        if (job.pack_frame) image[p] = pack_rgba8(a, fpack);
    }
    if (ws.totals) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            n_ext += __shfl_down_sync(kFull, n_ext, off);
            n_sh += __shfl_down_sync(kFull, n_sh, off);
            n_first += __shfl_down_sync(kFull, n_first, off);
        }
        if (lane_id() == 0u) {
            if (n_ext) atomicAdd(&ws.totals[0], (unsigned long long)n_ext);
            if (n_sh) atomicAdd(&ws.totals[1], (unsigned long long)n_sh);
            if (n_first) atomicAdd(&ws.totals[2], (unsigned long long)n_first);
        }
    }
}

__global__ void k_clear(float4* p, uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        p[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

template <int IS>
__global__ void __launch_bounds__(kThreads) k_trace(SceneView sc, const float* __restrict__ org,
                                                    const float* __restrict__ dir, uint64_t n, float* t_out,
                                                    int32_t* id_out)
{
    constexpr bool SMEM = IS == kIsSmem;
    extern __shared__ float4 s_sph[];
    if (SMEM) stage_spheres(sc, s_sph);
    const float4* sph = SMEM ? s_sph : sc.sph;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float3 o = mk3(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
        const float3 d = mk3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
        float t;
        const int32_t id = scene_nearest<IS>(sc, sph, o, d, t);
        t_out[i] = id < 0 ? -1.0f : t;
        id_out[i] = id;
    }
}

// The camera's per-pixel direction table (CameraView::dirs).
__global__ void k_dir_table(CameraView cam, float4* out)
{
    const uint64_t n = (uint64_t)cam.width * cam.height;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float3 d = primary_dir(cam, (uint32_t)(i % cam.width), (uint32_t)(i / cam.width));
        out[i] = make_float4(d.x, d.y, d.z, 0.0f);
    }
}

// Tile masks (CameraView::masks): one warp per tile of 32 pixels builds the
// cone of their primary directions as k_primary does (warp_cone over the same
// directions, primary_ray) and sets bit i where cone_meets passes sphere i, or
// every bit when the cone is too wide, which is what k_primary's per-warp
// loop would test.  A k_primary warp whose pixels are this tile, or part of
// it, has its directions inside this cone.
__global__ void __launch_bounds__(kThreads) k_tile_masks(SceneView sc, CameraView cam, uint32_t* masks)
{
    const uint64_t px = (uint64_t)cam.width * cam.height;
    const uint64_t tiles = (px + 31u) / 32u;
    const uint32_t words = tile_mask_words(sc.n_sph);
    const uint32_t lane = threadIdx.x & 31u;
    const float3 o = mk3(cam.pos[0], cam.pos[1], cam.pos[2]);
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32u);
    for (uint64_t t = (uint64_t)blockIdx.x * (blockDim.x / 32u) + threadIdx.x / 32u; t < tiles; t += warps) {
        const uint64_t p = 32u * t + lane;
        const bool me = p < px;
        float3 d = o;
        if (me) d = primary_ray(cam, (uint32_t)p);
        WarpCone cone;
        const bool ok = warp_cone(me, d, cone);
        for (uint32_t w = 0; w < words; ++w) {
            const uint32_t i = 32u * w + lane;
            bool pass = false;
            if (i < sc.n_sph) {
                const float4 s = __ldg(&sc.sph[i]);
                pass = !ok || cone_meets(cone, mk3(s.x - o.x, s.y - o.y, s.z - o.z), cone_radius(s.w), 0.0f, 0.0f);
            }
            const uint32_t bits = __ballot_sync(kFull, pass);
            if (lane == 0u) masks[t * words + w] = bits;
        }
    }
}

// Candidate spheres of one tile of an LBVH scene: a warp-cooperative walk of
// the 4-wide nodes (lbvh.cu k_pack_quads) with the tile's cone.  A slot is
// entered when the cone meets the ball around its box centre through the box
// corners, that radius also added to the distance in the float-error margin:
// this ball, inflated by cone_meets, contains the inflated test ball of every
// sphere inside the box, so a slot holding a sphere that passes the sphere
// test is entered.  A leaf cluster's spheres get the sphere test the
// brute-force masks use, one per lane.  All lanes call it and keep the same
// stack.  Returns the number of candidates (the first cap of them written to
// out when FILL), or kNoTileList when the walk overflows its stack or step
// budget or the list would pass kTileListMax.
template <bool FILL>
__device__ uint32_t tile_walk(const BvhView& b, const WarpCone& cone, float3 o, uint32_t* out, uint32_t cap)
{
    const uint32_t lane = lane_id();
    uint32_t stack[kBvhStack];
    int sp = 0;
    stack[sp++] = b.root;
    uint32_t count = 0u;
    uint32_t budget = 2u * b.n_leaves + 8u;
    while (sp > 0) {
        if (budget-- == 0u) return kNoTileList;
        const uint32_t node = stack[--sp];
        if (node >= b.n_leaves - 1u) continue;
        bool pass = false;
        uint32_t ref = 0u, cnt = 0u;
        if (lane < 4u) {   // lane k tests slot k
            const float4* p = b.quad + 8 * (size_t)node + 4 * (lane >> 1);
            const float4 r0 = __ldg(p), r1 = __ldg(p + 1), r2 = __ldg(p + 2), r3 = __ldg(p + 3);
            const bool hi = (lane & 1u) != 0u;
            ref = __float_as_uint(hi ? r3.y : r3.x);
            cnt = __float_as_uint(hi ? r3.w : r3.z);
            if (bvh_slot_ok(b, ref, cnt)) {
                const float cx = hi ? r0.y : r0.x, cy = hi ? r0.w : r0.z, cz = hi ? r1.y : r1.x;
                const float hx = hi ? r1.w : r1.z, hy = hi ? r2.y : r2.x, hz = hi ? r2.w : r2.z;
                // rounded up past the float error of the sum of squares and the root
                const float rb = sqrtf(hx * hx + hy * hy + hz * hz) * 1.000001f + 1e-6f;
                pass = cone_meets(cone, mk3(cx - o.x, cy - o.y, cz - o.z), rb, rb, 0.0f);
            }
        }
        uint32_t inner = __ballot_sync(kFull, pass && cnt == 0u);
        uint32_t leaves = __ballot_sync(kFull, pass && cnt != 0u);
        while (inner) {
            const int k = __ffs(inner) - 1;
            inner &= inner - 1u;
            const uint32_t r = __shfl_sync(kFull, ref, k);
            if (sp >= kBvhStack) return kNoTileList;
            stack[sp++] = r;
        }
        while (leaves) {
            const int k = __ffs(leaves) - 1;
            leaves &= leaves - 1u;
            const uint32_t first = __shfl_sync(kFull, ref, k);
            const uint32_t c = min(__shfl_sync(kFull, cnt, k), b.n_leaves - first);
            bool meets = false;
            if (lane < c) {
                const float4 sp4 = __ldg(&b.leaf_sph[first + lane]);
                meets = cone_meets(cone, mk3(sp4.x - o.x, sp4.y - o.y, sp4.z - o.z), cone_radius(sp4.w), 0.0f, 0.0f);
            }
            const uint32_t bits = __ballot_sync(kFull, meets);
            if (count + (uint32_t)__popc(bits) > kTileListMax) return kNoTileList;
            const uint32_t at = count + (uint32_t)__popc(bits & ((1u << lane) - 1u));
            if (FILL && meets && at < cap) out[at] = first + lane;
            count += (uint32_t)__popc(bits);
        }
    }
    return count;
}

// One warp per tile: the cone of the tile's primary directions (as k_primary
// and k_tile_masks build it) and its candidate walk.  FILL: only tiles with a
// list, written from lists + info[t].x.
template <bool FILL>
__global__ void __launch_bounds__(kThreads) k_tile_lists(SceneView sc, CameraView cam, uint2* info, uint32_t* lists)
{
    const uint64_t px = (uint64_t)cam.width * cam.height;
    const uint64_t tiles = (px + 31u) / 32u;
    const uint32_t lane = lane_id();
    const float3 o = mk3(cam.pos[0], cam.pos[1], cam.pos[2]);
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32u);
    for (uint64_t t = (uint64_t)blockIdx.x * (blockDim.x / 32u) + threadIdx.x / 32u; t < tiles; t += warps) {
        uint2 ti = make_uint2(0u, 0u);
        if (FILL) {
            ti = info[t];
            if (ti.y == kNoTileList || ti.y == 0u) continue;   // warp-uniform
        }
        const uint64_t p = 32u * t + lane;
        const bool me = p < px;
        float3 d = o;
        if (me) d = primary_ray(cam, (uint32_t)p);
        WarpCone cone;
        const bool ok = warp_cone(me, d, cone);
        if (FILL) {
            if (ok) tile_walk<true>(sc.bvh, cone, o, lists + ti.x, ti.y);
        } else {
            const uint32_t len = ok ? tile_walk<false>(sc.bvh, cone, o, nullptr, 0u) : kNoTileList;
            if (lane == 0u) info[t] = make_uint2(0u, len);
        }
    }
}

// Offsets of the tile lists: one block, chunks of kThreads tiles in order;
// tiles past 2^31 - 1 listed entries in all lose their list.
__global__ void __launch_bounds__(kThreads) k_tile_list_scan(uint2* info, uint64_t tiles, uint32_t* total)
{
    __shared__ uint32_t warp_sums[kThreads / 32];
    __shared__ uint64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const uint32_t lane = lane_id(), w = threadIdx.x / 32u;
    for (uint64_t base = 0; base < tiles; base += kThreads) {
        const uint64_t i = base + threadIdx.x;
        uint2 ti = i < tiles ? info[i] : make_uint2(0u, 0u);
        const uint32_t v = ti.y == kNoTileList ? 0u : ti.y;
        uint32_t x = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, x, off);
            if (lane >= (uint32_t)off) x += y;
        }
        if (lane == 31u) warp_sums[w] = x;
        __syncthreads();
        uint64_t pre = carry;
        for (uint32_t k = 0; k < w; ++k) pre += warp_sums[k];
        const uint64_t at = pre + x - v;
        if (i < tiles) {
            if (at + v > 0x7fffffffull) ti.y = kNoTileList;
            ti.x = ti.y == kNoTileList ? 0u : (uint32_t)at;
            info[i] = ti;
        }
        __syncthreads();
        if (threadIdx.x == kThreads - 1) carry = pre + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = (uint32_t)(carry < 0x7fffffffull ? carry : 0x7fffffffull);
}

__global__ void k_primary_dirs(CameraView cam, float* out)
{
    const uint64_t n = (uint64_t)cam.width * cam.height;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float3 d = primary_dir(cam, (uint32_t)(i % cam.width), (uint32_t)(i / cam.width));
        out[3 * i] = d.x;
        out[3 * i + 1] = d.y;
        out[3 * i + 2] = d.z;
    }
}

constexpr size_t kSmemSphereCap = 96 * 1024;  // 6144 spheres staged per CTA

int isect_mode(const SceneView& sc)
{
    if (sc.use_bvh) return kIsBvh;
    if (sc.n_sph > 0 && smem_table_bytes(sc.n_sph) <= kSmemSphereCap) return kIsSmem;
    return kIsGlobal;
}

int grid_for(uint64_t n, int threads, int cap)
{
    uint64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return (int)(b < (uint64_t)cap ? b : (uint64_t)cap);
}

// Calls f with the intersection mode as a compile-time constant.
template <class F>
void with_mode(int mode, F&& f)
{
    if (mode == kIsSmem) f(std::integral_constant<int, kIsSmem>{});
    else if (mode == kIsBvh) f(std::integral_constant<int, kIsBvh>{});
    else f(std::integral_constant<int, kIsGlobal>{});
}

template <int IS>
cudaError_t occupancy(int threads, size_t bytes, int* ext, int* sh, int* pr)
{
    if (bytes > 48 * 1024) {
        const int b = (int)bytes;
        const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
        cudaError_t e = cudaFuncSetAttribute(k_first<IS, false, false>, a, b);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bounce<IS>, a, b);
        if constexpr (IS != kIsBvh) {
            if (e == cudaSuccess) e = cudaFuncSetAttribute(k_first<IS, false, true>, a, b);
        }
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_primary<IS>, a, b);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_shadow<IS, false>, a, b);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_shadow<IS, true>, a, b);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_trace<IS>, a, b);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(ext, k_bounce<IS>, kExtendThreads, bytes);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(sh, k_shadow<IS, false>, threads, bytes);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(pr, k_primary<IS>, threads, bytes);
    return e;
}

}  // namespace

cudaError_t plan_launch(const SceneView& sc, int device, int threads, LaunchShape* out, int path_kernel)
{
    if (threads <= 0 || threads > kThreads) threads = kThreads;
    int sms = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    const int mode = isect_mode(sc);
    const size_t bytes = mode == kIsSmem ? smem_table_bytes(sc.n_sph) : 0;
    int ext = 0, sh = 0, pr = 0;
    with_mode(mode, [&](auto m) { e = occupancy<decltype(m)::value>(threads, bytes, &ext, &sh, &pr); });
    if (e != cudaSuccess) return e;
    out->threads = threads;
    out->blocks_extend = sms * (ext > 0 ? ext : 1);
    out->blocks_shadow = sms * (sh > 0 ? sh : 1);
    out->blocks_primary = sms * (pr > 0 ? pr : 1);
    out->smem_spheres = bytes;
    out->mode = mode;
    out->fused = mode == kIsBvh ? 0 : path_kernel == 2 ? 2 : (path_kernel == 0 && sc.n_sph <= kFusedMaxSpheres) ? 1 : 0;
    return cudaSuccess;
}

cudaError_t enqueue_wave(const SceneView& sc, const CameraView& cam, const WaveState& ws, const WaveJob& job,
                         const LaunchShape& shape, float4* accum, uint32_t* image, cudaStream_t stream,
                         uint32_t* launches, KernelTimer* timer)
{
    uint32_t nl = 0;
    const size_t sm = shape.smem_spheres;
    const int bounces = job.max_bounces;
    const uint64_t paths = (uint64_t)job.n_pixels * job.spp;
    auto begin = [&](int fam) { if (timer) timer->begin(fam, stream); };
    auto end = [&](int fam) { if (timer) timer->end(fam, stream); };
    if (shape.mode != kIsBvh && (shape.fused == 2 || (shape.fused == 1 && job.spp <= kFusedMaxSpp))) {
        // whole paths in one thread per pixel
        const int g = grid_for(job.n_pixels, kThreads, 1 << 20);
        begin(kFamExtend);
        if (shape.mode == kIsSmem) k_fused<kIsSmem><<<g, kThreads, sm, stream>>>(sc, cam, ws, job, accum, image);
        else k_fused<kIsGlobal><<<g, kThreads, 0, stream>>>(sc, cam, ws, job, accum, image);
        end(kFamExtend);
        if (launches) *launches += 1;
        return cudaGetLastError();
    }
    if (bounces > 0) {
        cudaError_t e = cudaMemsetAsync(ws.counters, 0, sizeof(uint32_t) * wave_counter_words(bounces), stream);
        if (e != cudaSuccess) return e;
        const int g0 = grid_for(paths, kExtendThreads, shape.blocks_extend);
        const bool share = wave_shares_primary(job);
        const bool vis = wave_light_vis(job, sc.n_lights);
        // a light buffer exists only for the brute-force tables
        const bool inl = shape.mode != kIsBvh && sc.lb.n_lights != 0u;
        with_mode(shape.mode, [&](auto m) {
            constexpr int IS = decltype(m)::value;
            if (share) {
                const int gp = grid_for(job.n_pixels, shape.threads, shape.blocks_primary);
                begin(kFamExtend);
                k_primary<IS><<<gp, shape.threads, sm, stream>>>(sc, cam, ws, job);
                end(kFamExtend);
                ++nl;
                if (vis) {   // bounce 0's shadow rays, one per (pixel, light), before the shading
                    begin(kFamShadow);
                    k_shadow<IS, true><<<shape.blocks_shadow, shape.threads, sm, stream>>>(sc, ws, 0);
                    end(kFamShadow);
                    ++nl;
                }
                // no sphere table needed: the nearest hit comes from k_primary
                begin(kFamExtend);
                if (inl) k_first<kIsGlobal, true, true><<<g0, kExtendThreads, 0, stream>>>(sc, cam, ws, job);
                else k_first<kIsGlobal, true, false><<<g0, kExtendThreads, 0, stream>>>(sc, cam, ws, job);
                end(kFamExtend);
            } else {
                begin(kFamExtend);
                if constexpr (IS != kIsBvh) {
                    if (inl) k_first<IS, false, true><<<g0, kExtendThreads, sm, stream>>>(sc, cam, ws, job);
                    else k_first<IS, false, false><<<g0, kExtendThreads, sm, stream>>>(sc, cam, ws, job);
                } else {
                    k_first<IS, false, false><<<g0, kExtendThreads, sm, stream>>>(sc, cam, ws, job);
                }
                end(kFamExtend);
            }
            ++nl;
            for (int b = 0; b < bounces; ++b) {
                if constexpr (IS != kIsBvh) {
                    if (inl && b >= kPathsFrom) {   // the late bounces in one persistent launch
                        // on half the resident blocks: the late bounces are a trickle of
                        // paths, and the blocks stay resident until their pools drain,
                        // holding slots the other lanes' kernels could use (+1%)
                        begin(kFamExtend);
                        k_paths<kIsGlobal><<<max(1, shape.blocks_extend / 2), kExtendThreads, 0, stream>>>(sc, ws, job,
                                                                                                           b);
                        end(kFamExtend);
                        ++nl;
                        break;
                    }
                }
                if (b > 0) {
                    begin(kFamExtend);
                    if constexpr (IS != kIsBvh) {
                        if (inl) k_shade<kIsGlobal><<<shape.blocks_extend, kExtendThreads, 0, stream>>>(sc, ws, job, b);
                        else k_bounce<IS><<<shape.blocks_extend, kExtendThreads, sm, stream>>>(sc, ws, job, b);
                    } else {
                        k_bounce<IS><<<shape.blocks_extend, kExtendThreads, sm, stream>>>(sc, ws, job, b);
                    }
                    end(kFamExtend);
                    ++nl;
                }
                if ((vis && b == 0) || inl) continue;   // tested in k_first / k_shade / k_paths
                begin(kFamShadow);
                k_shadow<IS, false><<<shape.blocks_shadow, shape.threads, sm, stream>>>(sc, ws, b);
                end(kFamShadow);
                ++nl;
            }
        });
    }
    begin(kFamAccumulate);
    k_accumulate<<<grid_for(job.n_pixels, kThreads, 4096), kThreads, 0, stream>>>(ws, job, accum, image);
    end(kFamAccumulate);
    ++nl;
    if (launches) *launches += nl;
    return cudaGetLastError();
}

cudaError_t enqueue_clear_accum(float4* accum, uint64_t n, cudaStream_t stream)
{
    k_clear<<<grid_for(n, kThreads, 4096), kThreads, 0, stream>>>(accum, n);
    return cudaGetLastError();
}

cudaError_t enqueue_trace_nearest(const SceneView& sc, const float* origins, const float* dirs, uint64_t n,
                                  float* t_out, int32_t* id_out, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    const int g = grid_for(n, kThreads, 4096);
    const int mode = isect_mode(sc);
    const size_t bytes = mode == kIsSmem ? smem_table_bytes(sc.n_sph) : 0;
    cudaError_t e = cudaSuccess;
    with_mode(mode, [&](auto m) {
        constexpr int IS = decltype(m)::value;
        if (bytes > 48 * 1024)
            e = cudaFuncSetAttribute(k_trace<IS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e == cudaSuccess) k_trace<IS><<<g, kThreads, bytes, stream>>>(sc, origins, dirs, n, t_out, id_out);
    });
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t enqueue_dir_table(const CameraView& cam, float4* out, cudaStream_t stream)
{
    const uint64_t n = (uint64_t)cam.width * cam.height;
    if (n == 0) return cudaSuccess;
    k_dir_table<<<grid_for(n, kThreads, 4096), kThreads, 0, stream>>>(cam, out);
    return cudaGetLastError();
}

cudaError_t enqueue_tile_masks(const SceneView& sc, const CameraView& cam, uint32_t* masks, cudaStream_t stream)
{
    const uint64_t px = (uint64_t)cam.width * cam.height;
    if (px == 0 || sc.n_sph == 0 || sc.n_sph > kTileMaskMaxSpheres) return cudaErrorInvalidValue;
    const uint64_t tiles = (px + 31u) / 32u;
    k_tile_masks<<<grid_for(tiles * 32u, kThreads, 4096), kThreads, 0, stream>>>(sc, cam, masks);
    return cudaGetLastError();
}

cudaError_t enqueue_tile_list_counts(const SceneView& sc, const CameraView& cam, uint2* info, uint32_t* total,
                                     cudaStream_t stream)
{
    const uint64_t px = (uint64_t)cam.width * cam.height;
    if (px == 0 || !sc.use_bvh || sc.bvh.n_leaves < 2) return cudaErrorInvalidValue;
    const uint64_t tiles = (px + 31u) / 32u;
    k_tile_lists<false><<<grid_for(tiles * 32u, kThreads, 4096), kThreads, 0, stream>>>(sc, cam, info, nullptr);
    k_tile_list_scan<<<1, kThreads, 0, stream>>>(info, tiles, total);
    return cudaGetLastError();
}

cudaError_t enqueue_tile_list_fill(const SceneView& sc, const CameraView& cam, const uint2* info, uint32_t* lists,
                                   cudaStream_t stream)
{
    const uint64_t px = (uint64_t)cam.width * cam.height;
    if (px == 0 || !sc.use_bvh || sc.bvh.n_leaves < 2) return cudaErrorInvalidValue;
    const uint64_t tiles = (px + 31u) / 32u;
    k_tile_lists<true><<<grid_for(tiles * 32u, kThreads, 4096), kThreads, 0, stream>>>(
        sc, cam, const_cast<uint2*>(info), lists);
    return cudaGetLastError();
}

cudaError_t enqueue_primary_dirs(const CameraView& cam, float* out, cudaStream_t stream)
{
    const uint64_t n = (uint64_t)cam.width * cam.height;
    if (n == 0) return cudaSuccess;
    k_primary_dirs<<<grid_for(n, kThreads, 4096), kThreads, 0, stream>>>(cam, out);
    return cudaGetLastError();
}

}  // namespace atx
