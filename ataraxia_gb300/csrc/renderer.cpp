// Renderer: the reference's Renderer::onResize / Render state machine
// (Renderer.cu:98-249) over the wavefront kernels, with explicit scene upload,
// device-side ray generation and status codes instead of exit()/stderr.
#include "renderer.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "lbvh.h"
#include "light_buffer.h"

namespace atx {

namespace {
constexpr uint32_t kDefaultWavePaths = 64u << 20;  // at most 64 Mi paths (8.7 GB of state) per wave
constexpr uint32_t kDefaultBvhThreshold = 1025;  // LBVH above the direction buffer's 1,024 spheres (64-scene mix: +23% over 512)
constexpr uint32_t kDefaultBvhLeaf = 16;   // fastest of 1..32 on the 65,536-sphere scene
constexpr uint32_t kMaxBounces = 4096;
}  // namespace

// ------------------------------------------------------------------ scene

atx_status SceneStore::upload(const atx_sphere* s, uint32_t n, const atx_material* m, uint32_t nm,
                              const atx_light* l, uint32_t nl, Budget* budget, cudaStream_t stream)
{
    if ((n && !s) || (nm && !m) || (nl && !l)) return fail(ATX_ERR_INVALID_ARG, "set_scene: null array");
    if (n > 0 && nm == 0) return fail(ATX_ERR_INVALID_ARG, "set_scene: spheres need at least one material");
    for (DeviceBuffer* b : {&this->sph, &sph_mat, &sph_rad, &mat, &lights, &bvh, &lbuf, &dbuf})
        b->use_stream_order(order);

    std::vector<float4> sph(n);
    std::vector<int32_t> smat(n);
    std::vector<float> srad(n);
    for (uint32_t i = 0; i < n; ++i) {
        const float r = s[i].radius;
        sph[i] = make_float4(s[i].center[0], s[i].center[1], s[i].center[2], r * r);
        // Renderer.cu:30-37: ids outside [0, materials) render with material 0
        smat[i] = ((uint32_t)s[i].material >= nm) ? 0 : s[i].material;
        srad[i] = r;
    }
    std::vector<DevMaterial> mats(nm);
    for (uint32_t i = 0; i < nm; ++i) {
        DevMaterial& d = mats[i];
        for (int k = 0; k < 3; ++k) {
            d.albedo[k] = m[i].albedo[k];
            d.f0[k] = m[i].f0[k];
            d.emission[k] = m[i].emission_color[k] * m[i].emission_intensity;  // Scene.h:41
        }
        d.roughness = m[i].roughness;
        d.metallic = m[i].metallic;
        d.emission_intensity = m[i].emission_intensity;
    }
    std::vector<DevLight> lts(nl);
    for (uint32_t i = 0; i < nl; ++i) {
        for (int k = 0; k < 3; ++k) {
            lts[i].pos[k] = l[i].position[k];
            lts[i].le[k] = l[i].color[k] * l[i].intensity;  // Renderer.cu:362
        }
        lts[i].pad0 = lts[i].pad1 = 0.0f;
    }

    ATX_TRY(sph.empty() ? ATX_OK : this->sph.ensure(n * sizeof(float4), budget, "sphere table"));
    ATX_TRY(smat.empty() ? ATX_OK : sph_mat.ensure(n * sizeof(int32_t), budget, "sphere materials"));
    ATX_TRY(srad.empty() ? ATX_OK : sph_rad.ensure(n * sizeof(float), budget, "sphere radii"));
    ATX_TRY(mats.empty() ? ATX_OK : mat.ensure(nm * sizeof(DevMaterial), budget, "materials"));
    ATX_TRY(lts.empty() ? ATX_OK : lights.ensure(nl * sizeof(DevLight), budget, "lights"));
    // The host vectors die at return: copy synchronously with respect to them.
    if (n) {
        ATX_CUDA(cudaMemcpyAsync(this->sph.get(), sph.data(), n * sizeof(float4), cudaMemcpyHostToDevice, stream));
        ATX_CUDA(cudaMemcpyAsync(sph_mat.get(), smat.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, stream));
        ATX_CUDA(cudaMemcpyAsync(sph_rad.get(), srad.data(), n * sizeof(float), cudaMemcpyHostToDevice, stream));
    }
    if (nm) ATX_CUDA(cudaMemcpyAsync(mat.get(), mats.data(), nm * sizeof(DevMaterial), cudaMemcpyHostToDevice, stream));
    if (nl) ATX_CUDA(cudaMemcpyAsync(lights.get(), lts.data(), nl * sizeof(DevLight), cudaMemcpyHostToDevice, stream));

    view = SceneView{};
    view.sph = n ? this->sph.as<float4>() : nullptr;
    view.sph_mat = n ? sph_mat.as<int32_t>() : nullptr;
    view.mat = nm ? mat.as<DevMaterial>() : nullptr;
    view.lights = nl ? lights.as<DevLight>() : nullptr;
    view.n_sph = n;
    view.n_mat = nm;
    view.n_lights = nl;
    view.light_mod = fastmod_multiplier(nl);

    const uint32_t thr = bvh_threshold ? bvh_threshold : kDefaultBvhThreshold;
    if (n >= thr && n > 1) {
        const uint64_t need = lbvh_bytes(n);
        ATX_TRY(bvh.ensure(need, budget, "lbvh"));
        BvhView bv{};
        ATX_CUDA(lbvh_build(view.sph, sph_rad.as<float>(), n, bvh_leaf ? bvh_leaf : kDefaultBvhLeaf, bvh.get(),
                            bvh.bytes(), &bv, stream));
        view.bvh = bv;
        view.use_bvh = 1;
    } else {
        bvh.reset();
    }
    ATX_TRY(build_cells(budget, stream));
    ATX_CUDA(cudaStreamSynchronize(stream));
    return ATX_OK;
}

atx_status SceneStore::build_cells(Budget* budget, cudaStream_t stream)
{
    const uint32_t n = view.n_sph, nl = view.n_lights;
    const uint32_t res = cell_res ? cell_res : default_cell_res(n);
    // light buffer for the shadow rays of the brute-force tables
    view.lb = LightBufferView{};
    if (!view.use_bvh && n >= 1 && n <= kLbMaxSpheres && nl >= 1 && nl <= kLbMaxLights) {
        ATX_TRY(lbuf.ensure(lb_bytes(nl, res), budget, "light buffer"));
        LightBufferView lv{};
        ATX_CUDA(lb_build(view.sph, sph_rad.as<float>(), n, view.lights, nl, res, lbuf.get(), lbuf.bytes(), &lv,
                          stream));
        view.lb = lv;
    } else {
        lbuf.reset();
    }
    // direction buffer for the extension rays of the brute-force tables
    view.db = DirBufferView{};
    if (!view.use_bvh && n >= 1 && n <= kDbMaxSpheres) {
        ATX_TRY(dbuf.ensure(db_bytes(n, res), budget, "direction buffer"));
        DirBufferView dv{};
        ATX_CUDA(db_build(view.sph, sph_rad.as<float>(), n, res, dbuf.get(), dbuf.bytes(), &dv, stream));
        view.db = dv;
    } else {
        dbuf.reset();
    }
    return ATX_OK;
}

uint32_t SceneStore::cells() const
{
    return view.db.n ? view.db.res : view.lb.n_lights ? view.lb.res : 0u;
}

atx_status SceneStore::rebuild_cells(uint32_t res, Budget* budget, cudaStream_t stream)
{
    if (res && (res < kCellResMin || res > kCellResMax))
        return fail(ATX_ERR_INVALID_ARG, "cell resolution %u outside %u..%u", res, kCellResMin, kCellResMax);
    cell_res = res;
    if (cells() == 0 || cells() == (res ? res : default_cell_res(view.n_sph))) return ATX_OK;
    ATX_TRY(build_cells(budget, stream));
    ATX_CUDA(cudaStreamSynchronize(stream));
    return ATX_OK;
}

uint32_t SceneStore::leaf_size() const
{
    return view.use_bvh ? view.bvh.leaf_size : 0u;
}

atx_status SceneStore::rebuild_bvh(uint32_t leaf, cudaStream_t stream)
{
    if (!view.use_bvh) return ATX_OK;
    if (leaf == 0) leaf = bvh_leaf ? bvh_leaf : kDefaultBvhLeaf;
    if (leaf == view.bvh.leaf_size) return ATX_OK;
    BvhView bv{};
    ATX_CUDA(lbvh_build(view.sph, sph_rad.as<float>(), view.n_sph, leaf, bvh.get(), bvh.bytes(), &bv, stream));
    view.bvh = bv;
    ATX_CUDA(cudaStreamSynchronize(stream));
    return ATX_OK;
}

// ------------------------------------------------------------------ waves

uint64_t WaveStore::bytes_for(uint32_t capacity, uint32_t max_bounces)
{
    const uint64_t c = capacity;
    return c * kWaveBytesPerPath + wave_counter_words((int)max_bounces) * sizeof(uint32_t) + 16 +
           (kWaveArrays + 1) * 256;
}

atx_status WaveStore::ensure(uint32_t capacity, uint32_t max_bounces, Budget* budget)
{
    if (view.capacity >= capacity && bounces >= max_bounces && buf.get()) return ATX_OK;
    const uint32_t cap = std::max(capacity, view.capacity);
    const uint32_t b = std::max(max_bounces, bounces);
    buf.reset();
    ATX_TRY(buf.ensure(bytes_for(cap, b), budget, "path state"));
    char* p = buf.as<char>();
    auto take = [&](uint64_t bytes) {
        char* r = p;
        p += (bytes + 255) & ~uint64_t(255);
        return r;
    };
    const uint64_t c = cap;
    view.ray_o = reinterpret_cast<float4*>(take(c * sizeof(float4)));
    view.ray_d = reinterpret_cast<float4*>(take(c * sizeof(float4)));
    view.thr = reinterpret_cast<float4*>(take(c * sizeof(float4)));
    view.col = reinterpret_cast<float4*>(take(c * sizeof(float4)));
    view.sh_o = reinterpret_cast<float4*>(take(c * sizeof(float4)));
    view.sh_d = reinterpret_cast<float4*>(take(c * sizeof(float4)));
    view.sh_c = reinterpret_cast<float4*>(take(c * sizeof(float4)));
    view.q[0] = reinterpret_cast<uint32_t*>(take(c * sizeof(uint32_t)));
    view.q[1] = reinterpret_cast<uint32_t*>(take(c * sizeof(uint32_t)));
    view.prim = reinterpret_cast<uint2*>(take(c * sizeof(uint2)));
    view.hitq = reinterpret_cast<uint32_t*>(take(c * sizeof(uint32_t)));
    view.vis = reinterpret_cast<uint32_t*>(take(c * sizeof(uint32_t)));
    view.counters = reinterpret_cast<uint32_t*>(take(wave_counter_words((int)b) * sizeof(uint32_t)));
    view.capacity = cap;
    bounces = b;
    return ATX_OK;
}

WavePlan plan_waves(uint64_t pixels, uint32_t spp, uint32_t capacity, uint32_t cap_spp)
{
    WavePlan p;
    // keep at least 256 pixels per wave so the first bounce fills the GPU
    uint32_t max_spp = std::max<uint32_t>(1, capacity / 256);
    if (cap_spp) max_spp = std::min(max_spp, cap_spp);
    p.spp_per_wave = std::min(spp, max_spp);
    uint64_t ppw = capacity / p.spp_per_wave;
    if (ppw < 1) ppw = 1;
    if (ppw > pixels) ppw = pixels;
    p.pixels_per_wave = (uint32_t)ppw;
    return p;
}

EventTimer::~EventTimer()
{
    for (auto& r : recs_) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (cudaEvent_t e : pool_) cudaEventDestroy(e);
}

cudaEvent_t EventTimer::take()
{
    if (!pool_.empty()) {
        cudaEvent_t e = pool_.back();
        pool_.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

void EventTimer::begin(int, cudaStream_t stream)
{
    open_ = take();
    if (open_) cudaEventRecord(open_, stream);
}

void EventTimer::end(int family, cudaStream_t stream)
{
    if (!open_) return;
    cudaEvent_t b = take();
    if (!b) {
        pool_.push_back(open_);
        open_ = nullptr;
        return;
    }
    cudaEventRecord(b, stream);
    recs_.push_back(Rec{family, open_, b});
    open_ = nullptr;
}

atx_status EventTimer::collect(atx_kernel_times* t)
{
    for (auto& r : recs_) {
        ATX_CUDA(cudaEventSynchronize(r.b));
        float ms = 0.0f;
        ATX_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        double* dst[4] = {&t->extend_ms, &t->shadow_ms, &t->accumulate_ms, &t->other_ms};
        uint64_t* cnt[4] = {&t->extend_launches, &t->shadow_launches, &t->accumulate_launches, &t->other_launches};
        *dst[r.family] += ms;
        *cnt[r.family] += 1;
        pool_.push_back(r.a);
        pool_.push_back(r.b);
    }
    recs_.clear();
    return ATX_OK;
}

atx_status enqueue_frames(const SceneView& sc, const CameraView& cam, WaveStore& ws, const LaunchShape& shape,
                          uint32_t frame0, uint32_t spp, int32_t max_bounces, int32_t sky, float4* accum,
                          uint32_t* image, uint32_t capacity, cudaStream_t stream, uint32_t* launches,
                          KernelTimer* timer, uint64_t* primary_rays, uint64_t pix_begin, uint64_t pix_end,
                          uint2* prim_cache, bool prim_cached, uint32_t wave_spp)
{
    const uint64_t all = (uint64_t)cam.width * cam.height;
    const uint64_t pend = std::min(pix_end, all);
    const uint64_t pbeg = std::min(pix_begin, pend);
    const WavePlan plan = plan_waves(pend - pbeg, spp, capacity, wave_spp);
    const uint32_t last_frame = frame0 + spp - 1;
    for (uint64_t p0 = pbeg; p0 < pend; p0 += plan.pixels_per_wave) {
        const uint32_t np = (uint32_t)std::min<uint64_t>(plan.pixels_per_wave, pend - p0);
        bool filled = prim_cached;   // primary hits of these pixels already traced
        for (uint32_t s0 = 0; s0 < spp; s0 += plan.spp_per_wave) {
            WaveJob job;
            job.pixel0 = (uint32_t)p0;
            job.n_pixels = np;
            job.spp = std::min(plan.spp_per_wave, spp - s0);
            job.frame0 = frame0 + s0;
            job.max_bounces = max_bounces;
            job.sky = sky;
            job.pack_frame = (s0 + job.spp >= spp && image) ? last_frame : 0u;
            job.prim_cache = prim_cache;
            // later sample chunks of the same pixels reuse the hits the first traced
            // (in the cache, or in the wave's own per-pixel rows, which only k_primary writes)
            job.prim_cached = filled ? 1 : 0;
            ATX_CUDA(enqueue_wave(sc, cam, ws.view, job, shape, accum, image, stream, launches, timer));
            if (wave_shares_primary(job)) filled = true;
            // primary rays traced: once per pixel when its samples share the hit, none when cached
            if (primary_rays && max_bounces > 0 && !job.prim_cached)
                *primary_rays += wave_shares_primary(job) ? np : (uint64_t)np * job.spp;
        }
    }
    return ATX_OK;
}

// ---------------------------------------------------------------- renderer

Renderer::Renderer(const atx_config& cfg) : cfg_(cfg), budget_(cfg.hbm_budget_bytes) {}

Renderer::~Renderer()
{
    if (cudaSetDevice(cfg_.device) == cudaSuccess) {
        if (stream_) cudaStreamSynchronize(stream_);
        for (int l = 0; l < kLanes; ++l)
            if (lane_stream_[l]) cudaStreamSynchronize(lane_stream_[l]);
        scene_ = SceneStore();
        for (WaveStore& w : wave_) w.buf.reset();
        if (fork_) cudaEventDestroy(fork_);
        for (int l = 0; l < kLanes; ++l) {
            if (join_[l]) cudaEventDestroy(join_[l]);
            if (lane_stream_[l] && lane_stream_[l] != stream_) cudaStreamDestroy(lane_stream_[l]);
        }
        if (time_stream_) cudaStreamDestroy(time_stream_);
        if (copy_stream_) cudaStreamSynchronize(copy_stream_);
        accum_.reset();
        image_.reset();
        image_alt_.reset();
        for (cudaEvent_t& e : read_done_)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t& e : ticket_ev_)
            if (e) cudaEventDestroy(e);
        if (src_ready_) cudaEventDestroy(src_ready_);
        if (copy_stream_) cudaStreamDestroy(copy_stream_);
        totals_.reset();
        if (ev_start_) cudaEventDestroy(ev_start_);
        if (ev_stop_) cudaEventDestroy(ev_stop_);
        if (stream_) cudaStreamDestroy(stream_);
    }
}

atx_status Renderer::activate() const
{
    ATX_CUDA(cudaSetDevice(cfg_.device));
    return ATX_OK;
}

atx_status Renderer::init()
{
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        (void)cudaGetLastError();
        return fail(ATX_ERR_NO_DEVICE, "no CUDA device visible (%s)", cudaGetErrorString(e));
    }
    if (cfg_.device < 0 || cfg_.device >= count)
        return fail(ATX_ERR_INVALID_ARG, "device %d out of range (%d visible)", cfg_.device, count);
    ATX_TRY(activate());
    ATX_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    overlap_ = (cfg_.flags & ATX_FLAG_OVERLAP_RENDERS) != 0;
    lane_stream_[0] = stream_;
    for (int l = overlap_ ? 0 : 1; l < kLanes; ++l) {
        ATX_CUDA(cudaStreamCreateWithFlags(&lane_stream_[l], cudaStreamNonBlocking));
        ATX_CUDA(cudaEventCreateWithFlags(&join_[l], cudaEventDisableTiming));
    }
    if (overlap_) ATX_CUDA(cudaStreamCreateWithFlags(&time_stream_, cudaStreamNonBlocking));
    ATX_CUDA(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking));
    for (cudaEvent_t& e : read_done_) ATX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (cudaEvent_t& e : ticket_ev_) ATX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ATX_CUDA(cudaEventCreateWithFlags(&src_ready_, cudaEventDisableTiming));
    ATX_CUDA(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
    ATX_CUDA(cudaEventCreate(&ev_start_));
    ATX_CUDA(cudaEventCreate(&ev_stop_));
    ATX_TRY(totals_.ensure(3 * sizeof(unsigned long long), &budget_, "ray totals"));
    ATX_CUDA(cudaMemsetAsync(totals_.get(), 0, 3 * sizeof(unsigned long long), stream_));
    scene_.bvh_threshold = cfg_.bvh_threshold;
    scene_.bvh_leaf = cfg_.bvh_leaf_size;
    // empty scene until set_scene
    ATX_TRY(scene_.upload(nullptr, 0, nullptr, 0, nullptr, 0, &budget_, stream_));
    return ATX_OK;
}

atx_status Renderer::resize(uint32_t w, uint32_t h)
{
    if (w == 0 || h == 0) return fail(ATX_ERR_INVALID_ARG, "resize: width and height must be non-zero");
    if ((uint64_t)w * h > 0xffffffffull) return fail(ATX_ERR_INVALID_ARG, "resize: more than 2^32 pixels");
    if (w == width_ && h == height_ && accum_.get()) return ATX_OK;  // Renderer.cu:100-101
    ATX_TRY(activate());
    ATX_TRY(join());
    ATX_CUDA(cudaStreamSynchronize(stream_));
    ATX_CUDA(cudaStreamSynchronize(copy_stream_));
    read_pending_[0] = read_pending_[1] = false;
    const uint64_t px = (uint64_t)w * h;
    accum_.reset();
    image_.reset();
    image_alt_.reset();
    ATX_TRY(accum_.ensure(px * sizeof(float4), &budget_, "accumulation buffer"));
    ATX_TRY(image_.ensure(px * sizeof(uint32_t), &budget_, "image buffer"));
    if (overlap_) ATX_TRY(image_alt_.ensure(px * sizeof(uint32_t), &budget_, "second image buffer"));
    img_last_ = img_next_ = 0;
    width_ = w;
    height_ = h;
    frame_ = 1;  // Renderer.cu:145
    cam_dirty_ = true;
    return ATX_OK;
}

atx_status Renderer::set_scene(const atx_sphere* s, uint32_t n, const atx_material* m, uint32_t nm,
                               const atx_light* l, uint32_t nl)
{
    ATX_TRY(activate());
    ATX_TRY(join());
    ATX_CUDA(cudaStreamSynchronize(stream_));
    shape_valid_ = false;
    masks_valid_ = false;
    prev_cam_valid_ = false;
    scene_.bvh_leaf = tune_.bvh_leaf_size ? tune_.bvh_leaf_size : cfg_.bvh_leaf_size;
    scene_.cell_res = tune_.cell_res;
    return scene_.upload(s, n, m, nm, l, nl, &budget_, stream_);
}

atx_status Renderer::set_settings(const atx_settings& s)
{
    if (s.max_bounces > (int32_t)kMaxBounces)
        return fail(ATX_ERR_INVALID_ARG, "max_bounces %d above the supported %u", s.max_bounces, kMaxBounces);
    settings_ = s;
    return ATX_OK;
}

atx_status Renderer::set_camera(const atx_camera& c)
{
    cam_desc_ = c;
    cam_from_desc_ = true;
    cam_dirty_ = true;
    return ATX_OK;
}

atx_status Renderer::set_camera_matrices(const float inv_view[16], const float inv_proj[16], const float pos[3])
{
    std::memcpy(camv_.inv_view, inv_view, sizeof(camv_.inv_view));
    std::memcpy(camv_.inv_proj, inv_proj, sizeof(camv_.inv_proj));
    std::memcpy(camv_.pos, pos, sizeof(camv_.pos));
    cam_from_desc_ = false;
    cam_dirty_ = false;
    return ATX_OK;
}

atx_status Renderer::refresh_dirs()
{
    // the table depends on the matrices and the viewport, not on the eye
    camv_.dirs = nullptr;
    const bool same = dirs_valid_ && dirs_cam_.width == camv_.width && dirs_cam_.height == camv_.height &&
                      std::memcmp(dirs_cam_.inv_proj, camv_.inv_proj, sizeof(camv_.inv_proj)) == 0 &&
                      std::memcmp(dirs_cam_.inv_view, camv_.inv_view, sizeof(camv_.inv_view)) == 0;
    if (!same) {
        const uint64_t px = (uint64_t)camv_.width * camv_.height;
        ATX_TRY(dirs_.ensure(px * sizeof(float4), &budget_, "primary directions"));
        ATX_CUDA(enqueue_dir_table(camv_, dirs_.as<float4>(), stream_));
        stream_dirty_ = true;
        dirs_cam_ = camv_;
        dirs_valid_ = true;
    }
    camv_.dirs = dirs_.as<float4>();
    return ATX_OK;
}

atx_status Renderer::refresh_masks()
{
    camv_.masks = nullptr;
    camv_.mask_words = 0;
    camv_.tile_info = nullptr;
    camv_.tile_lists = nullptr;
    const SceneView& sc = scene_.view;
    // the masks and lists depend on the directions (matrices, viewport), the eye and the spheres
    auto same_view = [](const CameraView& a, const CameraView& b) {
        return a.width == b.width && a.height == b.height &&
               std::memcmp(a.inv_proj, b.inv_proj, sizeof(a.inv_proj)) == 0 &&
               std::memcmp(a.inv_view, b.inv_view, sizeof(a.inv_view)) == 0 &&
               std::memcmp(a.pos, b.pos, sizeof(a.pos)) == 0;
    };
    const bool same = masks_valid_ && same_view(masks_cam_, camv_);
    // built for a camera that stayed put since the previous render only
    const bool still = prev_cam_valid_ && same_view(prev_cam_, camv_);
    prev_cam_ = camv_;
    prev_cam_valid_ = true;
    if (!same && !still) return ATX_OK;
    const uint64_t tiles = ((uint64_t)camv_.width * camv_.height + 31u) / 32u;
    if (sc.use_bvh) {
        if (sc.bvh.n_leaves < 2 || sc.bvh.n_leaves <= sc.bvh.leaf_size) return ATX_OK;
        if (!same) {
            ATX_TRY(tile_info_.ensure((tiles + 1) * sizeof(uint2), &budget_, "primary tile list heads"));
            uint2* info = tile_info_.as<uint2>();
            uint32_t* total = reinterpret_cast<uint32_t*>(info + tiles);
            ATX_CUDA(enqueue_tile_list_counts(sc, camv_, info, total, stream_));
            uint32_t n = 0;
            ATX_CUDA(cudaMemcpyAsync(&n, total, sizeof(n), cudaMemcpyDeviceToHost, stream_));
            ATX_CUDA(cudaStreamSynchronize(stream_));
            ATX_TRY(tile_lists_.ensure((uint64_t)(n ? n : 1u) * sizeof(uint32_t), &budget_, "primary tile lists"));
            ATX_CUDA(enqueue_tile_list_fill(sc, camv_, info, tile_lists_.as<uint32_t>(), stream_));
            stream_dirty_ = true;
            masks_cam_ = camv_;
            masks_valid_ = true;
        }
        camv_.tile_info = tile_info_.as<uint2>();
        camv_.tile_lists = tile_lists_.as<uint32_t>();
        return ATX_OK;
    }
    if (sc.n_sph == 0 || sc.n_sph > kTileMaskMaxSpheres) return ATX_OK;
    const uint32_t words = tile_mask_words(sc.n_sph);
    if (!same) {
        ATX_TRY(masks_.ensure(tiles * words * sizeof(uint32_t), &budget_, "primary tile masks"));
        ATX_CUDA(enqueue_tile_masks(sc, camv_, masks_.as<uint32_t>(), stream_));
        stream_dirty_ = true;
        masks_cam_ = camv_;
        masks_valid_ = true;
    }
    camv_.masks = masks_.as<uint32_t>();
    camv_.mask_words = words;
    return ATX_OK;
}

// Whether render() would put no work on stream_ for the per-camera tables:
// the directions are those of the current matrices and viewport, and the
// primary tile masks or lists (where the scene has them) those of the
// current camera, eye and scene.
bool Renderer::tables_current() const
{
    auto same_view = [](const CameraView& a, const CameraView& b) {
        return a.width == b.width && a.height == b.height &&
               std::memcmp(a.inv_proj, b.inv_proj, sizeof(a.inv_proj)) == 0 &&
               std::memcmp(a.inv_view, b.inv_view, sizeof(a.inv_view)) == 0 &&
               std::memcmp(a.pos, b.pos, sizeof(a.pos)) == 0;
    };
    const bool dirs = dirs_valid_ && dirs_cam_.width == camv_.width && dirs_cam_.height == camv_.height &&
                      std::memcmp(dirs_cam_.inv_proj, camv_.inv_proj, sizeof(camv_.inv_proj)) == 0 &&
                      std::memcmp(dirs_cam_.inv_view, camv_.inv_view, sizeof(camv_.inv_view)) == 0;
    if (!dirs) return false;
    const SceneView& sc = scene_.view;
    const bool has_tables = sc.use_bvh ? (sc.bvh.n_leaves >= 2 && sc.bvh.n_leaves > sc.bvh.leaf_size)
                                       : (sc.n_sph >= 1 && sc.n_sph <= kTileMaskMaxSpheres);
    return !has_tables || (masks_valid_ && same_view(masks_cam_, camv_));
}

atx_status Renderer::join()
{
    if (!joins_pending_) return ATX_OK;
    ATX_TRY(activate());
    for (uint32_t l = 0; l < pending_lanes_; ++l) ATX_CUDA(cudaStreamWaitEvent(stream_, join_[l], 0));
    joins_pending_ = false;
    stream_dirty_ = true;   // what follows on stream_ comes before the next render's lanes
    return ATX_OK;
}

atx_status Renderer::refresh_camera()
{
    camv_.width = width_;
    camv_.height = height_;
    if (cam_from_desc_ && (cam_dirty_ || cam_w_ != width_ || cam_h_ != height_)) {
        camera_matrices(cam_desc_, width_, height_, nullptr, camv_.inv_view, nullptr, camv_.inv_proj);
        std::memcpy(camv_.pos, cam_desc_.position, sizeof(camv_.pos));
        cam_w_ = width_;
        cam_h_ = height_;
        cam_dirty_ = false;
    }
    return ATX_OK;
}

atx_status Renderer::ensure_shape()
{
    if (shape_valid_) return ATX_OK;
    ATX_CUDA(plan_launch(scene_.view, cfg_.device, (int)(tune_.threads ? tune_.threads : cfg_.threads), &shape_,
                         (int)tune_.path_kernel));
    shape_valid_ = true;
    return ATX_OK;
}

atx_status Renderer::render(uint32_t spp)
{
    if (!width_ || !height_ || !accum_.get()) return fail(ATX_ERR_INVALID_ARG, "render: call atx_resize first");
    if (spp == 0) return ATX_OK;
    ATX_TRY(activate());
    ATX_TRY(refresh_camera());
    ATX_TRY(ensure_shape());
    // One wave per lane when it fits: fewer, fuller kernels (the state is
    // allocated for this launch's paths, rounded up to 1 Mi, and kept).  Up
    // to the lane count for the scene (at least 4 Mi paths each), one lane
    // when the caller fixed the wave size or kernels are being timed one by
    // one.  Scenes with light and direction buffers run their late bounces in
    // one persistent launch and, with each render joined, overlap best on two
    // lanes; LBVH scenes, and every scene with overlapped renders (whose lanes
    // run on from one render into the next), use four (large scene: 4 lanes
    // +11% over 2; medium scene overlapped: 4 lanes +12% over 2).
    const uint64_t px = (uint64_t)width_ * height_;
    const bool profile = (cfg_.flags & ATX_FLAG_PROFILE_KERNELS) != 0;
    uint32_t max_lanes = (!overlap_ && !scene_.view.use_bvh && scene_.view.lb.n_lights) ? kBufferedLanes
                                                                                         : kDefaultLanes;
    if (tune_.lanes) max_lanes = std::min<uint32_t>(tune_.lanes, kLanes);
    const uint32_t wave_paths = tune_.wave_paths ? tune_.wave_paths : cfg_.wave_paths;
    // at least 4 Mi paths per lane
    const uint64_t fill = std::max<uint64_t>(1, px * spp / (4ull << 20));
    const uint32_t lanes = ((cfg_.wave_paths && !tune_.lanes) || profile)
                               ? 1u
                               : (uint32_t)std::min<uint64_t>({(uint64_t)max_lanes, fill, px});
    const uint64_t lane_px = (px + lanes - 1) / lanes;
    uint32_t capacity = wave_paths;
    if (!capacity) {
        const uint64_t lane_paths = lane_px * spp;
        const uint64_t want = (lane_paths + (1u << 20) - 1) & ~uint64_t((1u << 20) - 1);
        capacity = (uint32_t)std::min<uint64_t>(want, kDefaultWavePaths);
    }
    const int32_t bounces = settings_.max_bounces;
    if (!settings_.accumulation) frame_ = 1;
    const uint32_t f0 = frame_;
    // overlapped renders: the lanes of earlier renders must be done before
    // this one puts work on stream_ (a clear, camera tables) or moves pixels
    // to another lane, and before a lane's path state is reallocated
    if (overlap_ && joins_pending_) {
        bool grow = false;
        for (uint32_t l = 0; l < lanes; ++l)
            grow = grow || wave_[l].view.capacity < capacity || wave_[l].bounces < (uint32_t)std::max(bounces, 0);
        if (f0 == 1 || !tables_current() || lanes != last_lanes_ || lane_px != last_lane_px_ || grow) ATX_TRY(join());
    }
    for (uint32_t l = 0; l < lanes; ++l) {
        ATX_TRY(wave_[l].ensure(capacity, bounces > 0 ? (uint32_t)bounces : 0u, &budget_));
        wave_[l].view.totals = totals_.as<unsigned long long>();
    }
    ATX_TRY(refresh_dirs());
    ATX_TRY(refresh_masks());

    uint32_t launches = 0;
    KernelTimer* timer = profile ? &timer_ : nullptr;
    if (!overlap_) ATX_CUDA(cudaEventRecord(ev_start_, stream_));
    if (f0 == 1) {  // Renderer.cu:181-182
        if (timer) timer->begin(kFamOther, stream_);
        ATX_CUDA(enqueue_clear_accum(accum_.as<float4>(), px, stream_));
        if (timer) timer->end(kFamOther, stream_);
        ++launches;
        stream_dirty_ = true;
    }
    uint64_t primary_rays = 0;
    const int32_t sky = settings_.sky_light ? 1 : 0;
    // the image buffer this render packs; an asynchronous read of its previous
    // contents must have landed first
    const int ib = overlap_ ? img_next_ : 0;
    if (read_pending_[ib]) {
        if (overlap_)
            for (uint32_t l = 0; l < lanes; ++l) ATX_CUDA(cudaStreamWaitEvent(lane_stream_[l], read_done_[ib], 0));
        else
            ATX_CUDA(cudaStreamWaitEvent(stream_, read_done_[ib], 0));
        read_pending_[ib] = false;
    }
    if (!overlap_ && lanes > 1) {
        ATX_CUDA(cudaEventRecord(fork_, stream_));
        for (uint32_t l = 1; l < lanes; ++l) ATX_CUDA(cudaStreamWaitEvent(lane_stream_[l], fork_, 0));
    } else if (overlap_ && stream_dirty_) {
        ATX_CUDA(cudaEventRecord(fork_, stream_));
        for (uint32_t l = 0; l < lanes; ++l) ATX_CUDA(cudaStreamWaitEvent(lane_stream_[l], fork_, 0));
        stream_dirty_ = false;
    }
    if (overlap_) ATX_CUDA(cudaEventRecord(ev_start_, lane_stream_[0]));
    for (uint32_t l = 0; l < lanes; ++l) {
        const uint64_t b = std::min(px, l * lane_px), e = std::min(px, (l + 1) * lane_px);
        ATX_TRY(enqueue_frames(scene_.view, camv_, wave_[l], shape_, f0, spp, bounces, sky, accum_.as<float4>(),
                               image_buf(ib), capacity, lane_stream_[l], &launches, l == 0 ? timer : nullptr,
                               &primary_rays, b, e, nullptr, false, tune_.wave_spp));
    }
    if (overlap_) {
        for (uint32_t l = 0; l < lanes; ++l) {
            ATX_CUDA(cudaEventRecord(join_[l], lane_stream_[l]));
            ATX_CUDA(cudaStreamWaitEvent(time_stream_, join_[l], 0));
        }
        ATX_CUDA(cudaEventRecord(ev_stop_, time_stream_));
        joins_pending_ = true;
        pending_lanes_ = lanes;
        last_lanes_ = lanes;
        last_lane_px_ = lane_px;
    } else {
        for (uint32_t l = 1; l < lanes; ++l) {
            ATX_CUDA(cudaEventRecord(join_[l], lane_stream_[l]));
            ATX_CUDA(cudaStreamWaitEvent(stream_, join_[l], 0));
        }
        ATX_CUDA(cudaEventRecord(ev_stop_, stream_));
    }
    timed_ = true;
    img_last_ = ib;
    img_next_ = overlap_ ? 1 - ib : 0;
    frame_ = settings_.accumulation ? f0 + spp : 1u;  // Renderer.cu:245-248
    st_.frames += spp;
    st_.paths += (uint64_t)width_ * height_ * spp;
    st_.kernel_launches += launches;
    totals_host_[0] += primary_rays;
    return ATX_OK;
}

atx_status Renderer::synchronize()
{
    ATX_TRY(activate());
    ATX_TRY(join());
    ATX_CUDA(cudaStreamSynchronize(stream_));
    return ATX_OK;
}

atx_status Renderer::read_accumulation(float* host, uint64_t n)
{
    if (!host) return fail(ATX_ERR_INVALID_ARG, "read_accumulation: null buffer");
    if (n > (uint64_t)width_ * height_) return fail(ATX_ERR_INVALID_ARG, "read_accumulation: %llu pixels > image",
                                                    (unsigned long long)n);
    ATX_TRY(activate());
    ATX_TRY(join());
    ATX_CUDA(cudaMemcpyAsync(host, accum_.get(), n * sizeof(float4), cudaMemcpyDeviceToHost, stream_));
    ATX_CUDA(cudaStreamSynchronize(stream_));
    return ATX_OK;
}

atx_status Renderer::read_image(uint32_t* host, uint64_t n)
{
    if (!host) return fail(ATX_ERR_INVALID_ARG, "read_image: null buffer");
    if (n > (uint64_t)width_ * height_) return fail(ATX_ERR_INVALID_ARG, "read_image: %llu pixels > image",
                                                    (unsigned long long)n);
    ATX_TRY(activate());
    ATX_TRY(join());
    ATX_CUDA(cudaMemcpyAsync(host, image_buf(img_last_), n * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_));
    ATX_CUDA(cudaStreamSynchronize(stream_));
    return ATX_OK;
}

atx_status Renderer::read_image_async(uint32_t* host, uint64_t n, uint64_t* ticket)
{
    if (!host || !ticket) return fail(ATX_ERR_INVALID_ARG, "read_image_async: null pointer");
    if (n > (uint64_t)width_ * height_) return fail(ATX_ERR_INVALID_ARG, "read_image_async: %llu pixels > image",
                                                    (unsigned long long)n);
    ATX_TRY(activate());
    // after the last render's lanes (without joining them into stream_), or
    // after stream_'s work when renders are joined
    if (overlap_ && joins_pending_) {
        for (uint32_t l = 0; l < pending_lanes_; ++l) ATX_CUDA(cudaStreamWaitEvent(copy_stream_, join_[l], 0));
    } else {
        ATX_CUDA(cudaEventRecord(src_ready_, stream_));
        ATX_CUDA(cudaStreamWaitEvent(copy_stream_, src_ready_, 0));
    }
    ATX_CUDA(cudaMemcpyAsync(host, image_buf(img_last_), n * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             copy_stream_));
    ATX_CUDA(cudaEventRecord(read_done_[img_last_], copy_stream_));
    read_pending_[img_last_] = true;
    const int slot = (int)(tickets_ % kTickets);
    if (tickets_ >= (uint64_t)kTickets) ATX_CUDA(cudaEventSynchronize(ticket_ev_[slot]));   // the ticket it replaces
    ATX_CUDA(cudaEventRecord(ticket_ev_[slot], copy_stream_));
    *ticket = tickets_++;
    return ATX_OK;
}

atx_status Renderer::wait_read(uint64_t ticket)
{
    if (ticket >= tickets_) return fail(ATX_ERR_INVALID_ARG, "wait_read: unknown ticket %llu",
                                        (unsigned long long)ticket);
    // a ticket whose slot was reused was waited for when it was
    if (ticket + kTickets < tickets_) return ATX_OK;
    ATX_TRY(activate());
    ATX_CUDA(cudaEventSynchronize(ticket_ev_[ticket % kTickets]));
    return ATX_OK;
}

atx_status Renderer::device_buffers(void** accum, void** image)
{
    ATX_TRY(join());
    if (accum) *accum = accum_.get();
    if (image) *image = image_buf(img_last_);
    return ATX_OK;
}

atx_status Renderer::stats(atx_stats* out)
{
    ATX_TRY(activate());
    ATX_TRY(join());
    ATX_CUDA(cudaStreamSynchronize(stream_));
    unsigned long long dev[3] = {0, 0, 0};
    ATX_CUDA(cudaMemcpy(dev, totals_.get(), sizeof(dev), cudaMemcpyDeviceToHost));
    if (timed_) {
        float ms = 0.0f;
        ATX_CUDA(cudaEventElapsedTime(&ms, ev_start_, ev_stop_));
        st_.last_render_ms = ms;
    }
    *out = st_;
    out->extension_rays = totals_host_[0] + dev[0];
    out->shadow_rays = dev[1];
    out->shaded_first = dev[2];
    out->device_bytes = budget_.used();
    out->bvh_in_use = scene_.view.use_bvh;
    return ATX_OK;
}

atx_status Renderer::kernel_times(atx_kernel_times* out)
{
    ATX_TRY(activate());
    ATX_TRY(timer_.collect(&ktimes_));
    *out = ktimes_;
    return ATX_OK;
}

// ------------------------------------------------------------- autotuner

namespace {

// Tuned settings kept per process, keyed by the GPU (SM count and compute
// capability) and a bucket of the workload: log2 of the sphere count, the
// nearest-hit structure (LBVH, or brute force with light buffer or without),
// log2 of the paths per launch and the bounce depth.
struct TuneKey {
    int sms, cc;
    int sph_bucket, kind, path_bucket, bounces;
    bool operator<(const TuneKey& o) const
    {
        return std::tie(sms, cc, sph_bucket, kind, path_bucket, bounces) <
               std::tie(o.sms, o.cc, o.sph_bucket, o.kind, o.path_bucket, o.bounces);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, atx_tuning> g_tune_cache;

int log2_bucket(uint64_t x)
{
    int b = 0;
    while (x > 1) {
        x >>= 1;
        ++b;
    }
    return b;
}

}  // namespace

atx_status Renderer::set_tuning(const atx_tuning& t)
{
    if (t.lanes > (uint32_t)kLanes) return fail(ATX_ERR_INVALID_ARG, "tuning: at most %d lanes", kLanes);
    if (t.threads && (t.threads % 32u || t.threads > 256u))
        return fail(ATX_ERR_INVALID_ARG, "tuning: threads must be a multiple of 32 up to 256");
    if (t.bvh_leaf_size > 64u) return fail(ATX_ERR_INVALID_ARG, "tuning: leaf size above 64");
    if (t.path_kernel > 2u) return fail(ATX_ERR_INVALID_ARG, "tuning: path_kernel is 0, 1 or 2");
    if (t.cell_res && (t.cell_res < kCellResMin || t.cell_res > kCellResMax))
        return fail(ATX_ERR_INVALID_ARG, "tuning: cell_res is 0 or %u..%u", kCellResMin, kCellResMax);
    ATX_TRY(activate());
    ATX_TRY(join());
    ATX_CUDA(cudaStreamSynchronize(stream_));
    for (int l = 0; l < kLanes; ++l)
        if (lane_stream_[l]) ATX_CUDA(cudaStreamSynchronize(lane_stream_[l]));
    if (t.bvh_leaf_size != tune_.bvh_leaf_size && scene_.view.use_bvh) {
        ATX_TRY(scene_.rebuild_bvh(t.bvh_leaf_size, stream_));
        masks_valid_ = false;       // the tile candidate lists walk the tree
        prev_cam_valid_ = false;
    }
    // light and direction buffers at another resolution (the lists change,
    // the frames do not)
    if (t.cell_res != tune_.cell_res) ATX_TRY(scene_.rebuild_cells(t.cell_res, &budget_, stream_));
    if (t.threads != tune_.threads || t.path_kernel != tune_.path_kernel) shape_valid_ = false;
    tune_ = t;
    tune_.from_cache = 0;
    tune_.ms = 0.0;
    return ATX_OK;
}

atx_status Renderer::tuning(atx_tuning* out)
{
    *out = tune_;
    out->bvh_leaf_size = scene_.leaf_size();
    out->cell_res = scene_.cells();
    return ATX_OK;
}

// Device time per render of renders issued back to back, as a caller renders:
// one interval on stream_ from before the first to after the last (with
// overlapped renders a render's own events would also hold the previous
// render's lanes).  The interval holds at least `passes` renders and about
// 20 ms of them: in a shorter one the first render's start and the last one's
// unoverlapped tail weigh enough to favour settings that overlap less (0.3 ms
// renders of the 256-sphere scene: two lanes over four in three renders).
atx_status Renderer::time_renders(uint32_t spp, uint32_t passes, double* ms)
{
    frame_ = 1;
    ATX_TRY(render(spp));   // the per-camera tables are built on the second render of a camera
    ATX_TRY(render(spp));
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    atx_status s = ATX_OK;
    auto block = [&](uint32_t k, double* per) {
        if (s == ATX_OK) s = join();
        if (s != ATX_OK || e != cudaSuccess) return;
        e = cudaEventRecord(ev[0], stream_);
        for (uint32_t i = 0; i < k && s == ATX_OK && e == cudaSuccess; ++i) s = render(spp);
        if (s == ATX_OK) s = join();
        if (s != ATX_OK || e != cudaSuccess) return;
        e = cudaEventRecord(ev[1], stream_);
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
        float t = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
        *per = (double)t / k;
    };
    double per = 0.0;
    block(passes, &per);
    constexpr double kBlockMs = 20.0;
    if (s == ATX_OK && e == cudaSuccess && per > 0.0 && per * passes < kBlockMs) {
        const uint32_t k = (uint32_t)std::min(256.0, std::ceil(kBlockMs / per));
        if (k > passes) block(k, &per);
    }
    *ms = per;
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    ATX_TRY(s);
    ATX_CUDA(e);
    return ATX_OK;
}

atx_status Renderer::autotune(uint32_t spp, uint32_t passes, bool use_cache, atx_tuning* out)
{
    if (!width_ || !height_ || !accum_.get()) return fail(ATX_ERR_INVALID_ARG, "autotune: call atx_resize first");
    if (!spp) return fail(ATX_ERR_INVALID_ARG, "autotune: spp must be positive");
    if (!passes) passes = 2;
    ATX_TRY(activate());
    ATX_TRY(refresh_camera());
    int sms = 0, major = 0, minor = 0;
    ATX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg_.device));
    ATX_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, cfg_.device));
    ATX_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, cfg_.device));
    const SceneView& sv = scene_.view;
    const int kind = sv.use_bvh ? 2 : (sv.lb.n_lights ? 1 : 0);
    const TuneKey key{sms, 10 * major + minor, log2_bucket(sv.n_sph + 1ull), kind,
                      log2_bucket((uint64_t)width_ * height_ * spp), settings_.max_bounces};
    if (use_cache) {
        atx_tuning hit{};
        bool found = false;
        {
            std::lock_guard<std::mutex> lock(g_tune_mu);
            auto it = g_tune_cache.find(key);
            if (it != g_tune_cache.end()) {
                hit = it->second;
                found = true;
            }
        }
        if (found) {
            ATX_TRY(set_tuning(hit));
            tune_.from_cache = 1;
            tune_.ms = hit.ms;
            frame_ = 1;
            return tuning(out);
        }
    }
    // coordinate descent from the defaults: leaf size, then lanes, path state,
    // block size and the wave's tile shape, each keeping the best so far
    atx_tuning best{};
    ATX_TRY(set_tuning(best));
    double best_ms = 0.0;
    ATX_TRY(time_renders(spp, passes, &best_ms));
    auto trial = [&](atx_tuning t) -> atx_status {
        ATX_TRY(set_tuning(t));
        double ms = 0.0;
        ATX_TRY(time_renders(spp, passes, &ms));
        if (ms < best_ms) {
            best_ms = ms;
            best = t;
        }
        return ATX_OK;
    };
    if (sv.use_bvh)
        for (uint32_t leaf : {4u, 8u, 12u, 24u, 32u}) {
            atx_tuning t = best;
            t.bvh_leaf_size = leaf;
            ATX_TRY(trial(t));
        }
    for (uint32_t lanes : {1u, 2u, 4u, 6u, 8u}) {
        atx_tuning t = best;
        t.lanes = lanes;
        ATX_TRY(trial(t));
    }
    for (uint32_t mi : {4u, 16u}) {
        atx_tuning t = best;
        t.wave_paths = mi << 20;
        ATX_TRY(trial(t));
    }
    for (uint32_t threads : {128u}) {
        atx_tuning t = best;
        t.threads = threads;
        ATX_TRY(trial(t));
    }
    if (!sv.use_bvh && (sv.db.n || sv.lb.n_lights))   // cells of the light and direction buffers
        for (uint32_t res : {16u, 24u, 32u}) {
            atx_tuning t = best;
            t.cell_res = res;
            ATX_TRY(trial(t));
        }
    if (!sv.use_bvh && sv.n_sph <= 256u)   // whole paths in one thread against the wavefront stages
        for (uint32_t pk : {1u, 2u}) {
            atx_tuning t = best;
            t.path_kernel = pk;
            ATX_TRY(trial(t));
        }
    for (uint32_t wspp : {1u, 4u}) {
        if (wspp >= spp) continue;
        atx_tuning t = best;
        t.wave_spp = wspp;
        ATX_TRY(trial(t));
    }
    ATX_TRY(set_tuning(best));
    tune_.ms = best_ms;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key] = tune_;
    }
    frame_ = 1;
    return tuning(out);
}

atx_status Renderer::trace_nearest(const float* o, const float* d, uint64_t n, float* t, int32_t* id)
{
    if (n == 0) return ATX_OK;
    if (!o || !d || !t || !id) return fail(ATX_ERR_INVALID_ARG, "trace_nearest: null array");
    ATX_TRY(activate());
    ATX_TRY(join());
    DeviceBuffer buf;
    ATX_TRY(buf.ensure(n * 8 * sizeof(float) + 1024, &budget_, "trace scratch"));
    float* dorg = buf.as<float>();
    float* ddir = dorg + 3 * n;
    float* dt = ddir + 3 * n;
    int32_t* did = reinterpret_cast<int32_t*>(dt + n);
    ATX_CUDA(cudaMemcpyAsync(dorg, o, 3 * n * sizeof(float), cudaMemcpyHostToDevice, stream_));
    ATX_CUDA(cudaMemcpyAsync(ddir, d, 3 * n * sizeof(float), cudaMemcpyHostToDevice, stream_));
    ATX_CUDA(enqueue_trace_nearest(scene_.view, dorg, ddir, n, dt, did, stream_));
    ATX_CUDA(cudaMemcpyAsync(t, dt, n * sizeof(float), cudaMemcpyDeviceToHost, stream_));
    ATX_CUDA(cudaMemcpyAsync(id, did, n * sizeof(int32_t), cudaMemcpyDeviceToHost, stream_));
    ATX_CUDA(cudaStreamSynchronize(stream_));
    return ATX_OK;
}

atx_status Renderer::primary_directions(float* host, uint64_t n)
{
    if (!width_ || !height_) return fail(ATX_ERR_INVALID_ARG, "primary_directions: call atx_resize first");
    const uint64_t px = (uint64_t)width_ * height_;
    if (!host || n < px) return fail(ATX_ERR_INVALID_ARG, "primary_directions: buffer smaller than W*H");
    ATX_TRY(activate());
    ATX_TRY(join());
    ATX_TRY(refresh_camera());
    DeviceBuffer buf;
    ATX_TRY(buf.ensure(px * 3 * sizeof(float), &budget_, "direction scratch"));
    ATX_CUDA(enqueue_primary_dirs(camv_, buf.as<float>(), stream_));
    ATX_CUDA(cudaMemcpyAsync(host, buf.get(), px * 3 * sizeof(float), cudaMemcpyDeviceToHost, stream_));
    ATX_CUDA(cudaStreamSynchronize(stream_));
    return ATX_OK;
}

}  // namespace atx
