// Batched renderer (batch_host.h): resident scenes, lanes of concurrent
// streams, one captured CUDA graph per pass.
#include "batch_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace atx {

namespace {
constexpr uint32_t kDefaultLanes = 8;
constexpr uint32_t kMaxLanes = 64;
constexpr uint32_t kDefaultLaneWavePaths = 16u << 20;  // 16 Mi paths (about 2.2 GB of path state) per lane
constexpr uint32_t kDefaultBvhThreshold = 1025;  // LBVH above the direction buffer's 1,024 spheres (64-scene mix: +23% over 512)

// Relative device time of one pass of a scene: paths x (1 + B/2) rays, each
// N brute-force tests or an LBVH walk, plus a fixed cost per dependent launch
// (about B + 3 per wave).  Only the order of the estimates matters (LPT).
double pass_cost(const SceneView& sc, uint64_t paths, int32_t bounces)
{
    const double b = std::max(0, bounces);
    const double per_ray = sc.use_bvh ? 100.0 * std::log2((double)sc.n_sph + 2.0) : (double)sc.n_sph + 8.0;
    return (double)paths * (1.0 + 0.5 * b) * per_ray + 2.0e7 * (b + 3.0);
}
}  // namespace

Batch::Batch(const atx_config& cfg) : cfg_(cfg), budget_(cfg.hbm_budget_bytes) {}

Batch::~Batch()
{
    if (cudaSetDevice(cfg_.device) == cudaSuccess) {
        if (up_stream_) cudaStreamSynchronize(up_stream_);
        if (stream_) cudaStreamSynchronize(stream_);
        for (Lane& l : lanes_)
            if (l.stream) cudaStreamSynchronize(l.stream);
        if (graph_) cudaGraphExecDestroy(graph_);
        slots_.clear();   // stream-ordered frees on stream_
        if (stream_) cudaStreamSynchronize(stream_);
        for (Lane& l : lanes_) {
            l.wave.buf.reset();
            if (l.done) cudaEventDestroy(l.done);
            if (l.mark) cudaEventDestroy(l.mark);
            if (l.stream) cudaStreamDestroy(l.stream);
        }
        totals_.reset();
        if (pool_) cudaMemPoolDestroy(pool_);
        if (fork_) cudaEventDestroy(fork_);
        if (ev0_) cudaEventDestroy(ev0_);
        if (ev1_) cudaEventDestroy(ev1_);
        if (uploaded_) cudaEventDestroy(uploaded_);
        if (up_stream_) cudaStreamDestroy(up_stream_);
        if (stream_) cudaStreamDestroy(stream_);
    }
}

atx_status Batch::init()
{
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        (void)cudaGetLastError();
        return fail(ATX_ERR_NO_DEVICE, "no CUDA device visible");
    }
    if (cfg_.device < 0 || cfg_.device >= count) return fail(ATX_ERR_INVALID_ARG, "device %d out of range", cfg_.device);
    ATX_CUDA(cudaSetDevice(cfg_.device));
    ATX_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    ATX_CUDA(cudaStreamCreateWithFlags(&up_stream_, cudaStreamNonBlocking));
    ATX_CUDA(cudaEventCreateWithFlags(&uploaded_, cudaEventDisableTiming));
    ATX_CUDA(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
    // scenes come and go between passes: their memory comes from a pool that
    // keeps freed blocks for reuse instead of returning them at every sync
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = cfg_.device;
    ATX_CUDA(cudaMemPoolCreate(&pool_, &props));
    uint64_t keep = ~0ull;
    ATX_CUDA(cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &keep));
    order_ = StreamOrder{pool_, up_stream_, stream_};
    ATX_CUDA(cudaEventCreate(&ev0_));
    ATX_CUDA(cudaEventCreate(&ev1_));
    ATX_TRY(totals_.ensure(3 * sizeof(unsigned long long), &scratch_, "ray totals"));
    ATX_CUDA(cudaMemsetAsync(totals_.get(), 0, 3 * sizeof(unsigned long long), stream_));
    tuning_.lanes = kDefaultLanes;
    tuning_.lane_wave_paths = cfg_.wave_paths ? cfg_.wave_paths : kDefaultLaneWavePaths;
    tuning_.threads = cfg_.threads;
    tuning_.bvh_threshold = cfg_.bvh_threshold ? cfg_.bvh_threshold : kDefaultBvhThreshold;
    tuning_.bvh_leaf_size = cfg_.bvh_leaf_size;
    tuning_.primary_cache = 1;
    return ATX_OK;
}

Batch::Slot* Batch::slot(uint32_t id)
{
    if (id >= slots_.size() || !slots_[id]) return nullptr;
    return slots_[id].get();
}

atx_status Batch::add_scene(const atx_batch_scene& d, uint32_t* id)
{
    if (d.width == 0 || d.height == 0 || (uint64_t)d.width * d.height > 0xffffffffull)
        return fail(ATX_ERR_INVALID_ARG, "batch_add_scene: bad viewport %ux%u", d.width, d.height);
    if (d.settings.max_bounces > 4096)
        return fail(ATX_ERR_INVALID_ARG, "batch_add_scene: max_bounces %d above 4096", d.settings.max_bounces);
    ATX_CUDA(cudaSetDevice(cfg_.device));
    auto s = std::make_unique<Slot>();
    s->scene.bvh_threshold = tuning_.bvh_threshold;
    s->scene.bvh_leaf = tuning_.bvh_leaf_size;
    s->scene.order = &order_;
    s->accum.use_stream_order(&order_);
    s->image.use_stream_order(&order_);
    s->prim.use_stream_order(&order_);
    s->dirs.use_stream_order(&order_);
    s->scene.cell_res = cell_res_;
    // on the upload stream: a pass running on the batch stream is not waited for
    ATX_TRY(s->scene.upload(d.spheres, d.n_spheres, d.materials, d.n_materials, d.lights, d.n_lights, &budget_,
                            up_stream_));
    const uint64_t px = (uint64_t)d.width * d.height;
    ATX_TRY(s->accum.ensure(px * sizeof(float4), &budget_, "batch accumulator"));
    ATX_TRY(s->image.ensure(px * sizeof(uint32_t), &budget_, "batch image"));
    ATX_TRY(s->prim.ensure(px * sizeof(uint2), &budget_, "batch primary hits"));
    ATX_TRY(s->dirs.ensure(px * sizeof(float4), &budget_, "batch primary directions"));
    s->w = d.width;
    s->h = d.height;
    s->settings = d.settings;
    s->desc = d.camera;
    camera_matrices(d.camera, d.width, d.height, nullptr, s->cam.inv_view, nullptr, s->cam.inv_proj);
    std::memcpy(s->cam.pos, d.camera.position, sizeof(s->cam.pos));
    s->cam.width = d.width;
    s->cam.height = d.height;
    s->cam.dirs = nullptr;
    ATX_CUDA(enqueue_dir_table(s->cam, s->dirs.as<float4>(), up_stream_));
    s->cam.dirs = s->dirs.as<float4>();
    ATX_CUDA(cudaEventRecord(uploaded_, up_stream_));
    ATX_CUDA(plan_launch(s->scene.view, cfg_.device, (int)tuning_.threads, &s->shape));
    uint32_t i = 0;   // reuse a free id
    while (i < slots_.size() && slots_[i]) ++i;
    if (i == slots_.size()) slots_.emplace_back();
    slots_[i] = std::move(s);
    *id = i;
    return ATX_OK;
}

void Batch::drop_graph()
{
    if (graph_) {
        cudaGraphExecDestroy(graph_);   // a graph still running is freed when it completes
        graph_ = nullptr;
    }
}

void Batch::release_scratch()
{
    drop_graph();
    for (Lane& l : lanes_) {
        if (l.stream) cudaStreamSynchronize(l.stream);
        l.wave.buf.reset();
        l.wave.view = WaveState{};
        l.wave.bounces = 0;
    }
}

atx_status Batch::remove_scene(uint32_t id)
{
    Slot* s = slot(id);
    if (!s) return fail(ATX_ERR_NOT_FOUND, "batch: no scene %u", id);
    ATX_CUDA(cudaSetDevice(cfg_.device));
    slots_[id].reset();   // freed on the batch stream after the passes queued there
    return ATX_OK;
}

atx_status Batch::set_spp(uint32_t id, uint32_t spp)
{
    Slot* s = slot(id);
    if (!s) return fail(ATX_ERR_NOT_FOUND, "batch: no scene %u", id);
    s->spp_next = spp;
    return ATX_OK;
}

atx_status Batch::reset(uint32_t id)
{
    Slot* s = slot(id);
    if (!s) return fail(ATX_ERR_NOT_FOUND, "batch: no scene %u", id);
    s->frame = 1;
    return ATX_OK;
}

atx_status Batch::frame_index(uint32_t id, uint32_t* f)
{
    Slot* s = slot(id);
    if (!s) return fail(ATX_ERR_NOT_FOUND, "batch: no scene %u", id);
    *f = s->frame;
    return ATX_OK;
}

atx_status Batch::set_camera(uint32_t id, const atx_camera& c)
{
    Slot* s = slot(id);
    if (!s) return fail(ATX_ERR_NOT_FOUND, "batch: no scene %u", id);
    s->desc = c;
    camera_matrices(c, s->w, s->h, nullptr, s->cam.inv_view, nullptr, s->cam.inv_proj);
    std::memcpy(s->cam.pos, c.position, sizeof(s->cam.pos));
    // passes already queued may still read the old direction table: from now
    // on the scene's directions are computed where needed
    s->cam.dirs = nullptr;
    s->frame = 1;   // a moved camera restarts the accumulation (main.cpp:24-29)
    s->prim_valid = false;
    return ATX_OK;
}

atx_status Batch::set_tuning(const atx_batch_tuning& t)
{
    ATX_CUDA(cudaSetDevice(cfg_.device));
    if (t.lanes) tuning_.lanes = std::min(t.lanes, kMaxLanes);   // <= 64: lane sets are 64-bit masks
    if (t.lane_wave_paths && t.lane_wave_paths != tuning_.lane_wave_paths) {
        tuning_.lane_wave_paths = std::max<uint32_t>(t.lane_wave_paths, 1u << 16);
        release_scratch();
    }
    if (t.threads && t.threads != tuning_.threads) {
        tuning_.threads = std::min<uint32_t>(1024, std::max<uint32_t>(32, t.threads & ~31u));
        for (auto& p : slots_)
            if (p) ATX_CUDA(plan_launch(p->scene.view, cfg_.device, (int)tuning_.threads, &p->shape));
    }
    if (t.primary_cache) {
        tuning_.primary_cache = t.primary_cache == 1 ? 1u : 2u;
        for (auto& p : slots_)
            if (p) p->prim_valid = false;
    }
    if (t.bvh_threshold) tuning_.bvh_threshold = t.bvh_threshold;   // scenes added from now on
    if (t.bvh_leaf_size && t.bvh_leaf_size != tuning_.bvh_leaf_size) {
        // resident LBVH scenes are rebuilt with the new leaf size (their frames do not change: the walk is
        // exact for any leaf size); the next pass captures a new graph with their new tree views
        if (t.bvh_leaf_size > 64u) return fail(ATX_ERR_INVALID_ARG, "batch tuning: leaf size above 64");
        tuning_.bvh_leaf_size = t.bvh_leaf_size;
        ATX_CUDA(cudaStreamSynchronize(stream_));
        for (auto& p : slots_)
            if (p && p->scene.view.use_bvh) {
                p->scene.bvh_leaf = t.bvh_leaf_size;
                ATX_TRY(p->scene.rebuild_bvh(t.bvh_leaf_size, up_stream_));
            }
        drop_graph();
    }
    return ATX_OK;
}

atx_status Batch::autotune(uint32_t passes, atx_batch_tuning* chosen)
{
    for (auto& p : slots_)
        if (p && p->frame != 1) return fail(ATX_ERR_INVALID_ARG, "batch_autotune: scenes must be at frame 1");
    if (!passes) passes = 2;
    // lanes x path state per lane (Mi paths); at 136 B per path the largest is ~37 GB
    const uint32_t cand[][2] = {{2, 64}, {4, 32}, {4, 16}, {8, 16}, {8, 32}, {16, 8}, {16, 16}};
    double best = 1e300;
    atx_batch_tuning pick = tuning_;
    auto reset_frames = [&]() {
        for (auto& p : slots_)
            if (p) p->frame = 1;
    };
    for (const auto& c : cand) {
        atx_batch_tuning t{};
        t.lanes = c[0];
        t.lane_wave_paths = c[1] << 20;
        ATX_TRY(set_tuning(t));
        ATX_TRY(run());   // a new shape, then its graph capture
        ATX_TRY(run());
        double ms = 0.0;
        for (uint32_t k = 0; k < passes; ++k) {
            ATX_TRY(run());
            atx_batch_stats st;
            ATX_TRY(stats(&st));   // synchronises
            ms += st.last_pass_ms;
        }
        reset_frames();
        if (ms < best) {
            best = ms;
            pick = tuning_;
        }
    }
    ATX_TRY(set_tuning(pick));
    // then the LBVH leaf size (when the mix has LBVH scenes) and the block size
    // of the primary and shadow kernels, one at a time from the pick
    auto trial = [&](atx_batch_tuning t) -> atx_status {
        ATX_TRY(set_tuning(t));
        ATX_TRY(run());
        ATX_TRY(run());
        double ms = 0.0;
        for (uint32_t k = 0; k < passes; ++k) {
            ATX_TRY(run());
            atx_batch_stats st;
            ATX_TRY(stats(&st));
            ms += st.last_pass_ms;
        }
        reset_frames();
        if (ms < best) {
            best = ms;
            pick = tuning_;
        }
        return ATX_OK;
    };
    bool any_bvh = false;
    for (auto& p : slots_)
        if (p && p->scene.view.use_bvh) any_bvh = true;
    // explicit values, so that putting the pick back restores them
    if (!pick.bvh_leaf_size) pick.bvh_leaf_size = 16;
    if (!pick.threads) pick.threads = 256;
    ATX_TRY(set_tuning(pick));
    if (any_bvh)
        for (uint32_t leaf : {8u, 12u, 24u, 32u}) {
            atx_batch_tuning t = pick;
            t.bvh_leaf_size = leaf;
            ATX_TRY(trial(t));
            ATX_TRY(set_tuning(pick));
        }
    for (uint32_t threads : {128u, 256u}) {
        atx_batch_tuning t = pick;
        t.threads = threads;
        ATX_TRY(trial(t));
        ATX_TRY(set_tuning(pick));
    }
    ATX_TRY(set_tuning(pick));
    reset_frames();
    if (chosen) *chosen = tuning_;
    return ATX_OK;
}

atx_status Batch::ensure_lanes(uint32_t n)
{
    while (lanes_.size() < n) {
        Lane l;
        ATX_CUDA(cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking));
        ATX_CUDA(cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming));
        ATX_CUDA(cudaEventCreateWithFlags(&l.mark, cudaEventDisableTiming));
        lanes_.push_back(std::move(l));
    }
    return ATX_OK;
}

atx_status Batch::run(cudaEvent_t done)
{
    ATX_CUDA(cudaSetDevice(cfg_.device));
    // Work items: a scene's pass, split into pixel ranges when it is larger
    // than one lane's wave so that a big scene spreads over several lanes
    // (ranges of pixels are independent: their accumulator rows are disjoint).
    struct Part {
        uint32_t id;
        double cost;
        uint64_t pix_begin, pix_end;
    };
    const uint32_t max_lanes = std::max<uint32_t>(tuning_.lanes, 1u);
    std::vector<Part> parts;
    uint64_t paths = 0;
    for (uint32_t i = 0; i < slots_.size(); ++i) {
        Slot* s = slots_[i].get();
        if (!s || s->spp_next == 0) continue;
        const uint64_t px = (uint64_t)s->w * s->h;
        const uint64_t p = px * s->spp_next;
        paths += p;
        const uint64_t want = (p + tuning_.lane_wave_paths - 1) / tuning_.lane_wave_paths;
        const uint32_t n = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>({want, max_lanes, px}));
        const double c = pass_cost(s->scene.view, p, s->settings.max_bounces) / n;
        for (uint32_t k = 0; k < n; ++k) parts.push_back({i, c, px * k / n, px * (k + 1) / n});
    }
    ++st_.passes;
    st_.waves_last_pass = 0;
    if (parts.empty()) {
        if (done) ATX_CUDA(cudaEventRecord(done, stream_));
        return ATX_OK;
    }

    // longest first onto the least-loaded lane
    std::stable_sort(parts.begin(), parts.end(), [](const Part& a, const Part& b) { return a.cost > b.cost; });
    const uint32_t nl = std::min<uint32_t>(max_lanes, (uint32_t)parts.size());
    ATX_TRY(ensure_lanes(nl));
    std::vector<std::vector<uint32_t>> plan(nl);
    std::vector<double> load(nl, 0.0);
    for (uint32_t k = 0; k < parts.size(); ++k) {
        const uint32_t lane = (uint32_t)(std::min_element(load.begin(), load.end()) - load.begin());
        plan[lane].push_back(k);
        load[lane] += parts[k].cost;
    }
    // path state: one buffer per lane, deep enough for its deepest scene
    for (uint32_t l = 0; l < nl; ++l) {
        int32_t maxb = 0;
        for (uint32_t k : plan[l]) maxb = std::max(maxb, slots_[parts[k].id]->settings.max_bounces);
        Lane& ln = lanes_[l];
        if (ln.wave.view.capacity < tuning_.lane_wave_paths || ln.wave.bounces < (uint32_t)maxb) drop_graph();
        ATX_TRY(ln.wave.ensure(tuning_.lane_wave_paths, (uint32_t)maxb, &scratch_));
        ln.wave.view.totals = totals_.as<unsigned long long>();
    }
    // frame bookkeeping (Renderer.cu:175-182, 245-248): this pass renders
    // frames [frame0, frame0 + spp) of each scene
    std::vector<uint32_t> frame0(slots_.size(), 0u);
    for (uint32_t i = 0; i < slots_.size(); ++i) {
        Slot* s = slots_[i].get();
        if (!s || s->spp_next == 0) continue;
        if (!s->settings.accumulation) s->frame = 1;
        frame0[i] = s->frame;
        s->frame = s->settings.accumulation ? s->frame + s->spp_next : 1u;
    }
    // lanes each scene's parts run on this pass
    std::vector<uint64_t> now_lanes(slots_.size(), 0u);
    for (uint32_t l = 0; l < nl; ++l)
        for (uint32_t k : plan[l]) now_lanes[parts[k].id] |= 1ull << l;

    // The graph's shape: lanes, their parts in order, whether each clears its
    // accumulator rows, its waves and bounces.  A pass of the same shape as
    // the last one replays the graph with updated kernel arguments; a pass of
    // a new shape (scenes come and go in a server) is launched directly,
    // since capturing and instantiating a graph used once costs more host time.
    auto part_waves = [&](const Part& q, uint32_t cap) {
        const Slot* s = slots_[q.id].get();
        const WavePlan wp = plan_waves(q.pix_end - q.pix_begin, s->spp_next, cap);
        return ((q.pix_end - q.pix_begin + wp.pixels_per_wave - 1) / wp.pixels_per_wave) *
               ((s->spp_next + wp.spp_per_wave - 1) / wp.spp_per_wave);
    };
    std::vector<uint64_t> sig;
    for (uint32_t l = 0; l < nl; ++l) {
        sig.push_back(0xffffffff00000000ull | l);
        for (uint32_t k : plan[l]) {
            const Part& q = parts[k];
            const Slot* s = slots_[q.id].get();
            sig.push_back(((uint64_t)q.id << 32) | (q.pix_begin & 0xffffffffu));
            sig.push_back(((uint64_t)(frame0[q.id] == 1) << 63) |
                          ((uint64_t)(uint32_t)s->settings.max_bounces << 32) |
                          part_waves(q, lanes_[l].wave.view.capacity));
        }
    }
    const bool graphs = !(cfg_.flags & ATX_FLAG_NO_GRAPHS) && sig == last_sig_;
    last_sig_.swap(sig);
    if (!graphs) drop_graph();
    uint32_t launches = 0, waves = 0;
    uint64_t prim = 0;
    // direct launch: a lane that takes over a scene, or part of one, from
    // other lanes waits for their queued work (the scene's last pass); a lane
    // continues with its own scenes in stream order
    std::vector<uint64_t> waits(nl, 0u);   // per lane: lanes whose marks it waits for
    if (!graphs) {
        for (uint32_t l = 0; l < nl; ++l)
            for (uint32_t k : plan[l]) waits[l] |= slots_[parts[k].id]->lanes & ~(1ull << l);
        for (Lane& ln : lanes_) ATX_CUDA(cudaEventRecord(ln.mark, ln.stream));
    }
    // A graph pass forks from the batch stream (a barrier); so does a direct
    // pass after a graph pass, whose kernels ran on the batch stream.
    const bool fork = graphs || last_graph_;
    if (fork) ATX_CUDA(cudaStreamWaitEvent(stream_, uploaded_, 0));   // scenes added since the last pass
    auto enqueue = [&]() -> atx_status {
        if (fork) ATX_CUDA(cudaEventRecord(fork_, stream_));
        for (uint32_t l = 0; l < nl; ++l) {
            Lane& ln = lanes_[l];
            if (fork) {
                ATX_CUDA(cudaStreamWaitEvent(ln.stream, fork_, 0));
            } else {
                ATX_CUDA(cudaStreamWaitEvent(ln.stream, uploaded_, 0));
                for (uint32_t from = 0; from < (uint32_t)lanes_.size() && from < 64u; ++from)
                    if (waits[l] >> from & 1u) ATX_CUDA(cudaStreamWaitEvent(ln.stream, lanes_[from].mark, 0));
            }
            for (uint32_t k : plan[l]) {
                const Part& q = parts[k];
                Slot* s = slots_[q.id].get();
                if (frame0[q.id] == 1) {
                    ATX_CUDA(enqueue_clear_accum(s->accum.as<float4>() + q.pix_begin, q.pix_end - q.pix_begin,
                                                 ln.stream));
                    ++launches;
                }
                waves += (uint32_t)part_waves(q, ln.wave.view.capacity);
                ATX_TRY(enqueue_frames(s->scene.view, s->cam, ln.wave, s->shape, frame0[q.id], s->spp_next,
                                       s->settings.max_bounces, s->settings.sky_light ? 1 : 0, s->accum.as<float4>(),
                                       s->image.as<uint32_t>(), ln.wave.view.capacity, ln.stream, &launches, nullptr,
                                       &prim, q.pix_begin, q.pix_end, s->prim.as<uint2>(),
                                       s->prim_valid && tuning_.primary_cache == 1));
            }
            ATX_CUDA(cudaEventRecord(ln.done, ln.stream));
            ATX_CUDA(cudaStreamWaitEvent(stream_, ln.done, 0));
        }
        return ATX_OK;
    };

    if (graphs) {
        ATX_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        const atx_status st = enqueue();
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(stream_, &g);
        if (st != ATX_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            (void)cudaGetLastError();
            drop_graph();
            return st != ATX_OK ? st : cuda_fail(e, "batch pass capture");
        }
        bool updated = false;
        if (graph_) {
            cudaGraphExecUpdateResultInfo info{};
            updated = cudaGraphExecUpdate(graph_, g, &info) == cudaSuccess;
            if (!updated) {
                (void)cudaGetLastError();
                drop_graph();
            }
        }
        cudaError_t ie = cudaSuccess;
        if (!updated) ie = cudaGraphInstantiate(&graph_, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            graph_ = nullptr;
            return cuda_fail(ie, "batch graph instantiate");
        }
        ATX_CUDA(cudaEventRecord(ev0_, stream_));
        ATX_CUDA(cudaGraphLaunch(graph_, stream_));
        ATX_CUDA(cudaEventRecord(ev1_, stream_));
        ++st_.graph_launches;
    } else {
        ATX_CUDA(cudaEventRecord(ev0_, stream_));
        ATX_TRY(enqueue());
        ATX_CUDA(cudaEventRecord(ev1_, stream_));
    }
    for (uint32_t i = 0; i < slots_.size(); ++i)
        if (slots_[i] && now_lanes[i]) {
            slots_[i]->lanes = now_lanes[i];
            slots_[i]->prim_valid = true;   // this pass traced every pixel's primary hit
        }
    last_graph_ = graphs;
    if (done) ATX_CUDA(cudaEventRecord(done, stream_));
    timed_ = true;
    st_.paths += paths;
    st_.kernel_launches += launches;
    st_.waves_last_pass = waves;
    primary_rays_ += prim;
    return ATX_OK;
}

atx_status Batch::synchronize()
{
    ATX_CUDA(cudaSetDevice(cfg_.device));
    ATX_CUDA(cudaStreamSynchronize(stream_));
    return ATX_OK;
}

atx_status Batch::read_accumulation(uint32_t id, float* host, uint64_t n)
{
    Slot* s = slot(id);
    if (!s) return fail(ATX_ERR_NOT_FOUND, "batch: no scene %u", id);
    if (!host || n > (uint64_t)s->w * s->h) return fail(ATX_ERR_INVALID_ARG, "batch_read_accumulation: bad buffer");
    ATX_CUDA(cudaSetDevice(cfg_.device));
    ATX_CUDA(cudaMemcpyAsync(host, s->accum.get(), n * sizeof(float4), cudaMemcpyDeviceToHost, stream_));
    ATX_CUDA(cudaStreamSynchronize(stream_));
    return ATX_OK;
}

atx_status Batch::read_image(uint32_t id, uint32_t* host, uint64_t n)
{
    Slot* s = slot(id);
    if (!s) return fail(ATX_ERR_NOT_FOUND, "batch: no scene %u", id);
    if (!host || n > (uint64_t)s->w * s->h) return fail(ATX_ERR_INVALID_ARG, "batch_read_image: bad buffer");
    ATX_CUDA(cudaSetDevice(cfg_.device));
    ATX_CUDA(cudaMemcpyAsync(host, s->image.get(), n * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_));
    ATX_CUDA(cudaStreamSynchronize(stream_));
    return ATX_OK;
}

atx_status Batch::read_async(uint32_t id, uint32_t* image, float* accum, uint64_t n)
{
    Slot* s = slot(id);
    if (!s) return fail(ATX_ERR_NOT_FOUND, "batch: no scene %u", id);
    if (n > (uint64_t)s->w * s->h) return fail(ATX_ERR_INVALID_ARG, "batch read: %llu pixels > image",
                                               (unsigned long long)n);
    ATX_CUDA(cudaSetDevice(cfg_.device));
    if (image) ATX_CUDA(cudaMemcpyAsync(image, s->image.get(), n * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_));
    if (accum) ATX_CUDA(cudaMemcpyAsync(accum, s->accum.get(), n * sizeof(float4), cudaMemcpyDeviceToHost, stream_));
    return ATX_OK;
}

atx_status Batch::stats(atx_batch_stats* out)
{
    ATX_CUDA(cudaSetDevice(cfg_.device));
    ATX_CUDA(cudaStreamSynchronize(stream_));
    unsigned long long rays[2] = {0, 0};
    ATX_CUDA(cudaMemcpy(rays, totals_.get(), sizeof(rays), cudaMemcpyDeviceToHost));
    if (timed_) {
        float ms = 0.0f;
        ATX_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
        st_.last_pass_ms = ms;
    }
    *out = st_;
    out->extension_rays = primary_rays_ + rays[0];
    out->shadow_rays = rays[1];
    out->device_bytes = budget_.used() + scratch_.used();
    uint32_t n = 0;
    for (auto& s : slots_) n += s ? 1 : 0;
    out->scenes = n;
    return ATX_OK;
}

}  // namespace atx
