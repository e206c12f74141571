// Host side of the batched persistent renderer: resident per-scene state,
// the per-pass work-item table and its CUDA-graph replay.
#include "batch_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace atx {

namespace {
constexpr uint32_t kDefaultTileW = 32, kDefaultTileH = 32;
constexpr uint32_t kDefaultBvhThreshold = 1024;
constexpr uint32_t kBatchSmemCap = 4096;   // spheres a CTA stages (64 KB)
}  // namespace

Batch::Batch(const atx_config& cfg) : cfg_(cfg), budget_(cfg.hbm_budget_bytes) {}

Batch::~Batch()
{
    if (cudaSetDevice(cfg_.device) == cudaSuccess) {
        if (stream_) cudaStreamSynchronize(stream_);
        if (graph_) cudaGraphExecDestroy(graph_);
        slots_.clear();
        if (h_scenes_) cudaFreeHost(h_scenes_);
        if (h_items_) cudaFreeHost(h_items_);
        if (ev0_) cudaEventDestroy(ev0_);
        if (ev1_) cudaEventDestroy(ev1_);
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
    ATX_CUDA(cudaEventCreate(&ev0_));
    ATX_CUDA(cudaEventCreate(&ev1_));
    ATX_TRY(counters_.ensure(64, &budget_, "batch counters"));
    ATX_CUDA(cudaMemsetAsync(counters_.get(), 0, 64, stream_));
    tuning_.tile_w = kDefaultTileW;
    tuning_.tile_h = kDefaultTileH;
    tuning_.threads = 256;
    tuning_.bvh_threshold = cfg_.bvh_threshold ? cfg_.bvh_threshold : kDefaultBvhThreshold;
    tuning_.bvh_leaf_size = cfg_.bvh_leaf_size;
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
    ATX_CUDA(cudaSetDevice(cfg_.device));
    auto s = std::make_unique<Slot>();
    s->scene.bvh_threshold = tuning_.bvh_threshold;
    s->scene.bvh_leaf = tuning_.bvh_leaf_size;
    ATX_TRY(s->scene.upload(d.spheres, d.n_spheres, d.materials, d.n_materials, d.lights, d.n_lights, &budget_,
                            stream_));
    const uint64_t px = (uint64_t)d.width * d.height;
    ATX_TRY(s->accum.ensure(px * sizeof(float4), &budget_, "batch accumulator"));
    ATX_TRY(s->image.ensure(px * sizeof(uint32_t), &budget_, "batch image"));
    s->w = d.width;
    s->h = d.height;
    s->settings = d.settings;
    camera_matrices(d.camera, d.width, d.height, nullptr, s->cam.inv_view, nullptr, s->cam.inv_proj);
    std::memcpy(s->cam.pos, d.camera.position, sizeof(s->cam.pos));
    s->cam.width = d.width;
    s->cam.height = d.height;
    // reuse a free slot id
    uint32_t i = 0;
    while (i < slots_.size() && slots_[i]) ++i;
    if (i == slots_.size()) slots_.emplace_back();
    slots_[i] = std::move(s);
    *id = i;
    return ATX_OK;
}

atx_status Batch::remove_scene(uint32_t id)
{
    Slot* s = slot(id);
    if (!s) return fail(ATX_ERR_NOT_FOUND, "batch: no scene %u", id);
    ATX_CUDA(cudaSetDevice(cfg_.device));
    ATX_CUDA(cudaStreamSynchronize(stream_));
    slots_[id].reset();
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

atx_status Batch::set_tuning(const atx_batch_tuning& t)
{
    if (t.tile_w) tuning_.tile_w = t.tile_w;
    if (t.tile_h) tuning_.tile_h = t.tile_h;
    if (t.threads) tuning_.threads = std::min<uint32_t>(256, std::max<uint32_t>(32, t.threads & ~31u));
    if (t.bvh_threshold) tuning_.bvh_threshold = t.bvh_threshold;
    if (t.bvh_leaf_size) tuning_.bvh_leaf_size = t.bvh_leaf_size;
    shape_valid_ = false;
    return ATX_OK;
}

// Relative cost of one path of a scene (a model for ordering work items,
// largest first): ~(1 + bounces/2) rays, each N brute-force tests or a
// logarithmic LBVH walk.
static double path_cost(const SceneView& sc, int32_t bounces, int mode)
{
    const double rays = 1.0 + 0.5 * std::max(0, bounces);
    const double per_ray = mode == 2 ? 24.0 * std::log2((double)sc.n_sph + 2.0) : (double)sc.n_sph + 8.0;
    return rays * per_ray;
}

atx_status Batch::run()
{
    ATX_CUDA(cudaSetDevice(cfg_.device));
    // the previous pass reads the pinned staging tables when it executes:
    // let it finish before they are rewritten
    ATX_CUDA(cudaStreamSynchronize(stream_));
    // order scenes by item cost, largest first; a scene's tiles stay together
    // so CTAs keep their staged sphere table
    struct Act { uint32_t id; double cost; };
    std::vector<Act> act;
    uint32_t smem_need = 0;
    for (uint32_t i = 0; i < slots_.size(); ++i) {
        Slot* s = slots_[i].get();
        if (!s || s->spp_next == 0) continue;
        const SceneView& sc = s->scene.view;
        s->mode = sc.use_bvh ? 2 : (sc.n_sph > 0 && sc.n_sph <= kBatchSmemCap ? 1 : 0);
        if (s->mode == 1) smem_need = std::max(smem_need, sc.n_sph);
        const double c = path_cost(sc, s->settings.max_bounces, s->mode) * s->spp_next * tuning_.tile_w *
                         tuning_.tile_h;
        act.push_back({i, c});
    }
    std::stable_sort(act.begin(), act.end(), [](const Act& a, const Act& b) { return a.cost > b.cost; });

    const uint32_t n_sc = (uint32_t)act.size();
    uint64_t n_items = 0;
    for (const Act& a : act) {
        const Slot* s = slots_[a.id].get();
        n_items += (uint64_t)((s->w + tuning_.tile_w - 1) / tuning_.tile_w) * ((s->h + tuning_.tile_h - 1) / tuning_.tile_h);
    }
    if (n_items > 0xffffffffull) return fail(ATX_ERR_INVALID_ARG, "batch: too many work items");
    ++st_.passes;
    st_.items_last_pass = (uint32_t)n_items;
    if (n_sc == 0) return ATX_OK;

    // staging (pinned, so a captured graph reads the current contents)
    if (n_sc > cap_scenes_) {
        if (h_scenes_) cudaFreeHost(h_scenes_);
        cap_scenes_ = std::max<uint32_t>(n_sc, 2 * cap_scenes_);
        ATX_CUDA(cudaMallocHost(&h_scenes_, cap_scenes_ * sizeof(BatchSceneDev)));
        ATX_TRY(d_scenes_.ensure(cap_scenes_ * sizeof(BatchSceneDev), &budget_, "batch scene table"));
        invalidate_graph();
    }
    if (n_items > cap_items_) {
        if (h_items_) cudaFreeHost(h_items_);
        cap_items_ = std::max<uint64_t>(n_items, 2 * cap_items_);
        ATX_CUDA(cudaMallocHost(&h_items_, cap_items_ * 2 * sizeof(uint32_t)));
        ATX_TRY(d_items_.ensure(cap_items_ * 2 * sizeof(uint32_t), &budget_, "batch work items"));
        invalidate_graph();
    }
    uint32_t* item_scene = static_cast<uint32_t*>(h_items_);
    uint32_t* item_tile = item_scene + cap_items_;
    uint64_t k = 0;
    uint64_t paths = 0;
    for (uint32_t j = 0; j < n_sc; ++j) {
        Slot* s = slots_[act[j].id].get();
        BatchSceneDev& d = h_scenes_[j];
        d.sc = s->scene.view;
        d.cam = s->cam;
        d.accum = s->accum.as<float4>();
        d.image = s->image.as<uint32_t>();
        d.max_bounces = s->settings.max_bounces;
        d.sky = s->settings.sky_light ? 1 : 0;
        if (!s->settings.accumulation) s->frame = 1;   // Renderer.cu:245-248
        d.frame0 = s->frame;
        d.spp = s->spp_next;
        d.tile_w = tuning_.tile_w;
        d.tile_h = tuning_.tile_h;
        d.tiles_x = (s->w + tuning_.tile_w - 1) / tuning_.tile_w;
        d.mode = s->mode;
        const uint32_t tiles = d.tiles_x * ((s->h + tuning_.tile_h - 1) / tuning_.tile_h);
        for (uint32_t t = 0; t < tiles; ++t, ++k) {
            item_scene[k] = j;
            item_tile[k] = t;
        }
        paths += (uint64_t)s->w * s->h * s->spp_next;
        s->frame = s->settings.accumulation ? s->frame + s->spp_next : 1u;
    }

    if (!shape_valid_ || smem_need > shape_smem_) {
        shape_smem_ = std::max(smem_need, 256u);
        ATX_CUDA(batch_plan(cfg_.device, (int)tuning_.threads, shape_smem_, &shape_));
        shape_valid_ = true;
        invalidate_graph();
    }

    BatchDev b;
    b.scenes = d_scenes_.as<BatchSceneDev>();
    b.item_scene = d_items_.as<uint32_t>();
    b.item_tile = d_items_.as<uint32_t>() + cap_items_;
    b.n_items = (uint32_t)n_items;
    b.next_item = counters_.as<uint32_t>();
    b.rays = reinterpret_cast<unsigned long long*>(counters_.as<char>() + 16);
    b.smem_cap = shape_smem_;

    const bool graphs = !(cfg_.flags & ATX_FLAG_NO_GRAPHS);
    if (graphs && graph_ && graph_scenes_ == n_sc && graph_items_ == n_items) {
        ATX_CUDA(cudaEventRecord(ev0_, stream_));
        ATX_CUDA(cudaGraphLaunch(graph_, stream_));
        ATX_CUDA(cudaEventRecord(ev1_, stream_));
        ++st_.graph_launches;
    } else {
        invalidate_graph();
        if (graphs) ATX_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = enqueue_pass(b, n_sc, n_items);
        if (graphs) {
            cudaGraph_t g = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(stream_, &g);
            if (e == cudaSuccess) e = e2;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&graph_, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                graph_ = nullptr;
                return cuda_fail(e, "batch graph capture");
            }
            graph_scenes_ = n_sc;
            graph_items_ = n_items;
            ATX_CUDA(cudaEventRecord(ev0_, stream_));
            ATX_CUDA(cudaGraphLaunch(graph_, stream_));
            ATX_CUDA(cudaEventRecord(ev1_, stream_));
        } else {
            if (e != cudaSuccess) return cuda_fail(e, "batch pass");
        }
    }
    timed_ = true;
    st_.paths += paths;
    st_.kernel_launches += 1;
    return ATX_OK;
}

cudaError_t Batch::enqueue_pass(const BatchDev& b, uint32_t n_sc, uint64_t n_items)
{
    const bool graphs = !(cfg_.flags & ATX_FLAG_NO_GRAPHS);
    if (!graphs) {
        cudaError_t e = cudaEventRecord(ev0_, stream_);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaMemcpyAsync(d_scenes_.get(), h_scenes_, n_sc * sizeof(BatchSceneDev), cudaMemcpyHostToDevice,
                                    stream_);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_items_.get(), h_items_, n_items * sizeof(uint32_t), cudaMemcpyHostToDevice, stream_);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_items_.as<uint32_t>() + cap_items_, static_cast<uint32_t*>(h_items_) + cap_items_,
                            n_items * sizeof(uint32_t), cudaMemcpyHostToDevice, stream_);
    if (e == cudaSuccess) e = cudaMemsetAsync(counters_.get(), 0, sizeof(uint32_t), stream_);
    if (e == cudaSuccess) e = enqueue_batch(b, shape_, stream_);
    if (!graphs && e == cudaSuccess) e = cudaEventRecord(ev1_, stream_);
    return e;
}

void Batch::invalidate_graph()
{
    if (graph_) {
        cudaStreamSynchronize(stream_);
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
    }
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

atx_status Batch::stats(atx_batch_stats* out)
{
    ATX_CUDA(cudaSetDevice(cfg_.device));
    ATX_CUDA(cudaStreamSynchronize(stream_));
    unsigned long long rays[2] = {0, 0};
    ATX_CUDA(cudaMemcpy(rays, counters_.as<char>() + 16, sizeof(rays), cudaMemcpyDeviceToHost));
    if (timed_) {
        float ms = 0.0f;
        ATX_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
        st_.last_pass_ms = ms;
    }
    *out = st_;
    out->extension_rays = rays[0];
    out->shadow_rays = rays[1];
    out->device_bytes = budget_.used();
    uint32_t n = 0;
    for (auto& s : slots_) n += s ? 1 : 0;
    out->scenes = n;
    return ATX_OK;
}

}  // namespace atx
