// Render server: a worker thread admits jobs when a slot and their device
// memory fit, queues batched passes over all active jobs (each renders a
// slice of its remaining frames) and retires jobs that reach their target
// (image and accumulator copied to host buffers, device memory released).
// Passes are pipelined: while pass k runs on the GPU the worker admits jobs,
// uploads their scenes and queues pass k+1 with the read-backs of the jobs it
// completes, then waits for pass k.  Submitters never touch the GPU.
#include "server.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>

#include "lbvh.h"
#include "light_buffer.h"

namespace atx {

namespace {
constexpr uint32_t kDefaultActive = 16;
constexpr uint32_t kDefaultPassSpp = 64;
constexpr uint64_t kDefaultPassPaths = 1ull << 30;
constexpr uint32_t kDefaultBvhThreshold = 1025;  // LBVH above the direction buffer's 1,024 spheres (64-scene mix: +23% over 512)
constexpr size_t kPassesInFlight = 2;                 // the one running and the next
constexpr uint64_t kMinSlicePaths = 16ull << 20;      // a job's slice fills at least a 16 Mi-path wave
constexpr uint64_t kPinnedCacheBytes = 4ull << 30;    // result buffers kept for reuse

uint64_t up256(uint64_t x) { return (x + 255u) & ~uint64_t(255u); }

bool finite3(const float* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

// The batched renderer.  Each commit records a pair of events around the pass
// and its read-backs; result buffers are page-locked, cached by size.
class BatchExecutor : public Executor {
public:
    explicit BatchExecutor(const atx_config& cfg) : b_(cfg), device_(cfg.device) { b_.set_cell_res(kCellResJobs); }
    ~BatchExecutor() override
    {
        if (cudaSetDevice(device_) != cudaSuccess) return;
        cudaStreamSynchronize(b_.stream());
        for (auto& kv : marks_) {
            cudaEventDestroy(kv.second.first);
            cudaEventDestroy(kv.second.second);
        }
        for (cudaEvent_t e : free_events_) cudaEventDestroy(e);
        for (auto& kv : pinned_)
            for (void* p : kv.second) cudaFreeHost(p);
    }
    atx_status init() override { return b_.init(); }
    atx_status add(const atx_batch_scene& d, uint64_t, uint32_t* slot) override { return b_.add_scene(d, slot); }
    atx_status remove(uint32_t slot) override { return b_.remove_scene(slot); }
    atx_status set_spp(uint32_t slot, uint32_t spp) override { return b_.set_spp(slot, spp); }
    atx_status set_camera(uint32_t slot, const atx_camera& c) override { return b_.set_camera(slot, c); }
    atx_status enqueue_pass() override
    {
        ATX_CUDA(cudaSetDevice(device_));
        if (!start_) ATX_TRY(take(&start_));
        ATX_CUDA(cudaEventRecord(start_, b_.stream()));
        return b_.run();
    }
    atx_status enqueue_read(uint32_t slot, uint32_t* image, float* accum, uint64_t n) override
    {
        return b_.read_async(slot, image, accum, n);
    }
    atx_status commit(uint64_t* ticket) override
    {
        ATX_CUDA(cudaSetDevice(device_));
        if (!start_) return fail(ATX_ERR_INVALID_ARG, "server: commit without a pass");
        cudaEvent_t end = nullptr;
        ATX_TRY(take(&end));
        ATX_CUDA(cudaEventRecord(end, b_.stream()));
        marks_[next_] = {start_, end};
        start_ = nullptr;
        *ticket = next_++;
        return ATX_OK;
    }
    atx_status wait(uint64_t ticket, double* device_ms) override
    {
        ATX_CUDA(cudaSetDevice(device_));
        auto it = marks_.find(ticket);
        if (it == marks_.end()) return fail(ATX_ERR_NOT_FOUND, "server: no pass %llu", (unsigned long long)ticket);
        const auto ev = it->second;
        marks_.erase(it);
        free_events_.push_back(ev.first);
        free_events_.push_back(ev.second);
        ATX_CUDA(cudaEventSynchronize(ev.second));
        float ms = 0.0f;
        ATX_CUDA(cudaEventElapsedTime(&ms, ev.first, ev.second));
        *device_ms = ms;
        return ATX_OK;
    }
    uint64_t device_bytes() const override { return b_.scene_bytes(); }
    void* host_alloc(uint64_t bytes) override
    {
        auto& list = pinned_[bytes];
        if (!list.empty()) {
            void* p = list.back();
            list.pop_back();
            cached_ -= bytes;
            return p;
        }
        if (cudaSetDevice(device_) != cudaSuccess) return nullptr;
        void* p = nullptr;
        if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) != cudaSuccess) {
            (void)cudaGetLastError();
            return nullptr;
        }
        return p;
    }
    void host_free(void* p, uint64_t bytes) override
    {
        if (!p) return;
        if (cached_ + bytes <= kPinnedCacheBytes) {
            pinned_[bytes].push_back(p);
            cached_ += bytes;
        } else {
            cudaFreeHost(p);
        }
    }

private:
    atx_status take(cudaEvent_t* e)
    {
        if (!free_events_.empty()) {
            *e = free_events_.back();
            free_events_.pop_back();
            return ATX_OK;
        }
        ATX_CUDA(cudaEventCreate(e));
        return ATX_OK;
    }

    Batch b_;
    int device_;
    cudaEvent_t start_ = nullptr;
    uint64_t next_ = 1;
    std::map<uint64_t, std::pair<cudaEvent_t, cudaEvent_t>> marks_;
    std::vector<cudaEvent_t> free_events_;
    std::map<uint64_t, std::vector<void*>> pinned_;
    uint64_t cached_ = 0;
};

// Host-only stand-in for the device, for scheduling tests without a GPU: a
// pass takes 1 ns of simulated device time per path on a timeline that runs
// behind the host like a stream; memory is accounted by the admission
// estimate; read-backs fill images with the frame count reached.  fail_pass
// > 0 makes that pass report an error, so failure handling is tested on the
// host.
class HostExecutor : public Executor {
    using Clock = std::chrono::steady_clock;

public:
    explicit HostExecutor(uint32_t fail_pass) : fail_pass_(fail_pass) {}
    atx_status init() override { return ATX_OK; }
    atx_status add(const atx_batch_scene& d, uint64_t bytes, uint32_t* slot) override
    {
        uint32_t i = 0;
        while (i < slots_.size() && slots_[i].used) ++i;
        if (i == slots_.size()) slots_.emplace_back();
        slots_[i] = Slot{true, d.width, d.height, 0, 0, bytes};
        bytes_ += bytes;
        *slot = i;
        return ATX_OK;
    }
    atx_status remove(uint32_t slot) override
    {
        if (slot >= slots_.size() || !slots_[slot].used) return fail(ATX_ERR_NOT_FOUND, "host executor: slot %u", slot);
        bytes_ -= slots_[slot].bytes;
        slots_[slot].used = false;
        return ATX_OK;
    }
    atx_status set_spp(uint32_t slot, uint32_t spp) override
    {
        if (slot >= slots_.size() || !slots_[slot].used) return fail(ATX_ERR_NOT_FOUND, "host executor: slot %u", slot);
        slots_[slot].spp = spp;
        return ATX_OK;
    }
    atx_status set_camera(uint32_t slot, const atx_camera&) override
    {
        if (slot >= slots_.size() || !slots_[slot].used) return fail(ATX_ERR_NOT_FOUND, "host executor: slot %u", slot);
        slots_[slot].frames = 0;
        return ATX_OK;
    }
    atx_status enqueue_pass() override
    {
        if (fail_pass_ && ++passes_ == fail_pass_) return fail(ATX_ERR_CUDA, "host executor: injected device error");
        uint64_t paths = 0;
        for (auto& s : slots_)
            if (s.used) {
                paths += (uint64_t)s.w * s.h * s.spp;
                s.frames += s.spp;
            }
        const Clock::time_point start = std::max(Clock::now(), busy_until_);
        busy_until_ = start + std::chrono::nanoseconds(paths);
        pass_ms_ += (double)paths * 1e-6;
        return ATX_OK;
    }
    atx_status enqueue_read(uint32_t slot, uint32_t* image, float* accum, uint64_t n) override
    {
        if (slot >= slots_.size() || !slots_[slot].used) return fail(ATX_ERR_NOT_FOUND, "host executor: slot %u", slot);
        reads_.push_back(Read{image, accum, n, slots_[slot].frames});
        return ATX_OK;
    }
    atx_status commit(uint64_t* ticket) override
    {
        marks_[next_] = Mark{busy_until_, pass_ms_, std::move(reads_)};
        reads_.clear();
        pass_ms_ = 0.0;
        *ticket = next_++;
        return ATX_OK;
    }
    atx_status wait(uint64_t ticket, double* device_ms) override
    {
        auto it = marks_.find(ticket);
        if (it == marks_.end()) return fail(ATX_ERR_NOT_FOUND, "server: no pass %llu", (unsigned long long)ticket);
        std::this_thread::sleep_until(it->second.ready);
        for (const Read& r : it->second.reads) {
            if (r.image) std::fill(r.image, r.image + r.n, r.frames);
            if (r.accum)
                for (uint64_t i = 0; i < r.n; ++i) {
                    r.accum[4 * i] = r.accum[4 * i + 1] = r.accum[4 * i + 2] = 0.0f;
                    r.accum[4 * i + 3] = (float)r.frames;
                }
        }
        *device_ms = it->second.ms;
        marks_.erase(it);
        return ATX_OK;
    }
    uint64_t device_bytes() const override { return bytes_; }
    void* host_alloc(uint64_t bytes) override { return std::malloc(bytes); }
    void host_free(void* p, uint64_t) override { std::free(p); }

private:
    struct Slot { bool used; uint32_t w, h, spp, frames; uint64_t bytes; };
    struct Read { uint32_t* image; float* accum; uint64_t n; uint32_t frames; };
    struct Mark { Clock::time_point ready; double ms; std::vector<Read> reads; };
    std::vector<Slot> slots_;
    std::vector<Read> reads_;
    std::map<uint64_t, Mark> marks_;
    uint64_t next_ = 1;
    uint64_t bytes_ = 0;
    uint32_t fail_pass_ = 0, passes_ = 0;
    Clock::time_point busy_until_{};
    double pass_ms_ = 0.0;
};
}  // namespace

std::unique_ptr<Executor> make_batch_executor(const atx_config& cfg) { return std::make_unique<BatchExecutor>(cfg); }
std::unique_ptr<Executor> make_host_executor(uint32_t fail_pass) { return std::make_unique<HostExecutor>(fail_pass); }

Server::Server(const atx_server_config& cfg) : cfg_(cfg)
{
    if (!cfg_.max_active_jobs) cfg_.max_active_jobs = kDefaultActive;
    auto_slice_ = cfg_.pass_spp == 0;   // explicit pass_spp: slices of exactly that many frames
    if (!cfg_.pass_spp) cfg_.pass_spp = kDefaultPassSpp;
    if (!cfg_.max_pass_paths) cfg_.max_pass_paths = kDefaultPassPaths;
    exec_ = (cfg_.base.flags & ATX_FLAG_HOST_EXECUTOR) ? make_host_executor(cfg_.host_fail_pass)
                                                        : make_batch_executor(cfg_.base);
}

Server::~Server()
{
    {
        std::lock_guard<std::mutex> lock(mu_);
        stop_ = true;
    }
    cv_work_.notify_all();
    if (worker_.joinable()) worker_.join();
    for (auto& kv : jobs_) free_results(kv.second);
}

atx_status Server::init()
{
    ATX_TRY(exec_->init());
    t0_ = std::chrono::steady_clock::now();
    worker_ = std::thread(&Server::loop, this);
    return ATX_OK;
}

double Server::now() const
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
}

uint64_t Server::job_bytes(const atx_batch_scene& s, uint32_t bvh_threshold)
{
    const uint64_t n = s.n_spheres;
    uint64_t b = up256(16 * n) + up256(4 * n) + up256(4 * n) + up256(48ull * s.n_materials) + up256(32ull * s.n_lights);
    const bool bvh = n >= (bvh_threshold ? bvh_threshold : kDefaultBvhThreshold) && n > 1;
    if (bvh) b += up256(lbvh_bytes((uint32_t)n));
    // light and direction buffers, as SceneStore::upload builds them
    if (!bvh && n >= 1 && n <= kLbMaxSpheres && s.n_lights >= 1 && s.n_lights <= kLbMaxLights)
        b += up256(lb_bytes(s.n_lights, kCellResJobs));
    if (!bvh && n >= 1 && n <= kDbMaxSpheres) b += up256(db_bytes((uint32_t)n, kCellResJobs));
    const uint64_t px = (uint64_t)s.width * s.height;
    b += up256(16 * px) + up256(4 * px) + up256(8 * px) + up256(16 * px);   // accumulator, image, primary hits, directions
    return b;
}

atx_status Server::submit(const atx_batch_scene& d, uint32_t target, uint32_t* id)
{
    if (target == 0) return fail(ATX_ERR_INVALID_ARG, "server_submit: target spp must be > 0");
    if (d.width == 0 || d.height == 0 || (uint64_t)d.width * d.height > 0xffffffffull)
        return fail(ATX_ERR_INVALID_ARG, "server_submit: bad viewport %ux%u", d.width, d.height);
    if ((d.n_spheres && !d.spheres) || (d.n_materials && !d.materials) || (d.n_lights && !d.lights))
        return fail(ATX_ERR_INVALID_ARG, "server_submit: null scene array");
    if (d.n_spheres && !d.n_materials) return fail(ATX_ERR_INVALID_ARG, "server_submit: spheres need a material");
    for (uint32_t i = 0; i < d.n_spheres; ++i)
        if (!finite3(d.spheres[i].center) || !std::isfinite(d.spheres[i].radius))
            return fail(ATX_ERR_INVALID_ARG, "server_submit: sphere %u is not finite", i);
    if (!finite3(d.camera.position) || !finite3(d.camera.direction))
        return fail(ATX_ERR_INVALID_ARG, "server_submit: camera is not finite");
    const uint64_t bytes = job_bytes(d, cfg_.base.bvh_threshold);
    const uint64_t cap = cfg_.base.hbm_budget_bytes;
    std::lock_guard<std::mutex> lock(mu_);
    if (cap && bytes > cap) {
        ++st_.rejected;
        return fail(ATX_ERR_OUT_OF_MEMORY, "server_submit: job needs %llu bytes, budget %llu",
                    (unsigned long long)bytes, (unsigned long long)cap);
    }
    if (cfg_.max_pending && pending_.size() >= cfg_.max_pending) {
        ++st_.rejected;
        return fail(ATX_ERR_BUSY, "server_submit: %u jobs queued", cfg_.max_pending);
    }
    const uint32_t jid = next_id_++;
    Job& j = jobs_[jid];
    j.spheres.assign(d.spheres, d.spheres + d.n_spheres);
    j.materials.assign(d.materials, d.materials + d.n_materials);
    j.lights.assign(d.lights, d.lights + d.n_lights);
    j.desc = d;
    j.desc.spheres = j.spheres.data();
    j.desc.materials = j.materials.data();
    j.desc.lights = j.lights.data();
    j.target = target;
    j.bytes = bytes;
    j.t_submit = now();
    pending_.push_back(jid);
    ++st_.submitted;
    *id = jid;
    cv_work_.notify_one();
    return ATX_OK;
}

// Moves queued jobs to the executor while slots and memory allow: in arrival
// order, or the job with the fewest pixel-samples first.
void Server::admit_locked()
{
    const uint64_t cap = cfg_.base.hbm_budget_bytes;
    while (!pending_.empty() && active_.size() < cfg_.max_active_jobs) {
        auto pick = pending_.begin();
        if (cfg_.policy == ATX_ADMIT_SMALLEST) {
            auto work = [&](uint32_t id) {
                const Job& j = jobs_[id];
                return (uint64_t)j.desc.width * j.desc.height * j.target;
            };
            for (auto it = pending_.begin(); it != pending_.end(); ++it)
                if (work(*it) < work(*pick)) pick = it;
        }
        const uint32_t jid = *pick;
        Job& j = jobs_[jid];
        if (cap && exec_->device_bytes() + j.bytes > cap) break;   // wait for a job to retire
        uint32_t slot = 0;
        const atx_status s = exec_->add(j.desc, j.bytes, &slot);
        if (s == ATX_ERR_OUT_OF_MEMORY && (!active_.empty() || !flights_.empty())) break;
        pending_.erase(pick);
        if (s != ATX_OK) {
            j.state = ATX_JOB_FAILED;
            j.t_done = now();
            ++st_.failed;
            cv_done_.notify_all();
            continue;
        }
        j.slot = slot;
        j.state = ATX_JOB_ACTIVE;
        j.t_admit = now();
        active_.push_back(jid);
        ++st_.admitted;
    }
}

void Server::free_results(Job& j)
{
    if (j.image) exec_->host_free(j.image, j.result_bytes);
    j.image = nullptr;
    j.accum = nullptr;
    j.result_bytes = 0;
}

atx_status Server::queue_pass_locked(bool* queued)
{
    *queued = false;
    // cancelled jobs leave now (their device memory after the queued passes);
    // a new camera restarts a job's accumulation
    std::vector<uint32_t> keep;
    for (uint32_t jid : active_) {
        Job& j = jobs_[jid];
        if (j.cancel) {
            ATX_TRY(exec_->remove(j.slot));
            j.state = ATX_JOB_CANCELLED;
            j.t_done = now();
            ++st_.cancelled;
            cv_done_.notify_all();
            continue;
        }
        if (j.restart) {
            ATX_TRY(exec_->set_camera(j.slot, j.desc.camera));
            j.restart = false;
            j.queued = 0;
            j.done = 0;
            ++j.epoch;
        }
        keep.push_back(jid);
    }
    active_.swap(keep);

    // slices: pass_spp frames per job (by default, more for small images so
    // that every slice is at least kMinSlicePaths: a small wave is mostly
    // launch latency and tail), scaled down so a pass stays within
    // max_pass_paths
    std::vector<std::pair<uint32_t, uint32_t>> plan;   // job, frames this pass
    uint64_t total = 0;
    for (uint32_t jid : active_) {
        const Job& j = jobs_[jid];
        const uint64_t px = (uint64_t)j.desc.width * j.desc.height;
        const uint64_t want =
            auto_slice_ ? std::max<uint64_t>(cfg_.pass_spp, (kMinSlicePaths + px - 1) / px) : cfg_.pass_spp;
        const uint32_t q = (uint32_t)std::min<uint64_t>(j.target - j.queued, want);
        plan.emplace_back(jid, q);
        total += (uint64_t)j.desc.width * j.desc.height * q;
    }
    if (plan.empty()) return ATX_OK;
    if (total > cfg_.max_pass_paths) {
        const double scale = (double)cfg_.max_pass_paths / (double)total;
        total = 0;
        for (auto& p : plan) {
            const Job& j = jobs_[p.first];
            p.second = std::max<uint32_t>(1, (uint32_t)std::floor(p.second * scale));
            total += (uint64_t)j.desc.width * j.desc.height * p.second;
        }
    }
    for (auto& p : plan) ATX_TRY(exec_->set_spp(jobs_[p.first].slot, p.second));
    ATX_TRY(exec_->enqueue_pass());

    Flight f;
    f.paths = total;
    std::vector<uint32_t> still;
    for (auto& p : plan) {
        Job& j = jobs_[p.first];
        j.queued += p.second;
        f.frames.push_back({p.first, p.second, j.epoch});
        if (j.queued < j.target) {
            still.push_back(p.first);
            continue;
        }
        // final pass: read the results back after it
        const uint64_t px = (uint64_t)j.desc.width * j.desc.height;
        j.result_bytes = px * (sizeof(uint32_t) + 4 * sizeof(float));
        void* buf = exec_->host_alloc(j.result_bytes);
        if (!buf) return fail(ATX_ERR_OUT_OF_MEMORY, "server: no host memory for a %llu-pixel result",
                              (unsigned long long)px);
        j.image = static_cast<uint32_t*>(buf);
        j.accum = reinterpret_cast<float*>(j.image + px);
        ATX_TRY(exec_->enqueue_read(j.slot, j.image, j.accum, px));
        ATX_TRY(exec_->set_spp(j.slot, 0));   // resident until the read-back is done, idle meanwhile
        j.draining = true;
        f.finishing.push_back(p.first);
    }
    ATX_TRY(exec_->commit(&f.ticket));
    active_.swap(still);
    flights_.push_back(std::move(f));
    *queued = true;
    return ATX_OK;
}

// Waits for the oldest queued pass and settles its jobs.
atx_status Server::finish_oldest()
{
    uint64_t ticket;
    {
        std::lock_guard<std::mutex> lock(mu_);
        ticket = flights_.front().ticket;
    }
    double ms = 0.0;
    const atx_status s = exec_->wait(ticket, &ms);   // without the lock: submitters keep going
    std::lock_guard<std::mutex> lock(mu_);
    if (s != ATX_OK) return s;
    Flight f = std::move(flights_.front());
    flights_.pop_front();
    st_.busy_s += ms * 1e-3;
    ++st_.passes;
    st_.paths += f.paths;
    for (const auto& e : f.frames) {
        auto it = jobs_.find(e.job);
        if (it != jobs_.end() && it->second.epoch == e.epoch) it->second.done += e.frames;
    }
    for (uint32_t jid : f.finishing) {
        Job& j = jobs_[jid];
        ATX_TRY(exec_->remove(j.slot));
        j.draining = false;
        j.state = ATX_JOB_DONE;
        j.t_done = now();
        ++st_.completed;
    }
    cv_done_.notify_all();
    return ATX_OK;
}

void Server::fail_all_locked(atx_status s)
{
    worker_error_ = s;
    std::snprintf(worker_msg_, sizeof(worker_msg_), "%s", last_error_message());
    auto fail_job = [&](uint32_t jid) {
        Job& j = jobs_[jid];
        if (j.state != ATX_JOB_ACTIVE) return;
        j.state = ATX_JOB_FAILED;
        j.t_done = now();
        j.draining = false;
        exec_->remove(j.slot);
        ++st_.failed;
    };
    for (uint32_t jid : active_) fail_job(jid);
    for (const Flight& f : flights_)
        for (const auto& e : f.frames) fail_job(e.job);
    active_.clear();
    flights_.clear();
    cv_done_.notify_all();
}

void Server::loop()
{
    for (;;) {
        bool queued = false;
        {
            std::unique_lock<std::mutex> lock(mu_);
            cv_work_.wait(lock, [&] { return stop_ || !pending_.empty() || !active_.empty() || !flights_.empty(); });
            if (stop_) break;
            admit_locked();
            if (flights_.size() < kPassesInFlight) {
                const atx_status s = queue_pass_locked(&queued);
                if (s != ATX_OK) {
                    fail_all_locked(s);
                    continue;
                }
            }
            if (!queued && flights_.empty()) {
                // nothing fits yet and nothing runs: wait for a submission or cancel
                if (!pending_.empty()) cv_work_.wait_for(lock, std::chrono::milliseconds(5));
                continue;
            }
            if (queued && flights_.size() < kPassesInFlight) continue;   // queue the next one first
        }
        const atx_status s = finish_oldest();
        if (s != ATX_OK) {
            std::lock_guard<std::mutex> lock(mu_);
            fail_all_locked(s);
        }
    }
    // let queued passes finish (their read-backs write into job buffers), then
    // cancel whatever is left
    while (true) {
        {
            std::lock_guard<std::mutex> lock(mu_);
            if (flights_.empty()) break;
        }
        if (finish_oldest() != ATX_OK) {
            std::lock_guard<std::mutex> lock(mu_);
            flights_.clear();
            break;
        }
    }
    std::lock_guard<std::mutex> lock(mu_);
    for (uint32_t jid : pending_) jobs_[jid].state = ATX_JOB_CANCELLED;
    for (uint32_t jid : active_) jobs_[jid].state = ATX_JOB_CANCELLED;
    pending_.clear();
    active_.clear();
    cv_done_.notify_all();
}

atx_status Server::poll(uint32_t id, atx_job_info* info)
{
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return fail(ATX_ERR_NOT_FOUND, "server: no job %u", id);
    const Job& j = it->second;
    info->state = j.state;
    info->frames_done = j.done;
    info->target_spp = j.target;
    info->width = j.desc.width;
    info->height = j.desc.height;
    info->reserved = 0;
    info->submit_s = j.t_submit;
    info->admit_s = j.t_admit;
    info->done_s = j.t_done;
    return ATX_OK;
}

atx_status Server::wait(uint32_t id, uint32_t timeout_ms)
{
    std::unique_lock<std::mutex> lock(mu_);
    auto finished = [&] {
        auto it = jobs_.find(id);
        return it == jobs_.end() || it->second.state >= ATX_JOB_DONE;
    };
    if (!cv_done_.wait_for(lock, std::chrono::milliseconds(timeout_ms), finished))
        return fail(ATX_ERR_TIMEOUT, "server_wait: job %u not done after %u ms", id, timeout_ms);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return fail(ATX_ERR_NOT_FOUND, "server: no job %u", id);
    if (it->second.state == ATX_JOB_CANCELLED) return fail(ATX_ERR_CANCELLED, "server: job %u cancelled", id);
    if (it->second.state == ATX_JOB_FAILED)
        return fail(worker_error_ != ATX_OK ? worker_error_ : ATX_ERR_CUDA, "server: job %u failed: %s", id,
                    worker_msg_);
    return ATX_OK;
}

atx_status Server::read_image(uint32_t id, uint32_t* host, uint64_t n)
{
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return fail(ATX_ERR_NOT_FOUND, "server: no job %u", id);
    const Job& j = it->second;
    if (j.state != ATX_JOB_DONE) return fail(ATX_ERR_BUSY, "server: job %u not done", id);
    if (!host || n > (uint64_t)j.desc.width * j.desc.height)
        return fail(ATX_ERR_INVALID_ARG, "server_read_image: bad buffer");
    std::memcpy(host, j.image, n * sizeof(uint32_t));
    return ATX_OK;
}

atx_status Server::read_accumulation(uint32_t id, float* host, uint64_t n)
{
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return fail(ATX_ERR_NOT_FOUND, "server: no job %u", id);
    const Job& j = it->second;
    if (j.state != ATX_JOB_DONE) return fail(ATX_ERR_BUSY, "server: job %u not done", id);
    if (!host || n > (uint64_t)j.desc.width * j.desc.height)
        return fail(ATX_ERR_INVALID_ARG, "server_read_accumulation: bad buffer");
    std::memcpy(host, j.accum, 4 * n * sizeof(float));
    return ATX_OK;
}

atx_status Server::cancel(uint32_t id)
{
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return fail(ATX_ERR_NOT_FOUND, "server: no job %u", id);
    Job& j = it->second;
    if (j.state == ATX_JOB_QUEUED) {
        pending_.erase(std::remove(pending_.begin(), pending_.end(), id), pending_.end());
        j.state = ATX_JOB_CANCELLED;
        j.t_done = now();
        ++st_.cancelled;
        cv_done_.notify_all();
        cv_work_.notify_all();
    } else if (j.state == ATX_JOB_ACTIVE && !j.draining) {
        j.cancel = true;   // retired by the worker before its next pass
        cv_work_.notify_all();
    }
    return ATX_OK;
}

atx_status Server::set_camera(uint32_t id, const atx_camera& c)
{
    if (!finite3(c.position) || !finite3(c.direction))
        return fail(ATX_ERR_INVALID_ARG, "server_set_camera: camera is not finite");
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return fail(ATX_ERR_NOT_FOUND, "server: no job %u", id);
    Job& j = it->second;
    if (j.state == ATX_JOB_QUEUED) {
        j.desc.camera = c;
        return ATX_OK;
    }
    if (j.state != ATX_JOB_ACTIVE || j.draining)
        return fail(ATX_ERR_BUSY, "server_set_camera: job %u is finishing or finished", id);
    j.desc.camera = c;
    j.restart = true;
    cv_work_.notify_all();
    return ATX_OK;
}

atx_status Server::release(uint32_t id)
{
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return fail(ATX_ERR_NOT_FOUND, "server: no job %u", id);
    if (it->second.state < ATX_JOB_DONE) return fail(ATX_ERR_BUSY, "server: job %u still running", id);
    free_results(it->second);
    jobs_.erase(it);
    return ATX_OK;
}

atx_status Server::stats(atx_server_stats* out)
{
    std::lock_guard<std::mutex> lock(mu_);
    *out = st_;
    out->device_bytes = exec_->device_bytes();
    size_t draining = 0;   // resident until their final pass and read-back finish
    for (const Flight& f : flights_) draining += f.finishing.size();
    out->active = (uint32_t)(active_.size() + draining);
    out->queued = (uint32_t)pending_.size();
    return ATX_OK;
}

}  // namespace atx
