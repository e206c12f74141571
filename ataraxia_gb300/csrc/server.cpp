// Render server: a worker thread admits jobs in arrival order when a slot and
// their device memory fit, runs batched passes over all active jobs (each
// renders a slice of its remaining frames), and retires jobs that reach their
// target: image and accumulator are copied to the host and the job's device
// memory is released.  Submitters never touch the GPU.
#include "server.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "lbvh.h"

namespace atx {

namespace {
constexpr uint32_t kDefaultActive = 64;
constexpr uint32_t kDefaultPassSpp = 16;
constexpr uint64_t kDefaultPassPaths = 1ull << 28;
constexpr uint32_t kDefaultBvhThreshold = 1024;

uint64_t up256(uint64_t x) { return (x + 255u) & ~uint64_t(255u); }

bool finite3(const float* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

// The batched renderer.
class BatchExecutor : public Executor {
public:
    explicit BatchExecutor(const atx_config& cfg) : b_(cfg) {}
    atx_status init() override { return b_.init(); }
    atx_status add(const atx_batch_scene& d, uint64_t, uint32_t* slot) override { return b_.add_scene(d, slot); }
    atx_status remove(uint32_t slot) override { return b_.remove_scene(slot); }
    atx_status set_spp(uint32_t slot, uint32_t spp) override { return b_.set_spp(slot, spp); }
    atx_status run_pass() override
    {
        ATX_TRY(b_.run());
        return b_.synchronize();
    }
    atx_status read_image(uint32_t slot, uint32_t* host, uint64_t n) override { return b_.read_image(slot, host, n); }
    atx_status read_accumulation(uint32_t slot, float* host, uint64_t n) override
    {
        return b_.read_accumulation(slot, host, n);
    }
    uint64_t device_bytes() const override { return b_.scene_bytes(); }

private:
    Batch b_;
};

// Host-only stand-in for the device: accounts memory by the admission
// estimate, takes 1 ns of wall time per path of a pass, and fills images with
// the number of frames rendered.  fail_pass > 0 makes that pass report an
// error, so failure handling can be tested without a GPU.
class HostExecutor : public Executor {
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
    atx_status run_pass() override
    {
        if (fail_pass_ && ++passes_ == fail_pass_) return fail(ATX_ERR_CUDA, "host executor: injected device error");
        uint64_t paths = 0;
        for (auto& s : slots_)
            if (s.used) {
                paths += (uint64_t)s.w * s.h * s.spp;
                s.frames += s.spp;
            }
        std::this_thread::sleep_for(std::chrono::nanoseconds(paths));
        return ATX_OK;
    }
    atx_status read_image(uint32_t slot, uint32_t* host, uint64_t n) override
    {
        std::fill(host, host + n, slots_[slot].frames);
        return ATX_OK;
    }
    atx_status read_accumulation(uint32_t slot, float* host, uint64_t n) override
    {
        for (uint64_t i = 0; i < n; ++i) {
            host[4 * i] = host[4 * i + 1] = host[4 * i + 2] = 0.0f;
            host[4 * i + 3] = (float)slots_[slot].frames;
        }
        return ATX_OK;
    }
    uint64_t device_bytes() const override { return bytes_; }

private:
    struct Slot { bool used; uint32_t w, h, spp, frames; uint64_t bytes; };
    std::vector<Slot> slots_;
    uint64_t bytes_ = 0;
    uint32_t fail_pass_ = 0, passes_ = 0;
};
}  // namespace

std::unique_ptr<Executor> make_batch_executor(const atx_config& cfg) { return std::make_unique<BatchExecutor>(cfg); }
std::unique_ptr<Executor> make_host_executor(uint32_t fail_pass) { return std::make_unique<HostExecutor>(fail_pass); }

Server::Server(const atx_server_config& cfg) : cfg_(cfg)
{
    if (!cfg_.max_active_jobs) cfg_.max_active_jobs = kDefaultActive;
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
    if (n >= (bvh_threshold ? bvh_threshold : kDefaultBvhThreshold) && n > 1) b += up256(lbvh_bytes((uint32_t)n));
    const uint64_t px = (uint64_t)s.width * s.height;
    b += up256(16 * px) + up256(4 * px);
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

// Moves queued jobs to the executor, in arrival order, while slots and memory allow.
void Server::admit_locked()
{
    const uint64_t cap = cfg_.base.hbm_budget_bytes;
    while (!pending_.empty() && active_.size() < cfg_.max_active_jobs) {
        const uint32_t jid = pending_.front();
        Job& j = jobs_[jid];
        if (cap && exec_->device_bytes() + j.bytes > cap) break;   // wait for a job to retire
        uint32_t slot = 0;
        const atx_status s = exec_->add(j.desc, j.bytes, &slot);
        if (s == ATX_ERR_OUT_OF_MEMORY && !active_.empty()) break;
        pending_.pop_front();
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

atx_status Server::run_pass()
{
    // slices: up to pass_spp frames per job, scaled so a pass stays bounded
    std::vector<std::pair<uint32_t, uint32_t>> plan;   // job, frames this pass
    uint64_t total = 0;
    {
        std::lock_guard<std::mutex> lock(mu_);
        for (uint32_t jid : active_) {
            const Job& j = jobs_[jid];
            const uint32_t q = std::min(j.target - j.done, cfg_.pass_spp);
            plan.emplace_back(jid, q);
            total += (uint64_t)j.desc.width * j.desc.height * q;
        }
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
    }
    const double t = now();
    ATX_TRY(exec_->run_pass());
    std::lock_guard<std::mutex> lock(mu_);
    st_.busy_s += now() - t;
    ++st_.passes;
    st_.paths += total;
    std::vector<uint32_t> still;
    for (auto& p : plan) {
        Job& j = jobs_[p.first];
        j.done += p.second;
        const bool finished = j.done >= j.target;
        if (finished || j.cancel) {
            if (finished) {
                const uint64_t px = (uint64_t)j.desc.width * j.desc.height;
                j.image.resize(px);
                j.accum.resize(4 * px);
                ATX_TRY(exec_->read_image(j.slot, j.image.data(), px));
                ATX_TRY(exec_->read_accumulation(j.slot, j.accum.data(), px));
                j.state = ATX_JOB_DONE;
                ++st_.completed;
            } else {
                j.state = ATX_JOB_CANCELLED;
                ++st_.cancelled;
            }
            j.t_done = now();
            ATX_TRY(exec_->remove(j.slot));
            cv_done_.notify_all();
        } else {
            still.push_back(p.first);
        }
    }
    active_.swap(still);
    return ATX_OK;
}

void Server::loop()
{
    for (;;) {
        {
            std::unique_lock<std::mutex> lock(mu_);
            cv_work_.wait(lock, [&] { return stop_ || !pending_.empty() || !active_.empty(); });
            if (stop_) break;
            admit_locked();
            if (active_.empty()) {
                // nothing fits yet and nothing runs: wait for a submission or cancel
                if (!pending_.empty()) cv_work_.wait_for(lock, std::chrono::milliseconds(5));
                continue;
            }
        }
        const atx_status s = run_pass();
        if (s != ATX_OK) {
            std::lock_guard<std::mutex> lock(mu_);
            worker_error_ = s;
            std::snprintf(worker_msg_, sizeof(worker_msg_), "%s", last_error_message());
            for (uint32_t jid : active_) {
                Job& j = jobs_[jid];
                j.state = ATX_JOB_FAILED;
                j.t_done = now();
                exec_->remove(j.slot);
                ++st_.failed;
            }
            active_.clear();
            cv_done_.notify_all();
        }
    }
    // cancel whatever is left
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
    if (it->second.state != ATX_JOB_DONE) return fail(ATX_ERR_BUSY, "server: job %u not done", id);
    if (!host || n > it->second.image.size()) return fail(ATX_ERR_INVALID_ARG, "server_read_image: bad buffer");
    std::memcpy(host, it->second.image.data(), n * sizeof(uint32_t));
    return ATX_OK;
}

atx_status Server::read_accumulation(uint32_t id, float* host, uint64_t n)
{
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return fail(ATX_ERR_NOT_FOUND, "server: no job %u", id);
    if (it->second.state != ATX_JOB_DONE) return fail(ATX_ERR_BUSY, "server: job %u not done", id);
    if (!host || 4 * n > it->second.accum.size())
        return fail(ATX_ERR_INVALID_ARG, "server_read_accumulation: bad buffer");
    std::memcpy(host, it->second.accum.data(), 4 * n * sizeof(float));
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
    } else if (j.state == ATX_JOB_ACTIVE) {
        j.cancel = true;   // retired by the worker after the current pass
    }
    return ATX_OK;
}

atx_status Server::release(uint32_t id)
{
    std::lock_guard<std::mutex> lock(mu_);
    auto it = jobs_.find(id);
    if (it == jobs_.end()) return fail(ATX_ERR_NOT_FOUND, "server: no job %u", id);
    if (it->second.state < ATX_JOB_DONE) return fail(ATX_ERR_BUSY, "server: job %u still running", id);
    jobs_.erase(it);
    return ATX_OK;
}

atx_status Server::stats(atx_server_stats* out)
{
    std::lock_guard<std::mutex> lock(mu_);
    *out = st_;
    out->device_bytes = exec_->device_bytes();
    out->active = (uint32_t)active_.size();
    out->queued = (uint32_t)pending_.size();
    return ATX_OK;
}

}  // namespace atx
