// Render server: continuous batching of progressive render jobs over the
// batched renderer (batch_host.h), or over a host-only simulated executor for
// scheduling tests on machines without a GPU.
#pragma once

#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "atx.h"
#include "batch_host.h"

namespace atx {

// What the server needs from the device: resident scenes and batched passes,
// queued asynchronously.  A pass, the read-backs queued after it and the
// completion marker of commit() run in order; wait(ticket) returns when
// everything up to that marker has finished.
class Executor {
public:
    virtual ~Executor() = default;
    virtual atx_status init() = 0;
    // Makes a scene resident; its uploads do not wait for queued passes.
    virtual atx_status add(const atx_batch_scene& d, uint64_t bytes, uint32_t* slot) = 0;
    // Frees a slot after the work already queued (passes, read-backs).
    virtual atx_status remove(uint32_t slot) = 0;
    virtual atx_status set_spp(uint32_t slot, uint32_t spp) = 0;
    virtual atx_status set_camera(uint32_t slot, const atx_camera& c) = 0;
    virtual atx_status enqueue_pass() = 0;
    virtual atx_status enqueue_read(uint32_t slot, uint32_t* image, float* accum, uint64_t n) = 0;
    virtual atx_status commit(uint64_t* ticket) = 0;
    // Blocks until the ticket's marker is reached; device time since the
    // previous commit (the pass and its read-backs).
    virtual atx_status wait(uint64_t ticket, double* device_ms) = 0;
    virtual uint64_t device_bytes() const = 0;
    // Host buffers for results (page-locked where that makes copies async).
    virtual void* host_alloc(uint64_t bytes) = 0;
    virtual void host_free(void* p, uint64_t bytes) = 0;
};

std::unique_ptr<Executor> make_batch_executor(const atx_config& cfg);
std::unique_ptr<Executor> make_host_executor(uint32_t fail_pass);

class Server {
public:
    explicit Server(const atx_server_config& cfg);
    ~Server();
    atx_status init();

    atx_status submit(const atx_batch_scene& scene, uint32_t target, uint32_t* id);
    atx_status poll(uint32_t id, atx_job_info* info);
    atx_status wait(uint32_t id, uint32_t timeout_ms);
    atx_status read_image(uint32_t id, uint32_t* host, uint64_t n);
    atx_status read_accumulation(uint32_t id, float* host, uint64_t n);
    atx_status cancel(uint32_t id);
    atx_status set_camera(uint32_t id, const atx_camera& c);
    atx_status release(uint32_t id);
    atx_status stats(atx_server_stats* out);
    double now() const;

    // Device bytes a job will hold while active (admission control).
    static uint64_t job_bytes(const atx_batch_scene& s, uint32_t bvh_threshold);

private:
    struct Job {
        atx_job_state state = ATX_JOB_QUEUED;
        std::vector<atx_sphere> spheres;
        std::vector<atx_material> materials;
        std::vector<atx_light> lights;
        atx_batch_scene desc{};
        uint32_t target = 0;
        uint32_t queued = 0;        // frames in passes queued so far
        uint32_t done = 0;          // frames finished on the device
        uint32_t slot = 0;          // executor scene id while resident
        uint64_t bytes = 0;
        double t_submit = 0, t_admit = 0, t_done = 0;
        uint32_t* image = nullptr;  // results, host buffers from the executor
        float* accum = nullptr;
        uint64_t result_bytes = 0;
        bool cancel = false;
        bool restart = false;       // camera changed: restart when its queued passes finish
        bool draining = false;      // final pass queued, read-back pending
        uint32_t epoch = 0;         // bumped by a camera change; older frames in flight do not count
    };
    // A queued pass: its marker, the frames it adds per job and the jobs whose
    // final read-back follows it.
    struct Flight {
        uint64_t ticket = 0;
        uint64_t paths = 0;
        struct Part {
            uint32_t job, frames, epoch;
        };
        std::vector<Part> frames;
        std::vector<uint32_t> finishing;
    };
    void loop();
    void admit_locked();
    // Plans and queues one pass over the active jobs (lock held); false if
    // there was nothing to render.
    atx_status queue_pass_locked(bool* queued);
    atx_status finish_oldest();
    void fail_all_locked(atx_status s);
    void free_results(Job& j);

    atx_server_config cfg_;
    bool auto_slice_ = true;
    std::unique_ptr<Executor> exec_;
    std::chrono::steady_clock::time_point t0_;
    std::thread worker_;
    mutable std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    bool stop_ = false;
    uint32_t next_id_ = 1;
    std::unordered_map<uint32_t, Job> jobs_;
    std::deque<uint32_t> pending_;
    std::vector<uint32_t> active_;
    std::deque<Flight> flights_;
    atx_server_stats st_{};
    atx_status worker_error_ = ATX_OK;
    char worker_msg_[256] = "";
};

}  // namespace atx
