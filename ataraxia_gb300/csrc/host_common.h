// Host-side helpers shared by the renderer, batch and server: status/error
// reporting, device buffers charged against an HBM budget, and the camera
// matrices.
#pragma once

#include <atomic>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "atx.h"

namespace atx {

// Records a formatted message as the calling thread's last error and returns st.
atx_status fail(atx_status st, const char* fmt, ...);
atx_status cuda_fail(cudaError_t e, const char* what);
const char* last_error_message();
void clear_error();

#define ATX_CUDA(call)                                           \
    do {                                                         \
        cudaError_t atx_e_ = (call);                             \
        if (atx_e_ != cudaSuccess) return ::atx::cuda_fail(atx_e_, #call); \
    } while (0)

#define ATX_TRY(expr)                              \
    do {                                           \
        atx_status atx_s_ = (expr);                \
        if (atx_s_ != ATX_OK) return atx_s_;       \
    } while (0)

// Device bytes held by one owner (a renderer, a server) against a cap.  The
// reference allocates with bare cudaMalloc (DeviceMemory.h:19-106); here every
// allocation is charged so that admission control can refuse work before the
// device runs out.
class Budget {
public:
    explicit Budget(uint64_t cap = 0) : cap_(cap) {}
    bool reserve(uint64_t bytes)
    {
        uint64_t cur = used_.load();
        for (;;) {
            if (cap_ && cur + bytes > cap_) return false;
            if (used_.compare_exchange_weak(cur, cur + bytes)) return true;
        }
    }
    void release(uint64_t bytes) { used_.fetch_sub(bytes); }
    uint64_t used() const { return used_.load(); }
    uint64_t cap() const { return cap_; }
    void set_cap(uint64_t c) { cap_ = c; }

private:
    uint64_t cap_;
    std::atomic<uint64_t> used_{0};
};

// Where a buffer is allocated and freed in stream order: allocated from pool
// on `alloc` (cudaMallocFromPoolAsync), freed on `release` (cudaFreeAsync)
// after the work already queued there.  Neither call synchronises the device,
// which lets a server admit and retire jobs while a pass is running.
struct StreamOrder {
    cudaMemPool_t pool = nullptr;
    cudaStream_t alloc = nullptr;
    cudaStream_t release = nullptr;
};

// Owning device allocation charged to a Budget.  By default freed with
// cudaFree, which synchronises the device (buffers are then replaced only on
// resize / scene upload); with a StreamOrder, allocated and freed in stream
// order.
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    ~DeviceBuffer() { reset(); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept { *this = static_cast<DeviceBuffer&&>(o); }
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept
    {
        if (this != &o) {
            reset();
            ptr_ = o.ptr_; bytes_ = o.bytes_; budget_ = o.budget_; order_ = o.order_;
            o.ptr_ = nullptr; o.bytes_ = 0; o.budget_ = nullptr;
        }
        return *this;
    }

    // Allocates bytes (rounded up to 256); keeps the current block when it is
    // already large enough.
    atx_status ensure(uint64_t bytes, Budget* budget, const char* what);
    void reset();

    void* get() const { return ptr_; }
    template <class T> T* as() const { return static_cast<T*>(ptr_); }
    uint64_t bytes() const { return bytes_; }
    // Allocate / free this buffer in stream order from now on (nullptr: cudaMalloc / cudaFree).
    // Takes effect when the buffer holds no memory.
    void use_stream_order(const StreamOrder* order)
    {
        if (!ptr_) order_ = order;
    }

private:
    void* ptr_ = nullptr;
    uint64_t bytes_ = 0;
    Budget* budget_ = nullptr;
    const StreamOrder* order_ = nullptr;
};

// Camera.cpp:134-159: perspective (right-handed, clip z in [-1, 1]) and lookAt
// from position toward position + direction with +Y up, plus both inverses.
void camera_matrices(const atx_camera& cam, uint32_t width, uint32_t height, float view[16], float inv_view[16],
                     float proj[16], float inv_proj[16]);
void mat4_inverse(const float m[16], float out[16]);

// Camera::onUpdate (Camera.cpp:31-108) with the input passed in (host_tools.cpp).
bool camera_on_update(atx_camera& cam, float last_mouse[2], const atx_camera_input& in, float dt);
// Image files (host_tools.cpp): ATX_IMAGE_PPM / ATX_IMAGE_PAM from RGBA8, PFM from float4 sums.
atx_status write_rgba8(const char* path, const uint32_t* px, uint32_t w, uint32_t h, int format);
atx_status write_pfm(const char* path, const float* acc, uint32_t w, uint32_t h);

}  // namespace atx
