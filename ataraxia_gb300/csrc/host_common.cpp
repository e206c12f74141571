// Status reporting, budgeted device buffers and the host camera matrices.
// Built with -ffp-contract=off so the matrices round the same way on x86-64
// and aarch64.
#include "host_common.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>

namespace atx {

namespace {
thread_local char g_last_error[512] = "";
}

atx_status fail(atx_status st, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return st;
}

atx_status cuda_fail(cudaError_t e, const char* what)
{
    atx_status st = ATX_ERR_CUDA;
    if (e == cudaErrorMemoryAllocation) st = ATX_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) st = ATX_ERR_NO_DEVICE;
    // clear a non-sticky error so the next call starts clean
    (void)cudaGetLastError();
    return fail(st, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

const char* last_error_message() { return g_last_error; }
void clear_error() { g_last_error[0] = '\0'; }

atx_status DeviceBuffer::ensure(uint64_t bytes, Budget* budget, const char* what)
{
    bytes = (bytes + 255u) & ~uint64_t(255u);
    if (bytes == 0) bytes = 256;
    if (ptr_ && bytes_ >= bytes && budget_ == budget) return ATX_OK;
    reset();
    if (budget && !budget->reserve(bytes))
        return fail(ATX_ERR_OUT_OF_MEMORY, "%s: %llu bytes exceed the HBM budget (%llu of %llu in use)", what,
                    (unsigned long long)bytes, (unsigned long long)budget->used(),
                    (unsigned long long)budget->cap());
    cudaError_t e = order_ ? cudaMallocFromPoolAsync(&ptr_, bytes, order_->pool, order_->alloc)
                           : cudaMalloc(&ptr_, bytes);
    if (e != cudaSuccess) {
        ptr_ = nullptr;
        if (budget) budget->release(bytes);
        return cuda_fail(e, what);
    }
    bytes_ = bytes;
    budget_ = budget;
    return ATX_OK;
}

void DeviceBuffer::reset()
{
    if (ptr_) {
        if (order_) cudaFreeAsync(ptr_, order_->release);
        else cudaFree(ptr_);
        if (budget_) budget_->release(bytes_);
    }
    ptr_ = nullptr;
    bytes_ = 0;
    budget_ = nullptr;
}

// Inverse by the Laplace expansion in complementary 2x2 minors of the top and
// bottom row pairs (D. Eberly, "The Laplace Expansion Theorem: Computing the
// Determinants and Inverses of Matrices").  Column-major.
void mat4_inverse(const float m[16], float out[16])
{
    auto A = [&](int r, int c) { return m[c * 4 + r]; };
    const float s0 = A(0, 0) * A(1, 1) - A(1, 0) * A(0, 1);
    const float s1 = A(0, 0) * A(1, 2) - A(1, 0) * A(0, 2);
    const float s2 = A(0, 0) * A(1, 3) - A(1, 0) * A(0, 3);
    const float s3 = A(0, 1) * A(1, 2) - A(1, 1) * A(0, 2);
    const float s4 = A(0, 1) * A(1, 3) - A(1, 1) * A(0, 3);
    const float s5 = A(0, 2) * A(1, 3) - A(1, 2) * A(0, 3);
    const float c5 = A(2, 2) * A(3, 3) - A(3, 2) * A(2, 3);
    const float c4 = A(2, 1) * A(3, 3) - A(3, 1) * A(2, 3);
    const float c3 = A(2, 1) * A(3, 2) - A(3, 1) * A(2, 2);
    const float c2 = A(2, 0) * A(3, 3) - A(3, 0) * A(2, 3);
    const float c1 = A(2, 0) * A(3, 2) - A(3, 0) * A(2, 2);
    const float c0 = A(2, 0) * A(3, 1) - A(3, 0) * A(2, 1);
    const float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    const float id = 1.0f / det;
    float b[4][4];
    b[0][0] = (A(1, 1) * c5 - A(1, 2) * c4 + A(1, 3) * c3) * id;
    b[0][1] = (-A(0, 1) * c5 + A(0, 2) * c4 - A(0, 3) * c3) * id;
    b[0][2] = (A(3, 1) * s5 - A(3, 2) * s4 + A(3, 3) * s3) * id;
    b[0][3] = (-A(2, 1) * s5 + A(2, 2) * s4 - A(2, 3) * s3) * id;
    b[1][0] = (-A(1, 0) * c5 + A(1, 2) * c2 - A(1, 3) * c1) * id;
    b[1][1] = (A(0, 0) * c5 - A(0, 2) * c2 + A(0, 3) * c1) * id;
    b[1][2] = (-A(3, 0) * s5 + A(3, 2) * s2 - A(3, 3) * s1) * id;
    b[1][3] = (A(2, 0) * s5 - A(2, 2) * s2 + A(2, 3) * s1) * id;
    b[2][0] = (A(1, 0) * c4 - A(1, 1) * c2 + A(1, 3) * c0) * id;
    b[2][1] = (-A(0, 0) * c4 + A(0, 1) * c2 - A(0, 3) * c0) * id;
    b[2][2] = (A(3, 0) * s4 - A(3, 1) * s2 + A(3, 3) * s0) * id;
    b[2][3] = (-A(2, 0) * s4 + A(2, 1) * s2 - A(2, 3) * s0) * id;
    b[3][0] = (-A(1, 0) * c3 + A(1, 1) * c1 - A(1, 2) * c0) * id;
    b[3][1] = (A(0, 0) * c3 - A(0, 1) * c1 + A(0, 2) * c0) * id;
    b[3][2] = (-A(3, 0) * s3 + A(3, 1) * s1 - A(3, 2) * s0) * id;
    b[3][3] = (A(2, 0) * s3 - A(2, 1) * s1 + A(2, 2) * s0) * id;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = b[r][c];
}

namespace {
void normalize(const float a[3], float out[3])
{
    const float d = (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2];
    const float inv = 1.0f / std::sqrt(d);
    out[0] = a[0] * inv;
    out[1] = a[1] * inv;
    out[2] = a[2] * inv;
}
void cross(const float a[3], const float b[3], float out[3])
{
    out[0] = a[1] * b[2] - b[1] * a[2];
    out[1] = a[2] * b[0] - b[2] * a[0];
    out[2] = a[0] * b[1] - b[0] * a[1];
}
float dot(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
}  // namespace

void camera_matrices(const atx_camera& cam, uint32_t width, uint32_t height, float view[16], float inv_view[16],
                     float proj[16], float inv_proj[16])
{
    const float aspect = (float)width / (float)height;
    const float fovy = cam.fov_deg * 0.01745329251994329576923690768489f;  // glm::radians
    const float th = std::tan(fovy / 2.0f);
    float P[16] = {0};
    P[0 * 4 + 0] = 1.0f / (aspect * th);
    P[1 * 4 + 1] = 1.0f / th;
    P[2 * 4 + 2] = -(cam.far_clip + cam.near_clip) / (cam.far_clip - cam.near_clip);
    P[2 * 4 + 3] = -1.0f;
    P[3 * 4 + 2] = -(2.0f * cam.far_clip * cam.near_clip) / (cam.far_clip - cam.near_clip);

    const float* pos = cam.position;
    const float center[3] = {pos[0] + cam.direction[0], pos[1] + cam.direction[1], pos[2] + cam.direction[2]};
    const float fwd[3] = {center[0] - pos[0], center[1] - pos[1], center[2] - pos[2]};
    const float up[3] = {0.0f, 1.0f, 0.0f};
    float f[3], s[3], u[3], sx[3];
    normalize(fwd, f);
    cross(f, up, sx);
    normalize(sx, s);
    cross(s, f, u);
    float V[16] = {0};
    V[0 * 4 + 0] = s[0]; V[1 * 4 + 0] = s[1]; V[2 * 4 + 0] = s[2];
    V[0 * 4 + 1] = u[0]; V[1 * 4 + 1] = u[1]; V[2 * 4 + 1] = u[2];
    V[0 * 4 + 2] = -f[0]; V[1 * 4 + 2] = -f[1]; V[2 * 4 + 2] = -f[2];
    V[3 * 4 + 0] = -dot(s, pos);
    V[3 * 4 + 1] = -dot(u, pos);
    V[3 * 4 + 2] = dot(f, pos);
    V[3 * 4 + 3] = 1.0f;

    if (proj) std::memcpy(proj, P, sizeof(P));
    if (view) std::memcpy(view, V, sizeof(V));
    if (inv_proj) mat4_inverse(P, inv_proj);
    if (inv_view) mat4_inverse(V, inv_view);
}

}  // namespace atx
