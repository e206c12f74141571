// Host-side pieces around the render call: the interactive camera update
// (Camera::onUpdate, Engine/src/Camera.cpp:31-108, with the window's input
// passed in instead of polled from GLFW) and headless image files in place of
// the reference's Vulkan image upload (Core/src/Image.cpp:183-271).
#include <cmath>
#include <cstdio>
#include <vector>

#include "atx.h"
#include "host_common.h"

namespace atx {
namespace {

struct Quat {
    float w, x, y, z;
};

void cross3(const float a[3], const float b[3], float out[3])
{
    out[0] = a[1] * b[2] - b[1] * a[2];
    out[1] = a[2] * b[0] - b[2] * a[0];
    out[2] = a[0] * b[1] - b[0] * a[1];
}

// glm::angleAxis: (cos(a/2), axis * sin(a/2)); the axis is not normalised.
Quat angle_axis(float angle, const float axis[3])
{
    const float s = std::sin(angle * 0.5f);
    return Quat{std::cos(angle * 0.5f), axis[0] * s, axis[1] * s, axis[2] * s};
}

// Hamilton product p q (glm::cross of two quaternions).
Quat qmul(const Quat& p, const Quat& q)
{
    return Quat{p.w * q.w - p.x * q.x - p.y * q.y - p.z * q.z, p.w * q.x + p.x * q.w + p.y * q.z - p.z * q.y,
                p.w * q.y + p.y * q.w + p.z * q.x - p.x * q.z, p.w * q.z + p.z * q.w + p.x * q.y - p.y * q.x};
}

Quat qnormalize(const Quat& q)
{
    const float len = std::sqrt((q.x * q.x + q.y * q.y) + (q.z * q.z + q.w * q.w));
    if (len <= 0.0f) return Quat{1.0f, 0.0f, 0.0f, 0.0f};
    const float inv = 1.0f / len;
    return Quat{q.w * inv, q.x * inv, q.y * inv, q.z * inv};
}

// q * v = v + 2 (w (q.xyz x v) + q.xyz x (q.xyz x v))
void qrotate(const Quat& q, const float v[3], float out[3])
{
    const float qv[3] = {q.x, q.y, q.z};
    float uv[3], uuv[3];
    cross3(qv, v, uv);
    cross3(qv, uv, uuv);
    for (int k = 0; k < 3; ++k) out[k] = v[k] + ((uv[k] * q.w) + uuv[k]) * 2.0f;
}

}  // namespace

bool camera_on_update(atx_camera& cam, float last_mouse[2], const atx_camera_input& in, float dt)
{
    const float mdx = (in.mouse[0] - last_mouse[0]) * 0.002f;   // Camera.cpp:33-35
    const float mdy = (in.mouse[1] - last_mouse[1]) * 0.002f;
    last_mouse[0] = in.mouse[0];
    last_mouse[1] = in.mouse[1];
    if (!in.right_button) return false;                          // Camera.cpp:37-41

    bool moved = false;
    const float up[3] = {0.0f, 1.0f, 0.0f};
    float right[3];
    cross3(cam.direction, up, right);                             // Camera.cpp:47
    const float speed = 5.0f;
    // Camera.cpp:51-88: each key pair is if / else if
    const float* axis[3] = {cam.direction, right, up};
    const uint8_t first[3] = {in.key_w, in.key_a, in.key_q};
    const uint8_t second[3] = {in.key_s, in.key_d, in.key_e};
    const float sign_first[3] = {1.0f, -1.0f, -1.0f};             // W: +dir, A: -right, Q: -up
    float step[3][3];
    for (int a = 0; a < 3; ++a)
        for (int k = 0; k < 3; ++k) step[a][k] = (axis[a][k] * speed) * dt;
    for (int a = 0; a < 3; ++a) {
        float sign = 0.0f;
        if (first[a]) sign = sign_first[a];
        else if (second[a]) sign = -sign_first[a];
        if (sign == 0.0f) continue;
        for (int k = 0; k < 3; ++k)
            cam.position[k] = (sign > 0.0f) ? cam.position[k] + step[a][k] : cam.position[k] - step[a][k];
        moved = true;
    }
    if (mdx != 0.0f || mdy != 0.0f) {                             // Camera.cpp:90-101
        const float yaw = mdx * 0.3f, pitch = mdy * 0.3f;         // getRotationSpeed() = 0.3
        const Quat q = qnormalize(qmul(angle_axis(-pitch, right), angle_axis(-yaw, up)));
        float nd[3];
        qrotate(q, cam.direction, nd);
        cam.direction[0] = nd[0];
        cam.direction[1] = nd[1];
        cam.direction[2] = nd[2];
        moved = true;
    }
    return moved;
}

// ------------------------------------------------------------ image files
//
// Rows of the renderer's buffers run from the bottom of the picture up (pixel
// y = 0 is the bottom row: Camera.cpp:180-182 maps y/H to NDC -1..1, and the
// reference shows the texture with its v axis flipped, main.cpp:186-187).
// PPM/PAM store the top row first, so they are written from row H-1 down;
// PFM stores the bottom row first, so it is written in buffer order.

atx_status write_rgba8(const char* path, const uint32_t* px, uint32_t w, uint32_t h, int format)
{
    if (!path || !px || !w || !h) return fail(ATX_ERR_INVALID_ARG, "write image: null pointer or empty image");
    if (format != ATX_IMAGE_PPM && format != ATX_IMAGE_PAM)
        return fail(ATX_ERR_INVALID_ARG, "write image: unknown format %d", format);
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ATX_ERR_INVALID_ARG, "write image: cannot open %s", path);
    const int ch = (format == ATX_IMAGE_PPM) ? 3 : 4;
    if (ch == 3) std::fprintf(f, "P6\n%u %u\n255\n", w, h);
    else std::fprintf(f, "P7\nWIDTH %u\nHEIGHT %u\nDEPTH 4\nMAXVAL 255\nTUPLTYPE RGB_ALPHA\nENDHDR\n", w, h);
    std::vector<unsigned char> row((size_t)w * ch);
    bool ok = true;
    for (uint32_t r = 0; r < h && ok; ++r) {
        const uint32_t* src = px + (size_t)(h - 1 - r) * w;
        for (uint32_t x = 0; x < w; ++x) {
            const uint32_t v = src[x];   // A<<24 | B<<16 | G<<8 | R (Renderer.h:70-78)
            unsigned char* d = &row[(size_t)x * ch];
            d[0] = (unsigned char)(v & 0xFFu);
            d[1] = (unsigned char)((v >> 8) & 0xFFu);
            d[2] = (unsigned char)((v >> 16) & 0xFFu);
            if (ch == 4) d[3] = (unsigned char)(v >> 24);
        }
        ok = std::fwrite(row.data(), 1, row.size(), f) == row.size();
    }
    if (std::fclose(f) != 0 || !ok) return fail(ATX_ERR_INVALID_ARG, "write image: cannot write %s", path);
    return ATX_OK;
}

atx_status write_pfm(const char* path, const float* acc, uint32_t w, uint32_t h)
{
    if (!path || !acc || !w || !h) return fail(ATX_ERR_INVALID_ARG, "write pfm: null pointer or empty image");
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ATX_ERR_INVALID_ARG, "write pfm: cannot open %s", path);
    const uint32_t probe = 1;
    const bool little = *(const unsigned char*)&probe == 1;
    std::fprintf(f, "PF\n%u %u\n%s\n", w, h, little ? "-1.0" : "1.0");
    std::vector<float> row((size_t)w * 3);
    bool ok = true;
    for (uint32_t y = 0; y < h && ok; ++y) {
        const float* src = acc + (size_t)y * w * 4;
        for (uint32_t x = 0; x < w; ++x) {
            const float n = src[4 * x + 3];   // frames accumulated (alpha adds 1 per frame)
            for (int c = 0; c < 3; ++c) row[3 * x + c] = (n > 0.0f) ? src[4 * x + c] / n : 0.0f;
        }
        ok = std::fwrite(row.data(), sizeof(float), row.size(), f) == row.size();
    }
    if (std::fclose(f) != 0 || !ok) return fail(ATX_ERR_INVALID_ARG, "write pfm: cannot write %s", path);
    return ATX_OK;
}

}  // namespace atx
