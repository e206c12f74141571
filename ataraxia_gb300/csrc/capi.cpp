// extern "C" entry points of libatx.so (declared in include/atx.h).  Each
// wrapper checks its handle, clears the thread's last error and converts C++
// exceptions into status codes so nothing unwinds across the C boundary.
#include <new>
#include <vector>

#include "atx.h"
#include "host_common.h"
#include "renderer.h"

struct atx_renderer {
    atx::Renderer impl;
    explicit atx_renderer(const atx_config& c) : impl(c) {}
};

namespace {

template <class F>
atx_status guarded(F&& f)
{
    atx::clear_error();
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return atx::fail(ATX_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (...) {
        return atx::fail(ATX_ERR_CUDA, "unexpected exception");
    }
}

#define NEED(r) \
    if (!(r)) return atx::fail(ATX_ERR_INVALID_ARG, "%s: null renderer", __func__)

}  // namespace

extern "C" {

ATX_API int atx_abi_version(void) { return ATX_ABI_VERSION; }

ATX_API const char* atx_status_string(atx_status s)
{
    switch (s) {
    case ATX_OK: return "ok";
    case ATX_ERR_INVALID_ARG: return "invalid argument";
    case ATX_ERR_OUT_OF_MEMORY: return "out of memory";
    case ATX_ERR_CUDA: return "CUDA error";
    case ATX_ERR_TIMEOUT: return "timeout";
    case ATX_ERR_BUSY: return "busy";
    case ATX_ERR_NOT_FOUND: return "not found";
    case ATX_ERR_CANCELLED: return "cancelled";
    case ATX_ERR_NO_DEVICE: return "no CUDA device";
    case ATX_ERR_PARSE: return "parse error";
    }
    return "unknown status";
}

ATX_API const char* atx_last_error(void) { return atx::last_error_message(); }

ATX_API atx_status atx_device_count(int32_t* count)
{
    return guarded([&]() -> atx_status {
        if (!count) return atx::fail(ATX_ERR_INVALID_ARG, "atx_device_count: null pointer");
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            *count = 0;
            return ATX_OK;
        }
        *count = n;
        return ATX_OK;
    });
}

ATX_API atx_status atx_renderer_create(const atx_config* config, atx_renderer** out)
{
    return guarded([&]() -> atx_status {
        if (!out) return atx::fail(ATX_ERR_INVALID_ARG, "atx_renderer_create: null out");
        *out = nullptr;
        atx_config c{};
        if (config) c = *config;
        atx_renderer* r = new atx_renderer(c);
        atx_status st = r->impl.init();
        if (st != ATX_OK) {
            delete r;
            return st;
        }
        *out = r;
        return ATX_OK;
    });
}

ATX_API atx_status atx_renderer_destroy(atx_renderer* r)
{
    return guarded([&]() -> atx_status {
        delete r;
        return ATX_OK;
    });
}

ATX_API atx_status atx_resize(atx_renderer* r, uint32_t w, uint32_t h)
{
    return guarded([&]() -> atx_status { NEED(r); return r->impl.resize(w, h); });
}

ATX_API atx_status atx_set_scene(atx_renderer* r, const atx_sphere* s, uint32_t n, const atx_material* m,
                                 uint32_t nm, const atx_light* l, uint32_t nl)
{
    return guarded([&]() -> atx_status { NEED(r); return r->impl.set_scene(s, n, m, nm, l, nl); });
}

ATX_API atx_status atx_set_settings(atx_renderer* r, const atx_settings* s)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!s) return atx::fail(ATX_ERR_INVALID_ARG, "atx_set_settings: null settings");
        return r->impl.set_settings(*s);
    });
}

ATX_API atx_status atx_get_settings(const atx_renderer* r, atx_settings* s)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!s) return atx::fail(ATX_ERR_INVALID_ARG, "atx_get_settings: null settings");
        *s = r->impl.settings();
        return ATX_OK;
    });
}

ATX_API atx_status atx_reset_frame_index(atx_renderer* r)
{
    return guarded([&]() -> atx_status { NEED(r); r->impl.reset_frame_index(); return ATX_OK; });
}

ATX_API atx_status atx_get_frame_index(const atx_renderer* r, uint32_t* f)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!f) return atx::fail(ATX_ERR_INVALID_ARG, "atx_get_frame_index: null pointer");
        *f = r->impl.frame_index();
        return ATX_OK;
    });
}

ATX_API atx_status atx_set_camera(atx_renderer* r, const atx_camera* c)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!c) return atx::fail(ATX_ERR_INVALID_ARG, "atx_set_camera: null camera");
        return r->impl.set_camera(*c);
    });
}

ATX_API atx_status atx_set_camera_matrices(atx_renderer* r, const float inv_view[16], const float inv_proj[16],
                                           const float position[3])
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!inv_view || !inv_proj || !position) return atx::fail(ATX_ERR_INVALID_ARG, "atx_set_camera_matrices: null");
        return r->impl.set_camera_matrices(inv_view, inv_proj, position);
    });
}

ATX_API atx_status atx_render(atx_renderer* r, uint32_t spp)
{
    return guarded([&]() -> atx_status { NEED(r); return r->impl.render(spp); });
}

ATX_API atx_status atx_read_image_async(atx_renderer* r, uint32_t* host_rgba8, uint64_t n_pixels, uint64_t* ticket)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        return r->impl.read_image_async(host_rgba8, n_pixels, ticket);
    });
}

ATX_API atx_status atx_wait_read(atx_renderer* r, uint64_t ticket)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        return r->impl.wait_read(ticket);
    });
}

ATX_API atx_status atx_join(atx_renderer* r)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        return r->impl.join();
    });
}

ATX_API atx_status atx_synchronize(atx_renderer* r)
{
    return guarded([&]() -> atx_status { NEED(r); return r->impl.synchronize(); });
}

ATX_API atx_status atx_read_accumulation(atx_renderer* r, float* host_rgba, uint64_t n)
{
    return guarded([&]() -> atx_status { NEED(r); return r->impl.read_accumulation(host_rgba, n); });
}

ATX_API atx_status atx_read_image(atx_renderer* r, uint32_t* host_rgba8, uint64_t n)
{
    return guarded([&]() -> atx_status { NEED(r); return r->impl.read_image(host_rgba8, n); });
}

ATX_API atx_status atx_device_buffers(atx_renderer* r, void** accumulation, void** image)
{
    return guarded([&]() -> atx_status { NEED(r); return r->impl.device_buffers(accumulation, image); });
}

ATX_API atx_status atx_get_stats(const atx_renderer* r, atx_stats* s)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!s) return atx::fail(ATX_ERR_INVALID_ARG, "atx_get_stats: null pointer");
        return const_cast<atx_renderer*>(r)->impl.stats(s);
    });
}

ATX_API atx_status atx_get_kernel_times(atx_renderer* r, atx_kernel_times* t)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!t) return atx::fail(ATX_ERR_INVALID_ARG, "atx_get_kernel_times: null pointer");
        return r->impl.kernel_times(t);
    });
}

ATX_API atx_status atx_reset_kernel_times(atx_renderer* r)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        atx_kernel_times drop{};
        ATX_TRY(r->impl.kernel_times(&drop));
        r->impl.reset_kernel_times();
        return ATX_OK;
    });
}

ATX_API atx_status atx_get_stream(atx_renderer* r, void** stream)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!stream) return atx::fail(ATX_ERR_INVALID_ARG, "atx_get_stream: null pointer");
        *stream = static_cast<void*>(r->impl.stream());
        return ATX_OK;
    });
}

ATX_API atx_status atx_autotune(atx_renderer* r, uint32_t spp, uint32_t passes, int32_t use_cache, atx_tuning* out)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!out) return atx::fail(ATX_ERR_INVALID_ARG, "atx_autotune: null pointer");
        return r->impl.autotune(spp, passes, use_cache != 0, out);
    });
}

ATX_API atx_status atx_get_tuning(atx_renderer* r, atx_tuning* out)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!out) return atx::fail(ATX_ERR_INVALID_ARG, "atx_get_tuning: null pointer");
        return r->impl.tuning(out);
    });
}

ATX_API atx_status atx_set_tuning(atx_renderer* r, const atx_tuning* t)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!t) return atx::fail(ATX_ERR_INVALID_ARG, "atx_set_tuning: null pointer");
        return r->impl.set_tuning(*t);
    });
}

ATX_API atx_status atx_host_alloc(uint64_t bytes, void** out)
{
    return guarded([&]() -> atx_status {
        if (!out) return atx::fail(ATX_ERR_INVALID_ARG, "atx_host_alloc: null out");
        *out = nullptr;
        ATX_CUDA(cudaMallocHost(out, bytes ? bytes : 1));
        return ATX_OK;
    });
}

ATX_API atx_status atx_host_free(void* p)
{
    return guarded([&]() -> atx_status {
        if (p) ATX_CUDA(cudaFreeHost(p));
        return ATX_OK;
    });
}

ATX_API atx_status atx_camera_matrices(const atx_camera* c, uint32_t w, uint32_t h, float view[16],
                                       float inv_view[16], float proj[16], float inv_proj[16])
{
    return guarded([&]() -> atx_status {
        if (!c) return atx::fail(ATX_ERR_INVALID_ARG, "atx_camera_matrices: null camera");
        if (w == 0 || h == 0) return atx::fail(ATX_ERR_INVALID_ARG, "atx_camera_matrices: zero viewport");
        atx::camera_matrices(*c, w, h, view, inv_view, proj, inv_proj);
        return ATX_OK;
    });
}

ATX_API atx_status atx_trace_nearest(atx_renderer* r, const float* origins, const float* dirs, uint64_t n,
                                     float* t_out, int32_t* id_out)
{
    return guarded([&]() -> atx_status { NEED(r); return r->impl.trace_nearest(origins, dirs, n, t_out, id_out); });
}

ATX_API atx_status atx_primary_directions(atx_renderer* r, float* host_dirs, uint64_t n_pixels)
{
    return guarded([&]() -> atx_status { NEED(r); return r->impl.primary_directions(host_dirs, n_pixels); });
}

ATX_API atx_status atx_camera_on_update(atx_camera* camera, float last_mouse[2], const atx_camera_input* input,
                                        float dt, int32_t* moved)
{
    return guarded([&]() -> atx_status {
        if (!camera || !last_mouse || !input)
            return atx::fail(ATX_ERR_INVALID_ARG, "atx_camera_on_update: null pointer");
        const bool m = atx::camera_on_update(*camera, last_mouse, *input, dt);
        if (moved) *moved = m ? 1 : 0;
        return ATX_OK;
    });
}

ATX_API atx_status atx_update_camera(atx_renderer* r, atx_camera* camera, float last_mouse[2],
                                     const atx_camera_input* input, float dt, int32_t* moved)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        if (!camera || !last_mouse || !input)
            return atx::fail(ATX_ERR_INVALID_ARG, "atx_update_camera: null pointer");
        const bool m = atx::camera_on_update(*camera, last_mouse, *input, dt);
        if (moved) *moved = m ? 1 : 0;
        if (!m) return ATX_OK;
        ATX_TRY(r->impl.set_camera(*camera));          // main.cpp:24-29
        r->impl.reset_frame_index();
        return ATX_OK;
    });
}

ATX_API atx_status atx_write_rgba8(const char* path, const uint32_t* rgba8, uint32_t width, uint32_t height,
                                   int32_t format)
{
    return guarded([&]() -> atx_status { return atx::write_rgba8(path, rgba8, width, height, format); });
}

ATX_API atx_status atx_write_pfm(const char* path, const float* accum, uint32_t width, uint32_t height)
{
    return guarded([&]() -> atx_status { return atx::write_pfm(path, accum, width, height); });
}

ATX_API atx_status atx_save_image(atx_renderer* r, const char* path, int32_t format)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        const uint32_t w = r->impl.width(), h = r->impl.height();
        if (!w || !h) return atx::fail(ATX_ERR_INVALID_ARG, "atx_save_image: no image (call atx_resize)");
        const uint64_t n = (uint64_t)w * h;
        if (format == ATX_IMAGE_PFM) {
            std::vector<float> acc(n * 4);
            ATX_TRY(r->impl.read_accumulation(acc.data(), n));
            return atx::write_pfm(path, acc.data(), w, h);
        }
        std::vector<uint32_t> img(n);
        ATX_TRY(r->impl.read_image(img.data(), n));
        return atx::write_rgba8(path, img.data(), w, h, format);
    });
}

}  // extern "C"

// ------------------------------------------------------------ scene graph

#include <cstdio>

#include "scene_io.h"

struct atx_scene {
    atx::SceneGraph g;
};

#define NEED_SCENE(s) \
    if (!(s)) return atx::fail(ATX_ERR_INVALID_ARG, "%s: null scene", __func__)
#define NEED_NODE(s, k) \
    if ((k) >= (s)->g.nodes.size()) return atx::fail(ATX_ERR_INVALID_ARG, "%s: no node %u", __func__, (unsigned)(k))

extern "C" {

ATX_API atx_status atx_scene_create(atx_scene** out)
{
    return guarded([&]() -> atx_status {
        if (!out) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_create: null out");
        *out = new atx_scene();
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_destroy(atx_scene* s)
{
    delete s;
    return ATX_OK;
}

ATX_API atx_status atx_scene_parse_json(const char* text, uint64_t len, atx_scene** out)
{
    return guarded([&]() -> atx_status {
        if (!out || (!text && len)) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_parse_json: null pointer");
        *out = nullptr;
        auto* s = new atx_scene();
        const atx_status st = s->g.parse(text ? text : "", (size_t)len);
        if (st != ATX_OK) {
            delete s;
            return st;
        }
        *out = s;
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_load(const char* path, atx_scene** out)
{
    return guarded([&]() -> atx_status {
        if (!path || !out) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_load: null pointer");
        *out = nullptr;
        std::FILE* f = std::fopen(path, "rb");
        if (!f) return atx::fail(ATX_ERR_NOT_FOUND, "atx_scene_load: cannot open %s", path);
        std::string text;
        char buf[65536];
        size_t n;
        while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
        const bool bad = std::ferror(f) != 0;
        std::fclose(f);
        if (bad) return atx::fail(ATX_ERR_NOT_FOUND, "atx_scene_load: cannot read %s", path);
        return atx_scene_parse_json(text.data(), text.size(), out);
    });
}

ATX_API atx_status atx_scene_to_json(const atx_scene* s, char* buf, uint64_t cap, uint64_t* len)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        if (!len) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_to_json: null len");
        const std::string j = s->g.to_json();
        *len = j.size();
        if (buf) std::memcpy(buf, j.data(), j.size() < cap ? j.size() : (size_t)cap);
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_save(const atx_scene* s, const char* path)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        if (!path) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_save: null path");
        const std::string j = s->g.to_json();
        std::FILE* f = std::fopen(path, "wb");
        if (!f) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_save: cannot open %s", path);
        const bool ok = std::fwrite(j.data(), 1, j.size(), f) == j.size();
        if (std::fclose(f) != 0 || !ok) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_save: cannot write %s", path);
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_get_info(const atx_scene* s, atx_scene_info* info)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        if (!info) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_get_info: null info");
        info->n_spheres = (uint32_t)s->g.sphere_count();
        info->n_materials = (uint32_t)s->g.materials.size();
        info->n_lights = (uint32_t)s->g.lights.size();
        info->n_nodes = (uint32_t)s->g.nodes.size();
        info->camera = s->g.camera;
        info->settings = s->g.settings;
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_flatten(const atx_scene* s, atx_sphere* out, uint64_t cap)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        std::vector<atx_sphere> v;
        s->g.flatten(v);
        if (!out && !v.empty()) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_flatten: null out");
        if (cap < v.size())
            return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_flatten: %zu spheres, room for %llu", v.size(),
                             (unsigned long long)cap);
        if (!v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(atx_sphere));
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_get_materials(const atx_scene* s, atx_material* out, uint64_t cap)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        const auto& v = s->g.materials;
        if (cap < v.size() || (!out && !v.empty()))
            return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_get_materials: room for %llu of %zu",
                             (unsigned long long)cap, v.size());
        if (!v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(atx_material));
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_get_lights(const atx_scene* s, atx_light* out, uint64_t cap)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        const auto& v = s->g.lights;
        if (cap < v.size() || (!out && !v.empty()))
            return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_get_lights: room for %llu of %zu",
                             (unsigned long long)cap, v.size());
        if (!v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(atx_light));
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_add_node(atx_scene* s, uint32_t parent, const char* name, uint32_t* node)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        NEED_NODE(s, parent);
        const uint32_t k = s->g.add_node(parent, name ? name : "Untitled");   // SceneNode() default name
        if (k == atx::kNoNode) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_add_node: graph too deep");
        if (node) *node = k;
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_set_transform(atx_scene* s, uint32_t node, const float position[3],
                                           const float rotation_xyzw[4], const float scale[3])
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        NEED_NODE(s, node);
        atx::GraphNode& n = s->g.nodes[node];
        if (position) std::memcpy(n.position, position, sizeof n.position);
        if (rotation_xyzw) std::memcpy(n.rotation, rotation_xyzw, sizeof n.rotation);
        if (scale) std::memcpy(n.scale, scale, sizeof n.scale);
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_add_spheres(atx_scene* s, uint32_t node, const atx_sphere* spheres, uint32_t n)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        NEED_NODE(s, node);
        if (n && !spheres) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_add_spheres: null spheres");
        auto& v = s->g.nodes[node].spheres;
        v.insert(v.end(), spheres, spheres + n);
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_set_materials(atx_scene* s, const atx_material* m, uint32_t n)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        if (n && !m) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_set_materials: null materials");
        s->g.materials.assign(m, m + n);
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_set_lights(atx_scene* s, const atx_light* l, uint32_t n)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        if (n && !l) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_set_lights: null lights");
        s->g.lights.assign(l, l + n);
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_set_camera(atx_scene* s, const atx_camera* c)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        if (!c) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_set_camera: null camera");
        s->g.camera = *c;
        return ATX_OK;
    });
}

ATX_API atx_status atx_scene_set_settings(atx_scene* s, const atx_settings* st)
{
    return guarded([&]() -> atx_status {
        NEED_SCENE(s);
        if (!st) return atx::fail(ATX_ERR_INVALID_ARG, "atx_scene_set_settings: null settings");
        s->g.settings = *st;
        return ATX_OK;
    });
}

ATX_API atx_status atx_set_scene_graph(atx_renderer* r, const atx_scene* s)
{
    return guarded([&]() -> atx_status {
        NEED(r);
        NEED_SCENE(s);
        std::vector<atx_sphere> v;
        s->g.flatten(v);
        return r->impl.set_scene(v.data(), (uint32_t)v.size(), s->g.materials.data(),
                                 (uint32_t)s->g.materials.size(), s->g.lights.data(), (uint32_t)s->g.lights.size());
    });
}

}  // extern "C"

// ------------------------------------------------------------------ batches

#include "batch_host.h"

struct atx_batch {
    atx::Batch impl;
    explicit atx_batch(const atx_config& c) : impl(c) {}
};

#define NEEDB(b) \
    if (!(b)) return atx::fail(ATX_ERR_INVALID_ARG, "%s: null batch", __func__)

extern "C" {

ATX_API atx_status atx_batch_create(const atx_config* config, atx_batch** out)
{
    return guarded([&]() -> atx_status {
        if (!out) return atx::fail(ATX_ERR_INVALID_ARG, "atx_batch_create: null out");
        *out = nullptr;
        atx_config c{};
        if (config) c = *config;
        atx_batch* b = new atx_batch(c);
        atx_status st = b->impl.init();
        if (st != ATX_OK) {
            delete b;
            return st;
        }
        *out = b;
        return ATX_OK;
    });
}

ATX_API atx_status atx_batch_destroy(atx_batch* b)
{
    return guarded([&]() -> atx_status { delete b; return ATX_OK; });
}

ATX_API atx_status atx_batch_add_scene(atx_batch* b, const atx_batch_scene* scene, uint32_t* id)
{
    return guarded([&]() -> atx_status {
        NEEDB(b);
        if (!scene || !id) return atx::fail(ATX_ERR_INVALID_ARG, "atx_batch_add_scene: null argument");
        return b->impl.add_scene(*scene, id);
    });
}

ATX_API atx_status atx_batch_remove_scene(atx_batch* b, uint32_t id)
{
    return guarded([&]() -> atx_status { NEEDB(b); return b->impl.remove_scene(id); });
}

ATX_API atx_status atx_batch_set_spp(atx_batch* b, uint32_t id, uint32_t spp)
{
    return guarded([&]() -> atx_status { NEEDB(b); return b->impl.set_spp(id, spp); });
}

ATX_API atx_status atx_batch_reset(atx_batch* b, uint32_t id)
{
    return guarded([&]() -> atx_status { NEEDB(b); return b->impl.reset(id); });
}

ATX_API atx_status atx_batch_frame_index(atx_batch* b, uint32_t id, uint32_t* f)
{
    return guarded([&]() -> atx_status {
        NEEDB(b);
        if (!f) return atx::fail(ATX_ERR_INVALID_ARG, "atx_batch_frame_index: null pointer");
        return b->impl.frame_index(id, f);
    });
}

ATX_API atx_status atx_batch_set_camera(atx_batch* b, uint32_t id, const atx_camera* c)
{
    return guarded([&]() -> atx_status {
        NEEDB(b);
        if (!c) return atx::fail(ATX_ERR_INVALID_ARG, "atx_batch_set_camera: null camera");
        return b->impl.set_camera(id, *c);
    });
}

ATX_API atx_status atx_batch_run(atx_batch* b)
{
    return guarded([&]() -> atx_status { NEEDB(b); return b->impl.run(); });
}

ATX_API atx_status atx_batch_synchronize(atx_batch* b)
{
    return guarded([&]() -> atx_status { NEEDB(b); return b->impl.synchronize(); });
}

ATX_API atx_status atx_batch_read_accumulation(atx_batch* b, uint32_t id, float* host, uint64_t n)
{
    return guarded([&]() -> atx_status { NEEDB(b); return b->impl.read_accumulation(id, host, n); });
}

ATX_API atx_status atx_batch_read_image(atx_batch* b, uint32_t id, uint32_t* host, uint64_t n)
{
    return guarded([&]() -> atx_status { NEEDB(b); return b->impl.read_image(id, host, n); });
}

ATX_API atx_status atx_batch_get_stats(atx_batch* b, atx_batch_stats* s)
{
    return guarded([&]() -> atx_status {
        NEEDB(b);
        if (!s) return atx::fail(ATX_ERR_INVALID_ARG, "atx_batch_get_stats: null pointer");
        return b->impl.stats(s);
    });
}

ATX_API atx_status atx_batch_set_tuning(atx_batch* b, const atx_batch_tuning* t)
{
    return guarded([&]() -> atx_status {
        NEEDB(b);
        if (!t) return atx::fail(ATX_ERR_INVALID_ARG, "atx_batch_set_tuning: null pointer");
        return b->impl.set_tuning(*t);
    });
}

ATX_API atx_status atx_batch_get_tuning(atx_batch* b, atx_batch_tuning* t)
{
    return guarded([&]() -> atx_status {
        NEEDB(b);
        if (!t) return atx::fail(ATX_ERR_INVALID_ARG, "atx_batch_get_tuning: null pointer");
        *t = b->impl.tuning();
        return ATX_OK;
    });
}

ATX_API atx_status atx_batch_autotune(atx_batch* b, uint32_t passes, atx_batch_tuning* chosen)
{
    return guarded([&]() -> atx_status { NEEDB(b); return b->impl.autotune(passes, chosen); });
}

}  // extern "C"

// ------------------------------------------------------------------ serving

#include "server.h"

struct atx_server {
    atx::Server impl;
    explicit atx_server(const atx_server_config& c) : impl(c) {}
};

#define NEEDS(s) \
    if (!(s)) return atx::fail(ATX_ERR_INVALID_ARG, "%s: null server", __func__)

extern "C" {

ATX_API atx_status atx_server_create(const atx_server_config* config, atx_server** out)
{
    return guarded([&]() -> atx_status {
        if (!out) return atx::fail(ATX_ERR_INVALID_ARG, "atx_server_create: null out");
        *out = nullptr;
        atx_server_config c{};
        if (config) c = *config;
        atx_server* s = new atx_server(c);
        atx_status st = s->impl.init();
        if (st != ATX_OK) {
            delete s;
            return st;
        }
        *out = s;
        return ATX_OK;
    });
}

ATX_API atx_status atx_server_destroy(atx_server* s)
{
    return guarded([&]() -> atx_status { delete s; return ATX_OK; });
}

ATX_API atx_status atx_server_submit(atx_server* s, const atx_batch_scene* scene, uint32_t target, uint32_t* job)
{
    return guarded([&]() -> atx_status {
        NEEDS(s);
        if (!scene || !job) return atx::fail(ATX_ERR_INVALID_ARG, "atx_server_submit: null argument");
        return s->impl.submit(*scene, target, job);
    });
}

ATX_API atx_status atx_server_poll(atx_server* s, uint32_t job, atx_job_info* info)
{
    return guarded([&]() -> atx_status {
        NEEDS(s);
        if (!info) return atx::fail(ATX_ERR_INVALID_ARG, "atx_server_poll: null info");
        return s->impl.poll(job, info);
    });
}

ATX_API atx_status atx_server_wait(atx_server* s, uint32_t job, uint32_t timeout_ms)
{
    return guarded([&]() -> atx_status { NEEDS(s); return s->impl.wait(job, timeout_ms); });
}

ATX_API atx_status atx_server_read_image(atx_server* s, uint32_t job, uint32_t* host, uint64_t n)
{
    return guarded([&]() -> atx_status { NEEDS(s); return s->impl.read_image(job, host, n); });
}

ATX_API atx_status atx_server_read_accumulation(atx_server* s, uint32_t job, float* host, uint64_t n)
{
    return guarded([&]() -> atx_status { NEEDS(s); return s->impl.read_accumulation(job, host, n); });
}

ATX_API atx_status atx_server_cancel(atx_server* s, uint32_t job)
{
    return guarded([&]() -> atx_status { NEEDS(s); return s->impl.cancel(job); });
}

ATX_API atx_status atx_server_set_camera(atx_server* s, uint32_t job, const atx_camera* c)
{
    return guarded([&]() -> atx_status {
        NEEDS(s);
        if (!c) return atx::fail(ATX_ERR_INVALID_ARG, "atx_server_set_camera: null camera");
        return s->impl.set_camera(job, *c);
    });
}

ATX_API atx_status atx_server_release(atx_server* s, uint32_t job)
{
    return guarded([&]() -> atx_status { NEEDS(s); return s->impl.release(job); });
}

ATX_API atx_status atx_server_get_stats(atx_server* s, atx_server_stats* st)
{
    return guarded([&]() -> atx_status {
        NEEDS(s);
        if (!st) return atx::fail(ATX_ERR_INVALID_ARG, "atx_server_get_stats: null pointer");
        return s->impl.stats(st);
    });
}

ATX_API atx_status atx_server_now(atx_server* s, double* seconds)
{
    return guarded([&]() -> atx_status {
        NEEDS(s);
        if (!seconds) return atx::fail(ATX_ERR_INVALID_ARG, "atx_server_now: null pointer");
        *seconds = s->impl.now();
        return ATX_OK;
    });
}

}  // extern "C"
