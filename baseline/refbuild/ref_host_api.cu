// C entry layer over the host half of the reference's render path, compiled
// together with the reference's unmodified Camera.cpp, SceneNode.cpp and
// Renderer.cu (baseline/refbuild/Makefile).  Test infrastructure: CPU tests
// load it to check the project's camera, camera-motion and scene-graph code
// against the reference's own, bit for bit.  Nothing here touches a GPU.
//
//   refh_camera         Camera(fov, near, far, pos, dir) + Resize(w, h):
//                       matrices (Camera.cpp:134-159) and the per-pixel ray
//                       directions (Camera.cpp:161-195)
//   refh_camera_update  Camera::onUpdate(dt) (Camera.cpp:31-108) with the
//                       input state set by the caller
//   refh_flatten        SceneNode::updateGlobalTransform (SceneNode.cpp:42-59)
//                       and Renderer::traverseSceneGraph (Renderer.cu:67-96)
//                       over a node tree given as flat arrays
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>
#include <curand_kernel.h>

// Renderer::traverseSceneGraph is a private static member; this file alone
// (not the reference's sources) opens the class's private section to call it.
#define private public
#include "Renderer.h"
#undef private
#include "input/Input.h"

namespace {
void mat_out(const glm::mat4& m, float* out)
{
    if (!out) return;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[c * 4 + r] = m[c][r];
}
}  // namespace

extern "C" {

__attribute__((visibility("default"))) int refh_camera(float fov, float near_clip, float far_clip, const float* pos,
                                                       const float* dir, uint32_t w, uint32_t h, float* dirs_out,
                                                       float* view, float* inv_view, float* proj, float* inv_proj)
{
    Camera cam(fov, near_clip, far_clip, glm::vec3(pos[0], pos[1], pos[2]), glm::vec3(dir[0], dir[1], dir[2]));
    // Resize returns early when the size is unchanged (the constructor's
    // 1600x900), before computing any ray direction; pass through 1x1 then.
    if (w == 1600 && h == 900) cam.Resize(1, 1);
    cam.Resize(w, h);
    const auto& d = cam.getRayDirection();
    if (d.size() != static_cast<size_t>(w) * h) return 1;
    if (dirs_out)
        for (size_t i = 0; i < d.size(); ++i) {
            dirs_out[3 * i + 0] = d[i].x;
            dirs_out[3 * i + 1] = d[i].y;
            dirs_out[3 * i + 2] = d[i].z;
        }
    mat_out(cam.getViewMatrix(), view);
    mat_out(cam.getInverseViewMatrix(), inv_view);
    mat_out(cam.getProjectionMatrix(), proj);
    mat_out(cam.getInverseProjectionMatrix(), inv_proj);
    return 0;
}

// keys: W, A, S, D, Q, E as 0/1.  The camera starts at pos/dir with its last
// mouse position at last_mouse (one update with the button up records it).
__attribute__((visibility("default"))) int refh_camera_update(float* pos, float* dir, float* last_mouse,
                                                              const uint8_t* keys, int right_button, float mouse_x,
                                                              float mouse_y, float dt)
{
    Camera cam(45.0f, 0.1f, 100.0f, glm::vec3(pos[0], pos[1], pos[2]), glm::vec3(dir[0], dir[1], dir[2]));
    cam.Resize(8, 8);   // keeps onUpdate's ray-direction pass small
    auto& st = Input::ref_input_state();
    std::memset(&st, 0, sizeof(st));
    st.mouse_x = last_mouse[0];
    st.mouse_y = last_mouse[1];
    cam.onUpdate(dt);
    const Input::KeyCode codes[6] = {Input::Key::W, Input::Key::A, Input::Key::S,
                                     Input::Key::D, Input::Key::Q, Input::Key::E};
    for (int k = 0; k < 6; ++k) st.keys[static_cast<unsigned>(codes[k])] = keys[k] != 0;
    st.right_button = right_button != 0;
    st.mouse_x = mouse_x;
    st.mouse_y = mouse_y;
    const bool moved = cam.onUpdate(dt);
    const glm::vec3 p = cam.getPosition(), d = cam.getDirection();
    pos[0] = p.x; pos[1] = p.y; pos[2] = p.z;
    dir[0] = d.x; dir[1] = d.y; dir[2] = d.z;
    last_mouse[0] = mouse_x;
    last_mouse[1] = mouse_y;
    return moved ? 1 : 0;
}

// Nodes 0..n_nodes-1, node 0 the root; parent[i] < i for i > 0.  Per node:
// position (3), rotation x, y, z, w (4), scale (3).  Spheres: owning node,
// centre (3), radius, material id.  Output: the flattened spheres, 5 floats
// each (centre, radius, id as float), in traversal order; returns the count.
__attribute__((visibility("default"))) int refh_flatten(int n_nodes, const int* parent, const float* trs,
                                                        int n_spheres, const int* owner, const float* sph,
                                                        const int* ids, float* out, int out_cap)
{
    std::vector<std::shared_ptr<SceneNode>> nodes;
    for (int i = 0; i < n_nodes; ++i) {
        auto nd = std::make_shared<SceneNode>("n");
        const float* t = trs + 10 * i;
        nd->setPosition(glm::vec3(t[0], t[1], t[2]));
        nd->setRotation(glm::quat(t[6], t[3], t[4], t[5]));
        nd->setScale(glm::vec3(t[7], t[8], t[9]));
        nodes.push_back(nd);
        if (i > 0) nodes[parent[i]]->addChild(nd);
    }
    for (int s = 0; s < n_spheres; ++s)
        nodes[owner[s]]->addSphere(Sphere(glm::vec3(sph[4 * s], sph[4 * s + 1], sph[4 * s + 2]), sph[4 * s + 3], ids[s]));
    std::vector<Sphere> flat;
    Renderer::traverseSceneGraph(nodes.empty() ? nullptr : nodes[0], glm::mat4(1.0f), flat);
    const int n = static_cast<int>(flat.size());
    for (int i = 0; i < n && i < out_cap; ++i) {
        out[5 * i + 0] = flat[i].center.x;
        out[5 * i + 1] = flat[i].center.y;
        out[5 * i + 2] = flat[i].center.z;
        out[5 * i + 3] = flat[i].radius;
        out[5 * i + 4] = static_cast<float>(flat[i].id);
    }
    return n;
}

}  // extern "C"
