// Scene files and the scene graph: the reference's JSON scene format
// (Engine/src/Utils.cpp:3-187, written and read with nlohmann::json), its node
// hierarchy (Engine/include/SceneNode.h, Engine/src/SceneNode.cpp) and the
// flattening of the hierarchy into world-space spheres that the renderer
// uploads (Engine/src/Renderer.cu:25-37, 67-96).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "atx.h"

namespace atx {

struct GraphNode {
    std::string name;
    float position[3] = {0.0f, 0.0f, 0.0f};
    float rotation[4] = {0.0f, 0.0f, 0.0f, 0.0f};   // quaternion x, y, z, w (file order)
    float scale[3] = {1.0f, 1.0f, 1.0f};
    std::vector<atx_sphere> spheres;
    std::vector<uint32_t> children;
    uint32_t depth = 0;   // root = 0
};

constexpr uint32_t kNoNode = 0xffffffffu;
constexpr uint32_t kMaxNodeDepth = 256;   // bounds the recursion of flatten / export

// Column-major 4x4 float matrix, m[c][r] = column c, row r (glm's storage).
struct Mat4 {
    float m[4][4];
};

class SceneGraph {
public:
    // Scene() (Engine/include/Scene.h:66-75): a root node named "Scene", the
    // reference's default camera (Camera.h:63-75) and settings (Scene.h:49-56).
    SceneGraph();

    // Utils::deserializeScene (Utils.cpp:97-137) of a JSON text.
    atx_status parse(const char* text, size_t len);
    // Utils::serializeScene + json::dump(4) (Utils.cpp:3-96): keys sorted, four
    // spaces of indent, numbers in nlohmann's shortest round-trip form.
    std::string to_json() const;

    // Renderer::traverseSceneGraph + allocateDeviceMemory (Renderer.cu:25-37,
    // 67-96): depth-first, a node's own spheres before its children's.
    void flatten(std::vector<atx_sphere>& out) const;
    size_t sphere_count() const;

    // Appends a child of `parent`; kNoNode if parent is unknown or the graph
    // would be deeper than kMaxNodeDepth.
    uint32_t add_node(uint32_t parent, const char* name);
    std::vector<GraphNode> nodes;   // nodes[0] is the root
    std::vector<atx_material> materials;
    std::vector<atx_light> lights;
    atx_camera camera;
    atx_settings settings;
};

// SceneNode::updateGlobalTransform's local matrix (SceneNode.cpp:44-46):
// translate(I, p) * mat4_cast(q) * scale(I, s).
Mat4 node_local_matrix(const GraphNode& n);
Mat4 mat4_mul(const Mat4& a, const Mat4& b);

}  // namespace atx
