"""Scene-graph flattening and scene-file reading restated in Python (the oracle).

TEST INFRASTRUCTURE ONLY: imported by tests/, never by the product.

Follows the reference:
  - Utils::deserializeScene / deserializeSceneNode (Engine/src/Utils.cpp:97-173):
    camera position/direction/fov, nodes with transformation position,
    rotation stored x, y, z, w and read as glm::quat(w, x, y, z), scale,
    spheres (center, radius, materialIndex) and children; the root keeps the
    name "Scene" that Scene() gave it; materials, lights, settings.
  - SceneNode::updateGlobalTransform (Engine/src/SceneNode.cpp:42-59):
    local = translate(I, p) * mat4_cast(q) * scale(I, s), global = parent * local.
  - Renderer::traverseSceneGraph (Engine/src/Renderer.cu:67-96): centre =
    (global * (c, 1)).xyz / w, radius *= mean of the lengths of the first three
    columns of global; depth first, own spheres before children.
  - Renderer::allocateDeviceMemory (Renderer.cu:30-37): material indexes
    outside [0, materials) become 0.

Arithmetic: every operation rounds to float32, in glm's order (column-major
matrices; mat*mat column by column as left-to-right sums; mat*vec4 as
(c0*v0 + c1*v1) + (c2*v2 + c3*v3); length as sqrt((x*x + y*y) + z*z)).  glm
is an un-vendored submodule of the reference (thirdparty/glm, fork
github.com/1neskk/glm, branch c5eaa, SHA not recoverable), so the summation
order is that of glm's published source as generally released: for
translation / unit-scale / identity-rotation graphs, the only kind the
reference's sample scene holds, every order gives the same bits.
"""
from __future__ import annotations

import json

import numpy as np

f32 = np.float32


def _identity():
    return [[f32(1.0) if c == r else f32(0.0) for r in range(4)] for c in range(4)]


def mat_mul(a, b):
    """glm mat4 * mat4: column c of the result = ((a0*b[c][0] + a1*b[c][1]) + a2*b[c][2]) + a3*b[c][3]."""
    out = []
    for c in range(4):
        col = []
        for k in range(4):
            s = f32(a[0][k] * b[c][0])
            s = f32(s + f32(a[1][k] * b[c][1]))
            s = f32(s + f32(a[2][k] * b[c][2]))
            s = f32(s + f32(a[3][k] * b[c][3]))
            col.append(s)
        out.append(col)
    return out


def mat_vec(m, v):
    return [f32(f32(f32(m[0][k] * v[0]) + f32(m[1][k] * v[1])) + f32(f32(m[2][k] * v[2]) + f32(m[3][k] * v[3])))
            for k in range(4)]


def local_matrix(position, rotation_xyzw, scale):
    """SceneNode.cpp:44-46."""
    I = _identity()
    p = [f32(x) for x in position]
    T = [list(c) for c in I]
    for k in range(4):
        s = f32(I[0][k] * p[0])
        s = f32(s + f32(I[1][k] * p[1]))
        s = f32(s + f32(I[2][k] * p[2]))
        T[3][k] = f32(s + I[3][k])
    x, y, z, w = (f32(v) for v in rotation_xyzw)
    xx, yy, zz = f32(x * x), f32(y * y), f32(z * z)
    xz, xy, yz = f32(x * z), f32(x * y), f32(y * z)
    wx, wy, wz = f32(w * x), f32(w * y), f32(w * z)
    one, two = f32(1.0), f32(2.0)
    R = [list(c) for c in I]
    R[0][0] = f32(one - f32(two * f32(yy + zz)))
    R[0][1] = f32(two * f32(xy + wz))
    R[0][2] = f32(two * f32(xz - wy))
    R[1][0] = f32(two * f32(xy - wz))
    R[1][1] = f32(one - f32(two * f32(xx + zz)))
    R[1][2] = f32(two * f32(yz + wx))
    R[2][0] = f32(two * f32(xz + wy))
    R[2][1] = f32(two * f32(yz - wx))
    R[2][2] = f32(one - f32(two * f32(xx + yy)))
    sc = [f32(v) for v in scale]
    S = [[f32(I[c][k] * sc[c]) if c < 3 else I[c][k] for k in range(4)] for c in range(4)]
    return mat_mul(mat_mul(T, R), S)


def _length(col):
    return f32(np.sqrt(f32(f32(f32(col[0] * col[0]) + f32(col[1] * col[1])) + f32(col[2] * col[2]))))


def flatten(node: dict, n_materials: int, parent=None, out=None):
    """Renderer.cu:67-96 over a parsed JSON node; returns [(cx, cy, cz, r, material)]."""
    out = [] if out is None else out
    parent = _identity() if parent is None else parent
    t = node["transformation"]
    g = mat_mul(parent, local_matrix(t["position"], t["rotation"], t["scale"]))
    scale = f32(f32(f32(_length(g[0]) + _length(g[1])) + _length(g[2])) / f32(3.0))
    for s in node.get("spheres") or []:
        c = mat_vec(g, [f32(s["center"][0]), f32(s["center"][1]), f32(s["center"][2]), f32(1.0)])
        m = int(s["materialIndex"])
        if m < 0 or m >= n_materials:
            m = 0
        out.append((f32(c[0] / c[3]), f32(c[1] / c[3]), f32(c[2] / c[3]), f32(f32(s["radius"]) * scale), m))
    for ch in node.get("children") or []:
        flatten(ch, n_materials, g, out)
    return out


def flatten_file_text(text: str):
    j = json.loads(text)
    n_mat = len(j.get("materials") or [])
    return flatten(j["sceneGraph"], n_mat) if "sceneGraph" in j else []


def flatten_f64(node: dict, n_materials: int, parent=None, out=None):
    """The same transform in float64 with numpy matrices: the tolerance reference."""
    out = [] if out is None else out
    parent = np.eye(4) if parent is None else parent
    t = node["transformation"]
    x, y, z, w = t["rotation"]
    R = np.eye(4)
    R[:3, :3] = np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
        [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
        [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    T = np.eye(4)
    T[:3, 3] = t["position"]
    S = np.diag(list(t["scale"]) + [1.0])
    g = parent @ T @ R @ S
    scale = np.mean(np.linalg.norm(g[:3, :3], axis=0))
    for s in node.get("spheres") or []:
        c = g @ np.array(list(s["center"]) + [1.0])
        m = int(s["materialIndex"])
        out.append((c[0] / c[3], c[1] / c[3], c[2] / c[3], s["radius"] * scale,
                    m if 0 <= m < n_materials else 0))
    for ch in node.get("children") or []:
        flatten_f64(ch, n_materials, g, out)
    return out
