"""The project's host-side pieces against the reference's own host code, compiled from its unmodified
sources (baseline/refbuild: Camera.cpp, SceneNode.cpp and the host half of Renderer.cu over the
project's minimal glm), bit for bit:

* camera matrices (Camera.cpp:134-159) and per-pixel ray directions (Camera.cpp:161-195) against the
  library's camera_matrices, the oracle's directions and the numpy restatement the GPU tests feed to the
  reference's kernel;
* Camera::onUpdate (Camera.cpp:31-108) against the library's CameraController;
* SceneNode::updateGlobalTransform + Renderer::traverseSceneGraph (SceneNode.cpp:42-59,
  Renderer.cu:67-96) against the library's scene-graph flattening.

The reference's host library exists only where the reference tree was built (x86 here); elsewhere these
tests skip.  What glm itself would compute is not pinned (the submodule is absent): the minimal glm
is the project's own, written from the mathematics."""
import json

import numpy as np
import pytest

import ataraxia_gb300 as atx
from ataraxia_gb300 import scenes
from baseline import refbuild as rb
from tests.test_camera_output import random_inputs
from tests.test_scene_io import random_scene

pytestmark = pytest.mark.skipif(rb.host_lib() is None, reason="the reference's host code was not built here")


def u32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32)).view(np.uint32)


CAMERAS = [
    ("config0", lambda: scenes.config0()),
    ("config1", lambda: scenes.config1()),
    ("config2_small", lambda: scenes.config2().with_resolution(384, 216)),
    ("odd", lambda: scenes.config1().with_resolution(97, 31)),
    ("default_1600x900", lambda: scenes.config0().with_resolution(1600, 900)),
]


@pytest.mark.parametrize("name,make", CAMERAS, ids=[c[0] for c in CAMERAS])
def test_camera_matches_reference_camera_cpp(po, name, make):
    sc = make()
    dirs, view, inv_view, proj, inv_proj = rb.ref_camera(sc.fov, sc.near, sc.far, sc.camera_position,
                                                         sc.camera_direction, sc.width, sc.height)
    cam = atx.Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction)
    ours = atx.camera_matrices(cam, sc.width, sc.height)
    for a, b in zip(ours, (view, inv_view, proj, inv_proj)):
        assert np.array_equal(u32(a).reshape(-1), u32(b))
    assert np.array_equal(u32(rb.ray_dirs(inv_view, inv_proj, sc.width, sc.height)), u32(dirs))
    v = po.make_view(inv_view, inv_proj, sc.camera_position, sc.width, sc.height)
    for mode in (po.EXACT, po.LITERAL):
        assert np.array_equal(u32(po.ray_dirs(v, mode)).reshape(-1, 3), u32(dirs))


@pytest.mark.parametrize("seed", range(3))
def test_camera_update_matches_reference_on_update(seed):
    cam = atx.Camera(position=(0.0, 2.0, 10.0), direction=(0.0, -0.2, -1.0))
    ctl = atx.CameraController(cam)
    pos = np.array(cam.position, dtype=np.float32)
    d = np.array(cam.direction, dtype=np.float32)
    lm = np.zeros(2, dtype=np.float32)
    for mouse, right, keys, dt in random_inputs(seed, n=120):
        moved = ctl.on_update(dt, mouse=mouse, right_button=right, keys=keys)
        m2, pos, d = rb.ref_camera_update(pos, d, lm, {k.lower(): True for k in keys}, right, mouse, dt)
        lm = np.array(mouse, dtype=np.float32)
        assert moved == m2
        assert np.array_equal(u32(ctl.camera.position), u32(pos))
        assert np.array_equal(u32(ctl.camera.direction), u32(d))


def _flat_graph(j: dict):
    """A scene file's node tree as the flat arrays refh_flatten takes (depth first, parents first)."""
    parents, trs, owners, spheres, ids = [], [], [], [], []

    def walk(node, parent):
        me = len(parents)
        parents.append(parent)
        t = node["transformation"]
        trs.append(list(t["position"]) + list(t["rotation"]) + list(t["scale"]))
        for s in node.get("spheres") or []:
            owners.append(me)
            spheres.append(list(s["center"]) + [s["radius"]])
            ids.append(int(s["materialIndex"]))
        for ch in node.get("children") or []:
            walk(ch, me)

    walk(j["sceneGraph"], -1)
    return (np.array(parents, np.int32), np.array(trs, np.float32).reshape(-1, 10), np.array(owners, np.int32),
            np.array(spheres, np.float32).reshape(-1, 4), np.array(ids, np.int32))


@pytest.mark.parametrize("seed", range(8))
def test_flatten_matches_reference_traverse_scene_graph(seed):
    j = random_scene(seed, unit_quat=seed % 3 != 0)
    n_mat = len(j["materials"])
    got = atx.SceneGraph.from_json(json.dumps(j)).flatten()
    ref = rb.ref_flatten(*_flat_graph(j))
    assert len(got) == len(ref)
    ours = np.array([list(s["center"]) + [s["radius"]] for s in got], dtype=np.float32).reshape(-1, 4)
    assert np.array_equal(u32(ours), u32(ref[:, :4]))
    # Renderer::allocateDeviceMemory (Renderer.cu:30-37) sends ids outside the table to 0
    ids = ref[:, 4].astype(np.int64)
    ids[(ids < 0) | (ids >= n_mat)] = 0
    assert np.array_equal(got["material"].astype(np.int64), ids)
