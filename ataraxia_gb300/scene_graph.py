"""Scene graph and scene files over libatx.so (atx_scene_*).

The reference keeps a scene as a tree of nodes with their own spheres
(Engine/include/SceneNode.h, Engine/src/SceneNode.cpp), stores it as JSON
(Engine/src/Utils.cpp) and flattens it into world-space spheres before upload
(Engine/src/Renderer.cu:25-37, 67-96).  SceneGraph wraps the library's
implementation of all three; it runs on the host and needs no GPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _native as N
from ._native import LIGHT_DTYPE, MATERIAL_DTYPE, SPHERE_DTYPE

ROOT = 0


class SceneGraph:
    """A scene tree: node 0 is the root ("Scene"), add_node() appends children."""

    def __init__(self, _handle=None):
        if _handle is None:
            _handle = C.c_void_p()
            N.check(N.lib().atx_scene_create(C.byref(_handle)))
        self._h = _handle

    # ---- construction from text / files (Utils::deserializeScene, importScene)
    @classmethod
    def from_json(cls, text: str | bytes) -> "SceneGraph":
        b = text.encode() if isinstance(text, str) else bytes(text)
        h = C.c_void_p()
        N.check(N.lib().atx_scene_parse_json(b, len(b), C.byref(h)))
        return cls(h)

    @classmethod
    def load(cls, path: str | os.PathLike) -> "SceneGraph":
        h = C.c_void_p()
        N.check(N.lib().atx_scene_load(os.fsencode(path), C.byref(h)))
        return cls(h)

    # ---- output (Utils::serializeScene, exportScene)
    def to_json(self) -> str:
        n = C.c_uint64()
        N.check(N.lib().atx_scene_to_json(self._h, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        N.check(N.lib().atx_scene_to_json(self._h, buf, n.value, C.byref(n)))
        return buf.raw[: n.value].decode()

    def save(self, path: str | os.PathLike):
        N.check(N.lib().atx_scene_save(self._h, os.fsencode(path)))

    # ---- contents
    def info(self) -> dict:
        i = N.SceneInfo()
        N.check(N.lib().atx_scene_get_info(self._h, C.byref(i)))
        c = i.camera
        return {"n_spheres": i.n_spheres, "n_materials": i.n_materials, "n_lights": i.n_lights,
                "n_nodes": i.n_nodes,
                "camera": {"position": tuple(c.position), "direction": tuple(c.direction), "fov": c.fov_deg,
                           "near": c.near_clip, "far": c.far_clip},
                "settings": {"accumulation": bool(i.settings.accumulation), "skyLight": bool(i.settings.sky_light),
                             "maxBounces": i.settings.max_bounces}}

    def flatten(self) -> np.ndarray:
        """World-space spheres (SPHERE_DTYPE) in Renderer::traverseSceneGraph order."""
        n = self.info()["n_spheres"]
        out = np.zeros(n, dtype=SPHERE_DTYPE)
        N.check(N.lib().atx_scene_flatten(self._h, N.ptr(out) if n else None, n))
        return out

    def materials(self) -> np.ndarray:
        n = self.info()["n_materials"]
        out = np.zeros(n, dtype=MATERIAL_DTYPE)
        N.check(N.lib().atx_scene_get_materials(self._h, N.ptr(out) if n else None, n))
        return out

    def lights(self) -> np.ndarray:
        n = self.info()["n_lights"]
        out = np.zeros(n, dtype=LIGHT_DTYPE)
        N.check(N.lib().atx_scene_get_lights(self._h, N.ptr(out) if n else None, n))
        return out

    # ---- editing (SceneNode::addChild, setPosition/Rotation/Scale, addSphere)
    def add_node(self, parent: int = ROOT, name: str = "Untitled") -> int:
        k = C.c_uint32()
        N.check(N.lib().atx_scene_add_node(self._h, parent, name.encode(), C.byref(k)))
        return k.value

    def set_transform(self, node: int, position=None, rotation_xyzw=None, scale=None):
        def f(v, n):
            return None if v is None else (C.c_float * n)(*[float(x) for x in v])
        N.check(N.lib().atx_scene_set_transform(self._h, node, f(position, 3), f(rotation_xyzw, 4), f(scale, 3)))

    def add_spheres(self, node: int, spheres: np.ndarray):
        s = np.ascontiguousarray(spheres, dtype=SPHERE_DTYPE)
        N.check(N.lib().atx_scene_add_spheres(self._h, node, N.ptr(s) if len(s) else None, len(s)))

    def set_materials(self, materials: np.ndarray):
        m = np.ascontiguousarray(materials, dtype=MATERIAL_DTYPE)
        N.check(N.lib().atx_scene_set_materials(self._h, N.ptr(m) if len(m) else None, len(m)))

    def set_lights(self, lights: np.ndarray):
        a = np.ascontiguousarray(lights, dtype=LIGHT_DTYPE)
        N.check(N.lib().atx_scene_set_lights(self._h, N.ptr(a) if len(a) else None, len(a)))

    def set_camera(self, desc: N.CameraDesc):
        N.check(N.lib().atx_scene_set_camera(self._h, C.byref(desc)))

    def set_settings(self, s: N.Settings):
        N.check(N.lib().atx_scene_set_settings(self._h, C.byref(s)))

    # ---- lifetime
    def close(self):
        if getattr(self, "_h", None):
            N.lib().atx_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h
