"""GB300 path tracer: a drop-in for the render call of 1neskk/Ataraxia.

Python mirror of the reference's Renderer / Scene / Camera interface
(Engine/include/Renderer.h, Scene.h, Camera.h) over the C ABI in
include/atx.h.  The reference's method names are kept as aliases
(onResize, Render, getSettings, setSettings, resetFrameIndex, getImage).
All rendering runs in libatx.so on the GPU; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _native as N
from ._native import AtxError, LIGHT_DTYPE, MATERIAL_DTYPE, SPHERE_DTYPE
from .scene_graph import ROOT, SceneGraph

__all__ = [
    "AtxError", "Batch", "Camera", "Light", "Material", "Renderer", "Scene", "Server", "Settings", "Sphere",
    "SPHERE_DTYPE", "MATERIAL_DTYPE", "LIGHT_DTYPE", "camera_matrices", "device_count",
    "SceneGraph", "ROOT", "import_scene", "export_scene", "scene_from_json", "scene_to_json",
    "importScene", "exportScene", "serializeScene", "deserializeScene",
    "CameraController", "write_image", "write_pfm",
]


@dataclass
class Sphere:
    """SceneNode.h:11-21."""
    center: Sequence[float] = (0.0, 0.0, 0.0)
    radius: float = 1.0
    id: int = 0


@dataclass
class Material:
    """Scene.h:28-47 (constructor argument order of Scene.h:44)."""
    albedo: Sequence[float] = (1.0, 1.0, 1.0)
    roughness: float = 0.0
    metallic: float = 0.0
    emissionColor: Sequence[float] = (0.0, 0.0, 0.0)
    emissionIntensity: float = 0.0
    id: int = 0
    F0: Sequence[float] = (0.04, 0.04, 0.04)


@dataclass
class Light:
    """Scene.h:17-26."""
    position: Sequence[float] = (0.0, 0.0, 0.0)
    color: Sequence[float] = (1.0, 1.0, 1.0)
    intensity: float = 1.0


@dataclass
class Settings:
    """Scene.h:49-56."""
    accumulation: bool = True
    skyLight: bool = False
    maxBounces: int = 15


@dataclass
class Camera:
    """Camera.h / Camera.cpp:14-21 defaults: fov 45, near 0.1, far 100, at (0, 0, 3) looking -Z."""
    fov: float = 45.0
    nearClip: float = 0.1
    farClip: float = 100.0
    position: Sequence[float] = (0.0, 0.0, 3.0)
    direction: Sequence[float] = (0.0, 0.0, -1.0)

    def desc(self) -> N.CameraDesc:
        d = N.CameraDesc()
        d.position[:] = [float(x) for x in self.position]
        d.direction[:] = [float(x) for x in self.direction]
        d.fov_deg, d.near_clip, d.far_clip = float(self.fov), float(self.nearClip), float(self.farClip)
        return d


@dataclass
class Scene:
    """Scene.h:58-75.  spheres/materials/lights may be lists of the dataclasses above or structured
    numpy arrays with SPHERE_DTYPE / MATERIAL_DTYPE / LIGHT_DTYPE.  With a scene graph (import_scene,
    or a SceneGraph built node by node) the spheres are the graph's, flattened as Renderer.cu:67-96
    does; otherwise `spheres` is already the world-space list."""
    spheres: object = field(default_factory=list)
    materials: object = field(default_factory=list)
    lights: object = field(default_factory=list)
    settings: Settings = field(default_factory=Settings)
    camera: Camera = field(default_factory=Camera)
    graph: SceneGraph | None = None

    def arrays(self):
        s = self.graph.flatten() if self.graph is not None else _as_spheres(self.spheres)
        return s, _as_materials(self.materials), _as_lights(self.lights)


def import_scene(path) -> Scene:
    """Utils::importScene (Utils.cpp:175-187): the scene file's graph, materials, lights, camera and
    settings.  A missing file raises AtxError (ATX_ERR_NOT_FOUND); the reference returns an empty Scene."""
    g = SceneGraph.load(path)
    return _scene_from_graph(g)


def _scene_from_graph(g: SceneGraph) -> Scene:
    i = g.info()
    c, st = i["camera"], i["settings"]
    return Scene(spheres=g.flatten(), materials=g.materials(), lights=g.lights(),
                 settings=Settings(st["accumulation"], st["skyLight"], st["maxBounces"]),
                 camera=Camera(c["fov"], c["near"], c["far"], c["position"], c["direction"]), graph=g)


def scene_from_json(text) -> Scene:
    """Utils::deserializeScene (Utils.cpp:97-137)."""
    return _scene_from_graph(SceneGraph.from_json(text))


def _graph_for(scene: Scene) -> SceneGraph:
    g = scene.graph
    if g is None:                       # a flat scene: every sphere on the root node
        g = SceneGraph()
        g.add_spheres(ROOT, _as_spheres(scene.spheres))
    g.set_materials(_as_materials(scene.materials))
    g.set_lights(_as_lights(scene.lights))
    g.set_camera(scene.camera.desc())
    st = scene.settings
    g.set_settings(N.Settings(int(bool(st.accumulation)), int(bool(st.skyLight)), (0, 0), int(st.maxBounces)))
    return g


def scene_to_json(scene: Scene) -> str:
    """Utils::serializeScene + dump(4) (Utils.cpp:3-51)."""
    return _graph_for(scene).to_json()


def export_scene(scene: Scene, path):
    """Utils::exportScene (Utils.cpp:53-62)."""
    _graph_for(scene).save(path)


importScene = import_scene
exportScene = export_scene
serializeScene = scene_to_json
deserializeScene = scene_from_json


def _as_spheres(x) -> np.ndarray:
    if isinstance(x, np.ndarray):
        return np.ascontiguousarray(x, dtype=SPHERE_DTYPE)
    a = np.zeros(len(x), dtype=SPHERE_DTYPE)
    for i, s in enumerate(x):
        a[i] = (tuple(s.center), s.radius, s.id)
    return a


def _as_materials(x) -> np.ndarray:
    if isinstance(x, np.ndarray):
        return np.ascontiguousarray(x, dtype=MATERIAL_DTYPE)
    a = np.zeros(len(x), dtype=MATERIAL_DTYPE)
    for i, m in enumerate(x):
        a[i] = (tuple(m.albedo), m.roughness, m.metallic, tuple(m.F0), tuple(m.emissionColor),
                m.emissionIntensity, m.id)
    return a


def _as_lights(x) -> np.ndarray:
    if isinstance(x, np.ndarray):
        return np.ascontiguousarray(x, dtype=LIGHT_DTYPE)
    a = np.zeros(len(x), dtype=LIGHT_DTYPE)
    for i, l in enumerate(x):
        a[i] = (tuple(l.position), tuple(l.color), l.intensity)
    return a


class CameraController:
    """Camera::onUpdate (Camera.cpp:31-108) with the window input passed in: keeps the camera and the
    previous cursor position (Camera::m_lastMousePos).  keys is a string of the held keys among
    "WSADQE"; nothing moves unless the right mouse button is held."""

    def __init__(self, camera: Camera | None = None, last_mouse=(0.0, 0.0)):
        self.camera = camera or Camera()
        self.last_mouse = (C.c_float * 2)(*[float(v) for v in last_mouse])

    @staticmethod
    def _input(mouse, right_button: bool, keys: str) -> N.CameraInput:
        k = keys.upper()
        return N.CameraInput((C.c_float * 2)(*[float(v) for v in mouse]), int(bool(right_button)),
                             int("W" in k), int("S" in k), int("A" in k), int("D" in k), int("Q" in k),
                             int("E" in k), 0)

    def _apply(self, fn, *head, dt, mouse, right_button, keys) -> bool:
        d = self.camera.desc()
        inp = self._input(mouse, right_button, keys)
        moved = C.c_int32(0)
        N.check(fn(*head, C.byref(d), self.last_mouse, C.byref(inp), float(dt), C.byref(moved)))
        self.camera = Camera(d.fov_deg, d.near_clip, d.far_clip, tuple(d.position), tuple(d.direction))
        return bool(moved.value)

    def on_update(self, dt: float, mouse=(0.0, 0.0), right_button: bool = False, keys: str = "") -> bool:
        return self._apply(N.lib().atx_camera_on_update, dt=dt, mouse=mouse, right_button=right_button, keys=keys)

    onUpdate = on_update


def write_image(path, rgba8: np.ndarray, fmt: str | None = None):
    """RGBA8 pixels (H, W) uint32 to a PPM (RGB) or PAM (RGBA) file, top row first (atx_write_rgba8)."""
    a = np.ascontiguousarray(rgba8, dtype=np.uint32)
    h, w = a.shape
    f = _image_format(path, fmt)
    if f == N.IMAGE_PFM:
        raise ValueError("PFM files are written from the float accumulator (write_pfm)")
    N.check(N.lib().atx_write_rgba8(os.fsencode(path), N.ptr(a), w, h, f))


def write_pfm(path, accum: np.ndarray):
    """Float4 accumulator (H, W, 4) to a PFM file of accumulated colour / frames (atx_write_pfm)."""
    a = np.ascontiguousarray(accum, dtype=np.float32)
    h, w = a.shape[:2]
    N.check(N.lib().atx_write_pfm(os.fsencode(path), N.ptr(a), w, h))


def _image_format(path, fmt) -> int:
    ext = (fmt or os.path.splitext(os.fspath(path))[1].lstrip(".")).lower()
    table = {"ppm": N.IMAGE_PPM, "pam": N.IMAGE_PAM, "pfm": N.IMAGE_PFM}
    if ext not in table:
        raise ValueError(f"unknown image format {ext!r} (ppm, pam, pfm)")
    return table[ext]


def device_count() -> int:
    n = C.c_int32(0)
    N.check(N.lib().atx_device_count(C.byref(n)))
    return n.value


def camera_matrices(camera: Camera, width: int, height: int):
    """Camera.cpp:134-159 on the host: (view, inv_view, proj, inv_proj) as 4x4 column-major float32
    arrays (element [c, r] = column c, row r, as glm stores them).  Needs no GPU."""
    out = [np.zeros(16, dtype=np.float32) for _ in range(4)]
    d = camera.desc()
    N.check(N.lib().atx_camera_matrices(C.byref(d), width, height, *[N.ptr(o) for o in out]))
    return tuple(o.reshape(4, 4) for o in out)


class Renderer:
    """Renderer.h:19-86 over libatx.so.

    Render(camera, scene, spp) follows Renderer.cu:173-249: the scene is uploaded when a different
    Scene object is passed or the frame index is 1, spp consecutive frames are traced, and the frame
    index advances (accumulation on) or stays 1 (off)."""

    def __init__(self, device: int = 0, wave_paths: int = 0, threads: int = 0, bvh_threshold: int = 0,
                 bvh_leaf_size: int = 0, hbm_budget_bytes: int = 0, flags: int = 0):
        cfg = N.Config(device, wave_paths, threads, bvh_threshold, bvh_leaf_size, flags, hbm_budget_bytes)
        h = C.c_void_p()
        N.check(N.lib().atx_renderer_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._scene_id = None
        self.width = 0
        self.height = 0

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            N.lib().atx_renderer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- reference interface
    def on_resize(self, width: int, height: int):
        N.check(N.lib().atx_resize(self._h, width, height))
        self.width, self.height = width, height

    onResize = on_resize

    def get_settings(self) -> Settings:
        s = N.Settings()
        N.check(N.lib().atx_get_settings(self._h, C.byref(s)))
        return Settings(bool(s.accumulation), bool(s.sky_light), int(s.max_bounces))

    getSettings = get_settings

    def set_settings(self, settings: Settings):
        s = N.Settings(int(bool(settings.accumulation)), int(bool(settings.skyLight)), (C.c_uint8 * 2)(),
                       int(settings.maxBounces))
        N.check(N.lib().atx_set_settings(self._h, C.byref(s)))

    setSettings = set_settings

    def reset_frame_index(self):
        N.check(N.lib().atx_reset_frame_index(self._h))

    resetFrameIndex = reset_frame_index

    @property
    def frame_index(self) -> int:
        f = C.c_uint32()
        N.check(N.lib().atx_get_frame_index(self._h, C.byref(f)))
        return f.value

    def render(self, camera: Camera, scene: Scene, spp: int = 1):
        if self._scene_id != id(scene) or self.frame_index == 1:
            self.set_scene(*scene.arrays())
            self._scene_id = id(scene)
        self.set_camera(camera)
        self.render_frames(spp)

    Render = render

    def get_image(self, out: np.ndarray | None = None) -> np.ndarray:
        """RGBA8 image as (H, W) uint32, A<<24 | B<<16 | G<<8 | R (Renderer.h:70-78); out, if given, is a
        contiguous uint32 buffer of W*H pixels to read into."""
        if out is None:
            out = np.empty(self.width * self.height, dtype=np.uint32)
        if out.dtype != np.uint32 or not out.flags.c_contiguous or out.size != self.width * self.height:
            raise ValueError("get_image: out must be a contiguous uint32 array of width*height pixels")
        N.check(N.lib().atx_read_image(self._h, N.ptr(out), out.size))
        return out.reshape(self.height, self.width)

    getImage = get_image

    # -- explicit API
    def set_scene(self, spheres: np.ndarray, materials: np.ndarray, lights: np.ndarray):
        s, m, l = _as_spheres(spheres), _as_materials(materials), _as_lights(lights)
        N.check(N.lib().atx_set_scene(self._h, N.ptr(s) if len(s) else None, len(s), N.ptr(m) if len(m) else None,
                                      len(m), N.ptr(l) if len(l) else None, len(l)))

    def update_camera(self, controller: CameraController, dt: float, mouse=(0.0, 0.0), right_button: bool = False,
                      keys: str = "") -> bool:
        """Ataraxia::onUpdate (main.cpp:22-32): Camera::onUpdate, and when it moved, the new camera
        with the frame index reset to 1 (atx_update_camera)."""
        return controller._apply(N.lib().atx_update_camera, self._h, dt=dt, mouse=mouse,
                                 right_button=right_button, keys=keys)

    def save_image(self, path, fmt: str | None = None):
        """The image (.ppm, .pam) or the accumulator (.pfm) written to a file (atx_save_image)."""
        N.check(N.lib().atx_save_image(self._h, os.fsencode(path), _image_format(path, fmt)))

    def set_scene_graph(self, graph: SceneGraph):
        """Flattens the graph (Renderer.cu:67-96) and uploads it (atx_set_scene_graph)."""
        N.check(N.lib().atx_set_scene_graph(self._h, graph.handle))

    def set_camera(self, camera: Camera):
        d = camera.desc()
        N.check(N.lib().atx_set_camera(self._h, C.byref(d)))

    def set_camera_matrices(self, inv_view: np.ndarray, inv_proj: np.ndarray, position):
        iv = np.ascontiguousarray(inv_view, dtype=np.float32).reshape(16)
        ip = np.ascontiguousarray(inv_proj, dtype=np.float32).reshape(16)
        p = np.ascontiguousarray(position, dtype=np.float32).reshape(3)
        N.check(N.lib().atx_set_camera_matrices(self._h, N.ptr(iv), N.ptr(ip), N.ptr(p)))

    def render_frames(self, spp: int = 1):
        N.check(N.lib().atx_render(self._h, spp))

    def read_image_async(self, out: np.ndarray) -> int:
        """Starts reading the last render's RGBA8 image into out (contiguous uint32, W*H; best page-locked)
        and returns a ticket for wait_read (atx_read_image_async); out must not be used before."""
        if out.dtype != np.uint32 or not out.flags.c_contiguous or out.size != self.width * self.height:
            raise ValueError("read_image_async: out must be a contiguous uint32 array of width*height pixels")
        t = C.c_uint64()
        N.check(N.lib().atx_read_image_async(self._h, N.ptr(out), out.size, C.byref(t)))
        return t.value

    def wait_read(self, ticket: int):
        N.check(N.lib().atx_wait_read(self._h, ticket))

    def join(self):
        """Orders the renderer's stream after every render so far (atx_join; with
        FLAG_OVERLAP_RENDERS renders are not joined into it until then)."""
        N.check(N.lib().atx_join(self._h))

    def synchronize(self):
        N.check(N.lib().atx_synchronize(self._h))

    def get_accumulation(self, out: np.ndarray | None = None) -> np.ndarray:
        """Float4 accumulator as (H, W, 4) float32."""
        if out is None:
            out = np.empty((self.height, self.width, 4), dtype=np.float32)
        N.check(N.lib().atx_read_accumulation(self._h, N.ptr(out), self.width * self.height))
        return out

    def stats(self) -> dict:
        s = N.Stats()
        N.check(N.lib().atx_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in N.Stats._fields_ if k != "reserved"}

    def kernel_times(self) -> dict:
        t = N.KernelTimes()
        N.check(N.lib().atx_get_kernel_times(self._h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in N.KernelTimes._fields_}

    def autotune(self, spp: int, passes: int = 2, use_cache: bool = True) -> dict:
        """Times launch settings (LBVH leaf size, lanes, path state, block size, wave shape) on the current
        scene, camera and viewport and keeps the fastest (atx_autotune); every setting renders the same
        frames bit for bit.  The renderer is left at frame 1."""
        t = N.Tuning()
        N.check(N.lib().atx_autotune(self._h, spp, passes, int(bool(use_cache)), C.byref(t)))
        return {k: getattr(t, k) for k, _ in N.Tuning._fields_}

    def tuning(self) -> dict:
        t = N.Tuning()
        N.check(N.lib().atx_get_tuning(self._h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in N.Tuning._fields_}

    def set_tuning(self, bvh_leaf_size=0, lanes=0, wave_paths=0, threads=0, wave_spp=0, path_kernel=0, cell_res=0):
        t = N.Tuning(bvh_leaf_size, lanes, wave_paths, threads, wave_spp, path_kernel, 0, cell_res, 0.0)
        N.check(N.lib().atx_set_tuning(self._h, C.byref(t)))

    def reset_kernel_times(self):
        N.check(N.lib().atx_reset_kernel_times(self._h))

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        N.check(N.lib().atx_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def trace_nearest(self, origins: np.ndarray, dirs: np.ndarray):
        o = np.ascontiguousarray(origins, dtype=np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(dirs, dtype=np.float32).reshape(-1, 3)
        n = len(o)
        t = np.empty(n, dtype=np.float32)
        ids = np.empty(n, dtype=np.int32)
        N.check(N.lib().atx_trace_nearest(self._h, N.ptr(o), N.ptr(d), n, N.ptr(t), N.ptr(ids)))
        return t, ids

    def primary_directions(self) -> np.ndarray:
        out = np.empty((self.height * self.width, 3), dtype=np.float32)
        N.check(N.lib().atx_primary_directions(self._h, N.ptr(out), self.width * self.height))
        return out

    def device_buffers(self):
        a, i = C.c_void_p(), C.c_void_p()
        N.check(N.lib().atx_device_buffers(self._h, C.byref(a), C.byref(i)))
        return a.value, i.value


class Batch:
    """Many resident scenes rendered together (atx_batch_*): each pass runs every scene with pending
    frames through the wavefront kernels on concurrent lanes, captured as one CUDA graph.

    add_scene(...) -> id; set_spp(id, spp); run() renders one pass for every scene with spp > 0.
    Each scene keeps the reference's per-scene frame semantics, so its results are bit-identical to
    rendering it alone with Renderer."""

    def __init__(self, device: int = 0, bvh_threshold: int = 0, bvh_leaf_size: int = 0, hbm_budget_bytes: int = 0,
                 flags: int = 0, lane_wave_paths: int = 0):
        cfg = N.Config(device, lane_wave_paths, 0, bvh_threshold, bvh_leaf_size, flags, hbm_budget_bytes)
        h = C.c_void_p()
        N.check(N.lib().atx_batch_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._sizes = {}
        self._keep = {}

    def close(self):
        if getattr(self, "_h", None):
            N.lib().atx_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_scene(self, spheres, materials, lights, camera: Camera, width: int, height: int,
                  settings: Settings = None) -> int:
        settings = settings or Settings()
        s, m, l = _as_spheres(spheres), _as_materials(materials), _as_lights(lights)
        d = N.BatchScene(N.ptr(s) if len(s) else None, len(s), N.ptr(m) if len(m) else None, len(m),
                         N.ptr(l) if len(l) else None, len(l), camera.desc(), width, height,
                         N.Settings(int(bool(settings.accumulation)), int(bool(settings.skyLight)),
                                    (C.c_uint8 * 2)(), int(settings.maxBounces)))
        i = C.c_uint32()
        N.check(N.lib().atx_batch_add_scene(self._h, C.byref(d), C.byref(i)))
        self._sizes[i.value] = (width, height)
        return i.value

    def add_synthetic(self, sc, settings: Settings = None) -> int:
        """Adds a scenes.SyntheticScene with its own camera and bounce depth."""
        cam = Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction)
        st = settings or Settings(accumulation=True, skyLight=sc.sky_light, maxBounces=sc.max_bounces)
        return self.add_scene(sc.spheres, sc.materials, sc.lights, cam, sc.width, sc.height, st)

    def remove_scene(self, i: int):
        N.check(N.lib().atx_batch_remove_scene(self._h, i))
        self._sizes.pop(i, None)

    def set_spp(self, i: int, spp: int):
        N.check(N.lib().atx_batch_set_spp(self._h, i, spp))

    def reset(self, i: int):
        N.check(N.lib().atx_batch_reset(self._h, i))

    def frame_index(self, i: int) -> int:
        f = C.c_uint32()
        N.check(N.lib().atx_batch_frame_index(self._h, i, C.byref(f)))
        return f.value

    def set_camera(self, i: int, camera: Camera):
        """New camera for scene i; its accumulation restarts (atx_batch_set_camera)."""
        d = camera.desc()
        N.check(N.lib().atx_batch_set_camera(self._h, i, C.byref(d)))

    def run(self):
        N.check(N.lib().atx_batch_run(self._h))

    def synchronize(self):
        N.check(N.lib().atx_batch_synchronize(self._h))

    def get_accumulation(self, i: int) -> np.ndarray:
        w, h = self._sizes[i]
        out = np.empty((h * w, 4), dtype=np.float32)
        N.check(N.lib().atx_batch_read_accumulation(self._h, i, N.ptr(out), w * h))
        return out

    def get_image(self, i: int) -> np.ndarray:
        w, h = self._sizes[i]
        out = np.empty(h * w, dtype=np.uint32)
        N.check(N.lib().atx_batch_read_image(self._h, i, N.ptr(out), w * h))
        return out

    def stats(self) -> dict:
        s = N.BatchStats()
        N.check(N.lib().atx_batch_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in N.BatchStats._fields_}

    def set_tuning(self, lanes=0, lane_wave_paths=0, threads=0, bvh_threshold=0, bvh_leaf_size=0,
                   primary_cache=None):
        pc = 0 if primary_cache is None else (1 if primary_cache else 2)
        t = N.BatchTuning(lanes, lane_wave_paths, threads, bvh_threshold, bvh_leaf_size, pc, (C.c_uint32 * 2)())
        N.check(N.lib().atx_batch_set_tuning(self._h, C.byref(t)))

    def autotune(self, passes: int = 2) -> dict:
        """Times lane / path-state settings on the current scenes (all at frame 1) and keeps the fastest
        (atx_batch_autotune); the scenes are back at frame 1 afterwards."""
        t = N.BatchTuning()
        N.check(N.lib().atx_batch_autotune(self._h, passes, C.byref(t)))
        return {k: getattr(t, k) for k, _ in N.BatchTuning._fields_ if k != "reserved"}

    def tuning(self) -> dict:
        t = N.BatchTuning()
        N.check(N.lib().atx_batch_get_tuning(self._h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in N.BatchTuning._fields_ if k != "reserved"}


def _batch_scene(spheres, materials, lights, camera: Camera, width: int, height: int, settings: Settings):
    s, m, l = _as_spheres(spheres), _as_materials(materials), _as_lights(lights)
    d = N.BatchScene(N.ptr(s) if len(s) else None, len(s), N.ptr(m) if len(m) else None, len(m),
                     N.ptr(l) if len(l) else None, len(l), camera.desc(), width, height,
                     N.Settings(int(bool(settings.accumulation)), int(bool(settings.skyLight)), (C.c_uint8 * 2)(),
                                int(settings.maxBounces)))
    return d, (s, m, l)


class Server:
    """Progressive render server with continuous batching (atx_server_*).

    submit() copies the scene and returns a job id at once; a worker thread admits jobs (policy "arrival":
    in arrival order; "smallest": fewest pixel-samples first) when a slot and their device memory fit the
    HBM budget and renders all active jobs together, a slice of frames per pass, until each reaches its
    target spp.  Passes are pipelined: the next one is queued while the current one runs."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, max_active_jobs: int = 0, pass_spp: int = 0,
                 max_pass_paths: int = 0, max_pending: int = 0, bvh_threshold: int = 0, flags: int = 0,
                 host_executor: bool = False, host_fail_pass: int = 0, policy: str = "arrival"):
        if host_executor:
            flags |= N.FLAG_HOST_EXECUTOR
        pol = {"arrival": N.ADMIT_ARRIVAL, "smallest": N.ADMIT_SMALLEST}[policy]
        cfg = N.ServerConfig(N.Config(device, 0, 0, bvh_threshold, 0, flags, hbm_budget_bytes), max_active_jobs,
                             pass_spp, max_pass_paths, max_pending, host_fail_pass, pol)
        h = C.c_void_p()
        N.check(N.lib().atx_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._sizes = {}

    def close(self):
        if getattr(self, "_h", None):
            N.lib().atx_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit_scene(self, spheres, materials, lights, camera: Camera, width: int, height: int,
                     settings: Settings, target_spp: int) -> int:
        d, keep = _batch_scene(spheres, materials, lights, camera, width, height, settings)
        j = C.c_uint32()
        N.check(N.lib().atx_server_submit(self._h, C.byref(d), target_spp, C.byref(j)))
        del keep
        self._sizes[j.value] = (width, height)
        return j.value

    def submit(self, sc, target_spp: int) -> int:
        """Submits a scenes.SyntheticScene with its own camera and bounce depth."""
        cam = Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction)
        st = Settings(accumulation=True, skyLight=sc.sky_light, maxBounces=sc.max_bounces)
        return self.submit_scene(sc.spheres, sc.materials, sc.lights, cam, sc.width, sc.height, st, target_spp)

    def poll(self, job: int) -> dict:
        i = N.JobInfo()
        N.check(N.lib().atx_server_poll(self._h, job, C.byref(i)))
        d = {k: getattr(i, k) for k, _ in N.JobInfo._fields_ if k != "reserved"}
        d["state"] = N.JOB_STATES.get(d["state"], d["state"])
        return d

    def wait(self, job: int, timeout_ms: int = 60000):
        N.check(N.lib().atx_server_wait(self._h, job, timeout_ms))

    def image(self, job: int) -> np.ndarray:
        w, h = self._sizes[job]
        out = np.empty(w * h, dtype=np.uint32)
        N.check(N.lib().atx_server_read_image(self._h, job, N.ptr(out), w * h))
        return out

    def accumulation(self, job: int) -> np.ndarray:
        w, h = self._sizes[job]
        out = np.empty((w * h, 4), dtype=np.float32)
        N.check(N.lib().atx_server_read_accumulation(self._h, job, N.ptr(out), w * h))
        return out

    def cancel(self, job: int):
        N.check(N.lib().atx_server_cancel(self._h, job))

    def set_camera(self, job: int, camera: Camera):
        """New camera for a queued or active job: it restarts from frame 1 (atx_server_set_camera)."""
        d = camera.desc()
        N.check(N.lib().atx_server_set_camera(self._h, job, C.byref(d)))

    def release(self, job: int):
        N.check(N.lib().atx_server_release(self._h, job))
        self._sizes.pop(job, None)

    def stats(self) -> dict:
        s = N.ServerStats()
        N.check(N.lib().atx_server_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in N.ServerStats._fields_}

    def now(self) -> float:
        t = C.c_double()
        N.check(N.lib().atx_server_now(self._h, C.byref(t)))
        return t.value
