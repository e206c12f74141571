"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, never by the product.  Pinned to the
reference's own kernel built from its sources (oracle.h says how).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
# Same source built with multiply-add contraction allowed (see oracle/Makefile).
CONTRACT_LIB_PATH = HERE / "_build" / "liboracle_contract.so"

EXACT = 0
LITERAL = 1

SPHERE_DTYPE = np.dtype([("center", "<f4", (3,)), ("radius", "<f4"), ("material", "<i4")])
MATERIAL_DTYPE = np.dtype([
    ("albedo", "<f4", (3,)), ("roughness", "<f4"), ("metallic", "<f4"), ("f0", "<f4", (3,)),
    ("emission_color", "<f4", (3,)), ("emission_intensity", "<f4"), ("id", "<i4"),
])
LIGHT_DTYPE = np.dtype([("position", "<f4", (3,)), ("color", "<f4", (3,)), ("intensity", "<f4")])


class OrcScene(C.Structure):
    _fields_ = [("spheres", C.c_void_p), ("n_spheres", C.c_int32), ("materials", C.c_void_p),
                ("n_materials", C.c_int32), ("lights", C.c_void_p), ("n_lights", C.c_int32)]


class OrcView(C.Structure):
    _fields_ = [("inv_view", C.c_float * 16), ("inv_proj", C.c_float * 16), ("position", C.c_float * 3),
                ("width", C.c_uint32), ("height", C.c_uint32)]


class OrcJob(C.Structure):
    _fields_ = [("max_bounces", C.c_int32), ("sky_light", C.c_int32), ("frame0", C.c_uint32),
                ("spp", C.c_uint32), ("pixels", C.c_void_p), ("n_pixels", C.c_uint64), ("threads", C.c_int32)]


class OrcStats(C.Structure):
    _fields_ = [("ext_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("shaded_hits", C.c_uint64),
                ("sphere_tests", C.c_uint64)]


_libs: dict = {}


def build() -> Path:
    """Compiles the oracle with oracle/Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib(contract: bool = False):
    path = CONTRACT_LIB_PATH if contract else LIB_PATH
    if path not in _libs:
        if not path.exists():
            build()
        h = C.CDLL(str(path))
        P = C.c_void_p
        h.orc_render_f32.argtypes = [C.c_int, C.POINTER(OrcScene), C.POINTER(OrcView), C.POINTER(OrcJob), P, P,
                                     C.POINTER(OrcStats)]
        h.orc_render_f64.argtypes = [C.POINTER(OrcScene), C.POINTER(OrcView), C.POINTER(OrcJob), P, P,
                                     C.POINTER(OrcStats)]
        h.orc_trace.argtypes = [C.c_int, P, C.c_int32, P, P, C.c_uint64, P, P]
        h.orc_trace.restype = None
        h.orc_camera_matrices.argtypes = [P, P, C.c_float, C.c_float, C.c_float, C.c_uint32, C.c_uint32, P, P, P, P]
        h.orc_camera_matrices.restype = None
        h.orc_mat4_inverse.argtypes = [P, P]
        h.orc_mat4_inverse.restype = None
        h.orc_ray_dirs.argtypes = [C.c_int, C.POINTER(OrcView), P]
        h.orc_ray_dirs.restype = None
        h.orc_pcg_hash.argtypes = [C.c_uint32]
        h.orc_pcg_hash.restype = C.c_uint32
        h.orc_pcg_float.argtypes = [C.POINTER(C.c_uint32)]
        h.orc_pcg_float.restype = C.c_float
        h.orc_sincos2pi.argtypes = [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        h.orc_sincos2pi.restype = None
        h.orc_cook_torrance.argtypes = [C.c_int, P, P, C.c_float, C.c_float, P, P, P, P]
        h.orc_cook_torrance.restype = None
        h.orc_sample_cosine.argtypes = [C.c_int, P, C.POINTER(C.c_uint32), P]
        h.orc_sample_cosine.restype = None
        h.orc_sample_ggx.argtypes = [C.c_int, P, C.c_float, C.POINTER(C.c_uint32), P]
        h.orc_sample_ggx.restype = None
        h.orc_pack_rgba8.argtypes = [P, C.c_uint64, C.c_uint32, P]
        h.orc_pack_rgba8.restype = None
        h.orc_max_threads.restype = C.c_int
        h.orc_camera_on_update.argtypes = [P, P, P, P, C.c_int, P, C.c_float]
        h.orc_camera_on_update.restype = C.c_int
        h.orc_decision_hash.argtypes = [C.c_int, C.POINTER(OrcScene), C.POINTER(OrcView), C.POINTER(OrcJob), P]
        h.orc_decision_events.argtypes = [C.c_int, C.POINTER(OrcScene), C.POINTER(OrcView), C.POINTER(OrcJob), P,
                                          C.c_int32]
        _libs[path] = h
    return _libs[path]


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def f32vec(x) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.float32)


def camera_matrices(position, direction, fov=45.0, near=0.1, far=100.0, width=1280, height=720):
    """(view, inv_view, proj, inv_proj), each a flat column-major float32[16]."""
    out = [np.zeros(16, dtype=np.float32) for _ in range(4)]
    pos, dirv = f32vec(position), f32vec(direction)      # keep the arrays alive across the call
    lib().orc_camera_matrices(_p(pos), _p(dirv), fov, near, far, width, height, *[_p(o) for o in out])
    return tuple(out)


def make_view(inv_view, inv_proj, position, width, height) -> OrcView:
    v = OrcView()
    v.inv_view[:] = [float(x) for x in np.asarray(inv_view, dtype=np.float32).reshape(16)]
    v.inv_proj[:] = [float(x) for x in np.asarray(inv_proj, dtype=np.float32).reshape(16)]
    v.position[:] = [float(x) for x in np.asarray(position, dtype=np.float32).reshape(3)]
    v.width, v.height = width, height
    return v


def view_for(scene) -> OrcView:
    """View of a SyntheticScene computed by the oracle's own camera code."""
    _, iv, _, ip = camera_matrices(scene.camera_position, scene.camera_direction, scene.fov, scene.near,
                                   scene.far, scene.width, scene.height)
    return make_view(iv, ip, scene.camera_position, scene.width, scene.height)


def _scene(spheres, materials, lights):
    s = np.ascontiguousarray(spheres, dtype=SPHERE_DTYPE)
    m = np.ascontiguousarray(materials, dtype=MATERIAL_DTYPE)
    l = np.ascontiguousarray(lights, dtype=LIGHT_DTYPE)
    sc = OrcScene(_p(s) if len(s) else None, len(s), _p(m) if len(m) else None, len(m),
                  _p(l) if len(l) else None, len(l))
    return sc, (s, m, l)


def render(spheres, materials, lights, view: OrcView, *, max_bounces=5, sky=False, frame0=1, spp=1,
           pixels=None, mode=EXACT, threads=0, accum=None, samples=False, f64=False, contract=False):
    """Runs the oracle.  Returns (accum [n,4], samples [n,spp,4] or None, stats dict).
    accum (if given) is the starting accumulator, updated in frame order.  contract=True runs the
    build with multiply-add contraction allowed (meaningful for mode=LITERAL)."""
    sc, keep = _scene(spheres, materials, lights)
    px = None if pixels is None else np.ascontiguousarray(pixels, dtype=np.uint32)
    n = (view.width * view.height) if px is None else len(px)
    dt = np.float64 if f64 else np.float32
    acc = np.zeros((n, 4), dtype=dt) if accum is None else np.ascontiguousarray(accum, dtype=dt).reshape(n, 4).copy()
    smp = np.zeros((n, spp, 4), dtype=dt) if samples else None
    job = OrcJob(max_bounces, int(bool(sky)), frame0, spp, _p(px), 0 if px is None else len(px), threads)
    st = OrcStats()
    h = lib(contract)
    if f64:
        rc = h.orc_render_f64(C.byref(sc), C.byref(view), C.byref(job), _p(acc), _p(smp), C.byref(st))
    else:
        rc = h.orc_render_f32(mode, C.byref(sc), C.byref(view), C.byref(job), _p(acc), _p(smp), C.byref(st))
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    del keep
    return acc, smp, {k: getattr(st, k) for k, _ in OrcStats._fields_}


F64 = 2
EV_HIT, EV_SHADOW, EV_ROULETTE, EV_FRAME = 1, 2, 3, 4


def decision_hash(spheres, materials, lights, view: OrcView, *, max_bounces=5, sky=False, frame0=1, spp=1,
                  pixels=None, variant=EXACT, contract=False, threads=0) -> np.ndarray:
    """Per pixel, a 64-bit hash of the branch decisions of its frames (oracle.h, orc_decision_hash).
    variant EXACT, LITERAL or F64; contract=True runs the literal expressions with contraction."""
    sc, keep = _scene(spheres, materials, lights)
    px = None if pixels is None else np.ascontiguousarray(pixels, dtype=np.uint32)
    n = (view.width * view.height) if px is None else len(px)
    out = np.zeros(n, dtype=np.uint64)
    job = OrcJob(max_bounces, int(bool(sky)), frame0, spp, _p(px), 0 if px is None else len(px), threads)
    if lib(contract).orc_decision_hash(variant, C.byref(sc), C.byref(view), C.byref(job), _p(out)) != 0:
        raise ValueError("oracle rejected the arguments")
    del keep
    return out


def decision_events(spheres, materials, lights, view: OrcView, pixels, *, max_bounces=5, sky=False, frame0=1,
                    spp=1, variant=EXACT, contract=False, threads=0) -> np.ndarray:
    """Branch-decision events [pixel, frame, event] of the listed pixels (oracle.h, orc_decision_events)."""
    sc, keep = _scene(spheres, materials, lights)
    px = np.ascontiguousarray(pixels, dtype=np.uint32)
    cap = 4 * max(int(max_bounces), 1) + 4
    out = np.zeros((len(px), spp, cap), dtype=np.uint32)
    job = OrcJob(max_bounces, int(bool(sky)), frame0, spp, _p(px), len(px), threads)
    if len(px) and lib(contract).orc_decision_events(variant, C.byref(sc), C.byref(view), C.byref(job), _p(out),
                                                     cap) != 0:
        raise ValueError("oracle rejected the arguments")
    del keep
    return out


def trace(spheres, origins, dirs, mode=EXACT):
    s = np.ascontiguousarray(spheres, dtype=SPHERE_DTYPE)
    o = f32vec(origins).reshape(-1, 3)
    d = f32vec(dirs).reshape(-1, 3)
    n = len(o)
    t = np.empty(n, dtype=np.float32)
    ids = np.empty(n, dtype=np.int32)
    lib().orc_trace(mode, _p(s) if len(s) else None, len(s), _p(o), _p(d), n, _p(t), _p(ids))
    return t, ids


def ray_dirs(view: OrcView, mode=EXACT) -> np.ndarray:
    out = np.empty((view.width * view.height, 3), dtype=np.float32)
    lib().orc_ray_dirs(mode, C.byref(view), _p(out))
    return out


def pcg_hash(seed: int) -> int:
    return lib().orc_pcg_hash(seed & 0xFFFFFFFF)


def pcg_float(seed: int):
    s = C.c_uint32(seed & 0xFFFFFFFF)
    f = lib().orc_pcg_float(C.byref(s))
    return f, s.value


def sincos2pi(u: float):
    c, s = C.c_float(), C.c_float()
    lib().orc_sincos2pi(u, C.byref(c), C.byref(s))
    return c.value, s.value


def camera_on_update(position, direction, last_mouse, mouse, right_button: bool, keys: str, dt: float):
    """Camera::onUpdate restated (orc_camera_on_update); returns (moved, position, direction, last_mouse)."""
    pos, d, lm, m = f32vec(position), f32vec(direction), f32vec(last_mouse), f32vec(mouse)
    k = np.array([int(c in keys.upper()) for c in "WSADQE"], dtype=np.int32)
    moved = lib().orc_camera_on_update(_p(pos), _p(d), _p(lm), _p(m), int(bool(right_button)), _p(k), dt)
    return bool(moved), pos, d, lm


def cook_torrance(albedo, f0, metallic, roughness, n, v, l, mode=EXACT):
    out = np.zeros(3, dtype=np.float32)
    a, f, nn, vv, ll = (f32vec(x) for x in (albedo, f0, n, v, l))
    lib().orc_cook_torrance(mode, _p(a), _p(f), metallic, roughness, _p(nn), _p(vv), _p(ll), _p(out))
    return out


def sample_cosine(n, seed, mode=EXACT):
    out = np.zeros(3, dtype=np.float32)
    s = C.c_uint32(seed & 0xFFFFFFFF)
    nn = f32vec(n)
    lib().orc_sample_cosine(mode, _p(nn), C.byref(s), _p(out))
    return out, s.value


def sample_ggx(n, roughness, seed, mode=EXACT):
    out = np.zeros(3, dtype=np.float32)
    s = C.c_uint32(seed & 0xFFFFFFFF)
    nn = f32vec(n)
    lib().orc_sample_ggx(mode, _p(nn), roughness, C.byref(s), _p(out))
    return out, s.value


def pack_rgba8(accum, frame: int) -> np.ndarray:
    a = np.ascontiguousarray(accum, dtype=np.float32).reshape(-1, 4)
    out = np.empty(len(a), dtype=np.uint32)
    lib().orc_pack_rgba8(_p(a), len(a), frame, _p(out))
    return out


def max_threads() -> int:
    return lib().orc_max_threads()
