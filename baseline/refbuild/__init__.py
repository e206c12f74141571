"""The reference's own render path, compiled from its unmodified sources: loaders for tests and bench.py.

Two parts, both test and benchmark infrastructure (the product never loads them):

* ``baseline/refbuild/_ref/kernel_render*.cubin`` -- the reference's Renderer.cu + BRDF.cu device code
  (kernelRender, perPixel, traceRay, BRDF, Random), built by ``baseline/refbuild/Makefile`` where the
  reference tree is present and shipped as device images.  ``libreflaunch.so`` (``ref_launch.cu``,
  built on any machine) loads one and launches kernelRender as Renderer::Render does.
* ``baseline/refbuild/_ref/libref_host.so`` -- the reference's Camera.cpp, SceneNode.cpp and the
  host half of Renderer.cu for x86 CPU tests (present only where the reference tree was built).

Variants of the device image: ``fast`` (the reference's flags, -use_fast_math), ``nofmad`` (the same
without multiply-add contraction) and ``ieee`` (IEEE arithmetic, no contraction).
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_OUT = HERE / "_ref"
LAUNCH_LIB = HERE / "_build" / "libreflaunch.so"
HOST_LIB = REF_OUT / "libref_host.so"
VARIANTS = {"fast": "kernel_render.cubin", "nofmad": "kernel_render_nofmad.cubin",
            "ieee": "kernel_render_ieee.cubin"}


def cubin(variant: str = "fast") -> Path:
    return REF_OUT / VARIANTS[variant]


def build_reference(ref_root: str | os.PathLike | None = None) -> bool:
    """Runs the Makefile over the reference tree; False (nothing built) when the tree is absent."""
    root = Path(ref_root or os.environ.get("ATX_REFERENCE_ROOT", "/root/reference"))
    if not (root / "Engine" / "src" / "Renderer.cu").exists():
        return False
    subprocess.run(["make", "-s", "-j4", "-C", str(HERE), f"REF={root}"], check=True)
    return True


def build(force: bool = False) -> Path:
    """Compiles the launcher (host code only) for this machine."""
    src = HERE / "ref_launch.cu"
    if LAUNCH_LIB.exists() and not force and LAUNCH_LIB.stat().st_mtime > src.stat().st_mtime:
        return LAUNCH_LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    LAUNCH_LIB.parent.mkdir(exist_ok=True)
    subprocess.run([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-Xcompiler",
                    "-fPIC,-fvisibility=hidden", "-shared", "-cudart=static", "-o", str(LAUNCH_LIB), str(src),
                    "-Xlinker", "--exclude-libs,ALL"], check=True)
    return LAUNCH_LIB


def available(variant: str = "fast") -> bool:
    return cubin(variant).exists()


# --------------------------------------------------------------------------- camera (host side)

def ray_dirs(inv_view, inv_proj, width: int, height: int) -> np.ndarray:
    """Camera::UpdateRayDirection (Engine/src/Camera.cpp:161-195) in float32, as the reference computes it
    on the host: coord = (x/W, y/H)*2 - 1; target = invProj * (cx, cy, 1, 1) with the matrix-vector
    product summed pairwise over columns; dir = normalize(vec3(invView * (normalize(target.xyz/target.w),
    0))) with normalize(v) = v * (1/sqrt((x*x + y*y) + z*z)).  numpy rounds every operation to float32 and
    fuses nothing.  Checked bit for bit against the reference's Camera.cpp built here (CPU test)."""
    f = np.float32
    IP = np.asarray(inv_proj, dtype=f).reshape(4, 4)      # [col][row]
    IV = np.asarray(inv_view, dtype=f).reshape(4, 4)
    x = np.arange(width, dtype=f)[None, :] / f(width)
    y = np.arange(height, dtype=f)[:, None] / f(height)
    cx = np.broadcast_to(x * f(2) - f(1), (height, width))
    cy = np.broadcast_to(y * f(2) - f(1), (height, width))
    t = [(IP[0, r] * cx + IP[1, r] * cy) + (IP[2, r] * f(1) + IP[3, r] * f(1)) for r in range(4)]
    v = [t[0] / t[3], t[1] / t[3], t[2] / t[3]]

    def normalize(a, b, c):
        inv = f(1) / np.sqrt((a * a + b * b) + c * c)
        return a * inv, b * inv, c * inv

    v = normalize(*v)
    d = [(IV[0, r] * v[0] + IV[1, r] * v[1]) + (IV[2, r] * v[2] + IV[3, r] * f(0)) for r in range(3)]
    d = normalize(*d)
    return np.ascontiguousarray(np.stack(d, axis=-1).reshape(-1, 3), dtype=f)


# --------------------------------------------------------------------------- GPU kernel

_launch = None


def _lib():
    global _launch
    if _launch is None:
        lib = C.CDLL(str(build()))
        P, U = C.c_void_p, C.c_uint32
        lib.refk_last_error.restype = C.c_char_p
        lib.refk_load.argtypes = [C.c_char_p, C.POINTER(P)]
        lib.refk_kernel_info.argtypes = [P, C.c_char_p, C.c_int, C.POINTER(C.c_int)]
        lib.refk_create.argtypes = [P, P, U, P, U, P, U, U, U, P, P, P, C.c_int, C.c_int, C.c_int, C.POINTER(P)]
        lib.refk_frame.argtypes = [P, C.c_int]
        lib.refk_time_frames.argtypes = [P, C.c_int, C.c_int, C.POINTER(C.c_float)]
        lib.refk_set_frame.argtypes = [P, U]
        lib.refk_frame_index.argtypes = [P]
        lib.refk_frame_index.restype = U
        lib.refk_read_accum.argtypes = [P, P]
        lib.refk_read_image.argtypes = [P, P]
        lib.refk_destroy.argtypes = [P]
        _launch = lib
    return _launch


def _check(rc: int, what: str):
    if rc:
        raise RuntimeError(f"{what}: {_lib().refk_last_error().decode(errors='replace')}")


def load_kernel(variant: str = "fast"):
    """The device image's kernelRender (loaded once per process); raises if the image is missing."""
    path = cubin(variant)
    if not path.exists():
        raise FileNotFoundError(f"{path} not built (baseline/refbuild/Makefile needs the reference tree)")
    h = C.c_void_p()
    _check(_lib().refk_load(str(path).encode(), C.byref(h)), "refk_load")
    return h


def kernel_info(variant: str = "fast"):
    h = load_kernel(variant)
    name = C.create_string_buffer(512)
    block = C.c_int()
    _lib().refk_kernel_info(h, name, 512, C.byref(block))
    return name.value.decode(), block.value


class RefRenderer:
    """One reference Renderer over a flat scene: spheres/materials/lights as the numpy structured arrays
    of ataraxia_gb300 (the reference's POD layouts), ray directions from ray_dirs()."""

    def __init__(self, spheres, materials, lights, width, height, dirs, position, direction, max_bounces,
                 accumulation=True, sky_light=False, variant="fast"):
        lib = _lib()
        k = load_kernel(variant)
        self._keep = [np.ascontiguousarray(a) for a in (spheres, materials, lights)]
        d = np.ascontiguousarray(dirs, dtype=np.float32)
        p = np.ascontiguousarray(position, dtype=np.float32)
        v = np.ascontiguousarray(direction, dtype=np.float32)
        ptr = [C.c_void_p(a.ctypes.data) if len(a) else None for a in self._keep]
        h = C.c_void_p()
        _check(lib.refk_create(k, ptr[0], len(self._keep[0]), ptr[1], len(self._keep[1]), ptr[2],
                               len(self._keep[2]), width, height, C.c_void_p(d.ctypes.data),
                               C.c_void_p(p.ctypes.data), C.c_void_p(v.ctypes.data), int(max_bounces),
                               int(bool(accumulation)), int(bool(sky_light)), C.byref(h)), "refk_create")
        self.h = h
        self.width, self.height = width, height

    def frame(self, full: bool = False):
        _check(_lib().refk_frame(self.h, int(full)), "refk_frame")

    def frames(self, n: int, full: bool = False):
        for _ in range(n):
            self.frame(full)

    def time_frames(self, n: int, full: bool = False) -> float:
        ms = C.c_float()
        _check(_lib().refk_time_frames(self.h, n, int(full), C.byref(ms)), "refk_time_frames")
        return ms.value

    def set_frame(self, f: int):
        _lib().refk_set_frame(self.h, f)

    @property
    def frame_index(self) -> int:
        return _lib().refk_frame_index(self.h)

    def accumulation(self) -> np.ndarray:
        out = np.empty((self.width * self.height, 4), dtype=np.float32)
        _check(_lib().refk_read_accum(self.h, C.c_void_p(out.ctypes.data)), "refk_read_accum")
        return out

    def image(self) -> np.ndarray:
        out = np.empty(self.width * self.height, dtype=np.uint32)
        _check(_lib().refk_read_image(self.h, C.c_void_p(out.ctypes.data)), "refk_read_image")
        return out

    def close(self):
        if self.h:
            _lib().refk_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# --------------------------------------------------------------------------- host library (CPU tests)

_host = None


def host_lib():
    """libref_host.so, or None where it was not built (no reference tree, or another architecture)."""
    global _host
    if _host is None:
        if not HOST_LIB.exists():
            return None
        try:
            lib = C.CDLL(str(HOST_LIB))
        except OSError:
            return None
        P, F, U = C.c_void_p, C.c_float, C.c_uint32
        lib.refh_camera.argtypes = [F, F, F, P, P, U, U, P, P, P, P, P]
        lib.refh_camera_update.argtypes = [P, P, P, P, C.c_int, F, F, F]
        lib.refh_flatten.argtypes = [C.c_int, P, P, C.c_int, P, P, P, P, C.c_int]
        _host = lib
    return _host


def _fp(a):
    return C.c_void_p(a.ctypes.data)


def ref_camera(fov, near, far, position, direction, width, height):
    """The reference's Camera: (ray directions (W*H, 3), view, inv_view, proj, inv_proj), matrices flat
    column-major."""
    lib = host_lib()
    pos = np.asarray(position, np.float32)
    d = np.asarray(direction, np.float32)
    dirs = np.empty((width * height, 3), np.float32)
    mats = [np.empty(16, np.float32) for _ in range(4)]
    rc = lib.refh_camera(fov, near, far, _fp(pos), _fp(d), width, height, _fp(dirs), *[_fp(m) for m in mats])
    if rc:
        raise RuntimeError("refh_camera failed")
    return (dirs, *mats)


def ref_camera_update(position, direction, last_mouse, keys, right_button, mouse, dt):
    """Camera::onUpdate once: returns (moved, position, direction)."""
    lib = host_lib()
    pos = np.array(position, np.float32)
    d = np.array(direction, np.float32)
    lm = np.array(last_mouse, np.float32)
    k = np.array([1 if keys.get(c) else 0 for c in "wasdqe"], np.uint8)
    moved = lib.refh_camera_update(_fp(pos), _fp(d), _fp(lm), _fp(k), int(bool(right_button)),
                                   float(mouse[0]), float(mouse[1]), float(dt))
    return bool(moved), pos, d


def ref_flatten(parents, trs, owners, spheres, ids):
    """Renderer::traverseSceneGraph over SceneNode::updateGlobalTransform: rows (cx, cy, cz, r, id)."""
    lib = host_lib()
    parents = np.ascontiguousarray(parents, np.int32)
    trs = np.ascontiguousarray(trs, np.float32)
    owners = np.ascontiguousarray(owners, np.int32)
    spheres = np.ascontiguousarray(spheres, np.float32)
    ids = np.ascontiguousarray(ids, np.int32)
    out = np.empty((max(len(owners), 1), 5), np.float32)
    n = lib.refh_flatten(len(parents), _fp(parents), _fp(trs), len(owners), _fp(owners), _fp(spheres), _fp(ids),
                         _fp(out), len(out))
    return out[:n]
