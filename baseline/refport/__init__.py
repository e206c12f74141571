"""Loader for the restated reference render kernel (refport.cu), a GPU measuring stick for bench.py.

build() compiles refport.cu for sm_103a with the reference's own flags (-use_fast_math, default
multiply-add contraction) into baseline/refport/_build/librefport.so.
"""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "librefport.so"


def build(force: bool = False) -> Path:
    src = HERE / "refport.cu"
    if LIB.exists() and not force and LIB.stat().st_mtime > src.stat().st_mtime:
        return LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    LIB.parent.mkdir(exist_ok=True)
    subprocess.run([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O3", "-use_fast_math", "-std=c++17",
                    "-Xcompiler", "-fPIC,-fvisibility=hidden", "-shared", "-cudart=static", "-o", str(LIB), str(src),
                    "-Xlinker", "--exclude-libs,ALL"], check=True)
    return LIB


def ray_dirs(inv_view: np.ndarray, inv_proj: np.ndarray, width: int, height: int) -> np.ndarray:
    """Camera.cpp:173-187 in float32 (the reference computes these on the host)."""
    f = np.float32
    IP = np.asarray(inv_proj, dtype=f).reshape(4, 4)      # [col][row]
    IV = np.asarray(inv_view, dtype=f).reshape(4, 4)
    x = np.arange(width, dtype=f)[None, :] / f(width)
    y = np.arange(height, dtype=f)[:, None] / f(height)
    cx = np.broadcast_to(x * f(2) - f(1), (height, width))
    cy = np.broadcast_to(y * f(2) - f(1), (height, width))
    t = [IP[0, r] * cx + IP[1, r] * cy + IP[2, r] + IP[3, r] for r in range(4)]
    v = np.stack([t[0] / t[3], t[1] / t[3], t[2] / t[3]], axis=-1)
    v = v / np.sqrt((v * v).sum(-1, keepdims=True))
    d = np.stack([IV[0, r] * v[..., 0] + IV[1, r] * v[..., 1] + IV[2, r] * v[..., 2] for r in range(3)], axis=-1)
    d = d / np.sqrt((d * d).sum(-1, keepdims=True))
    return np.ascontiguousarray(d.reshape(-1, 3), dtype=f)


class RefPort:
    def __init__(self, spheres, materials, lights, width, height, dirs, position, max_bounces):
        self.lib = C.CDLL(str(build()))
        self.lib.refport_create.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                            C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int,
                                            C.POINTER(C.c_void_p)]
        self.lib.refport_frame.argtypes = [C.c_void_p, C.c_int]
        self.lib.refport_read_accum.argtypes = [C.c_void_p, C.c_void_p]
        self.lib.refport_destroy.argtypes = [C.c_void_p]
        self.lib.refport_block.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
        self._keep = [np.ascontiguousarray(a) for a in (spheres, materials, lights)]
        d = np.ascontiguousarray(dirs, dtype=np.float32)
        p = np.ascontiguousarray(position, dtype=np.float32)
        h = C.c_void_p()
        rc = self.lib.refport_create(*[C.c_void_p(a.ctypes.data) if len(a) else None for a in self._keep[:1]],
                                     len(self._keep[0]), C.c_void_p(self._keep[1].ctypes.data), len(self._keep[1]),
                                     C.c_void_p(self._keep[2].ctypes.data) if len(self._keep[2]) else None,
                                     len(self._keep[2]), width, height, C.c_void_p(d.ctypes.data),
                                     C.c_void_p(p.ctypes.data), max_bounces, C.byref(h))
        if rc:
            raise RuntimeError("refport_create failed")
        self.h = h
        self.width, self.height = width, height

    def frame(self, full: bool = False):
        if self.lib.refport_frame(self.h, int(full)):
            raise RuntimeError("refport_frame failed")

    def sync(self):
        self.lib.refport_sync()

    def block(self):
        bx, by = C.c_int(), C.c_int()
        self.lib.refport_block(C.byref(bx), C.byref(by))
        return bx.value, by.value

    def accumulation(self) -> np.ndarray:
        out = np.empty((self.width * self.height, 4), dtype=np.float32)
        self.lib.refport_read_accum(self.h, C.c_void_p(out.ctypes.data))
        return out

    def close(self):
        if self.h:
            self.lib.refport_destroy(self.h)
            self.h = None
