"""FP32 pipe peak of the GPU for bench.py's FP32 roofline (fp32_peak.cu, built on first use)."""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libfp32peak.so"


def build(force: bool = False) -> Path:
    src = HERE / "fp32_peak.cu"
    if LIB.exists() and not force and LIB.stat().st_mtime > src.stat().st_mtime:
        return LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    LIB.parent.mkdir(exist_ok=True)
    subprocess.run([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler",
                    "-fPIC,-fvisibility=hidden", "-shared", "-cudart=static", "-o", str(LIB), str(src),
                    "-Xlinker", "--exclude-libs,ALL"], check=True)
    return LIB


def peak_tflops(device: int = 0) -> float:
    """FP32 fused multiply-add throughput (FMA = 2 FLOP) of `device`, TFLOP/s: best of five timed
    launches of independent register-resident FFMA chains on every SM."""
    lib = C.CDLL(str(build()))
    lib.fp32_peak_tflops.argtypes = [C.c_int, C.POINTER(C.c_double)]
    t = C.c_double()
    rc = lib.fp32_peak_tflops(device, C.byref(t))
    if rc:
        raise RuntimeError(f"fp32 peak probe failed (cudaError {rc})")
    return t.value
