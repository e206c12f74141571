"""Builds libatx.so in-tree (ataraxia_gb300/_lib/) for sm_103a.

CUDA sources go through nvcc with one -gencode (compute_103a -> sm_103a),
host C++ through g++; both with -ffp-contract=off (host) / -fmad=false
(device) so no multiply-add is fused unless the source spells it.  The CUDA
runtime is linked statically so the library loads on a machine without a GPU
(entry points then return ATX_ERR_NO_DEVICE).

    python -m ataraxia_gb300.build [-v] [--force]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_lib"
OBJ_DIR = OUT_DIR / "obj"
LIB = OUT_DIR / "libatx.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libatx.so")
    return cand


def _cuda_home(nvcc: str) -> Path:
    return Path(nvcc).resolve().parent.parent


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    return cu, cpp


def _headers():
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def _stale(obj: Path, src: Path, headers) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(h.stat().st_mtime > t for h in headers)


def build(verbose: bool = False, force: bool = False, jobs: int | None = None) -> Path:
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    cu, cpp = _sources()
    headers = _headers()
    inc = [f"-I{INCLUDE}", f"-I{CSRC}"]
    cmds = []
    objs = []
    for src in cu:
        obj = OBJ_DIR / (src.stem + ".cu.o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            cmds.append([nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
                         "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
                         *inc, "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = OBJ_DIR / (src.stem + ".cpp.o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off",
                         "-Wall", "-Wextra", *inc, f"-I{cuda / 'include'}", "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)

    if cmds:
        with ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
            list(ex.map(run, cmds))
    if force or cmds or not LIB.exists():
        link = [nvcc, ARCH, "-shared", "-cudart=static", "-o", str(LIB), *map(str, objs),
                "-Xlinker", "--exclude-libs,ALL", "-lpthread", "-ldl", "-lrt"]
        run(link)
    return LIB


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    p = build(verbose=a.verbose, force=a.force)
    print(p)
    return 0


if __name__ == "__main__":
    sys.exit(main())
