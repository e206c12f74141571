"""Generates tests/golden/*.npz: small fixed cases of the oracle (ORC_EXACT, ORC_LITERAL, f64) with
their full inputs, the PCG hash computed with Python integers, and the matched-order sin/cos table.

    python tests/golden/make_golden.py

The reference ships no golden vectors; these fixtures pin the oracle against itself across machines
(generated on x86-64; the GPU machine is aarch64) and give the GPU tests a fixed target."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from ataraxia_gb300 import scenes  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

CASES = {
    "config0_32x18": (scenes.config0, (32, 18), 3, False),
    "config1_40x24": (scenes.config1, (40, 24), 4, False),
    "default_24x16_sky": (scenes.reference_default_scene, (24, 16), 2, True),
}


def pcg_int(s: int) -> int:
    state = (s * 747796405 + 2891336453) & 0xFFFFFFFF
    word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & 0xFFFFFFFF
    return ((word >> 22) ^ word) & 0xFFFFFFFF


def main() -> None:
    po.build()
    for name, (fn, res, frames, sky) in CASES.items():
        sc = fn().with_resolution(*res)
        v = po.view_for(sc)
        kw = dict(max_bounces=sc.max_bounces, sky=sky, spp=frames)
        ex, _, _ = po.render(sc.spheres, sc.materials, sc.lights, v, mode=po.EXACT, **kw)
        li, _, _ = po.render(sc.spheres, sc.materials, sc.lights, v, mode=po.LITERAL, **kw)
        d64, _, _ = po.render(sc.spheres, sc.materials, sc.lights, v, f64=True, **kw)
        np.savez_compressed(HERE / f"{name}.npz", spheres=sc.spheres, materials=sc.materials, lights=sc.lights,
                            inv_view=np.array(v.inv_view, np.float32), inv_proj=np.array(v.inv_proj, np.float32),
                            position=np.array(v.position, np.float32), width=res[0], height=res[1],
                            max_bounces=sc.max_bounces, sky=int(sky), frames=frames,
                            accum_exact=ex, accum_literal=li, accum_f64=d64,
                            image_exact=po.pack_rgba8(ex, frames))
    seeds = np.array([0, 1, 2, 3, 255, 65535, 123456789, 2**31 - 1, 2**31, 2**32 - 1] +
                     list(np.random.default_rng(0).integers(0, 2**32, 246, dtype=np.uint64)), dtype=np.uint64)
    us = np.concatenate([np.linspace(0, 1, 257, dtype=np.float32), np.random.default_rng(1).random(255, dtype=np.float32)])
    sc_tab = np.array([po.sincos2pi(float(u)) for u in us], dtype=np.float32)
    np.savez_compressed(HERE / "rng_tables.npz", seeds=seeds.astype(np.uint32),
                        pcg=np.array([pcg_int(int(s)) for s in seeds], dtype=np.uint32), u=us, sincos=sc_tab)
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")))


if __name__ == "__main__":
    main()
