"""Committed fixtures (tests/golden/, made by make_golden.py on x86-64): the oracle reproduces them on
this machine (bit for bit in the matched order; within rounding for the libm-based modes), and the GPU
reproduces the matched-order accumulators and images bit for bit."""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ["config0_32x18", "config1_40x24", "default_24x16_sky"]


def load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def view_of(po, g):
    return po.make_view(g["inv_view"], g["inv_proj"], g["position"], int(g["width"]), int(g["height"]))


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(po, name):
    g = load(name)
    v = view_of(po, g)
    kw = dict(max_bounces=int(g["max_bounces"]), sky=bool(g["sky"]), spp=int(g["frames"]))
    ex, _, _ = po.render(g["spheres"], g["materials"], g["lights"], v, mode=po.EXACT, **kw)
    assert np.array_equal(ex.view(np.uint32), g["accum_exact"].view(np.uint32))
    assert np.array_equal(po.pack_rgba8(ex, int(g["frames"])), g["image_exact"])
    li, _, _ = po.render(g["spheres"], g["materials"], g["lights"], v, mode=po.LITERAL, **kw)
    d64, _, _ = po.render(g["spheres"], g["materials"], g["lights"], v, f64=True, **kw)
    # libm may differ by an ulp between machines: compare image means, not bits
    assert abs(li[:, :3].mean() - g["accum_literal"][:, :3].mean()) <= 1e-3 * max(1.0, abs(g["accum_literal"][:, :3].mean()))
    assert abs(d64[:, :3].mean() - g["accum_f64"][:, :3].mean()) <= 1e-3 * max(1.0, abs(g["accum_f64"][:, :3].mean()))


def test_rng_tables(po):
    g = load("rng_tables")
    for s, h in zip(g["seeds"], g["pcg"]):
        assert po.pcg_hash(int(s)) == int(h)
    for u, (c, s) in zip(g["u"], g["sincos"]):
        assert po.sincos2pi(float(u)) == (float(c), float(s))


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_reproduces_golden(name):
    from ataraxia_gb300 import Renderer, Settings

    g = load(name)
    w, h, frames = int(g["width"]), int(g["height"]), int(g["frames"])
    with Renderer() as r:
        r.on_resize(w, h)
        r.set_scene(g["spheres"], g["materials"], g["lights"])
        r.set_camera_matrices(g["inv_view"], g["inv_proj"], g["position"])
        r.set_settings(Settings(accumulation=True, skyLight=bool(g["sky"]), maxBounces=int(g["max_bounces"])))
        r.render_frames(frames)
        acc = r.get_accumulation().reshape(-1, 4)
        img = r.get_image().reshape(-1)
    assert np.array_equal(acc.view(np.uint32), g["accum_exact"].view(np.uint32))
    assert np.array_equal(img, g["image_exact"])
