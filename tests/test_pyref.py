"""The C oracle (matched order) against the independent pure-Python restatement in tests/pyref.py:
bit-identical per-frame colours on small images of three scenes, with sky light and emission."""
import numpy as np
import pytest

from ataraxia_gb300 import scenes
from tests import pyref


def _case(sc, pixels, frames, sky, po):
    view = po.view_for(sc)
    ip = [np.float32(x) for x in view.inv_proj]
    iv = [np.float32(x) for x in view.inv_view]
    pos = [np.float32(x) for x in view.position]
    _, smp, _ = po.render(sc.spheres, sc.materials, sc.lights, view, max_bounces=sc.max_bounces, sky=sky,
                          spp=frames, pixels=np.array(pixels, dtype=np.uint32), samples=True)
    for k, p in enumerate(pixels):
        x, y = p % sc.width, p // sc.width
        for f in range(frames):
            col = pyref.per_pixel((sc.spheres, sc.materials, sc.lights), ip, iv, pos, sc.width, sc.height, x, y,
                                  1 + f, sc.max_bounces, sky)
            got = smp[k, f, :3]
            assert np.array_equal(np.array(col, dtype=np.float32).view(np.uint32), got.view(np.uint32)), \
                (sc.name, p, f, col, got)


def test_pyref_config0(po):
    sc = scenes.config0().with_resolution(48, 27)
    rng = np.random.default_rng(0)
    _case(sc, sorted(rng.choice(sc.pixels, 40, replace=False)), 2, False, po)


def test_pyref_default_scene_with_sky(po):
    sc = scenes.reference_default_scene().with_resolution(40, 24)
    rng = np.random.default_rng(1)
    _case(sc, sorted(rng.choice(sc.pixels, 30, replace=False)), 2, True, po)


@pytest.mark.slow
def test_pyref_config1_subset_with_emission(po):
    sc = scenes.config1().with_resolution(64, 36)
    sph = sc.spheres[:48].copy()
    mats = sc.materials.copy()
    mats["emission_color"][3] = [0.5, 1.0, 0.25]
    mats["emission_intensity"][3] = 2.0
    sc = scenes.SyntheticScene(**{**sc.__dict__, "spheres": sph, "materials": mats, "max_bounces": 4})
    rng = np.random.default_rng(2)
    _case(sc, sorted(rng.choice(sc.pixels, 24, replace=False)), 2, False, po)
