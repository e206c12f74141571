"""Whole paths in one thread (k_fused, the path kernel of small brute-force scenes): bit for bit the
oracle's matched-order frames, exactly as the wavefront stages, across light counts around the
per-pixel visibility cache's 32 lights, sky and emission, bounce depths, one sample per call and many,
accumulation off, and the batch's primary-hit cache.  Each case is rendered with path_kernel = 2
(forced on, also for scenes that default to the wavefront) and, for the small scene, with the default."""
import numpy as np
import pytest

from ataraxia_gb300 import Batch, Renderer, Settings, scenes
from tests.helpers import bit_mismatches, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


def _lights(n, seed):
    rng = np.random.default_rng(seed)
    lt = np.zeros(n, dtype=scenes.LIGHT_DTYPE)
    lt["position"] = rng.normal(0.0, 12.0, (n, 3))
    lt["color"] = rng.uniform(0.5, 1.0, (n, 3))
    lt["intensity"] = rng.uniform(20.0, 200.0, n)
    return lt


def _cases():
    small = scenes.config0().with_resolution(96, 54)
    mats = small.materials.copy()
    mats["emission_color"][2] = [1.0, 0.5, 0.25]
    mats["emission_intensity"][2] = 3.0
    yield "small", small, 4, {}
    yield "small_1spp", small, 1, {}
    yield "small_sky_emission", scenes.SyntheticScene(**{**small.__dict__, "materials": mats}), 3, {"sky": True}
    yield "small_0_lights", scenes.SyntheticScene(**{**small.__dict__, "lights": small.lights[:0]}), 2, {}
    for n in (32, 33, 70):
        yield f"small_{n}_lights", scenes.SyntheticScene(**{**small.__dict__, "lights": _lights(n, n)}), 6, {}
    for b in (0, 1, 12):
        yield f"small_{b}_bounces", small, 3, {"max_bounces": b}
    yield "medium_256_spheres", scenes.config1().with_resolution(64, 36), 3, {}


CASES = list(_cases())


@pytest.mark.parametrize("name,sc,spp,kw", CASES, ids=[c[0] for c in CASES])
def test_fused_paths_bit_exact(po, name, sc, spp, kw):
    ref, _, _ = oracle_render(sc, spp, **kw)
    for pk in ((0, 2) if name.startswith("small") else (2,)):
        with Renderer() as r:
            r.set_tuning(path_kernel=pk)
            acc, img = gpu_render(sc, spp, renderer=r, **kw)
        assert bit_mismatches(acc, ref) == 0, pk
        assert np.array_equal(img, po.pack_rgba8(ref, spp)), pk


def test_fused_accumulation_off_equals_frames_1_to_spp(po):
    sc = scenes.config0().with_resolution(64, 36)
    with Renderer() as r:
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        view = po.view_for(sc)
        r.set_camera_matrices(np.array(view.inv_view), np.array(view.inv_proj), sc.camera_position)
        r.set_settings(Settings(accumulation=False, skyLight=False, maxBounces=sc.max_bounces))
        for _ in range(3):
            r.render_frames(4)
        acc = r.get_accumulation().reshape(-1, 4)
    ref, _, _ = oracle_render(sc, 4)
    assert bit_mismatches(acc, ref) == 0


def test_fused_in_the_batch_with_primary_cache(po):
    """Small scenes of a batch render through k_fused with the batch's per-pixel primary-hit cache:
    three passes equal rendering each scene alone."""
    mix = [scenes.config0().with_resolution(80, 45),
           scenes.SyntheticScene(**{**scenes.config0(seed=5).__dict__, "width": 48, "height": 32})]
    with Batch() as b:
        ids = [b.add_synthetic(sc) for sc in mix]
        for i in ids:
            b.set_spp(i, 2)
        for _ in range(3):
            b.run()
        for i, sc in zip(ids, mix):
            ref, _, _ = oracle_render(sc, 6)
            assert bit_mismatches(b.get_accumulation(i), ref) == 0
