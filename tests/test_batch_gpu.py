"""Batched renderer: every scene's accumulator and image are bit-identical to rendering
the scene alone (Renderer / atx_render) and to the oracle, whatever else shares the pass."""
import numpy as np
import pytest

from ataraxia_gb300 import Batch, Camera, Renderer, Settings, scenes
from tests.helpers import bit_mismatches, oracle_render

pytestmark = pytest.mark.gpu


def small_mix(count=6, scale=8):
    """Scenes of the batched mix at 1/scale of their resolution (spp capped for test time)."""
    out = []
    for sc in scenes.config3(count=count):
        out.append(scenes.SyntheticScene(**{**sc.__dict__, "width": max(8, sc.width // scale),
                                            "height": max(8, sc.height // scale), "spp": min(sc.spp, 12)}))
    return out


def alone(sc, spp, frames_before=0):
    with Renderer() as r:
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        r.set_camera(Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction))
        r.set_settings(Settings(accumulation=True, skyLight=sc.sky_light, maxBounces=sc.max_bounces))
        if frames_before:
            r.render_frames(frames_before)
        r.render_frames(spp)
        return r.get_accumulation().reshape(-1, 4).copy(), r.get_image().reshape(-1).copy()


def test_mix_equals_alone_three_passes():
    mix = small_mix()
    with Batch() as b:
        ids = [b.add_synthetic(sc) for sc in mix]
        for i, sc in zip(ids, mix):
            b.set_spp(i, sc.spp)
        b.run()                       # a new shape: launched directly
        b.run()                       # continues each accumulation (no clear): another new shape
        b.run()                       # same shape as the last: replayed from the captured graph
        for i, sc in zip(ids, mix):
            acc, img = b.get_accumulation(i), b.get_image(i)
            ref_acc, ref_img = alone(sc, sc.spp, frames_before=2 * sc.spp)
            assert bit_mismatches(acc, ref_acc) == 0, sc.name
            assert np.array_equal(img, ref_img), sc.name
            assert b.frame_index(i) == 1 + 3 * sc.spp
        st = b.stats()
        assert st["passes"] == 3 and st["graph_launches"] == 1
        assert st["paths"] == 3 * sum(sc.width * sc.height * sc.spp for sc in mix)


def test_batch_matches_oracle_and_lbvh_scene(po):
    sc0 = scenes.config0().with_resolution(64, 36)
    sc1 = scenes.config1().with_resolution(48, 27)
    big = scenes.config2().with_resolution(32, 18)          # 65,536 spheres: LBVH in the batch
    with Batch() as b:
        ids = [b.add_synthetic(s) for s in (sc0, sc1, big)]
        for i in ids:
            b.set_spp(i, 3)
        b.run()
        for i, s in zip(ids, (sc0, sc1, big)):
            ref, _, _ = oracle_render(s, 3)
            assert bit_mismatches(b.get_accumulation(i), ref) == 0, s.name


def test_idle_scenes_remove_and_reuse_ids():
    mix = small_mix(4)
    with Batch() as b:
        ids = [b.add_synthetic(sc) for sc in mix]
        b.set_spp(ids[0], 4)
        b.run()                                  # only scene 0 renders
        assert b.frame_index(ids[0]) == 5 and b.frame_index(ids[1]) == 1
        b.remove_scene(ids[1])
        j = b.add_synthetic(mix[1])
        assert j == ids[1]
        b.set_spp(ids[0], 0)
        b.set_spp(j, 2)
        b.run()
        ref, _ = alone(mix[1], 2)
        assert bit_mismatches(b.get_accumulation(j), ref) == 0


def test_edge_scenes_in_batch(po):
    base = scenes.config0().with_resolution(37, 23)
    empty = scenes.SyntheticScene(**{**base.__dict__, "spheres": base.spheres[:0], "sky_light": True})
    nolight = scenes.SyntheticScene(**{**base.__dict__, "lights": base.lights[:0], "sky_light": True})
    deep = scenes.SyntheticScene(**{**base.__dict__, "max_bounces": 40})
    zero = scenes.SyntheticScene(**{**base.__dict__, "max_bounces": 0})
    tiny = base.with_resolution(1, 1)
    cases = [empty, nolight, deep, zero, tiny]
    with Batch() as b:
        ids = [b.add_synthetic(s) for s in cases]
        for i in ids:
            b.set_spp(i, 2)
        b.run()
        for i, s in zip(ids, cases):
            ref, _, _ = oracle_render(s, 2, sky=s.sky_light)
            assert bit_mismatches(b.get_accumulation(i), ref) == 0


def test_accumulation_off_in_batch():
    sc = small_mix(1)[0]
    with Batch() as b:
        i = b.add_synthetic(sc, Settings(accumulation=False, skyLight=False, maxBounces=sc.max_bounces))
        b.set_spp(i, 1)
        b.run()
        b.run()
        assert b.frame_index(i) == 1
        ref, _ = alone(scenes.SyntheticScene(**{**sc.__dict__}), 1)
        assert bit_mismatches(b.get_accumulation(i), ref) == 0


@pytest.mark.parametrize("lanes,wave,cache", [(1, 1 << 16, True), (3, 1 << 17, False), (16, 1 << 20, True)])
def test_tunings_do_not_change_results(lanes, wave, cache):
    """Lane count, path-state size (down to several waves and pixel-range parts per scene) and the
    primary-hit cache leave results unchanged."""
    mix = small_mix(3)
    with Batch() as b:
        b.set_tuning(lanes=lanes, lane_wave_paths=wave, primary_cache=cache)
        ids = [b.add_synthetic(sc) for sc in mix]
        for i, sc in zip(ids, mix):
            b.set_spp(i, 3)
        b.run()
        for i, sc in zip(ids, mix):
            ref, _ = alone(sc, 3)
            assert bit_mismatches(b.get_accumulation(i), ref) == 0
        assert b.stats()["waves_last_pass"] >= len(mix)


def test_set_camera_restarts_accumulation():
    sc = small_mix(1)[0]
    with Batch() as b:
        i = b.add_synthetic(sc)
        b.set_spp(i, 2)
        b.run()
        assert b.frame_index(i) == 3
        cam = Camera(sc.fov, sc.near, sc.far, tuple(p + 0.5 for p in sc.camera_position), sc.camera_direction)
        b.set_camera(i, cam)
        assert b.frame_index(i) == 1
        b.run()
        moved = scenes.SyntheticScene(**{**sc.__dict__, "camera_position": cam.position})
        ref, _ = alone(moved, 2)
        assert bit_mismatches(b.get_accumulation(i), ref) == 0


def test_autotune_leaves_no_trace():
    """Autotuning renders the scenes under several settings, then puts them back at frame 1: the
    passes after it equal rendering each scene alone."""
    mix = small_mix(4)
    with Batch() as b:
        ids = [b.add_synthetic(sc) for sc in mix]
        for i, sc in zip(ids, mix):
            b.set_spp(i, 2)
        chosen = b.autotune(passes=1)
        assert chosen["lanes"] in (4, 8, 16) and chosen["lane_wave_paths"] >= 8 << 20
        assert all(b.frame_index(i) == 1 for i in ids)
        b.run()
        for i, sc in zip(ids, mix):
            ref, _ = alone(sc, 2)
            assert bit_mismatches(b.get_accumulation(i), ref) == 0
        b.run()
        with pytest.raises(Exception):
            b.autotune()                       # scenes have rendered frames now


def test_leaf_size_change_rebuilds_resident_trees():
    """A new LBVH leaf size rebuilds the resident LBVH scenes' trees (the autotuner's leaf trials): the
    next passes still equal rendering each scene alone."""
    big = scenes.config2()
    lbvh = scenes.SyntheticScene(**{**big.__dict__, "spheres": big.spheres[:3000].copy(), "width": 160,
                                    "height": 90, "max_bounces": 5, "spp": 3})
    mix = [lbvh] + small_mix(2)
    with Batch() as b:
        ids = [b.add_synthetic(sc) for sc in mix]
        for i, sc in zip(ids, mix):
            b.set_spp(i, 3)
        for leaf in (8, 24):
            b.set_tuning(bvh_leaf_size=leaf)
            assert b.tuning()["bvh_leaf_size"] == leaf
            for i in ids:
                b.reset(i)
            b.run()
            for i, sc in zip(ids, mix):
                ref, _ = alone(sc, 3)
                assert bit_mismatches(b.get_accumulation(i), ref) == 0, (leaf, sc.name)
