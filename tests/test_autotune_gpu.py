"""The launch tuner (atx_autotune / atx_set_tuning): every setting it can pick renders the same frames
bit for bit (the LBVH walk is exact for any leaf size, the light and direction buffers' lists for any
cell resolution; lanes, path state, block size and wave shape only change how the same paths are
scheduled), the tuner keeps one of them, and its cache answers a second call for the same GPU and
workload bucket without timing."""
import numpy as np
import pytest

from ataraxia_gb300 import Renderer, Settings, scenes
from tests.helpers import bit_mismatches

pytestmark = pytest.mark.gpu

SETTINGS = [dict(), dict(bvh_leaf_size=4), dict(bvh_leaf_size=8), dict(bvh_leaf_size=32), dict(lanes=1),
            dict(lanes=2), dict(lanes=4), dict(wave_paths=1 << 20), dict(threads=128), dict(wave_spp=1),
            dict(path_kernel=1), dict(path_kernel=2), dict(cell_res=8), dict(cell_res=16), dict(cell_res=24),
            dict(bvh_leaf_size=12, lanes=4, wave_paths=4 << 20, threads=128, wave_spp=4, cell_res=16)]


def _scene(kind):
    if kind == "lbvh":   # 8,192 clustered spheres: the LBVH (from 1,025 spheres)
        big = scenes.config2()
        return scenes.SyntheticScene(**{**big.__dict__, "spheres": big.spheres[:8192].copy(), "width": 1280,
                                        "height": 720, "max_bounces": 6})
    return scenes.config1().with_resolution(1280, 720)


def _render(r, sc, spp):
    r.reset_frame_index()
    r.render_frames(1)            # the first render of a camera goes without the per-camera tables
    r.render_frames(spp - 1)
    return r.get_accumulation().reshape(-1, 4).copy(), r.get_image().reshape(-1).copy()


@pytest.mark.parametrize("kind", ["lbvh", "brute_force"])
def test_every_tuning_renders_the_same_frames(po, kind):
    sc = _scene(kind)
    spp = 24                     # 22 Mi paths: enough for four lanes
    with Renderer() as r:
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        view = po.view_for(sc)
        r.set_camera_matrices(np.array(view.inv_view), np.array(view.inv_proj), sc.camera_position)
        r.set_settings(Settings(accumulation=True, skyLight=False, maxBounces=sc.max_bounces))
        ref_acc, ref_img = _render(r, sc, spp)
        assert r.stats()["bvh_in_use"] == (1 if kind == "lbvh" else 0)
        for t in SETTINGS[1:]:
            r.set_tuning(**t)
            got = r.tuning()
            if kind == "lbvh" and "bvh_leaf_size" in t:
                assert got["bvh_leaf_size"] == t["bvh_leaf_size"]
            # the brute-force scene (256 spheres) has light and direction buffers, by default with 32 cells
            # along a face's edge
            assert got["cell_res"] == (0 if kind == "lbvh" else t.get("cell_res", 32))
            acc, img = _render(r, sc, spp)
            assert bit_mismatches(acc, ref_acc) == 0, t
            assert np.array_equal(img, ref_img), t
        r.set_tuning()
        # the scene set again keeps a tuned leaf size
        r.set_tuning(bvh_leaf_size=8, cell_res=16)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        if kind == "lbvh":
            assert r.tuning()["bvh_leaf_size"] == 8
        else:
            assert r.tuning()["cell_res"] == 16
        acc, _ = _render(r, sc, spp)
        assert bit_mismatches(acc, ref_acc) == 0


def test_autotune_picks_a_setting_and_caches_it():
    sc = _scene("lbvh")
    spp = 8
    with Renderer() as r:
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        r.set_camera(__import__("ataraxia_gb300").Camera(sc.fov, sc.near, sc.far, sc.camera_position,
                                                          sc.camera_direction))
        r.set_settings(Settings(accumulation=True, skyLight=False, maxBounces=sc.max_bounces))
        ref_acc, _ = _render(r, sc, spp)
        t1 = r.autotune(spp, passes=1, use_cache=False)
        assert t1["from_cache"] == 0 and t1["ms"] > 0.0
        assert t1["bvh_leaf_size"] in (4, 8, 12, 16, 24, 32)
        assert r.frame_index == 1
        acc, _ = _render(r, sc, spp)
        assert bit_mismatches(acc, ref_acc) == 0
        t2 = r.autotune(spp, passes=1, use_cache=True)
        assert t2["from_cache"] == 1
        assert {k: t2[k] for k in ("bvh_leaf_size", "lanes", "wave_paths", "threads", "wave_spp", "path_kernel")} == \
               {k: t1[k] for k in ("bvh_leaf_size", "lanes", "wave_paths", "threads", "wave_spp", "path_kernel")}


@pytest.mark.parametrize("res", [4, 7, 33, 64])
def test_cell_resolution_outside_its_range_is_rejected(res):
    from ataraxia_gb300 import AtxError

    sc = scenes.config1().with_resolution(64, 36)
    with Renderer() as r:
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        with pytest.raises(AtxError):
            r.set_tuning(cell_res=res)
        assert r.tuning()["cell_res"] == 32
