"""GPU parity: the wavefront kernels against the CPU oracle through the C ABI.

The kernels evaluate the reference's estimator in the oracle's ORC_EXACT order,
so accumulators and images must be bit-identical to it.  Against the literal
restatement (reference expression order, no fused multiply-adds) the number of
pixels outside 1e-3 relative is counted and bounded by what FMA contraction
alone does to the reference's own expressions (the contracted oracle build).
"""
import numpy as np
import pytest

from ataraxia_gb300 import AtxError, Renderer, Settings, scenes
from tests.helpers import bit_mismatches, frac_outside, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


def test_camera_matrices_match_oracle(po):
    from ataraxia_gb300 import Camera, camera_matrices

    for pos, d, fov, w, h in [((0, 2, 10), (0, -0.196116, -0.980581), 45.0, 1280, 720),
                              ((0, 0, 3), (0, 0, -1), 45.0, 1600, 900),
                              ((-0.47, 2.13, 8.05), (0.2125, -0.2746, -0.9378), 60.0, 333, 777)]:
        cam = Camera(fov, 0.1, 100.0, pos, d)
        ours = camera_matrices(cam, w, h)
        ref = po.camera_matrices(pos, d, fov, 0.1, 100.0, w, h)
        for a, b in zip(ours, ref):
            assert bit_mismatches(a.reshape(-1), b) == 0


def test_primary_directions_bit_exact(po):
    sc = scenes.config0().with_resolution(320, 180)
    view = po.view_for(sc)
    with Renderer() as r:
        r.on_resize(sc.width, sc.height)
        r.set_camera_matrices(np.array(view.inv_view), np.array(view.inv_proj), sc.camera_position)
        gpu = r.primary_directions()
    ref = po.ray_dirs(view, po.EXACT)
    assert bit_mismatches(gpu, ref) == 0


def test_nearest_hit_index_and_t_bit_exact(po):
    rng = np.random.default_rng(7)
    sc = scenes.config1()
    n = 20000
    o = rng.uniform(-25, 25, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    with Renderer() as r:
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        t, ids = r.trace_nearest(o, d)
    rt, rids = po.trace(sc.spheres, o, d, po.EXACT)
    assert np.array_equal(ids, rids)
    assert bit_mismatches(t, rt) == 0
    assert (ids >= 0).mean() > 0.05


def test_nearest_hit_ties_lowest_index_and_inside_origin(po):
    from ataraxia_gb300 import SPHERE_DTYPE, MATERIAL_DTYPE

    s = np.zeros(4, dtype=SPHERE_DTYPE)
    s["center"] = [[0, 0, -5], [0, 0, -5], [0, 0, 0], [0, 0, -20]]   # 0 and 1 coincide, origin inside 2
    s["radius"] = [1, 1, 2, 1]
    m = np.zeros(1, dtype=MATERIAL_DTYPE)
    o = np.zeros((2, 3), dtype=np.float32)
    d = np.array([[0, 0, -1], [0, 0, 1]], dtype=np.float32)
    with Renderer() as r:
        r.set_scene(s, m, np.zeros(0, dtype=scenes.LIGHT_DTYPE))
        t, ids = r.trace_nearest(o, d)
    assert ids[0] == 0 and abs(t[0] - 4.0) < 1e-5       # lowest index wins the tie; sphere 2 never hit
    assert ids[1] == -1 and t[1] == -1.0                  # only the enclosing sphere lies that way
    rt, rids = po.trace(s, o, d, po.EXACT)
    assert np.array_equal(ids, rids)


@pytest.mark.parametrize("name,res,spp", [("config0", (160, 90), 4), ("config1", (192, 108), 16),
                                          ("default", (160, 90), 3)])
def test_frames_bit_exact(po, name, res, spp):
    sc = {"config0": scenes.config0, "config1": scenes.config1,
          "default": scenes.reference_default_scene}[name]().with_resolution(*res)
    acc, img = gpu_render(sc, spp)
    ref, _, _ = oracle_render(sc, spp)
    assert bit_mismatches(acc, ref) == 0
    assert np.array_equal(img, po.pack_rgba8(ref, spp))


def test_split_launches_equal_one_launch_and_frame_index(po):
    sc = scenes.config0().with_resolution(128, 72)
    view = po.view_for(sc)
    with Renderer() as r:
        acc, _ = gpu_render(sc, 5, frames_before=3, renderer=r, view=view)
        assert r.frame_index == 9
    ref, _, _ = oracle_render(sc, 8)
    assert bit_mismatches(acc, ref) == 0


def test_many_small_waves_bit_exact(po):
    # wave capacity far below the image forces pixel ranges and sample chunks
    sc = scenes.config1().with_resolution(97, 31)
    acc, img = gpu_render(sc, 40, wave_paths=1000)
    ref, _, _ = oracle_render(sc, 40)
    assert bit_mismatches(acc, ref) == 0
    assert np.array_equal(img, po.pack_rgba8(ref, 40))


def test_accumulation_off_and_reset(po):
    sc = scenes.config0().with_resolution(64, 36)
    view = po.view_for(sc)
    with Renderer() as r:
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        r.set_camera_matrices(np.array(view.inv_view), np.array(view.inv_proj), sc.camera_position)
        r.set_settings(Settings(accumulation=False, skyLight=False, maxBounces=5))
        r.render_frames(1)
        r.render_frames(1)
        assert r.frame_index == 1
        a1 = r.get_accumulation().reshape(-1, 4).copy()
        ref1, _, _ = oracle_render(sc, 1)
        assert bit_mismatches(a1, ref1) == 0
        r.set_settings(Settings(accumulation=True, skyLight=False, maxBounces=5))
        r.render_frames(2)
        assert r.frame_index == 3
        r.reset_frame_index()
        r.render_frames(1)
        a2 = r.get_accumulation().reshape(-1, 4)
        assert bit_mismatches(a2, ref1) == 0
        r.on_resize(32, 16)
        assert r.frame_index == 1


@pytest.mark.parametrize("res", [(1, 1), (37, 23), (3, 200)])
def test_ragged_sizes(po, res):
    sc = scenes.config1().with_resolution(*res)
    acc, img = gpu_render(sc, 3)
    ref, _, _ = oracle_render(sc, 3)
    assert bit_mismatches(acc, ref) == 0


@pytest.mark.parametrize("bounces", [0, 1, 2, 40])
def test_bounce_depths(po, bounces):
    sc = scenes.config0().with_resolution(48, 27)
    acc, _ = gpu_render(sc, 2, max_bounces=bounces)
    ref, _, _ = oracle_render(sc, 2, max_bounces=bounces)
    assert bit_mismatches(acc, ref) == 0


def test_sky_light_and_emission(po):
    sc = scenes.config0().with_resolution(64, 36)
    mats = sc.materials.copy()
    mats["emission_color"][2] = [1.0, 0.5, 0.25]
    mats["emission_intensity"][2] = 3.0
    sc = scenes.SyntheticScene(**{**sc.__dict__, "materials": mats})
    acc, _ = gpu_render(sc, 3, sky=True)
    ref, _, _ = oracle_render(sc, 3, sky=True)
    assert bit_mismatches(acc, ref) == 0


@pytest.mark.parametrize("n_lights,spp", [(32, 8), (33, 8), (5, 1), (31, 40), (70, 3)])
def test_first_bounce_light_visibility_per_pixel(po, n_lights, spp):
    # up to 32 lights a pixel's samples share one shadow ray per distinct light
    # at the first bounce; above that every sample casts its own.  Up to 64
    # lights shadow rays go through the light buffer, above that the whole table
    sc = scenes.config1().with_resolution(72, 40)
    rng = np.random.default_rng(n_lights)
    lights = np.zeros(n_lights, dtype=scenes.LIGHT_DTYPE)
    lights["position"] = rng.normal(0.0, 25.0, (n_lights, 3))
    lights["color"] = rng.uniform(0.5, 1.0, (n_lights, 3))
    lights["intensity"] = rng.uniform(20.0, 200.0, n_lights)
    sc = scenes.SyntheticScene(**{**sc.__dict__, "lights": lights})
    acc, img = gpu_render(sc, spp)
    ref, _, _ = oracle_render(sc, spp)
    assert bit_mismatches(acc, ref) == 0
    assert np.array_equal(img, po.pack_rgba8(ref, spp))


def _cone_scene(kind):
    st = scenes.Stream(7, "cone-" + kind)
    mats = scenes.draw_materials(st, 8)
    if kind == "far_narrow":     # distant camera, 3 deg: most primary rays pass within float error of a sphere
        n = 500                  # below the LBVH threshold: brute-force tables with their buffers
        c = st.uniform(3 * n, -5, 5).reshape(n, 3)
        r = st.uniform(n, 0.05, 0.45)
        cam, look, fov, far = (0.0, 30.0, 400.0), (0.0, -30.0, -400.0), 3.0, 1000.0
        lts = scenes.draw_lights(st, 4, 8.0)
    elif kind == "inside":       # camera inside a large sphere, small spheres around it and behind it
        n = 200
        c = np.concatenate([np.zeros((1, 3)), st.uniform(3 * (n - 1), -30, 30).reshape(n - 1, 3)])
        r = np.concatenate([[50.0], st.uniform(n - 1, 0.2, 2.0)])
        cam, look, fov, far = (0.0, 0.0, 5.0), (0.3, -0.2, -1.0), 60.0, 100.0
        lts = scenes.draw_lights(st, 6, 10.0)
    else:                        # spheres touching the near plane; lights on and inside sphere surfaces
        n = 64
        c = np.concatenate([[[0.6, 0.0, 0.0]], st.uniform(3 * (n - 1), -3, 3).reshape(n - 1, 3)])
        r = np.concatenate([[0.45], st.uniform(n - 1, 0.05, 0.6)])
        cam, look, fov, far = (0.0, 0.0, 0.5), (0.0, 0.0, -1.0), 70.0, 100.0
        lts = np.zeros(3, dtype=scenes.LIGHT_DTYPE)
        lts["position"] = [c[1], c[2] + [0.0, r[2], 0.0], [0.0, 4.0, 2.0]]
        lts["color"] = 1.0
        lts["intensity"] = [30.0, 60.0, 90.0]
    sph = np.zeros(n, dtype=scenes.SPHERE_DTYPE)
    sph["center"] = c
    sph["radius"] = r
    sph["material"] = np.arange(n) % 8
    return scenes.SyntheticScene("cone-" + kind, sph, mats, lts, cam, look, fov=fov, far=far, width=96, height=64,
                                 max_bounces=4)


@pytest.mark.parametrize("kind", ["far_narrow", "inside", "near"])
def test_warp_cone_culling_edge_cases(po, kind):
    # the warp-cone culling of primary rays and first-bounce shadow rays must
    # never drop a sphere the float test accepts: grazing rays from far away,
    # a camera inside a sphere, spheres at the near plane, lights on surfaces
    sc = _cone_scene(kind)
    acc, img = gpu_render(sc, 6)
    ref, _, _ = oracle_render(sc, 6)
    assert bit_mismatches(acc, ref) == 0
    assert np.array_equal(img, po.pack_rgba8(ref, 6))
    o = np.repeat(np.asarray(sc.camera_position, np.float32)[None], sc.pixels, 0)
    d = np.asarray(po.ray_dirs(po.view_for(sc), po.EXACT), np.float32).reshape(-1, 3)
    _, rids = po.trace(sc.spheres, o, d, po.EXACT)
    assert (rids >= 0).mean() > 0.05    # the primary rays do meet spheres


@pytest.mark.parametrize("n", [1024, 1025])
def test_direction_buffer_limit_and_packed_spheres(po, n):
    # touching and overlapping spheres (continuation rays leave one sphere and
    # graze its neighbours), lights in the gaps, at the direction buffer's
    # 1,024-sphere limit and one sphere above it (the LBVH)
    st = scenes.Stream(11, "packed")
    g = int(np.ceil(n ** (1.0 / 3.0)))
    ijk = np.stack(np.meshgrid(np.arange(g), np.arange(g), np.arange(g), indexing="ij"), -1).reshape(-1, 3)[:n]
    c = (ijk - (g - 1) / 2.0).astype(np.float64)
    r = np.where(np.arange(n) % 3 == 0, 0.5, 0.5 + 0.02 * st.uniform(n, 0.0, 1.0))
    sph = np.zeros(n, dtype=scenes.SPHERE_DTYPE)
    sph["center"] = c
    sph["radius"] = r
    sph["material"] = np.arange(n) % 8
    lts = np.zeros(4, dtype=scenes.LIGHT_DTYPE)
    lts["position"] = [[0.5, 0.5, 0.5], [-1.5, 0.5, 2.5], [0.0, 0.3 * g, 1.5 * g], [0.0, 2.0 * g, 0.0]]
    lts["color"] = 1.0
    lts["intensity"] = [20.0, 40.0, 800.0, 500.0]
    sc = scenes.SyntheticScene("packed", sph, scenes.draw_materials(st, 8), lts, (0.0, 0.6 * g, 2.0 * g),
                               (0.0, -0.6 * g, -2.0 * g), fov=50.0, far=1000.0, width=48, height=32, max_bounces=6)
    acc, img = gpu_render(sc, 4)
    ref, _, _ = oracle_render(sc, 4)
    assert bit_mismatches(acc, ref) == 0
    assert np.array_equal(img, po.pack_rgba8(ref, 4))


def test_empty_scene_no_lights_and_bad_material_ids(po):
    sc = scenes.config0().with_resolution(40, 20)
    empty = scenes.SyntheticScene(**{**sc.__dict__, "spheres": sc.spheres[:0]})
    acc, _ = gpu_render(empty, 2, sky=True)
    ref, _, _ = oracle_render(empty, 2, sky=True)
    assert bit_mismatches(acc, ref) == 0

    nolight = scenes.SyntheticScene(**{**sc.__dict__, "lights": sc.lights[:0]})
    acc, _ = gpu_render(nolight, 2, sky=True)
    ref, _, _ = oracle_render(nolight, 2, sky=True)
    assert bit_mismatches(acc, ref) == 0

    sph = sc.spheres.copy()
    sph["material"][:3] = [-1, 8, 1000]       # out of range -> material 0 (Renderer.cu:30-37)
    bad = scenes.SyntheticScene(**{**sc.__dict__, "spheres": sph})
    acc, _ = gpu_render(bad, 2)
    ref, _, _ = oracle_render(bad, 2)
    assert bit_mismatches(acc, ref) == 0


def test_invalid_arguments_raise():
    sc = scenes.config0()
    with Renderer() as r:
        with pytest.raises(AtxError) as e:
            r.on_resize(0, 10)
        assert e.value.status == 1
        with pytest.raises(AtxError):
            r.render_frames(1)                      # no resize yet
        with pytest.raises(AtxError):
            r.set_scene(sc.spheres, sc.materials[:0], sc.lights)   # spheres without materials
        r.on_resize(8, 8)
        r.render_frames(0)                          # no-op
        assert r.frame_index == 1


def test_literal_reference_order_within_fma_contraction_spread(po):
    """Counted and reported: pixels outside 1e-3 against the reference's expressions evaluated
    literally.  The reference's quadratic loses ~1e-4 in t at camera distance ~60 (cancellation in
    b^2 - a c), more than its 1e-4 surface offset, so the literal expressions compiled with and
    without FMA contraction already disagree on a few percent of pixels; the kernels stay within 1.25
    times that spread plus 0.1% (measured: 0.09% vs 0.05% on the small scene, 2.05% vs 1.87% on the
    medium one)."""
    for sc, spp in [(scenes.config0().with_resolution(160, 90), 4), (scenes.config1().with_resolution(192, 108), 4)]:
        acc, _ = gpu_render(sc, spp)
        lit, _, _ = oracle_render(sc, spp, mode=po.LITERAL)
        con, _, _ = oracle_render(sc, spp, mode=po.LITERAL, contract=True)
        ours = frac_outside(acc, lit)
        spread = frac_outside(con, lit)
        print(f"{sc.name}: outside 1e-3 vs literal {ours:.4%}; contraction spread {spread:.4%}")
        assert ours <= 1.25 * spread + 0.001


def test_converged_image_within_3_sigma_of_float64(po):
    """4096 frames of the medium scene at its full 1920x1080 on the GPU against the reference's
    expressions evaluated in float64 with the same random stream: each pixel's mean lies within 3
    standard errors (estimated from the float64 per-frame samples) on at least 99.5% of (pixel,
    channel) pairs, over 2,000 pixels drawn from those whose primary ray hits a sphere (the others are
    exact closed forms).  The random stream is the same, so the differences are the float32
    evaluation's own: a glossy lobe amplifies the quadratic's cancellation error into a percent of
    radiance on a few pixels (measured: 99.77% of 6,000 pairs within 3 sigma)."""
    sc = scenes.config1()
    spp = 4096
    view = po.view_for(sc)
    dirs = po.ray_dirs(view)
    origins = np.repeat(np.asarray(sc.camera_position, dtype=np.float32)[None, :], len(dirs), axis=0)
    _, ids = po.trace(sc.spheres, origins, dirs)
    hit_px = np.flatnonzero(ids >= 0)
    rng = np.random.default_rng(0)
    px = np.sort(rng.choice(hit_px, size=min(2000, len(hit_px)), replace=False)).astype(np.uint32)
    acc, _ = gpu_render(sc, spp)
    ref, smp, _ = po.render(sc.spheres, sc.materials, sc.lights, view, max_bounces=sc.max_bounces, spp=spp,
                            pixels=px, f64=True, samples=True)
    gpu_mean = acc[px, :3].astype(np.float64) / spp
    f64_mean = ref[:, :3] / spp
    sem = smp[:, :, :3].std(axis=1) / np.sqrt(spp)
    ok = np.abs(gpu_mean - f64_mean) <= 3.0 * sem + 1e-6
    print(f"within 3 sigma: {ok.mean():.4%} of {ok.size} (pixel, channel) pairs; "
          f"max |diff| / sigma {np.max(np.abs(gpu_mean - f64_mean) / (sem + 1e-12)):.2f}")
    assert ok.mean() >= 0.995


@pytest.mark.parametrize("bvh_threshold", [0, 1])
def test_primary_tile_masks_follow_scene_and_eye(po, bvh_threshold):
    """The per-camera primary tile masks (brute-force tables) and tile candidate lists (LBVH, forced
    with bvh_threshold=1) are rebuilt when the spheres or the eye change: renders after a scene change
    under the same camera and after an eye move are bit-exact against fresh oracle renders (stale
    masks or lists would miss the moved spheres)."""
    base = scenes.config1().with_resolution(96, 54)
    moved = scenes.SyntheticScene(**{**base.__dict__, "spheres": base.spheres.copy()})
    moved.spheres["center"] += np.array([3.0, -1.5, 2.0], dtype=np.float32)
    eye = scenes.SyntheticScene(**{**moved.__dict__, "camera_position": tuple(
        float(v) + dv for v, dv in zip(moved.camera_position, (4.0, 2.0, -3.0)))})
    with Renderer(bvh_threshold=bvh_threshold) as r:
        r.on_resize(base.width, base.height)
        r.set_settings(Settings(accumulation=True, skyLight=False, maxBounces=base.max_bounces))
        for sc in (base, moved, eye):
            view = po.view_for(sc)
            r.set_scene(sc.spheres, sc.materials, sc.lights)
            r.set_camera_matrices(np.array(view.inv_view), np.array(view.inv_proj), sc.camera_position)
            r.reset_frame_index()
            r.render_frames(1)   # camera or scene just changed: no masks or lists yet
            r.render_frames(2)   # the camera stayed put: built for it
            acc = r.get_accumulation().reshape(-1, 4).copy()
            ref, _, _ = oracle_render(sc, 3)
            assert bit_mismatches(acc, ref) == 0
            assert r.stats()["bvh_in_use"] == (1 if bvh_threshold == 1 else 0)
