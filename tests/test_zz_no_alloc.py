"""atx_render_noalloc: the render entry point for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc: code embedded in a runtime that owns every device allocation
through its own pool, or code that must not allocate because cudaMalloc/cudaFree synchronise the
device or are not allowed where it runs.  atx_render_noalloc takes the caller's device buffers for
inputs and outputs and keeps all of its scratch in a fixed array inside libatx.so.  This test calls it
through the C ABI twice in a row (the second call continues the first's accumulation) and checks
both results bit for bit against the allocating entry point (atx_render on a renderer).  The inputs
here are placed on the device by torch; the entry point itself allocates nothing.

Kept in its own file named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, arr: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.uint8).copy()).cuda()


def test_noalloc_matches_renderer_on_two_calls(po):
    torch = pytest.importorskip("torch")
    from ataraxia_gb300 import Renderer, Settings, scenes
    from ataraxia_gb300 import _native as N
    from tests.helpers import bit_mismatches

    sc = scenes.config1().with_resolution(320, 180)      # two waves of the fixed scratch
    view = po.view_for(sc)
    iv = np.array(view.inv_view, dtype=np.float32)
    ip = np.array(view.inv_proj, dtype=np.float32)
    pos = np.array(sc.camera_position, dtype=np.float32)
    px = sc.width * sc.height

    d_sph, d_mat, d_lts = _dev(torch, sc.spheres), _dev(torch, sc.materials), _dev(torch, sc.lights)
    d_acc = torch.full((px * 4,), 7.0, dtype=torch.float32, device="cuda")   # stale contents: frame 1 clears
    d_img = torch.zeros((px,), dtype=torch.int32, device="cuda")
    settings = N.Settings(1, 0, (C.c_uint8 * 2)(), sc.max_bounces)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def noalloc(frame_index, spp):
        st = N.lib().atx_render_noalloc(
            C.c_void_p(d_sph.data_ptr()), len(sc.spheres), C.c_void_p(d_mat.data_ptr()), len(sc.materials),
            C.c_void_p(d_lts.data_ptr()), len(sc.lights), N.ptr(iv), N.ptr(ip), N.ptr(pos), sc.width, sc.height,
            C.byref(settings), frame_index, spp, C.c_void_p(d_acc.data_ptr()), C.c_void_p(d_img.data_ptr()), stream)
        N.check(st)
        torch.cuda.synchronize()
        return d_acc.cpu().numpy().reshape(-1, 4), d_img.cpu().numpy().view(np.uint32)

    with Renderer() as r:
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        r.set_camera_matrices(iv, ip, pos)
        r.set_settings(Settings(accumulation=True, skyLight=False, maxBounces=sc.max_bounces))
        for frame_index, spp in ((1, 8), (9, 8)):
            acc, img = noalloc(frame_index, spp)
            r.render_frames(spp)
            ref_acc = r.get_accumulation().reshape(-1, 4)
            ref_img = r.get_image().reshape(-1)
            assert bit_mismatches(acc, ref_acc) == 0
            assert np.array_equal(img, ref_img)


def _limit_scene(case: str):
    """Scenes at the entry point's documented limits, each at a small resolution."""
    from ataraxia_gb300 import scenes

    base = scenes.config1().with_resolution(64, 36)
    if case == "spheres_16384":
        big = scenes.config2()
        return scenes.SyntheticScene(**{**big.__dict__, "spheres": big.spheres[:16384].copy(),
                                        "width": 64, "height": 36, "max_bounces": 4}), True, True
    if case == "lights_1024":
        lts = scenes.draw_lights(scenes.Stream(11, "noalloc-lights"), 1024, 30.0)
        return scenes.SyntheticScene(**{**base.__dict__, "lights": lts}), True, True
    if case == "lights_33_accumulation_off_no_image":
        lts = scenes.draw_lights(scenes.Stream(12, "noalloc-lights"), 33, 30.0)
        return scenes.SyntheticScene(**{**base.__dict__, "lights": lts}), False, False
    if case == "bounces_1024":
        # the camera inside a large white sphere whose albedo is 1: roulette keeps p = 1, so every path
        # that hits runs all 1,024 bounces
        sph = np.concatenate([base.spheres, base.spheres[:1].copy()])
        sph["center"][-1] = 0.0
        sph["radius"][-1] = 200.0
        sph["material"][-1] = len(base.materials)
        white = base.materials[:1].copy()
        white["albedo"] = 1.0
        white["metallic"] = 0.0
        white["f0"] = 0.04
        white["roughness"] = 1.0
        mats = np.concatenate([base.materials, white])
        return scenes.SyntheticScene(**{**base.__dict__, "spheres": sph, "materials": mats, "width": 32,
                                        "height": 18, "max_bounces": 1024}), True, True
    raise ValueError(case)


LIMIT_CASES = ["spheres_16384", "lights_1024", "lights_33_accumulation_off_no_image", "bounces_1024"]


@pytest.mark.parametrize("case", LIMIT_CASES)
def test_noalloc_at_its_limits_matches_renderer(po, case):
    """The documented limits rendered on the GPU, twice in a row, bit for bit against atx_render:
    16,384 spheres (a sphere table beyond shared memory), 1,024 lights (one shadow ray per sample, no
    light buffer), 33 lights with accumulation off and no image, 1,024 bounces (the deepest counter
    layout)."""
    torch = pytest.importorskip("torch")
    from ataraxia_gb300 import Renderer, Settings
    from ataraxia_gb300 import _native as N
    from tests.helpers import bit_mismatches

    sc, accumulate, with_image = _limit_scene(case)
    view = po.view_for(sc)
    iv = np.array(view.inv_view, dtype=np.float32)
    ip = np.array(view.inv_proj, dtype=np.float32)
    pos = np.array(sc.camera_position, dtype=np.float32)
    px = sc.width * sc.height
    d_sph, d_mat, d_lts = _dev(torch, sc.spheres), _dev(torch, sc.materials), _dev(torch, sc.lights)
    d_acc = torch.full((px * 4,), 3.0, dtype=torch.float32, device="cuda")
    d_img = torch.full((px,), 0x5A5A5A5A, dtype=torch.int32, device="cuda")
    settings = N.Settings(int(accumulate), 0, (C.c_uint8 * 2)(), sc.max_bounces)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    spp = 2
    with Renderer() as r:
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        r.set_camera_matrices(iv, ip, pos)
        r.set_settings(Settings(accumulation=accumulate, skyLight=False, maxBounces=sc.max_bounces))
        for call in range(2):
            frame_index = 1 + call * spp if accumulate else 1
            st = N.lib().atx_render_noalloc(
                C.c_void_p(d_sph.data_ptr()), len(sc.spheres), C.c_void_p(d_mat.data_ptr()), len(sc.materials),
                C.c_void_p(d_lts.data_ptr()), len(sc.lights), N.ptr(iv), N.ptr(ip), N.ptr(pos), sc.width,
                sc.height, C.byref(settings), frame_index, spp, C.c_void_p(d_acc.data_ptr()),
                C.c_void_p(d_img.data_ptr()) if with_image else None, stream)
            N.check(st)
            torch.cuda.synchronize()
            r.render_frames(spp)
            acc = d_acc.cpu().numpy().reshape(-1, 4)
            assert bit_mismatches(acc, r.get_accumulation().reshape(-1, 4)) == 0
            img = d_img.cpu().numpy().view(np.uint32)
            if with_image:
                assert np.array_equal(img, r.get_image().reshape(-1))
            else:
                assert np.all(img == 0x5A5A5A5A)          # image = NULL: never written


def test_noalloc_rejects_frames_past_the_index_range():
    from ataraxia_gb300 import _native as N

    settings = N.Settings(1, 0, (C.c_uint8 * 2)(), 8)
    m = np.zeros(16, dtype=np.float32)
    dummy = C.c_void_p(16)            # never dereferenced: the argument checks come first
    st = N.lib().atx_render_noalloc(dummy, 1, dummy, 1, None, 0, N.ptr(m), N.ptr(m), N.ptr(m), 8, 8,
                                    C.byref(settings), 0xFFFFFFF0, 32, dummy, None, None)
    assert st == 1 and b"frame index" in N.lib().atx_last_error()


def test_noalloc_rejects_sizes_beyond_its_limits():
    from ataraxia_gb300 import _native as N

    settings = N.Settings(1, 0, (C.c_uint8 * 2)(), 8)
    m = np.zeros(16, dtype=np.float32)
    dummy = C.c_void_p(16)            # never dereferenced: the size checks come first
    st = N.lib().atx_render_noalloc(dummy, 16385, dummy, 1, None, 0, N.ptr(m), N.ptr(m), N.ptr(m), 8, 8,
                                    C.byref(settings), 1, 1, dummy, None, None)
    assert st == 1 and b"16384" in N.lib().atx_last_error()
    big = N.Settings(1, 0, (C.c_uint8 * 2)(), 5000)
    st = N.lib().atx_render_noalloc(dummy, 1, dummy, 1, None, 0, N.ptr(m), N.ptr(m), N.ptr(m), 8, 8, C.byref(big),
                                    1, 1, dummy, None, None)
    assert st == 1 and b"max_bounces" in N.lib().atx_last_error()
