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
