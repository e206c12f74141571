"""Overlapped renders (ATX_FLAG_OVERLAP_RENDERS): consecutive atx_render calls run their lanes without
joining them into the renderer's stream, so the next render starts while the previous one's sparse
last bounces finish.  Every frame must equal the joined renderer's bit for bit, across reads between
renders, camera changes (camera tables rebuilt on the stream), a new lane split, accumulation off and
a resize."""
import numpy as np
import pytest

from ataraxia_gb300 import Camera, Renderer, Settings, scenes
from ataraxia_gb300 import _native as N
from tests.helpers import bit_mismatches

pytestmark = pytest.mark.gpu


def _setup(r, sc, accumulation=True):
    r.on_resize(sc.width, sc.height)
    r.set_scene(sc.spheres, sc.materials, sc.lights)
    r.set_camera(Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction))
    r.set_settings(Settings(accumulation=accumulation, skyLight=False, maxBounces=sc.max_bounces))


@pytest.mark.parametrize("kind", ["brute_force", "lbvh"])
def test_overlapped_renders_equal_joined_renders(kind):
    if kind == "lbvh":
        big = scenes.config2()
        sc = scenes.SyntheticScene(**{**big.__dict__, "spheres": big.spheres[:4096].copy(), "width": 1280,
                                      "height": 720, "max_bounces": 6})
    else:
        sc = scenes.config1().with_resolution(1280, 720)
    moved = Camera(sc.fov, sc.near, sc.far, tuple(v + dv for v, dv in zip(sc.camera_position, (2.0, 1.0, -3.0))),
                   sc.camera_direction)
    # 24 frames of 1280x720 are 22 Mi paths: enough for four lanes
    script = [("render", 24), ("render", 24), ("render", 8), ("read", None), ("render", 24), ("render", 24),
              ("camera", moved), ("render", 12), ("render", 12), ("render", 12), ("lanes", 1), ("render", 24),
              ("lanes", 4), ("render", 24), ("render", 24), ("read", None), ("render", 24)]
    outs = []
    for flags in (0, N.FLAG_OVERLAP_RENDERS):
        got = []
        with Renderer(flags=flags) as r:
            _setup(r, sc)
            for op, arg in script:
                if op == "render":
                    r.render_frames(arg)
                elif op == "read":
                    got.append(r.get_image().reshape(-1).copy())
                elif op == "camera":
                    r.set_camera(arg)
                    r.reset_frame_index()
                elif op == "lanes":
                    r.set_tuning(lanes=arg)
            got.append(r.get_accumulation().reshape(-1, 4).copy())
            got.append(r.get_image().reshape(-1).copy())
            assert r.frame_index == 1 + 12 * 3 + 24 * 4
        outs.append(got)
    for a, b in zip(*outs):
        if a.dtype == np.float32:
            assert bit_mismatches(a, b) == 0
        else:
            assert np.array_equal(a, b)


def test_overlapped_accumulation_off_resize_and_join():
    sc = scenes.config1().with_resolution(960, 540)
    with Renderer() as ref, Renderer(flags=N.FLAG_OVERLAP_RENDERS) as r:
        for x in (ref, r):
            _setup(x, sc, accumulation=False)
            for _ in range(3):
                x.render_frames(16)
        r.join()
        assert bit_mismatches(r.get_accumulation().reshape(-1, 4), ref.get_accumulation().reshape(-1, 4)) == 0
        big = sc.with_resolution(1280, 720)
        for x in (ref, r):
            x.on_resize(big.width, big.height)
            x.set_settings(Settings(accumulation=True, skyLight=False, maxBounces=big.max_bounces))
            x.render_frames(16)
            x.render_frames(16)
        assert bit_mismatches(r.get_accumulation().reshape(-1, 4), ref.get_accumulation().reshape(-1, 4)) == 0
        assert np.array_equal(r.get_image(), ref.get_image())


@pytest.mark.parametrize("flags", [0, N.FLAG_OVERLAP_RENDERS])
def test_async_image_reads_double_buffered(flags):
    """atx_read_image_async after every render into two alternating host buffers, each waited for one
    render later (while the next render runs): every image equals a synchronous read of the joined
    renderer after the same render."""
    sc = scenes.config1().with_resolution(1280, 720)
    want = []
    with Renderer() as ref:
        _setup(ref, sc)
        for k in range(6):
            ref.render_frames(16 if k % 3 else 8)
            want.append(ref.get_image().reshape(-1).copy())
    got = []
    with Renderer(flags=flags) as r:
        _setup(r, sc)
        bufs = [np.zeros(sc.width * sc.height, np.uint32) for _ in range(2)]
        tickets = []
        for k in range(6):
            r.render_frames(16 if k % 3 else 8)
            tickets.append(r.read_image_async(bufs[k % 2]))
            if k >= 1:
                r.wait_read(tickets[k - 1])
                got.append(bufs[(k - 1) % 2].copy())
        r.wait_read(tickets[-1])
        got.append(bufs[5 % 2].copy())
        r.wait_read(tickets[0])                  # an old ticket: already landed
        with pytest.raises(Exception):
            r.wait_read(len(tickets))            # never issued
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
