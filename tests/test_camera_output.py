"""Interactive camera update (Camera::onUpdate, Camera.cpp:31-108; reset on motion, main.cpp:22-32)
against the oracle's restatement, and the headless image files (PPM / PAM / PFM) that stand in for
the reference's Vulkan image upload."""
import numpy as np
import pytest

import ataraxia_gb300 as atx


def bits(a):
    return np.asarray(a, dtype=np.float32).view(np.uint32).tolist()


def random_inputs(seed, n=300):
    rng = np.random.default_rng(seed)
    mouse = np.zeros(2)
    out = []
    for _ in range(n):
        if rng.uniform() < 0.7:
            mouse = mouse + rng.integers(-40, 41, 2)
        keys = "".join(k for k in "WSADQE" if rng.uniform() < 0.25)
        out.append((tuple(float(v) for v in mouse), bool(rng.uniform() < 0.8), keys, float(rng.uniform(0.001, 0.05))))
    return out


@pytest.mark.parametrize("seed", range(4))
def test_camera_update_bit_exact_vs_oracle(po, seed):
    cam = atx.Camera(position=(0.0, 2.0, 10.0), direction=(0.0, -0.2, -1.0))
    ctl = atx.CameraController(cam)
    pos = np.array(cam.position, dtype=np.float32)
    d = np.array(cam.direction, dtype=np.float32)
    lm = np.zeros(2, dtype=np.float32)
    for mouse, right, keys, dt in random_inputs(seed):
        moved = ctl.on_update(dt, mouse=mouse, right_button=right, keys=keys)
        m2, pos, d, lm = po.camera_on_update(pos, d, lm, mouse, right, keys, dt)
        assert moved == m2
        assert bits(ctl.camera.position) == bits(pos)
        assert bits(ctl.camera.direction) == bits(d)
        assert bits(list(ctl.last_mouse)) == bits(lm)


def test_camera_update_semantics():
    ctl = atx.CameraController(atx.Camera(position=(0.0, 0.0, 0.0), direction=(0.0, 0.0, -1.0)))
    # without the right button nothing moves, but the cursor position is remembered
    assert not ctl.on_update(0.1, mouse=(100.0, 50.0), right_button=False, keys="W")
    assert tuple(ctl.camera.position) == (0.0, 0.0, 0.0) and list(ctl.last_mouse) == [100.0, 50.0]
    # no delta, no key: not moved
    assert not ctl.on_update(0.1, mouse=(100.0, 50.0), right_button=True)
    # W wins over S; speed 5 along the direction
    assert ctl.on_update(0.1, mouse=(100.0, 50.0), right_button=True, keys="WS")
    np.testing.assert_allclose(ctl.camera.position, (0.0, 0.0, -0.5), atol=1e-6)
    # A wins over D: right = direction x up = (1, 0, 0) here, A moves along -right
    ctl.on_update(0.1, mouse=(100.0, 50.0), right_button=True, keys="AD")
    np.testing.assert_allclose(ctl.camera.position, (-0.5, 0.0, -0.5), atol=1e-6)
    # Q wins over E and moves down
    ctl.on_update(0.1, mouse=(100.0, 50.0), right_button=True, keys="QE")
    np.testing.assert_allclose(ctl.camera.position, (-0.5, -0.5, -0.5), atol=1e-6)
    # a mouse delta of 100 px to the right turns the view 0.06 rad to the right (angleAxis(-yaw, +Y))
    ctl.on_update(0.1, mouse=(200.0, 50.0), right_button=True)
    d = np.array(ctl.camera.direction, dtype=np.float64)
    assert np.isclose(np.linalg.norm(d), 1.0, atol=1e-6)
    assert np.isclose(np.arctan2(d[0], -d[2]), 0.06, atol=1e-5) and d[1] == 0.0


# ------------------------------------------------------------ image files

def read_pnm(path):
    data = path.read_bytes()
    if data.startswith(b"P6"):
        _, w, h, mx, _ = data.split(maxsplit=4)
        off = len(b"P6\n%s %s\n%s\n" % (w, h, mx))
        w, h = int(w), int(h)
        return np.frombuffer(data[off:], dtype=np.uint8).reshape(h, w, 3)
    assert data.startswith(b"P7")
    end = data.index(b"ENDHDR\n") + len(b"ENDHDR\n")
    fields = dict(line.split(b" ", 1) for line in data[:end].split(b"\n")[1:-2])
    w, h, depth = int(fields[b"WIDTH"]), int(fields[b"HEIGHT"]), int(fields[b"DEPTH"])
    assert fields[b"TUPLTYPE"] == b"RGB_ALPHA" and fields[b"MAXVAL"] == b"255"
    return np.frombuffer(data[end:], dtype=np.uint8).reshape(h, w, depth)


def read_pfm(path):
    data = path.read_bytes()
    lines = data.split(b"\n", 3)
    assert lines[0] == b"PF"
    w, h = (int(v) for v in lines[1].split())
    scale = float(lines[2])
    assert scale < 0  # little endian
    return np.frombuffer(lines[3], dtype="<f4").reshape(h, w, 3)


def test_ppm_pam_row_order_and_channels(tmp_path):
    h, w = 3, 4
    rng = np.random.default_rng(0)
    rgba = rng.integers(0, 256, (h, w, 4), dtype=np.uint32)
    px = (rgba[..., 3] << 24) | (rgba[..., 2] << 16) | (rgba[..., 1] << 8) | rgba[..., 0]
    atx.write_image(tmp_path / "a.ppm", px)
    atx.write_image(tmp_path / "a.pam", px)
    ppm = read_pnm(tmp_path / "a.ppm")
    pam = read_pnm(tmp_path / "a.pam")
    # file row 0 is the top of the picture = buffer row h-1
    assert np.array_equal(ppm, rgba[::-1, :, :3].astype(np.uint8))
    assert np.array_equal(pam, rgba[::-1].astype(np.uint8))


def test_pfm_is_accumulated_colour_over_frames(tmp_path):
    h, w = 2, 3
    acc = np.zeros((h, w, 4), dtype=np.float32)
    acc[..., 0] = np.arange(h * w).reshape(h, w)
    acc[..., 1] = 1.5
    acc[..., 2] = -2.0
    acc[..., 3] = 4.0
    acc[1, 2, 3] = 0.0          # no frames: written as 0
    atx.write_pfm(tmp_path / "a.pfm", acc)
    got = read_pfm(tmp_path / "a.pfm")
    want = acc[..., :3] / np.where(acc[..., 3:] > 0, acc[..., 3:], 1)
    want[1, 2] = 0
    assert np.array_equal(got, want.astype(np.float32))     # bottom row first, as the buffer


def test_image_file_errors(tmp_path):
    with pytest.raises(ValueError):
        atx.write_image(tmp_path / "a.png", np.zeros((2, 2), dtype=np.uint32))
    with pytest.raises(atx.AtxError):
        atx.write_image(tmp_path / "a.ppm", np.zeros((0, 2), dtype=np.uint32))
    with pytest.raises(atx.AtxError):
        atx.write_image(tmp_path / "no_such_dir" / "a.ppm", np.zeros((2, 2), dtype=np.uint32))


# ------------------------------------------------------------------- GPU

@pytest.mark.gpu
def test_update_camera_resets_accumulation(tmp_path):
    from ataraxia_gb300 import scenes

    sc = scenes.config0().with_resolution(64, 36)
    cam = atx.Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction)
    with atx.Renderer() as r:
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        r.set_camera(cam)
        r.set_settings(atx.Settings(True, False, sc.max_bounces))
        r.render_frames(3)
        assert r.frame_index == 4
        ctl = atx.CameraController(cam)
        assert not r.update_camera(ctl, 0.016, mouse=(0.0, 0.0), right_button=True)
        assert r.frame_index == 4                       # no motion: accumulation continues
        assert r.update_camera(ctl, 0.016, mouse=(0.0, 0.0), right_button=True, keys="W")
        assert r.frame_index == 1                       # motion: restart
        r.render_frames(2)
        moved_acc = r.get_accumulation().copy()
        # the same camera set directly renders the same frames
        with atx.Renderer() as r2:
            r2.on_resize(sc.width, sc.height)
            r2.set_scene(sc.spheres, sc.materials, sc.lights)
            r2.set_camera(ctl.camera)
            r2.set_settings(atx.Settings(True, False, sc.max_bounces))
            r2.render_frames(2)
            assert np.array_equal(r2.get_accumulation().view(np.uint32), moved_acc.view(np.uint32))
        r.save_image(tmp_path / "out.ppm")
        r.save_image(tmp_path / "out.pfm")
        img = r.get_image()
        atx.write_image(tmp_path / "ref.ppm", img)
        assert (tmp_path / "out.ppm").read_bytes() == (tmp_path / "ref.ppm").read_bytes()
        pfm = read_pfm(tmp_path / "out.pfm")
        acc = r.get_accumulation().reshape(sc.height, sc.width, 4)
        assert np.array_equal(pfm, (acc[..., :3] / acc[..., 3:]).astype(np.float32))
