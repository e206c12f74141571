"""The C-ABI library: loads without a GPU, exports every entry point include/*.h declares, and its
host-only helpers work on the CPU.  No compute call is made here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        names.update(re.findall(r"ATX_API\s+[\w\s\*]+?\b(atx_\w+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported(native):
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, missing


def test_binding_covers_every_symbol():
    from ataraxia_gb300 import _native as N

    assert set(declared_symbols()) <= set(N.SIGNATURES), set(declared_symbols()) - set(N.SIGNATURES)


def test_struct_layouts_match_reference_sizes():
    from ataraxia_gb300 import LIGHT_DTYPE, MATERIAL_DTYPE, SPHERE_DTYPE
    from ataraxia_gb300 import _native as N

    assert SPHERE_DTYPE.itemsize == 20        # SceneNode.h:11-21
    assert MATERIAL_DTYPE.itemsize == 52      # Scene.h:28-47
    assert LIGHT_DTYPE.itemsize == 28         # Scene.h:17-26
    assert C.sizeof(N.Settings) == 8          # Scene.h:49-56 (bool, bool, int)
    assert N.Settings.max_bounces.offset == 4
    assert C.sizeof(N.Config) == 32 and C.sizeof(N.Stats) == 72


def test_version_and_status_strings(native):
    from ataraxia_gb300 import _native as N

    assert native.atx_abi_version() == 1
    for code, name in N.STATUS.items():
        s = native.atx_status_string(code)
        assert s and isinstance(s, bytes)
    assert native.atx_status_string(999) == b"unknown status"


def test_no_device_is_reported_not_fatal(native):
    import ataraxia_gb300 as atx

    if atx.device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(atx.AtxError) as e:
        atx.Renderer()
    assert e.value.status == 8                # ATX_ERR_NO_DEVICE
    assert b"device" in native.atx_last_error().lower()


def test_null_arguments_are_invalid(native):
    from ataraxia_gb300 import _native as N

    assert native.atx_renderer_create(None, None) == 1
    assert native.atx_resize(None, 4, 4) == 1
    assert native.atx_render(None, 1) == 1
    assert native.atx_get_stats(None, None) == 1
    assert native.atx_camera_matrices(None, 4, 4, None, None, None, None) == 1
    d = N.CameraDesc()
    assert native.atx_camera_matrices(C.byref(d), 0, 4, None, None, None, None) == 1


def test_host_camera_matrices_match_oracle(po):
    from ataraxia_gb300 import Camera, camera_matrices

    for pos, d, fov, near, far, w, h in [((0, 2, 10), (0, -0.19611613, -0.98058068), 45.0, 0.1, 100.0, 1280, 720),
                                         ((0, 12, 60), (0, -0.19611613, -0.98058068), 45.0, 0.1, 100.0, 1920, 1080),
                                         ((3, -1, 2), (-0.6, 0.2, -0.77), 75.0, 0.5, 500.0, 641, 479)]:
        ours = camera_matrices(Camera(fov, near, far, pos, d), w, h)
        ref = po.camera_matrices(pos, d, fov, near, far, w, h)
        for a, b in zip(ours, ref):
            assert np.array_equal(a.reshape(-1).view(np.uint32), b.view(np.uint32))


def test_reference_interface_names_exist():
    import ataraxia_gb300 as atx

    for name in ("onResize", "Render", "getSettings", "setSettings", "resetFrameIndex", "getImage"):
        assert callable(getattr(atx.Renderer, name))
    s = atx.Settings()
    assert (s.accumulation, s.skyLight, s.maxBounces) == (True, False, 15)     # Scene.h:51-53
    c = atx.Camera()
    assert (c.fov, c.nearClip, c.farClip, tuple(c.position), tuple(c.direction)) == \
        (45.0, 0.1, 100.0, (0.0, 0.0, 3.0), (0.0, 0.0, -1.0))                 # Camera.cpp:14-21
