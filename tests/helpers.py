"""Shared test helpers: render a synthetic scene on the GPU through the C ABI with the oracle's own
camera matrices, and compare accumulators."""
from __future__ import annotations

import numpy as np


def gpu_render(sc, spp, *, frames_before=0, renderer=None, sky=False, max_bounces=None, view=None, **cfg):
    """Renders frames 1+frames_before .. frames_before+spp of scene sc; returns (accum [n,4], image [n])."""
    from ataraxia_gb300 import Renderer, Settings
    from oracle import pyoracle as po

    view = view or po.view_for(sc)
    own = renderer is None
    r = renderer or Renderer(device=0, **cfg)
    try:
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        r.set_camera_matrices(np.array(view.inv_view), np.array(view.inv_proj), sc.camera_position)
        mb = sc.max_bounces if max_bounces is None else max_bounces
        r.set_settings(Settings(accumulation=True, skyLight=sky, maxBounces=mb))
        if frames_before:
            r.render_frames(frames_before)
        if spp > 1 and not frames_before:
            # the first render under a new camera goes without the per-camera primary tile masks or
            # lists (built once the camera stays put), the next one with them: both paths checked
            r.render_frames(1)
            r.render_frames(spp - 1)
        else:
            r.render_frames(spp)
        acc = r.get_accumulation().reshape(-1, 4).copy()
        img = r.get_image().reshape(-1).copy()
        return acc, img
    finally:
        if own:
            r.close()


def oracle_render(sc, spp, *, frame0=1, sky=False, max_bounces=None, mode=None, pixels=None, **kw):
    from oracle import pyoracle as po

    view = po.view_for(sc)
    mb = sc.max_bounces if max_bounces is None else max_bounces
    acc, smp, st = po.render(sc.spheres, sc.materials, sc.lights, view, max_bounces=mb, sky=sky, frame0=frame0,
                             spp=spp, mode=po.EXACT if mode is None else mode, pixels=pixels, **kw)
    return acc, smp, st


def bit_mismatches(a: np.ndarray, b: np.ndarray) -> int:
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    assert a.shape == b.shape, (a.shape, b.shape)
    return int(np.count_nonzero(a.view(np.uint32) != b.view(np.uint32)))


def frac_outside(a: np.ndarray, ref: np.ndarray, rel: float = 1e-3, floor: float = 1e-3) -> float:
    """Fraction of pixels whose rgb differs from ref by more than rel (relative to max(|ref|, floor))."""
    d = np.abs(a[:, :3].astype(np.float64) - ref[:, :3]) / np.maximum(np.abs(ref[:, :3]), floor)
    return float((d.max(axis=1) > rel).mean())


def job_bytes_bound(sc):
    """Upper bound of a served job's device bytes: accumulator, image, primary hits and primary
    directions, scene tables, and the LBVH (1,025 spheres and up) or the light and direction buffers."""
    n, nl = len(sc.spheres), len(sc.lights)
    px = sc.width * sc.height
    tables = 24 * n + 48 * len(sc.materials) + 32 * nl + 8 * 256
    bvh = 264 * n if n >= 1025 else 0
    # the server builds its jobs' light and direction buffers at 16 cells along a cube face's edge
    cells = 6 * 16 * 16 * 65          # per light / per sphere: a count and 32 indices per direction cell
    cones = 6 * 16 * 16 * 20 + 4096   # build scratch: the cells' bounding cones
    lb = cells * nl + cones if n < 1025 and 1 <= nl <= 64 else 0
    db = cells * n + cones if n < 1025 else 0
    return tables + bvh + lb + db + 44 * px + 1024
