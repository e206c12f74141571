"""LBVH nearest hit: bit-identical to the brute-force loop (index and t) on a 1M-ray sample of the
large clustered scene, and bit-identical frames when the LBVH is forced on for smaller scenes."""
import numpy as np
import pytest

from ataraxia_gb300 import Renderer, scenes
from tests.helpers import bit_mismatches, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


def _rays(sc, n, rng):
    """Half camera-to-scene rays, half secondary-like rays leaving sphere surfaces in random directions."""
    h = n // 2
    cam = np.array(sc.camera_position, dtype=np.float32)
    tgt = sc.spheres["center"][rng.integers(0, len(sc.spheres), h)] + rng.normal(0, 2.0, (h, 3))
    d1 = tgt - cam
    d1 /= np.linalg.norm(d1, axis=1, keepdims=True)
    o1 = np.broadcast_to(cam, (h, 3))
    k = rng.integers(0, len(sc.spheres), n - h)
    nrm = rng.normal(size=(n - h, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    o2 = sc.spheres["center"][k] + nrm * (sc.spheres["radius"][k][:, None] + 1e-4)
    d2 = rng.normal(size=(n - h, 3)) + nrm
    d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
    o = np.concatenate([o1, o2]).astype(np.float32)
    d = np.concatenate([d1, d2]).astype(np.float32)
    return o, d


def test_lbvh_bit_exact_vs_brute_force_1m_rays(po):
    sc = scenes.config2()
    rng = np.random.default_rng(42)
    o, d = _rays(sc, 1 << 20, rng)
    with Renderer(bvh_threshold=1) as rb, Renderer(bvh_threshold=1 << 30) as rf:
        rb.set_scene(sc.spheres, sc.materials, sc.lights)
        rf.set_scene(sc.spheres, sc.materials, sc.lights)
        assert rb.stats()["bvh_in_use"] == 1 and rf.stats()["bvh_in_use"] == 0
        tb, ib = rb.trace_nearest(o, d)
        tf, i_f = rf.trace_nearest(o, d)
    assert (ib >= 0).mean() > 0.3
    assert np.array_equal(ib, i_f), f"{np.count_nonzero(ib != i_f)} index mismatches"
    assert bit_mismatches(tb, tf) == 0
    # a subset against the CPU oracle's brute force
    sel = rng.choice(len(o), 3000, replace=False)
    rt, ri = po.trace(sc.spheres, o[sel], d[sel], po.EXACT)
    assert np.array_equal(ib[sel], ri)
    assert bit_mismatches(tb[sel], rt) == 0


@pytest.mark.parametrize("leaf", [1, 2, 4, 8])
def test_lbvh_leaf_sizes_and_ties(po, leaf):
    # duplicated spheres create exact ties in t: the lowest index must win as in the brute-force loop
    sc = scenes.config1()
    sph = np.concatenate([sc.spheres, sc.spheres[::3]])
    rng = np.random.default_rng(leaf)
    o = rng.uniform(-25, 25, (50000, 3)).astype(np.float32)
    d = rng.normal(size=(50000, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    with Renderer(bvh_threshold=1, bvh_leaf_size=leaf) as rb:
        rb.set_scene(sph, sc.materials, sc.lights)
        tb, ib = rb.trace_nearest(o, d)
    rt, ri = po.trace(sph, o, d, po.EXACT)
    assert np.array_equal(ib, ri)
    assert bit_mismatches(tb, rt) == 0


@pytest.mark.parametrize("name,res,spp", [("config1", (160, 90), 8), ("config0", (96, 54), 4)])
def test_lbvh_frames_bit_exact(po, name, res, spp):
    sc = {"config0": scenes.config0, "config1": scenes.config1}[name]().with_resolution(*res)
    acc, img = gpu_render(sc, spp, bvh_threshold=1)
    ref, _, _ = oracle_render(sc, spp)
    assert bit_mismatches(acc, ref) == 0
    assert np.array_equal(img, po.pack_rgba8(ref, spp))


def test_large_scene_frames_bit_exact(po):
    sc = scenes.config2().with_resolution(48, 27)
    acc, _ = gpu_render(sc, 2)
    ref, _, _ = oracle_render(sc, 2)
    assert bit_mismatches(acc, ref) == 0


def test_small_scenes_bvh_edge_counts(po):
    from ataraxia_gb300 import LIGHT_DTYPE

    sc = scenes.config1()
    rng = np.random.default_rng(3)
    o = rng.uniform(-25, 25, (4000, 3)).astype(np.float32)
    d = rng.normal(size=(4000, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    for n in (2, 3, 17, 33):
        sph = sc.spheres[:n]
        with Renderer(bvh_threshold=1) as rb:
            rb.set_scene(sph, sc.materials, np.zeros(0, dtype=LIGHT_DTYPE))
            tb, ib = rb.trace_nearest(o, d)
        rt, ri = po.trace(sph, o, d, po.EXACT)
        assert np.array_equal(ib, ri), n
        assert bit_mismatches(tb, rt) == 0


@pytest.mark.parametrize("leaf", [1, 8])
def test_lbvh_axis_aligned_rays(po, leaf):
    """Rays with zero direction components (inverse direction +-inf, slab products +-inf or NaN):
    along the axes through sphere centres and box-aligned offsets, and diagonals in the axis planes."""
    sc = scenes.config2()
    rng = np.random.default_rng(7 + leaf)
    n = 1 << 16
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    s = np.float32(np.sqrt(0.5))
    diag = np.array([[s, s, 0], [s, 0, -s], [0, -s, s], [-s, -s, 0]], np.float32)
    dirs = np.concatenate([axes, diag])
    d = dirs[rng.integers(0, len(dirs), n)]
    k = rng.integers(0, len(sc.spheres), n)
    c = sc.spheres["center"][k].astype(np.float32)
    r = sc.spheres["radius"][k].astype(np.float32)
    # start 40 units behind the target point: a centre (every third ray), a point one radius off the
    # centre across the ray (grazing), or a random point in the scene's extent
    off = rng.integers(0, 3, n)
    side = np.roll(d, 1, axis=1) * r[:, None]
    tgt = np.where(off[:, None] == 0, c, np.where(off[:, None] == 1, c + side,
                   rng.uniform(sc.spheres["center"].min(0), sc.spheres["center"].max(0), (n, 3))))
    o = (tgt - 40.0 * d).astype(np.float32)
    with Renderer(bvh_threshold=1, bvh_leaf_size=leaf) as rb:
        rb.set_scene(sc.spheres, sc.materials, sc.lights)
        tb, ib = rb.trace_nearest(o, d)
    sel = rng.choice(n, 4000, replace=False)
    rt, ri = po.trace(sc.spheres, o[sel], d[sel], po.EXACT)
    assert (ib >= 0).mean() > 0.3
    assert np.array_equal(ib[sel], ri)
    assert bit_mismatches(tb[sel], rt) == 0
