"""CPU checks of the oracle's pieces against closed forms and independent evaluations.

The reference has no tests or golden vectors, so each restated function is checked here against
an independent computation: the PCG hash against Python integer arithmetic, sin/cos against
float64 libm, the matrices against their defining identities, the BRDF against a float64
evaluation of BRDF.cu's formulas and the samplers against their geometry and distributions.
"""
import math

import numpy as np
import pytest

from ataraxia_gb300 import scenes


def pcg_ref(seed: int) -> int:
    """Random.h:59-64 in Python integers (mod 2^32)."""
    state = (seed * 747796405 + 2891336453) & 0xFFFFFFFF
    word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & 0xFFFFFFFF
    return ((word >> 22) ^ word) & 0xFFFFFFFF


def test_pcg_hash_known_answers(po):
    seeds = [0, 1, 2, 3, 7, 255, 65535, 123456789, 2**31 - 1, 2**31, 2**32 - 1, 2073600 * 17]
    for s in seeds:
        assert po.pcg_hash(s) == pcg_ref(s)
    rng = np.random.default_rng(1)
    for s in rng.integers(0, 2**32, 2000, dtype=np.uint64):
        assert po.pcg_hash(int(s)) == pcg_ref(int(s))


def test_pcg_float_is_hash_over_2_32(po):
    for s in [0, 1, 99, 2**32 - 1, 3141592653]:
        f, s2 = po.pcg_float(s)
        h = pcg_ref(s)
        assert s2 == h                                   # PcgFloat advances the seed to the hash
        assert f == np.float32(np.float32(h) / np.float32(4294967296.0))
        assert 0.0 <= f <= 1.0


def test_sincos2pi_error_bound(po):
    us = np.concatenate([np.linspace(0, 1, 4097, dtype=np.float32),
                         np.random.default_rng(3).random(5000, dtype=np.float32),
                         np.float32([0.125, 0.375, 0.625, 0.875, 1.0, 1e-8, 0.99999994])])
    worst = 0.0
    for u in us:
        c, s = po.sincos2pi(float(u))
        th = 2.0 * math.pi * float(u)
        worst = max(worst, abs(c - math.cos(th)), abs(s - math.sin(th)))
    assert worst < 3e-7


def test_camera_matrices_identities(po):
    pos, d = (0.0, 2.0, 10.0), (0.0, -0.19611613, -0.98058068)
    view, inv_view, proj, inv_proj = po.camera_matrices(pos, d, 45.0, 0.1, 100.0, 1280, 720)
    V, IV = view.reshape(4, 4).T, inv_view.reshape(4, 4).T        # row-major for numpy
    P, IP = proj.reshape(4, 4).T, inv_proj.reshape(4, 4).T
    assert np.allclose(V @ IV, np.eye(4), atol=1e-5)
    assert np.allclose(P @ IP, np.eye(4), atol=1e-5)
    # perspective entries (glm::perspective, right-handed, z in [-1, 1])
    th = math.tan(math.radians(45.0) / 2)
    assert P[0, 0] == pytest.approx(1 / (1280 / 720 * th), rel=1e-6)
    assert P[1, 1] == pytest.approx(1 / th, rel=1e-6)
    assert P[3, 2] == -1.0
    # the view maps the eye to the origin and looks down -Z
    eye = V @ np.array([*pos, 1.0])
    assert np.allclose(eye[:3], 0, atol=1e-5)
    fwd = V[:3, :3] @ np.array(d)
    assert np.allclose(fwd, [0, 0, -1], atol=1e-6)


def test_primary_directions_geometry(po):
    sc = scenes.config0().with_resolution(64, 36)
    v = po.view_for(sc)
    dirs = po.ray_dirs(v, po.EXACT).reshape(36, 64, 3)
    assert np.allclose(np.linalg.norm(dirs, axis=2), 1.0, atol=1e-6)
    # pixel (W/2, H/2) has NDC (0, 0): the camera direction
    assert np.allclose(dirs[18, 32], sc.camera_direction, atol=1e-6)
    # y = 0 is the bottom row (NDC -1), x grows to the right
    assert dirs[0, 32, 1] < dirs[35, 32, 1]
    # every mode computes the directions as the reference's host code does (nothing fused)
    lit = po.ray_dirs(v, po.LITERAL)
    assert np.array_equal(lit.view(np.uint32), dirs.reshape(-1, 3).view(np.uint32))


def cook_torrance_f64(albedo, f0, metallic, rough, n, v, l):
    """BRDF.cu:9-70 in float64."""
    albedo, f0, n, v, l = (np.asarray(x, dtype=np.float64) for x in (albedo, f0, n, v, l))
    h = (v + l) / np.linalg.norm(v + l)
    ndl = max(n @ l, 1e-7)
    ndv = max(n @ v, 1e-7)
    ndh = max(n @ h, 0.0)
    vdh = max(v @ h, 0.0)
    F = f0 + (1 - f0) * (1 - min(max(vdh, 0), 1)) ** 5
    a2 = (rough * rough) ** 2
    D = a2 / (math.pi * (ndh * ndh * (a2 - 1) + 1) ** 2)
    k = (rough + 1) ** 2 / 8
    G = (ndv / (ndv * (1 - k) + k)) * (ndl / (ndl * (1 - k) + k))
    kd = (1 - F) * (1 - metallic)
    spec = D * G * F / (4 * ndl * ndv + 0.001)
    return (kd * (1 - F) * albedo / math.pi + spec) * ndl


def test_cook_torrance_matches_f64(po):
    rng = np.random.default_rng(5)
    for _ in range(300):
        n = rng.normal(size=3); n /= np.linalg.norm(n)
        v = rng.normal(size=3); v /= np.linalg.norm(v)
        l = rng.normal(size=3); l /= np.linalg.norm(l)
        if n @ v < 0:
            v = -v
        if n @ l < 0:
            l = -l
        albedo = rng.random(3)
        metal = float(rng.random() < 0.3)
        f0 = albedo if metal else np.full(3, 0.04)
        rough = float(rng.uniform(0.2, 1.0))
        ref = cook_torrance_f64(albedo, f0, metal, rough, n, v, l)
        for mode in (po.EXACT, po.LITERAL):
            got = po.cook_torrance(albedo, f0, metal, rough, n, v, l, mode)
            assert np.allclose(got, ref, rtol=2e-4, atol=1e-6), (got, ref)


def test_samplers_hemisphere_and_distribution(po):
    rng = np.random.default_rng(9)
    cos_cos, cos_ggx = [], []
    for i in range(4000):
        n = rng.normal(size=3).astype(np.float32); n /= np.linalg.norm(n)
        d, s2 = po.sample_cosine(n, 1000 + i)
        assert s2 != 1000 + i                             # two PcgFloat draws advanced the seed
        assert abs(np.linalg.norm(d) - 1) < 1e-5
        cos_cos.append(float(n @ d))
        g, _ = po.sample_ggx(n, 0.5, 7000 + i)
        cos_ggx.append(float(n @ g))
    cos_cos = np.array(cos_cos)
    assert cos_cos.min() > -1e-5
    # cosine-weighted: E[cos theta] = 2/3
    assert abs(cos_cos.mean() - 2 / 3) < 0.02
    # GGX half vector with alpha = r^2 = 0.25: cos^2 = (1-u)/(1+(a^2-1)u) -> mostly near the normal
    cos_ggx = np.array(cos_ggx)
    assert cos_ggx.min() > -1e-5 and np.median(cos_ggx) > 0.95


def test_sampler_exact_vs_literal_close(po):
    rng = np.random.default_rng(11)
    for i in range(500):
        n = rng.normal(size=3).astype(np.float32); n /= np.linalg.norm(n)
        a, sa = po.sample_cosine(n, i * 7919, po.EXACT)
        b, sb = po.sample_cosine(n, i * 7919, po.LITERAL)
        assert sa == sb and np.abs(a - b).max() < 2e-6


def test_trace_rules(po):
    from oracle.pyoracle import SPHERE_DTYPE

    s = np.zeros(4, dtype=SPHERE_DTYPE)
    s["center"] = [[0, 0, -5], [0, 0, -5], [0, 0, 0], [0, 0, 5]]
    s["radius"] = [1, 1, 2, 1]
    o = np.zeros((3, 3), dtype=np.float32)
    d = np.array([[0, 0, -1], [0, 0, 1], [1, 0, 0]], dtype=np.float32)
    for mode in (po.EXACT, po.LITERAL):
        t, ids = po.trace(s, o, d, mode)
        assert ids[0] == 0 and t[0] == pytest.approx(4.0)    # tie between 0 and 1 -> lowest index
        assert ids[1] == 3 and t[1] == pytest.approx(4.0)    # origin inside sphere 2: never hits it
        assert ids[2] == -1 and t[2] == -1.0


def test_render_modes_agree_statistically(po):
    sc = scenes.config0().with_resolution(64, 36)
    v = po.view_for(sc)
    ex, _, st = po.render(sc.spheres, sc.materials, sc.lights, v, max_bounces=5, spp=4, mode=po.EXACT)
    li, _, _ = po.render(sc.spheres, sc.materials, sc.lights, v, max_bounces=5, spp=4, mode=po.LITERAL)
    d64, _, _ = po.render(sc.spheres, sc.materials, sc.lights, v, max_bounces=5, spp=4, f64=True)
    assert np.all(ex[:, 3] == 4.0)
    assert st["ext_rays"] >= 64 * 36 * 4
    for other in (li, d64):
        assert abs(ex[:, :3].mean() - other[:, :3].mean()) < 1e-3 * max(1.0, abs(ex[:, :3].mean()))


def test_pixel_subset_and_accumulator_input(po):
    sc = scenes.config0().with_resolution(40, 20)
    v = po.view_for(sc)
    full, _, _ = po.render(sc.spheres, sc.materials, sc.lights, v, max_bounces=5, spp=3)
    px = np.array([0, 5, 799, 400], dtype=np.uint32)
    sub, _, _ = po.render(sc.spheres, sc.materials, sc.lights, v, max_bounces=5, spp=3, pixels=px)
    assert np.array_equal(sub, full[px])
    a1, _, _ = po.render(sc.spheres, sc.materials, sc.lights, v, max_bounces=5, spp=1)
    a2, _, _ = po.render(sc.spheres, sc.materials, sc.lights, v, max_bounces=5, spp=2, frame0=2, accum=a1)
    assert np.array_equal(a2, full)


def test_pack_rgba8(po):
    acc = np.array([[0.0, 0.5, 1.0, 1.0], [2.0, -1.0, 0.25, 1.0], [np.nan, 0.1, 0.2, 1.0]], dtype=np.float32)
    out = po.pack_rgba8(acc, 1)
    assert out[0] == (255 << 24) | (255 << 16) | (127 << 8) | 0
    assert out[1] == (255 << 24) | (63 << 16) | (0 << 8) | 255
    assert out[2] & 0xFF == 0
