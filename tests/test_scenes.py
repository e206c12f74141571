"""Synthetic workload generators: determinism, counts, ranges and distributions."""
import math

import numpy as np

from ataraxia_gb300 import scenes


def test_stream_determinism_and_independence():
    a = scenes.Stream(5, "x").u64(100)
    b = scenes.Stream(5, "x").u64(100)
    c = scenes.Stream(5, "y").u64(100)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    s = scenes.Stream(1, "z")
    first = s.u64(10)
    rest = s.u64(10)
    assert np.array_equal(np.concatenate([first, rest]), scenes.Stream(1, "z").u64(20))
    u = scenes.Stream(3, "u").uniform(100000)
    assert 0.0 <= u.min() and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.01
    z = scenes.Stream(3, "n").normal(100000)
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1.0) < 0.02


def test_config0_shapes_and_rules():
    sc = scenes.config0()
    assert len(sc.spheres) == 9 and len(sc.materials) == 8 and len(sc.lights) == 1
    c = sc.spheres["center"][:8]
    assert (c[:, 0] >= -5).all() and (c[:, 0] <= 5).all() and (c[:, 1] >= 0).all() and (c[:, 1] <= 3).all()
    assert tuple(sc.spheres["center"][8]) == (0.0, -1000.0, 0.0) and sc.spheres["radius"][8] == 1000.0
    assert tuple(sc.lights["position"][0]) == (0.0, 8.0, 0.0) and sc.lights["intensity"][0] == 50.0
    assert (sc.width, sc.height, sc.max_bounces, sc.spp, sc.frames) == (1280, 720, 5, 1, 64)
    assert np.allclose(sc.camera_direction, np.array([0, -2, -10]) / math.sqrt(104), atol=1e-7)
    assert np.array_equal(sc.spheres, scenes.config0().spheres)


def test_materials_rules():
    m = scenes.draw_materials(scenes.Stream(0, "m"), 4000)
    metal = m["metallic"] > 0
    assert set(np.unique(m["metallic"])) <= {0.0, 1.0}
    assert abs(metal.mean() - 0.3) < 0.03
    assert np.array_equal(m["f0"][metal], m["albedo"][metal])
    assert np.all(m["f0"][~metal] == np.float32(0.04))
    assert m["roughness"].min() >= 0.05 and m["roughness"].max() <= 1.0
    assert np.all(m["emission_intensity"] == 0)


def test_config1_and_2_distributions():
    sc = scenes.config1()
    assert len(sc.spheres) == 256 and len(sc.materials) == 64 and len(sc.lights) == 8
    assert np.abs(sc.spheres["center"]).max() <= 20
    assert np.allclose(np.linalg.norm(sc.lights["position"], axis=1), 30.0, rtol=1e-5)
    assert (sc.width, sc.height, sc.max_bounces, sc.spp) == (1920, 1080, 8, 16)
    lr = np.log(sc.spheres["radius"])
    assert abs(lr.mean() + 0.5) < 0.1 and abs(lr.std() - 0.5) < 0.1
    big = scenes.config2()
    assert len(big.spheres) == 65536 and len(big.materials) == 256 and len(big.lights) == 16
    lr = np.log(big.spheres["radius"])
    assert abs(lr.mean() + 1.5) < 0.01 and abs(lr.std() - 0.5) < 0.01
    assert (big.width, big.height, big.spp) == (3840, 2160, 4)


def test_config3_mix_ranges():
    mix = scenes.config3()
    assert len(mix) == 64
    ns = np.array([len(s.spheres) for s in mix])
    assert ns.min() >= 8 and ns.max() <= 8192 and 100 < np.median(ns) < 600
    assert {(s.width, s.height) for s in mix} <= set(scenes.RESOLUTIONS)
    assert all(2 <= s.max_bounces <= 12 and 4 <= s.spp <= 64 and 1 <= len(s.lights) <= 16 for s in mix)


def test_config4_poisson_arrivals():
    jobs = scenes.config4(rate=200.0, duration_s=5.0)
    assert 800 < len(jobs) < 1200
    t = np.array([j.arrival_s for j in jobs])
    assert np.all(np.diff(t) > 0) and t.max() < 5.0
    assert {j.target_spp for j in jobs} <= set(scenes.TARGET_SPP)
