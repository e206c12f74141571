"""Seeded synthetic scenes for the benchmark and test workloads.

The reference ships one hand-made scene (sample-scene-data/scene.json) and no
benchmark scenes; these generators stand in for its render inputs with the
shapes, counts and value distributions of the five workloads this project
measures.  They use their own counter-based SplitMix64 stream (not numpy's
generators, whose streams may change between versions), so a seed gives the
same float32 scene on every machine.

Materials (all workloads): albedo U[0,1]^3, roughness U[0.05,1], metallic
Bernoulli(0.3) in {0,1}, F0 = 0.04 for dielectrics and the albedo for metals,
no emission.  Sky light off.  Sphere material indices are uniform over the
material table.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from ._native import LIGHT_DTYPE, MATERIAL_DTYPE, SPHERE_DTYPE

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _fnv1a(text: str) -> int:
    h = 0xCBF29CE484222325
    for b in text.encode():
        h = ((h ^ b) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


def _mix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


class Stream:
    """Counter-based SplitMix64: value i of stream (seed, label) is mix(key + (i+1)*gamma)."""

    def __init__(self, seed: int, label: str):
        with np.errstate(over="ignore"):
            k = np.uint64((seed * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF) ^ np.uint64(_fnv1a(label))
            self.key = _mix(np.array([k], dtype=np.uint64))[0]
        self.ctr = 0

    def u64(self, n: int) -> np.ndarray:
        i = np.arange(self.ctr + 1, self.ctr + n + 1, dtype=np.uint64)
        self.ctr += n
        with np.errstate(over="ignore"):
            return _mix(self.key + i * _GAMMA)

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        u = (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def normal(self, n: int) -> np.ndarray:
        u1 = 1.0 - self.uniform(n)          # (0, 1]
        u2 = self.uniform(n)
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)

    def lognormal(self, mu: float, sigma: float, n: int) -> np.ndarray:
        return np.exp(mu + sigma * self.normal(n))

    def integers(self, lo: int, hi: int, n: int) -> np.ndarray:
        """Uniform integers in [lo, hi)."""
        return (lo + np.floor(self.uniform(n) * (hi - lo))).astype(np.int64).clip(lo, hi - 1)


@dataclass
class SyntheticScene:
    name: str
    spheres: np.ndarray
    materials: np.ndarray
    lights: np.ndarray
    camera_position: tuple
    camera_direction: tuple
    fov: float = 45.0
    near: float = 0.1
    far: float = 100.0
    width: int = 1280
    height: int = 720
    max_bounces: int = 5
    spp: int = 1             # samples per pixel per launch
    frames: int = 1          # total frames (samples per pixel) of the workload
    sky_light: bool = False
    meta: dict = field(default_factory=dict)

    @property
    def pixels(self) -> int:
        return self.width * self.height

    def with_resolution(self, width: int, height: int) -> "SyntheticScene":
        """Same scene and camera, another viewport (for oracle-sized checks)."""
        import dataclasses
        return dataclasses.replace(self, width=width, height=height)


def draw_materials(st: Stream, n: int) -> np.ndarray:
    m = np.zeros(n, dtype=MATERIAL_DTYPE)
    albedo = st.uniform(3 * n).reshape(n, 3).astype(np.float32)
    rough = st.uniform(n, 0.05, 1.0).astype(np.float32)
    metal = (st.uniform(n) < 0.3).astype(np.float32)
    m["albedo"] = albedo
    m["roughness"] = rough
    m["metallic"] = metal
    f0 = np.full((n, 3), np.float32(0.04), dtype=np.float32)
    f0[metal > 0] = albedo[metal > 0]
    m["f0"] = f0
    m["id"] = np.arange(n, dtype=np.int32)
    return m


def draw_lights(st: Stream, n: int, radius: float) -> np.ndarray:
    """Positions uniform on a sphere of the given radius, colour U[0.5,1]^3, intensity U[20,200]."""
    lt = np.zeros(n, dtype=LIGHT_DTYPE)
    v = st.normal(3 * n).reshape(n, 3)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    lt["position"] = (radius * v).astype(np.float32)
    lt["color"] = st.uniform(3 * n, 0.5, 1.0).reshape(n, 3).astype(np.float32)
    lt["intensity"] = st.uniform(n, 20.0, 200.0).astype(np.float32)
    return lt


def _look_at(position) -> tuple:
    p = np.asarray(position, dtype=np.float64)
    d = -p / np.linalg.norm(p)
    return tuple(float(np.float32(x)) for x in p), tuple(float(np.float32(x)) for x in d)


def _spheres(centres: np.ndarray, radii: np.ndarray, mats: np.ndarray) -> np.ndarray:
    s = np.zeros(len(radii), dtype=SPHERE_DTYPE)
    s["center"] = centres.astype(np.float32)
    s["radius"] = radii.astype(np.float32)
    s["material"] = mats.astype(np.int32)
    return s


def config0(seed: int = 0) -> SyntheticScene:
    """Small scene: 8 spheres (centres U([-5,5]x[0,3]x[-5,5]), radii lognormal(0, 0.4)) plus a
    radius-1000 ground at (0,-1000,0); 8 materials; one white light of intensity 50 at (0,8,0);
    camera at (0,2,10) looking at the origin, 45 deg; 1280x720, 5 bounces, 1 spp x 64 frames."""
    st = Stream(seed, "config0")
    n = 8
    c = np.stack([st.uniform(n, -5, 5), st.uniform(n, 0, 3), st.uniform(n, -5, 5)], axis=1)
    r = st.lognormal(0.0, 0.4, n)
    mats = draw_materials(st, 8)
    mid = st.integers(0, 8, n + 1)
    c = np.vstack([c, [[0.0, -1000.0, 0.0]]])
    r = np.append(r, 1000.0)
    lt = np.zeros(1, dtype=LIGHT_DTYPE)
    lt["position"] = [0.0, 8.0, 0.0]
    lt["color"] = [1.0, 1.0, 1.0]
    lt["intensity"] = 50.0
    pos, d = _look_at((0.0, 2.0, 10.0))
    return SyntheticScene("config0", _spheres(c, r, mid), mats, lt, pos, d, width=1280, height=720,
                          max_bounces=5, spp=1, frames=64)


def config1(seed: int = 1) -> SyntheticScene:
    """Medium scene: 256 spheres U([-20,20]^3), radii lognormal(-0.5, 0.5); 64 materials; 8 lights on
    a radius-30 sphere; 1920x1080, 8 bounces, 16 spp per launch, 256 frames.  Camera (chosen here,
    the workload names none): (0, 12, 60) looking at the origin, outside the scene's bounding sphere."""
    st = Stream(seed, "config1")
    n = 256
    c = st.uniform(3 * n, -20, 20).reshape(n, 3)
    r = st.lognormal(-0.5, 0.5, n)
    mats = draw_materials(st, 64)
    mid = st.integers(0, 64, n)
    lts = draw_lights(st, 8, 30.0)
    pos, d = _look_at((0.0, 12.0, 60.0))
    return SyntheticScene("config1", _spheres(c, r, mid), mats, lts, pos, d, width=1920, height=1080,
                          max_bounces=8, spp=16, frames=256)


def config2(seed: int = 2) -> SyntheticScene:
    """Large scene: 65,536 spheres in 32 Gaussian clusters (centres U([-100,100]^3), sigma 5), radii
    lognormal(-1.5, 0.5); 256 materials; 16 lights on a radius-30 sphere; 3840x2160, 8 bounces,
    4 spp per launch.  Camera (chosen here): (0, 40, 320) looking at the origin, far clip 1000."""
    st = Stream(seed, "config2")
    n, k = 65536, 32
    centres = st.uniform(3 * k, -100, 100).reshape(k, 3)
    which = st.integers(0, k, n)
    c = centres[which] + 5.0 * st.normal(3 * n).reshape(n, 3)
    r = st.lognormal(-1.5, 0.5, n)
    mats = draw_materials(st, 256)
    mid = st.integers(0, 256, n)
    lts = draw_lights(st, 16, 30.0)
    pos, d = _look_at((0.0, 40.0, 320.0))
    return SyntheticScene("config2", _spheres(c, r, mid), mats, lts, pos, d, far=1000.0, width=3840,
                          height=2160, max_bounces=8, spp=4, frames=4)


RESOLUTIONS = ((256, 256), (640, 480), (1280, 720), (1920, 1080))


def batch_scene(st: Stream, index: int) -> SyntheticScene:
    """One scene of the batched mix: sphere count lognormal(ln 256, 1) clipped to [8, 8192]; centres
    U([-L,L]^3) with L = 20 (N/256)^(1/3) (the medium scene's density); radii lognormal(-0.5, 0.5);
    16 materials; 1-16 lights on a sphere of radius 1.5 L; resolution from RESOLUTIONS; bounces
    U{2..12}; 4-64 spp per pass.  Camera (chosen here): (0, 0.6 L, 3 L) looking at the origin."""
    n = int(np.clip(np.rint(st.lognormal(math.log(256.0), 1.0, 1)[0]), 8, 8192))
    L = 20.0 * (n / 256.0) ** (1.0 / 3.0)
    c = st.uniform(3 * n, -L, L).reshape(n, 3)
    r = st.lognormal(-0.5, 0.5, n)
    mats = draw_materials(st, 16)
    mid = st.integers(0, 16, n)
    nl = int(st.integers(1, 17, 1)[0])
    lts = draw_lights(st, nl, 1.5 * L)
    w, h = RESOLUTIONS[int(st.integers(0, len(RESOLUTIONS), 1)[0])]
    bounces = int(st.integers(2, 13, 1)[0])
    spp = int(st.integers(4, 65, 1)[0])
    pos, d = _look_at((0.0, 0.6 * L, 3.0 * L))
    return SyntheticScene(f"mix{index}", _spheres(c, r, mid), mats, lts, pos, d, far=max(100.0, 8.0 * L),
                          width=w, height=h, max_bounces=bounces, spp=spp, frames=spp)


def config3(seed: int = 3, count: int = 64) -> list[SyntheticScene]:
    """Batched mix: `count` independent scenes drawn by batch_scene."""
    st = Stream(seed, "config3")
    return [batch_scene(st, i) for i in range(count)]


TARGET_SPP = (16, 64, 256, 1024)


@dataclass
class Job:
    arrival_s: float
    scene: SyntheticScene
    target_spp: int
    pool_index: int = -1


def scene_pool(seed: int = 4, size: int = 512) -> list[SyntheticScene]:
    """A pool of scenes drawn from the batched-mix distribution (batch_scene) for the serving stream."""
    st = Stream(seed, "config4-pool")
    return [batch_scene(st, i) for i in range(size)]


def config4(seed: int = 4, rate: float = 50.0, duration_s: float = 60.0, pool: list | None = None) -> list[Job]:
    """Serving stream: Poisson arrivals at `rate` jobs/s over `duration_s`; each job a scene of the
    batched-mix distribution, drawn uniformly from a seeded pool of such scenes (scene_pool; generating a
    distinct scene per job in Python would throttle arrivals at 800 jobs/s), with a target spp drawn from
    TARGET_SPP."""
    pool = pool if pool is not None else scene_pool(seed)
    st = Stream(seed, f"config4-{rate}")
    jobs: list[Job] = []
    t = 0.0
    while True:
        t += -math.log(1.0 - float(st.uniform(1)[0])) / rate
        if t >= duration_s:
            break
        k = int(st.integers(0, len(pool), 1)[0])
        target = TARGET_SPP[int(st.integers(0, len(TARGET_SPP), 1)[0])]
        jobs.append(Job(t, pool[k], target, k))
    return jobs


def reference_default_scene() -> SyntheticScene:
    """The reference's built-in scene (Engine/src/main.cpp:235-265), flattened: spheres at the
    origin, (2,0,0) and (2,2,0), radius 1, materials 0..2, one light at (10,10,0); default camera
    (Camera.cpp:14-21)."""
    s = np.zeros(3, dtype=SPHERE_DTYPE)
    s["center"] = [[0.0, 0.0, 0.0], [2.0, 0.0, 0.0], [2.0, 2.0, 0.0]]
    s["radius"] = 1.0
    s["material"] = [0, 1, 2]
    m = np.zeros(3, dtype=MATERIAL_DTYPE)
    m["albedo"] = [[1.022, 0.782, 0.344], [1.0, 0.0, 0.0], [0.972, 0.960, 0.915]]
    m["roughness"] = [1.0, 0.3, 0.25]
    m["metallic"] = [0.0, 0.0, 1.0]
    m["f0"] = np.float32(0.04)
    m["id"] = [0, 1, 2]
    lt = np.zeros(1, dtype=LIGHT_DTYPE)
    lt["position"] = [10.0, 10.0, 0.0]
    lt["color"] = [1.0, 1.0, 1.0]
    lt["intensity"] = 1.0
    return SyntheticScene("reference-default", s, m, lt, (0.0, 0.0, 3.0), (0.0, 0.0, -1.0),
                          width=1600, height=900, max_bounces=15, spp=1, frames=1)
