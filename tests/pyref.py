"""Independent pure-Python restatement of the per-pixel path in the matched evaluation order.

Written from the reference's semantics (Renderer.cu:251-409, BRDF.cu:9-117, Random.h:59-70,
Camera.cpp:161-195) and the evaluation order the oracle's ORC_EXACT mode documents, without
sharing code with the C oracle.  float32 arithmetic uses numpy float32 scalars (IEEE single,
round to nearest); fused multiply-add is computed exactly with fractions and rounded once.
Slow (small cases only): it exists to pin the C oracle, which the GPU kernels then match.
"""
from __future__ import annotations

from fractions import Fraction

import numpy as np

F = np.float32
ONE = F(1.0)
ZERO = F(0.0)
FLT_MAX = F(3.4028234663852886e38)
PI = F(np.float32(3.14159265358979323846))


def round_f32(q: Fraction) -> np.float32:
    if q == 0:
        return ZERO
    f = F(float(q))
    cands = [np.nextafter(f, F(-np.inf)), f, np.nextafter(f, F(np.inf))]
    return min(cands, key=lambda x: (abs(Fraction(float(x)) - q), int(np.array(x, dtype=np.float32).view(np.uint32)) & 1))


def fma(a, b, c) -> np.float32:
    return round_f32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def v(x, y, z):
    return (F(x), F(y), F(z))


def add(a, b): return (a[0] + b[0], a[1] + b[1], a[2] + b[2])
def sub(a, b): return (a[0] - b[0], a[1] - b[1], a[2] - b[2])
def mul(a, b): return (a[0] * b[0], a[1] * b[1], a[2] * b[2])
def muls(a, s): return (a[0] * s, a[1] * s, a[2] * s)


def dot(a, b):
    return fma(a[2], b[2], fma(a[1], b[1], a[0] * b[0]))


def normalize(a):
    inv = ONE / np.sqrt(dot(a, a))
    return muls(a, inv)


def normalize_host(a):
    """Camera.cpp's normalisation on the host: (x*x + y*y) + z*z, nothing fused."""
    inv = ONE / np.sqrt((a[0] * a[0] + a[1] * a[1]) + a[2] * a[2])
    return muls(a, inv)


def cross(a, b):
    return (a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1])


def gmax(a, b): return b if a < b else a
def gmin(a, b): return b if b < a else a


def pcg_hash(s: int) -> int:
    state = (s * 747796405 + 2891336453) & 0xFFFFFFFF
    word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & 0xFFFFFFFF
    return ((word >> 22) ^ word) & 0xFFFFFFFF


class Seed:
    def __init__(self, s): self.s = s & 0xFFFFFFFF

    def float(self):
        self.s = pcg_hash(self.s)
        return F(self.s) / F(4294967296.0)


S9, S7, S5, S3, S1 = (F(float.fromhex(h)) for h in ("0x1.507834p+5", "-0x1.32d2ccp+6", "0x1.466bc6p+6",
                                                       "-0x1.4abbcep+5", "0x1.921fb6p+2"))
C10, C8, C6, C4, C2 = (F(float.fromhex(h)) for h in ("-0x1.a6d1f2p+4", "0x1.e1f506p+5", "-0x1.55d3c8p+6",
                                                        "0x1.03c1f0p+6", "-0x1.3bd3ccp+4"))


def sincos2pi(u):
    u = F(u)
    vv = u - F(np.rint(u))
    q = F(np.rint(vv * F(4.0)))
    w = fma(q, F(-0.25), vv)
    w2 = w * w
    ps = fma(w2, S9, S7); ps = fma(w2, ps, S5); ps = fma(w2, ps, S3); ps = fma(w2, ps, S1)
    sn = w * ps
    pc = fma(w2, C10, C8); pc = fma(w2, pc, C6); pc = fma(w2, pc, C4); pc = fma(w2, pc, C2)
    cs = fma(w2, pc, ONE)
    k = int(q) & 3
    return [(cs, sn), (-sn, cs), (-cs, -sn), (sn, -cs)][k]


def primary_dir(ip, iv, W, H, x, y):
    qx = F(x) / F(W)
    qy = F(y) / F(H)
    cx = qx * F(2.0) - ONE
    cy = qy * F(2.0) - ONE
    t = [(ip[0 * 4 + r] * cx + ip[1 * 4 + r] * cy) + (ip[2 * 4 + r] + ip[3 * 4 + r]) for r in range(4)]
    tv = normalize_host((t[0] / t[3], t[1] / t[3], t[2] / t[3]))
    d = [(iv[0 * 4 + r] * tv[0] + iv[1 * 4 + r] * tv[1]) + (iv[2 * 4 + r] * tv[2] + iv[3 * 4 + r] * F(0.0))
         for r in range(3)]
    return normalize_host(tuple(d))


def sphere_t(c, r2, o, d, a):
    ox, oy, oz = o[0] - c[0], o[1] - c[1], o[2] - c[2]
    b = fma(oz, d[2], fma(oy, d[1], ox * d[0]))
    cc = fma(oz, oz, fma(oy, oy, fma(ox, ox, -r2)))
    disc = fma(b, b, -(a * cc))
    if disc < ZERO:
        return None
    return -(b + np.sqrt(disc)) / a


def nearest(sph, o, d):
    a = dot(d, d)
    best, tm = -1, FLT_MAX
    for i, (c, r2) in enumerate(sph):
        t = sphere_t(c, r2, o, d, a)
        if t is not None and t > ZERO and t < tm:
            tm, best = t, i
    return best, tm


def occluded(sph, o, d, dist2):
    a = dot(d, d)
    for c, r2 in sph:
        t = sphere_t(c, r2, o, d, a)
        if t is not None and t > ZERO and t * t < dist2:
            return True
    return False


def cook_torrance(albedo, f0, metal, rough, n, vv, l):
    h = normalize(add(vv, l))
    ndl = gmax(dot(n, l), F(1e-7))
    ndv = gmax(dot(n, vv), F(1e-7))
    ndh = gmax(dot(n, h), ZERO)
    vdh = gmax(dot(vv, h), ZERO)
    m = ONE - gmin(gmax(vdh, ZERO), ONE)
    m2 = m * m
    p5 = (m2 * m2) * m
    Fr = tuple(f0[k] + (ONE - f0[k]) * p5 for k in range(3))
    a = rough * rough
    a2 = a * a
    den = (ndh * ndh) * (a2 - ONE) + ONE
    den = PI * den * den
    rr = rough + ONE
    k = (rr * rr) * F(0.125)
    gv = ndv * (ONE - k) + k
    gl = ndl * (ONE - k) + k
    one_f = sub(v(1, 1, 1), Fr)
    kd = muls(one_f, ONE - metal)
    denom = F(4.0) * ndl * ndv + F(0.001)
    # matched grouping: F * (D * G) / denom = F * (a2 ndv ndl) / (den gv gl denom); / pi as * (1 / pi)
    x = ((a2 * ndv) * ndl) / (((den * gv) * gl) * denom)
    spec = muls(Fr, x)
    diffuse = muls(mul(one_f, albedo), ONE / PI)
    return muls(add(mul(kd, diffuse), spec), ndl)


def div_v(a, s):
    """a / s as the kernels evaluate it: a * (1 / s)."""
    return muls(a, ONE / s)


def frame(n):
    if abs(n[0]) > abs(n[1]):
        t = div_v((-n[2], ZERO, n[0]), np.sqrt(n[0] * n[0] + n[2] * n[2]))
    else:
        t = div_v((ZERO, -n[2], n[1]), np.sqrt(n[1] * n[1] + n[2] * n[2]))
    return t, cross(n, t)


def to_world(x, y, z, t, b, n):
    return add(add(muls(t, x), muls(b, y)), muls(n, z))


def sample_cosine(n, seed: Seed):
    u1, u2 = seed.float(), seed.float()
    r = np.sqrt(u1)
    c, s = sincos2pi(u2)
    t, b = frame(n)
    return to_world(r * c, r * s, np.sqrt(ONE - u1), t, b, n)


def sample_ggx(n, rough, seed: Seed):
    u1, u2 = seed.float(), seed.float()
    a = rough * rough
    cos_t = np.sqrt((ONE - u1) / (ONE + (a * a - ONE) * u1))
    sin_t = np.sqrt(ONE - cos_t * cos_t)
    c, s = sincos2pi(u2)
    t, b = frame(n)
    return to_world(sin_t * c, sin_t * s, cos_t, t, b, n)


def per_pixel(scene, ip, iv, pos, W, H, x, y, frame_index, max_bounces, sky=False):
    spheres, materials, lights = scene
    sph = [((F(s["center"][0]), F(s["center"][1]), F(s["center"][2])), F(s["radius"]) * F(s["radius"]))
           for s in spheres]
    o = v(*pos)
    d = primary_dir(ip, iv, W, H, x, y)
    color = v(0, 0, 0)
    thr = v(1, 1, 1)
    seed = Seed(((x + y * W) & 0xFFFFFFFF) * frame_index)
    for i in range(max_bounces):
        seed.s = (seed.s + i) & 0xFFFFFFFF
        idx, t = nearest(sph, o, d)
        if idx < 0:
            if sky:
                color = add(color, mul(v(0.6, 0.7, 0.9), thr))
            break
        c, _ = sph[idx]
        p = add(sub(o, c), muls(d, t))
        nrm = normalize(p)
        hp = add(p, c)
        mid = int(spheres[idx]["material"])
        if mid < 0 or mid >= len(materials):
            mid = 0
        m = materials[mid]
        albedo = tuple(F(x_) for x_ in m["albedo"])
        metal, rough = F(m["metallic"]), F(m["roughness"])
        if F(m["emission_intensity"]) > ZERO:
            e = muls(tuple(F(x_) for x_ in m["emission_color"]), F(m["emission_intensity"]))
            color = add(color, mul(e, thr))
        base = add(muls(tuple(F(x_) for x_ in m["f0"]), ONE - metal), muls(albedo, metal))
        if len(lights):
            lt = lights[pcg_hash(seed.s) % len(lights)]
            L = sub(tuple(F(x_) for x_ in lt["position"]), hp)
            dist2 = dot(L, L)
            L = muls(L, ONE / np.sqrt(dist2))
            so = add(hp, muls(nrm, F(0.0001)))
            if not occluded(sph, so, L, dist2):
                f = cook_torrance(albedo, base, metal, rough, nrm, (-d[0], -d[1], -d[2]), L)
                le = muls(tuple(F(x_) for x_ in lt["color"]), F(lt["intensity"]))
                color = add(color, mul(mul(le, f), thr))
        if i + 1 >= max_bounces:
            break
        thr = mul(thr, albedo)
        o = add(hp, muls(nrm, F(0.0001)))
        pr = gmax(F(0.1), gmin(ONE, np.sqrt(dot(thr, thr))))
        if seed.float() > pr:
            break
        thr = div_v(thr, pr)
        d = sample_ggx(nrm, rough, seed) if metal > ZERO else sample_cosine(nrm, seed)
    return color
