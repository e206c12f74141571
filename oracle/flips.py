"""Branch flips between arithmetic modes of the oracle: which pixels a rounding difference can send down
another path, and why.

TEST INFRASTRUCTURE ONLY: imported by tests/ and bench.py's reference legs, never by the product.

Renderer.cu's path (perPixel, :287-387) branches on floating-point comparisons: the nearest hit
(:256-279, including a continuation or shadow ray hitting the sphere it leaves), the occlusion test
t^2 < d^2 (:352), Russian roulette (:376) and the samplers' tangent frame (BRDF.cu:85, :109).  A pixel is
"flip-free" when the oracle's matched-order mode (what the kernels compute, bit for bit), its literal
mode, the literal mode with multiply-add contraction and the literal mode in float64 take the same
branches in every frame; elsewhere the first decision in which the matched-order mode differs from the
literal mode (else from float64, else from the contracted literal mode) names the pixel's class.
"""
from __future__ import annotations

import numpy as np

from oracle import pyoracle as po

CLASSES = ("primary_hit", "extension_hit", "self_intersection", "occlusion_t2_d2", "occluder",
           "self_occlusion", "roulette", "sampler_frame", "other_variant_only")

_KIND = lambda e: (e >> 28) & 0xF          # noqa: E731
_BOUNCE = lambda e: (e >> 20) & 0xFF       # noqa: E731
_VALUE = lambda e: e & 0xFFFFF             # noqa: E731


def _decision(e: int) -> int:
    return e & ~(0x3FFFF << 2) if _KIND(e) == po.EV_SHADOW else e


def classify_path(a: np.ndarray, b: np.ndarray) -> str | None:
    """The class of the first differing decision of two event rows of one path, or None if none differs."""
    prev_hit = [-1, -1]
    for ea, eb in zip(a.tolist(), b.tolist()):
        if _decision(ea) == _decision(eb):
            if _KIND(ea) == po.EV_HIT:
                prev_hit = [_VALUE(ea) - 1, _VALUE(eb) - 1]
            if ea == 0:
                return None
            continue
        kind = _KIND(ea) or _KIND(eb)
        if kind == po.EV_HIT:
            if _BOUNCE(ea) == 0 and _BOUNCE(eb) == 0:
                return "primary_hit"
            ha, hb = _VALUE(ea) - 1, _VALUE(eb) - 1
            return "self_intersection" if prev_hit[0] in (ha, hb) or prev_hit[1] in (ha, hb) else "extension_hit"
        if kind == po.EV_SHADOW:
            sa, sb = (_VALUE(ea) >> 2) - 1, (_VALUE(eb) >> 2) - 1
            if sa == sb:
                return "occlusion_t2_d2"
            return "self_occlusion" if prev_hit[0] in (sa, sb) or prev_hit[1] in (sa, sb) else "occluder"
        if kind == po.EV_ROULETTE:
            return "roulette"
        if kind == po.EV_FRAME:
            return "sampler_frame"
        return "extension_hit"
    return None


def flip_map(sc, spp: int, *, frame0: int = 1, max_classified: int = 20000, seed: int = 0):
    """(flip-free mask over the pixels, {class: pixels}, pixels flagged) for frames frame0 .. frame0+spp-1
    of scene sc under the oracle's camera.  Classes are counted on at most max_classified flagged pixels
    (a seeded sample) and scaled to all of them."""
    view = po.view_for(sc)
    kw = dict(max_bounces=sc.max_bounces, sky=sc.sky_light, frame0=frame0, spp=spp)
    args = (sc.spheres, sc.materials, sc.lights, view)
    h_ex = po.decision_hash(*args, variant=po.EXACT, **kw)
    flagged = np.zeros(len(h_ex), dtype=bool)
    for variant, contract in ((po.LITERAL, False), (po.LITERAL, True), (po.F64, False)):
        flagged |= po.decision_hash(*args, variant=variant, contract=contract, **kw) != h_ex
    idx = np.flatnonzero(flagged)
    counts = {c: 0 for c in CLASSES}
    if len(idx):
        rng = np.random.default_rng(seed)
        pick = np.sort(rng.choice(idx, size=min(len(idx), max_classified), replace=False)).astype(np.uint32)
        ev_ex = po.decision_events(*args, pick, variant=po.EXACT, **kw)
        others = [po.decision_events(*args, pick, variant=v, contract=c, **kw)
                  for v, c in ((po.LITERAL, False), (po.F64, False), (po.LITERAL, True))]
        scale = len(idx) / len(pick)
        raw = {c: 0 for c in CLASSES}
        for k in range(len(pick)):
            cls = None
            for ev in others:
                for f in range(spp):
                    cls = classify_path(ev_ex[k, f], ev[k, f])
                    if cls:
                        break
                if cls:
                    break
            raw[cls or "other_variant_only"] += 1
        counts = {c: int(round(v * scale)) for c, v in raw.items()}
    return ~flagged, counts, int(len(idx))


def rel_diff(a: np.ndarray, b: np.ndarray, floor: float = 1e-3) -> np.ndarray:
    """Per pixel, the largest relative difference of the rgb channels of accumulators a and b."""
    return (np.abs(a[:, :3].astype(np.float64) - b[:, :3]) / np.maximum(np.abs(b[:, :3]), floor)).max(axis=1)


def well_conditioned(sc, spp: int, matched: np.ndarray, *, frame0: int = 1, tol: float = 1e-3):
    """Pixels whose result the reference's arithmetic determines to within tol: no branch can flip
    (flip_map) and both single-precision evaluations (matched-order, given as `matched`, and literal)
    lie within tol/2 of the float64 evaluation of the same path, so any two evaluation orders agree to
    tol.  Where a rounding error is amplified
    without a branch flip (the quadratic's cancellation at a distance moving a hit point by ~1e-4, then
    a glossy GGX lobe turning that into a percent of radiance) the reference's own builds disagree too.
    Returns (mask, flip-free mask, classes, flagged count)."""
    free, classes, flagged = flip_map(sc, spp, frame0=frame0)
    view = po.view_for(sc)
    kw = dict(max_bounces=sc.max_bounces, sky=sc.sky_light, frame0=frame0, spp=spp)
    lit, _, _ = po.render(sc.spheres, sc.materials, sc.lights, view, mode=po.LITERAL, **kw)
    d64, _, _ = po.render(sc.spheres, sc.materials, sc.lights, view, f64=True, **kw)
    mask = free & (rel_diff(matched, d64) <= tol / 2) & (rel_diff(lit, d64) <= tol / 2)
    return mask, free, classes, flagged

