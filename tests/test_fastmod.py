"""The light pick's remainder by multiplication (wavefront.h fastmod_multiplier,
wavefront.cu light_pick) restated with Python integers: for every 32-bit x and
divisor d >= 1 it must equal x % d, since it replaces PcgHash(seed) % lights
(Renderer.cu:339) bit for bit."""
import numpy as np

M64 = (1 << 64) - 1


def fastmod(x: int, d: int) -> int:
    m = (M64 // d + 1) & M64          # 2^64 wraps to 0 for d = 1
    low = (m * x) & M64
    return (low * d) >> 64


def test_fastmod_equals_remainder():
    rng = np.random.default_rng(3)
    divisors = [1, 2, 3, 5, 7, 8, 9, 16, 31, 32, 33, 63, 64, 100, 1000, 4096, 65535, 65537,
                2**31 - 1, 2**31, 2**31 + 1, 2**32 - 1]
    xs = [0, 1, 2, 2**31 - 1, 2**31, 2**32 - 2, 2**32 - 1] + [int(v) for v in rng.integers(0, 2**32, 3000)]
    for d in divisors:
        for x in xs:
            assert fastmod(x, d) == x % d, (x, d)


def test_fastmod_exhaustive_small_divisors_on_boundaries():
    # every multiple of d near the top of the 32-bit range and its neighbours
    for d in range(1, 70):
        top = (2**32 - 1) // d * d
        for x in range(max(0, top - 3 * d), 2**32):
            assert fastmod(x, d) == x % d
