"""The reference's general-position perturbation sequence restated
(preproc.cpp:2621-2627): std::mt19937 (Matsumoto & Nishimura 1998) seeded
with the first output of std::default_random_engine(1) (minstd_rand0:
16807 * 1 mod 2^31 - 1), and std::uniform_real_distribution<double>(-1, 1)
built on generate_canonical<double, 53> (two 32-bit draws,
(x0 + x1 * 2^32) / 2^64, below 1). Pinned against the C++ library's own
output in tests/golden/gp_rng.json."""
import math


def _mt19937(seed):
    mt = [0] * 624
    mt[0] = seed & 0xFFFFFFFF
    for i in range(1, 624):
        mt[i] = (1812433253 * (mt[i - 1] ^ (mt[i - 1] >> 30)) + i) & 0xFFFFFFFF
    idx = 624
    while True:
        if idx >= 624:
            for i in range(624):
                y = (mt[i] & 0x80000000) | (mt[(i + 1) % 624] & 0x7FFFFFFF)
                mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            idx = 0
        y = mt[idx]
        idx += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        yield y


def draws(n):
    """The first n uniform(-1, 1) values of a fresh sequence."""
    g = _mt19937(16807)
    out = []
    for _ in range(n):
        a, b = next(g), next(g)
        c = float(a + b * 2 ** 32) / 2 ** 64
        if c >= 1.0:
            c = math.nextafter(1.0, 0.0)
        out.append(2.0 * c - 1.0)
    return out


def perturbations(n, scale):
    """The first n perturbation vectors (3 draws each, times scale)."""
    d = draws(3 * n)
    return [tuple(d[3 * k + j] * scale for j in range(3)) for k in range(n)]
