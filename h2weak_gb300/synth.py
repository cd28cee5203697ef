"""Seeded synthetic inputs shared by the library, its tests and bench.py.

Counter-based splitmix64 (Steele, Lea, Flood 2014): draw i of stream `seed`
is mix(seed + (i + 1) * 0x9E3779B97F4A7C15). Uniform doubles take the top 53
bits, so points are bit-identical wherever they are generated (Python, C++,
CUDA). Normal right-hand sides use Box-Muller on consecutive pairs and are
generated once here and passed to every implementation as data.
"""
import numpy as np

_G = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, n):
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (np.arange(1, n + 1, dtype=np.uint64) * _G)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform01(seed, n):
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def uniform_pm1(seed, n):
    """Uniform doubles in [-1, 1): 2u - 1 is exact for 53-bit u."""
    return 2.0 * uniform01(seed, n) - 1.0


def normal(seed, n):
    m = (n + 1) // 2
    u = uniform01(seed, 2 * m)
    r = np.sqrt(-2.0 * np.log1p(-u[0::2]))
    t = 2.0 * np.pi * u[1::2]
    z = np.empty(2 * m)
    z[0::2] = r * np.cos(t)
    z[1::2] = r * np.sin(t)
    return z[:n]


def config_seed(cfg, instance=0):
    """Per-workload seed: configuration number c, instance i."""
    return 0x5EED0000 + 1000 * cfg + instance


def uniform_points(seed, n, dim):
    """n points uniform in [-1, 1)^dim, row-major (n, dim)."""
    return uniform_pm1(seed, n * dim).reshape(n, dim)
