"""Seeded synthetic point sets.

The reference measures on synthetic generators only (qdt_bench.cpp:637-783);
no public dataset is involved. This module produces, from fixed seeds, the
inputs the tests and the benchmark use:

* the reference benchmark's own uniform generator (splitmix64, extent 1000,
  qdt_bench.cpp:264-293 and :637-648), whose triangle counts the reference
  README publishes -- used as known answers;
* the single-set workloads (uniform square, integer lattice with exact
  duplicates, Gaussian mixture, unit circle, noisy line);
* the many-set workload (log-uniform sizes, square or disk, some snapped to a
  grid) and the request stream of the serving loop.

Every generator is vectorised numpy and deterministic for a given seed.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_MIX1 = np.uint64(0xBF58476D1CE4E5B9)
_MIX2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int) -> np.ndarray:
    """The first `count` outputs of splitmix64 started at `seed`
    (qdt_bench.cpp:264-276)."""
    with np.errstate(over="ignore"):
        i = np.arange(1, count + 1, dtype=np.uint64)
        s = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GOLDEN
        z = (s ^ (s >> np.uint64(30))) * _MIX1
        z = (z ^ (z >> np.uint64(27))) * _MIX2
        return z ^ (z >> np.uint64(31))


def bench_uniform(n: int, seed: int, extent: float = 1000.0) -> np.ndarray:
    """gen_uniform of the reference benchmark (qdt_bench.cpp:639-648): for each
    point x then y, each `extent * ((next() >> 11) * 2^-53)`."""
    z = splitmix64(seed, 2 * n)
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return (extent * u).reshape(n, 2)


# The reference README's batch table (README.md:507-512): n -> triangles, for
# bench_uniform(n, 20260607 + n).
BENCH_KNOWN_COUNTS = {
    100: 185,
    1000: 1976,
    10000: 19968,
    100000: 199958,
    1000000: 1999963,
    2624409: 5248777,
}
BENCH_SEED = 20260607


def uniform(n: int, seed: int = 12345) -> np.ndarray:
    """n points i.i.d. uniform in [0,1)^2."""
    rng = np.random.default_rng(seed)
    return rng.random((n, 2))


def lattice_with_duplicates(side: int = 1024, dup_frac: float = 0.01, seed: int = 7) -> np.ndarray:
    """The side x side integer lattice as float64 plus round(dup_frac * side^2)
    exact copies of random lattice points, shuffled."""
    rng = np.random.default_rng(seed)
    g = np.arange(side, dtype=np.float64)
    xx, yy = np.meshgrid(g, g, indexing="ij")
    base = np.stack([xx.ravel(), yy.ravel()], axis=1)
    k = int(round(dup_frac * side * side))
    dups = base[rng.integers(0, base.shape[0], size=k)]
    pts = np.concatenate([base, dups], axis=0)
    return pts[rng.permutation(pts.shape[0])]


def gaussian_mixture(n: int, k: int = 64, seed: int = 11) -> np.ndarray:
    """n points from a mixture of k isotropic Gaussians, centres uniform in
    [0,1)^2, sigma log-uniform in [1e-4, 1e-1]."""
    rng = np.random.default_rng(seed)
    c = rng.random((k, 2))
    sig = np.exp(rng.uniform(np.log(1e-4), np.log(1e-1), size=k))
    lab = rng.integers(0, k, size=n)
    return c[lab] + sig[lab, None] * rng.standard_normal((n, 2))


def unit_circle(n: int, seed: int = 13) -> np.ndarray:
    """n points (cos t, sin t), t uniform in [0, 2 pi), rounded to float64."""
    rng = np.random.default_rng(seed)
    t = rng.uniform(0.0, 2.0 * np.pi, size=n)
    return np.stack([np.cos(t), np.sin(t)], axis=1)


def noisy_line(n: int, seed: int = 17) -> np.ndarray:
    """n points on y = 0.5 x, x uniform in [0,1), moved perpendicular to the
    line by a uniform offset in [-2^-40, 2^-40]."""
    rng = np.random.default_rng(seed)
    x = rng.random(n)
    off = rng.uniform(-2.0 ** -40, 2.0 ** -40, size=n)
    inv = 1.0 / np.sqrt(1.25)
    # unit normal of the direction (1, 0.5)
    nx, ny = -0.5 * inv, 1.0 * inv
    return np.stack([x + off * nx, 0.5 * x + off * ny], axis=1)


def many_sets(count: int = 4096, lo: int = 16, hi: int = 65536, seed: int = 23):
    """The many-set workload: `count` independent sets, sizes log-uniform in
    [lo, hi]; per set a coin flip between the unit square and the unit disk;
    10% of the sets snapped to a 256 x 256 grid. Returns a list of arrays."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64)
    sizes = np.clip(sizes, lo, hi)
    out = []
    for i in range(count):
        n = int(sizes[i])
        if rng.random() < 0.5:
            p = rng.random((n, 2))
        else:
            r = np.sqrt(rng.random(n))
            t = rng.uniform(0.0, 2.0 * np.pi, size=n)
            p = np.stack([0.5 + 0.5 * r * np.cos(t), 0.5 + 0.5 * r * np.sin(t)], axis=1)
        if rng.random() < 0.1:
            p = np.floor(p * 256.0) / 256.0
        out.append(np.ascontiguousarray(p))
    return out


def request_stream(count: int, rate_per_s: float, lo: int = 100, hi: int = 2_000_000, seed: int = 29):
    """An open-loop Poisson stream: (arrival time s, points) pairs; sizes
    log-uniform in [lo, hi]; distribution per request drawn from uniform
    square, Gaussian mixture and snapped grid."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, size=count)
    t = np.cumsum(gaps)
    sizes = np.clip(np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64), lo, hi)
    reqs = []
    for i in range(count):
        n = int(sizes[i])
        kind = int(rng.integers(0, 3))
        s = int(rng.integers(0, 2 ** 31))
        if kind == 0:
            p = uniform(n, s)
        elif kind == 1:
            p = gaussian_mixture(n, seed=s)
        else:
            p = np.floor(uniform(n, s) * 256.0) / 256.0
        reqs.append((float(t[i]), p))
    return reqs
