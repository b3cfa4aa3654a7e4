"""The oracle against the reference library itself, on inputs that are not
in the committed fixtures.

Where the reference was compiled from its own sources into oracle/_ref
(oracle/build_ref.sh; only where the reference tree is present), this draws
fresh seeded inputs of the kinds the fixtures hold -- small integer grids
with duplicates, wide magnitude spreads, cocircular and collinear sets,
power-of-two scales down to the subnormal range -- and requires the C
restatement (serial and threaded drivers) to give the reference's canonical
triangles and used flags. Elsewhere it is skipped; the committed fixtures
(tests/test_oracle.py) pin the oracle there.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.skipif(
    not (O.reference_available() and os.path.exists(os.path.join(O.REF_DIR, "libqdt_dump_ref.so"))),
    reason="the reference is not compiled here (oracle/_ref)")


@pytest.fixture(scope="module")
def ref():
    from libqdt_gb300 import qdt_api as Q
    from tests.golden import make_golden as M
    lib = Q.load(O.REF_LIB_PATH)
    return lambda pts, par: M.run_ref(lib, pts, par)


def _used_from(res, n):
    used = np.zeros(n, dtype=np.uint8)
    if res.tris.shape[0]:
        used[np.arange(n)[res.rep == np.arange(n)]] = 1
    return used


def _inputs(seed):
    rng = np.random.default_rng(seed)
    kind = seed % 6
    n = int(rng.integers(3, 2000 if seed % 5 == 0 else 300))
    if kind == 0:      # small integer grid: duplicates, collinear and cocircular quadruples
        R = int(rng.choice([2, 3, 5, 8, 20]))
        return rng.integers(-R, R + 1, size=(n, 2)).astype(np.float64)
    if kind == 1:      # magnitudes from 1 to 2^40 in one set
        e = rng.integers(0, 41, size=(n, 1))
        return (rng.integers(-8, 9, size=(n, 2)) * np.ldexp(1.0, e)).astype(np.float64)
    if kind == 2:      # integer points on one circle
        r = 1 << int(rng.integers(10, 26))
        a = 2 * np.pi * rng.random(n)
        return np.stack([np.round(r * np.cos(a)), np.round(r * np.sin(a))], axis=1)
    if kind == 3:      # points on a few lines, some exactly collinear
        t = rng.integers(-1000, 1001, size=n).astype(np.float64)
        k = rng.integers(0, 3, size=n)
        return np.stack([t, k * t * 0.5 + k], axis=1)
    if kind == 4:      # a grid scaled by a power of two, down to subnormal coordinates
        s = np.ldexp(1.0, int(rng.choice([-1074, -1060, -600, -64, 64, 600, 960])))
        return rng.integers(-6, 7, size=(n, 2)).astype(np.float64) * s
    # uniform doubles snapped to a coarse grid, with repeated points
    p = np.round(rng.random((n, 2)) * 64) / 64
    return np.concatenate([p, p[rng.integers(0, n, size=n // 4)]])


@pytest.mark.parametrize("block", range(6))
def test_oracle_equals_reference_on_fresh_inputs(ref, block):
    nonempty = 0
    for seed in range(970000 + 250 * block, 970000 + 250 * (block + 1)):
        pts = _inputs(seed)
        for par in (False, True):
            st, tris, used = ref(pts, par)
            r = O.triangulate(pts, threaded=par, nthreads=4)
            assert r.status == st, seed
            assert np.array_equal(O.canonical(r.tris), O.canonical(tris)), (seed, par)
            assert np.array_equal(_used_from(r, pts.shape[0]), used), (seed, par)
            nonempty += tris.shape[0] > 0
    assert nonempty > 300   # most inputs are not all collinear
