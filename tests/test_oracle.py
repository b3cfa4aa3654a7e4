"""The CPU oracle against the reference's own outputs.

The fixtures under tests/golden were produced by the reference library
(compiled from its sources; tests/golden/make_golden.py). Here the C
restatement in oracle/ must reproduce them: canonical triangle sets, used
flags, and the reference README's published triangle counts.
"""
import hashlib
import json
import os
from fractions import Fraction

import numpy as np
import pytest

from oracle import oracle as O
from tests.golden import cases as C

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _used_from(res, n):
    used = np.zeros(n, dtype=np.uint8)
    if res.tris.shape[0]:
        used[np.arange(n)[res.rep == np.arange(n)]] = 1
    return used


def _small():
    d = np.load(os.path.join(GOLDEN, "small_cases.npz"))
    names = sorted({k.split("/")[0] for k in d.files})
    return d, names


def test_small_cases_serial_and_threaded():
    d, names = _small()
    assert len(names) > 200
    for name in names:
        pts = d[name + "/pts"]
        for thr in (False, True):
            r = O.triangulate(pts, threaded=thr, nthreads=4)
            assert r.status == 0, name
            assert np.array_equal(O.canonical(r.tris), d[name + "/tris"]), name
            assert np.array_equal(_used_from(r, pts.shape[0]), d[name + "/used"]), name


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


with open(os.path.join(GOLDEN, "digests.json")) as _f:
    # the CPU suite pins the oracle on the fixtures up to 4M points; the GPU
    # tests compare the library with every one, 16M points included
    _DIGESTS = [s for s in json.load(_f)["cases"] if s["npts"] <= 4_000_000]


@pytest.mark.parametrize("spec", _DIGESTS, ids=[s["name"] for s in _DIGESTS])
def test_large_cases_match_reference_digests(spec):
    pts = C.make_large(spec)
    r = O.triangulate(pts, threaded=True)
    ct = O.canonical(r.tris).astype(np.int64)
    assert ct.shape[0] == spec["serial"]["ntri"]
    if "known_ntri" in spec:
        assert ct.shape[0] == spec["known_ntri"]
    assert _digest(ct) == spec["serial"]["tri_digest"]
    assert _digest(_used_from(r, pts.shape[0])) == spec["serial"]["used_digest"]
    # the reference's serial and threaded modes agree on every fixture
    assert spec["serial"]["tri_digest"] == spec["threaded"]["tri_digest"]


def test_config_b_sets_match_reference():
    """Every 16th set of the 4,096-set workload through the oracle against
    the reference's per-set digests (tests/golden/config_b.npz)."""
    ref = np.load(os.path.join(GOLDEN, "config_b.npz"))
    sets = C.config_b_sets()
    for i in range(0, len(sets), 16):
        r = O.triangulate(sets[i])
        used = _used_from(r, sets[i].shape[0])
        got = C.set_record(r.status, r.tris, used)
        want = (int(ref["status"][i]), int(ref["ntri"][i]), int(ref["tri_digest"][i]), int(ref["used_digest"][i]))
        assert got == want, i


def test_check_input_order():
    assert O.check_input(np.zeros((0, 2))) == 0
    assert O.check_input(None) == -2
    bad = np.zeros((5, 2))
    bad[3, 1] = np.nan
    assert O.check_input(bad) == -4
    bad[3, 1] = np.inf
    assert O.check_input(bad) == -4


def _orient_exact(a, b, c):
    ax, ay, bx, by, cx, cy = (Fraction(float(v)) for v in (*a, *b, *c))
    d = (ax - cx) * (by - cy) - (ay - cy) * (bx - cx)
    return (d > 0) - (d < 0)


def _incircle_exact(a, b, c, d):
    F = [Fraction(float(v)) for v in (*a, *b, *c, *d)]
    ax, ay, bx, by, cx, cy, dx, dy = F
    adx, ady, bdx, bdy, cdx, cdy = ax - dx, ay - dy, bx - dx, by - dy, cx - dx, cy - dy
    det = ((adx * adx + ady * ady) * (bdx * cdy - cdx * bdy) + (bdx * bdx + bdy * bdy) * (cdx * ady - adx * cdy)
           + (cdx * cdx + cdy * cdy) * (adx * bdy - bdx * ady))
    return (det > 0) - (det < 0)


def test_predicates_exact_on_adversarial_inputs():
    rng = np.random.default_rng(5)
    for t in range(400):
        kind = t % 4
        if kind == 0:  # nearly collinear / cocircular around 1
            base = rng.random(2)
            pts = [base + rng.integers(-2, 3, size=2) * 2.0 ** -52 for _ in range(4)]
        elif kind == 1:  # lattice
            pts = [rng.integers(0, 4, size=2).astype(float) for _ in range(4)]
        elif kind == 2:  # scaled lattice
            s = np.ldexp(1.0, int(rng.integers(-900, 900)))
            pts = [rng.integers(0, 4, size=2).astype(float) * s for _ in range(4)]
        else:  # points on the unit circle
            a = rng.random(4) * 2 * np.pi
            pts = [np.array([np.cos(x), np.sin(x)]) for x in a]
        a, b, c, d = pts
        assert O.orient2d(a, b, c) == _orient_exact(a, b, c)
        assert O.orient2d(a, b, c, exact=True) == _orient_exact(a, b, c)
        assert O.incircle(a, b, c, d) == _incircle_exact(a, b, c, d)
        assert O.incircle(a, b, c, d, exact=True) == _incircle_exact(a, b, c, d)
