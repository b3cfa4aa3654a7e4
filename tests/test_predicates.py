"""The engine's predicates against the oracle's exact signs.

The library's orient2d / in-circle (float pre-filter, then the reference's
double filter, then exact integer evaluation) must return the exact sign on
every input; the float pre-filter alone must never return a wrong sign (0 =
undecided is allowed) and must decide almost every well-conditioned input.
The host copies run here on the CPU; the same source compiled for the GPU is
checked by the gpu-marked test.
"""
from fractions import Fraction

import numpy as np
import pytest

import libqdt_gb300 as G
from oracle import delaunay_check as D


def _adversarial(kind, n, seed):
    rng = np.random.default_rng(seed)
    k = 3 if kind == "orient" else 4
    out = []
    per = n // 9
    # 1) uniform in the unit square
    out.append(rng.random((per, k, 2)))
    # 2) nearly collinear / cocircular: lattice points perturbed by a few ulps
    base = rng.integers(0, 8, size=(per, k, 2)).astype(np.float64)
    out.append(base + rng.integers(-3, 4, size=(per, k, 2)) * 2.0 ** -50)
    # 3) exact lattice (many exact zeros)
    out.append(rng.integers(0, 4, size=(per, k, 2)).astype(np.float64))
    # 4) far from the origin, tiny spread
    out.append(1e6 + rng.random((per, k, 2)) * 1e-6)
    # 5) points on the unit circle (in-circle nearly zero)
    a = rng.random((per, k)) * 2 * np.pi
    out.append(np.stack([np.cos(a), np.sin(a)], axis=2))
    # 6) scaled far outside the float range of the pre-filter
    s = np.ldexp(1.0, rng.integers(-900, 900, size=(per, 1, 1)))
    out.append(rng.integers(0, 5, size=(per, k, 2)).astype(np.float64) * s)
    # 7) mixed magnitudes
    m = rng.random((per, k, 2)) * np.ldexp(1.0, rng.integers(-40, 40, size=(per, k, 2)))
    out.append(m)
    # 8) nearly collinear along a line with random slopes, tiny noise
    t = rng.random((per, k, 1))
    d = rng.standard_normal((per, 1, 2))
    out.append(0.5 + t * d + rng.standard_normal((per, k, 2)) * 2.0 ** -45)
    # 9) degenerate at float resolution: lattice points moved by a few 2^-30,
    # below what rounding the coordinates to float keeps
    base = rng.integers(0, 64, size=(per, k, 2)).astype(np.float64) / 64
    out.append(base + rng.integers(-4, 5, size=(per, k, 2)) * 2.0 ** -30)
    return np.concatenate(out, axis=0)


def _exact(kind, pts):
    k = pts.shape[1]
    flat = np.ascontiguousarray(pts.reshape(-1, 2))
    idx = np.arange(flat.shape[0], dtype=np.int64).reshape(-1, k)
    return D.orient_signs(flat, idx) if kind == "orient" else D.incircle_signs(flat, idx)


@pytest.mark.parametrize("kind", ["orient", "incircle"])
def test_host_predicates_exact(kind):
    pts = _adversarial(kind, 80000, 1 if kind == "orient" else 2)
    want = _exact(kind, pts)
    coords = pts.reshape(pts.shape[0], -1)
    got = G.eval_predicates(kind, coords, "full")
    assert np.array_equal(got, want)
    ex = G.eval_predicates(kind, coords, "exact")
    assert np.array_equal(ex, want)
    f = G.eval_predicates(kind, coords, "f32")
    decided = f != 0
    assert np.array_equal(f[decided], want[decided])   # never a wrong sign
    # the uniform block is decided almost always
    per = pts.shape[0] // 9
    assert decided[:per].mean() > 0.98


def _range_edges(kind, n, seed):
    """Inputs at the edges of the float pre-filter's accepted range: the
    coordinate differences of an orient2d are accepted in [2^-60, 2^60), of
    an in-circle in [2^-30, 2^30) (zero always). Differences exactly at,
    one ulp inside and one ulp outside each end; mixed ends in one
    predicate; exact and near (one-ulp) degeneracies at the smallest
    accepted scale, where products and their differences fall toward the
    float subnormal range; subnormal doubles."""
    rng = np.random.default_rng(seed)
    k = 3 if kind == "orient" else 4
    lo, hi = (-60, 59) if kind == "orient" else (-30, 29)
    ends = np.array([lo - 2, lo - 1, lo, lo + 1, hi - 1, hi, hi + 1, hi + 2])
    per = n // 6
    out = []

    def nudge(p):
        d = rng.integers(-1, 2, size=p.shape)
        return np.where(d > 0, np.nextafter(p, np.inf), np.where(d < 0, np.nextafter(p, -np.inf), p))

    def last_at_zero(p):
        p[: p.shape[0] // 2, -1, :] = 0.0       # differences equal the coordinates
        return p

    # 1) one edge scale per predicate, small integers, one-ulp nudges
    E = rng.choice(ends, size=(per, 1, 1))
    out.append(last_at_zero(nudge(np.ldexp(rng.integers(-4, 5, size=(per, k, 2)).astype(np.float64), E))))
    # 2) an edge scale per coordinate (both ends inside one predicate)
    E = rng.choice(ends, size=(per, k, 2))
    out.append(last_at_zero(np.ldexp(rng.integers(-3, 4, size=(per, k, 2)).astype(np.float64), E)))
    # 3) magnitudes 2^e, 2^e (1 + 2^-52) and 2^(e+1) (1 - 2^-53) at the ends
    E = rng.choice(ends, size=(per, k, 2))
    frac = rng.choice(np.array([1.0, 1.0 + 2.0 ** -52, 2.0 - 2.0 ** -52]), size=(per, k, 2))
    sign = rng.choice(np.array([-1.0, 1.0]), size=(per, k, 2))
    p = np.ldexp(sign * frac, E)
    p[:, -1, :] = 0.0
    out.append(p)
    # 4) exact degeneracies at the smallest accepted scale, one-ulp nudges:
    # collinear multiples (orient) or Pythagorean points on one circle
    # (in-circle), so products and their difference fall toward 2^-126
    s = np.ldexp(1.0, lo + rng.integers(0, 3, size=(per, 1, 1)))
    if kind == "orient":
        u = rng.integers(1, 6, size=(per, 1, 2)).astype(np.float64)
        t = rng.integers(-3, 4, size=(per, k, 1)).astype(np.float64)
        base = t * u
    else:
        circ = np.array([[5, 0], [0, 5], [-5, 0], [0, -5], [3, 4], [4, 3], [-3, 4], [-4, -3], [3, -4]], np.float64)
        base = circ[rng.integers(0, circ.shape[0], size=(per, k))]
    out.append(nudge(base * s))
    # 5) the same at the largest accepted scale
    out.append(nudge(base * np.ldexp(1.0, hi - 3 + rng.integers(0, 3, size=(per, 1, 1)))))
    # 6) subnormal and smallest normal doubles
    tiny = rng.choice(np.array([5e-324, 1e-323, 2.2250738585072014e-308, 0.0]), size=(per, k, 2))
    out.append(tiny * rng.choice(np.array([-1.0, 1.0]), size=(per, k, 2)))
    return np.concatenate(out, axis=0)


def _exact_fraction(kind, pts):
    """Signs by exact rational arithmetic (Python Fractions of the doubles):
    independent of both the library and the oracle."""
    out = np.zeros(pts.shape[0], dtype=np.int8)
    for i, q in enumerate(pts):
        f = [(Fraction(float(x)), Fraction(float(y))) for x, y in q]
        if kind == "orient":
            (ax, ay), (bx, by), (cx, cy) = f
            d = (ax - cx) * (by - cy) - (ay - cy) * (bx - cx)
        else:
            (ax, ay), (bx, by), (cx, cy), (dx, dy) = f
            adx, ady, bdx, bdy, cdx, cdy = ax - dx, ay - dy, bx - dx, by - dy, cx - dx, cy - dy
            d = ((adx * adx + ady * ady) * (bdx * cdy - cdx * bdy) + (bdx * bdx + bdy * bdy) * (cdx * ady - adx * cdy)
                 + (cdx * cdx + cdy * cdy) * (adx * bdy - bdx * ady))
        out[i] = (d > 0) - (d < 0)
    return out


@pytest.mark.parametrize("kind", ["orient", "incircle"])
def test_prefilter_range_edges_host(kind):
    pts = _range_edges(kind, 6000, 31 if kind == "orient" else 32)
    want = _exact_fraction(kind, pts)
    # The oracle follows the reference's expansion arithmetic, which scales
    # by the largest coordinate only (robust.hxx:297-306): with a subnormal
    # coordinate beside larger ones its products underflow and its sign can
    # be 0 or wrong. Everywhere else it is exact.
    a = np.abs(pts.reshape(pts.shape[0], -1))
    subnormal = ((a > 0) & (a < 2.2250738585072014e-308)).any(axis=1)
    orc = _exact(kind, pts)
    assert np.array_equal(orc[~subnormal], want[~subnormal])
    coords = pts.reshape(pts.shape[0], -1)
    assert np.array_equal(G.eval_predicates(kind, coords, "full"), want)
    f = G.eval_predicates(kind, coords, "f32")
    assert np.array_equal(f[f != 0], want[f != 0])      # never a wrong sign at the range edges
    assert (f != 0).any() and (f == 0).any()            # both outcomes occur in these blocks


def test_host_single_calls():
    lib = G.load()
    a = np.array([0.0, 0.0])
    b = np.array([1.0, 0.0])
    c = np.array([0.0, 1.0])
    d = np.array([1.0, 1.0])
    e = np.array([0.5, 0.5])
    P = lambda v: v.ctypes.data  # noqa: E731
    assert lib.qdtg_orient2d(P(a), P(b), P(c)) == 1
    assert lib.qdtg_orient2d(P(a), P(c), P(b)) == -1
    assert lib.qdtg_orient2d(P(a), P(e), P(d)) == 0
    assert lib.qdtg_incircle(P(a), P(b), P(c), P(d)) == 0
    assert lib.qdtg_incircle(P(a), P(b), P(c), P(e)) == 1


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["orient", "incircle"])
def test_device_predicates_exact(kind):
    pts = _adversarial(kind, 160000, 3 if kind == "orient" else 4)
    want = _exact(kind, pts)
    coords = pts.reshape(pts.shape[0], -1)
    for mode in ("full", "exact"):
        assert np.array_equal(G.eval_predicates(kind, coords, mode, device=True), want)
    f = G.eval_predicates(kind, coords, "f32", device=True)
    assert np.array_equal(f[f != 0], want[f != 0])
    # host and device pre-filters take the same decisions
    assert np.array_equal(f, G.eval_predicates(kind, coords, "f32"))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["orient", "incircle"])
def test_prefilter_range_edges_device(kind):
    pts = _range_edges(kind, 6000, 33 if kind == "orient" else 34)
    want = _exact_fraction(kind, pts)
    coords = pts.reshape(pts.shape[0], -1)
    for mode in ("full", "exact"):
        assert np.array_equal(G.eval_predicates(kind, coords, mode, device=True), want)
    f = G.eval_predicates(kind, coords, "f32", device=True)
    assert np.array_equal(f[f != 0], want[f != 0])
    assert np.array_equal(f, G.eval_predicates(kind, coords, "f32"))
