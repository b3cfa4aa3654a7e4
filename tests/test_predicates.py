"""The engine's predicates against the oracle's exact signs.

The library's orient2d / in-circle (float pre-filter, then the reference's
double filter, then exact integer evaluation) must return the exact sign on
every input; the float pre-filter alone must never return a wrong sign (0 =
undecided is allowed) and must decide almost every well-conditioned input.
The host copies run here on the CPU; the same source compiled for the GPU is
checked by the gpu-marked test.
"""
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
