"""Inputs of the golden fixtures and of the parity tests.

The small cases follow the shapes of the reference harness's batch-path
scenarios (qdt_verify.cpp: `structured` :1033-1163, `batch` :1165-1190,
`magnitudes` :1192-1231, `scale` :1233-1258, `circle` :1260-1298, and the
example inputs :745-787), generated here with numpy seeds of our own. The
large specs are the workloads of the benchmark and the reference README's
known-answer sizes.
"""
from __future__ import annotations

import numpy as np

from libqdt_gb300 import workloads as W


def _structured():
    out = []
    g = [(i, j) for i in range(40) for j in range(40)]
    out.append(("grid40", g))
    out.append(("collinear_diagonal", [(i, 2 * i) for i in range(50)]))
    out.append(("collinear_horizontal", [(i, 7) for i in range(50)]))
    out.append(("collinear_vertical", [(7, i) for i in range(50)]))
    out.append(("line_plus_one", [(i, 7) for i in range(50)] + [(25, 8)]))
    out.append(("parabola", [(i, i * i) for i in range(30)]))
    out.append(("all_duplicates", [(5, 5)] * 100))
    r = 1 << 27
    out.append(("near_circle_2p27", [(int(np.round(r * np.cos(2 * np.pi * i / 200))),
                                      int(np.round(r * np.sin(2 * np.pi * i / 200)))) for i in range(200)]))
    out.append(("two_rows", [p for i in range(100) for p in ((i, 0), (i, 1))]))
    out.append(("triangle_with_duplicates", [p for _ in range(20) for p in ((0, 0), (1, 0), (0, 1))]))
    out.append(("empty", []))
    out.append(("one_point", [(1, 1)]))
    out.append(("two_points", [(1, 1), (2, 3)]))
    out.append(("three_collinear", [(0, 0), (1, 1), (2, 2)]))
    out.append(("three_points", [(0, 0), (5, 0), (0, 5)]))
    m = 1 << 28
    out.append(("coords_2p28", [(-m, -m), (m, -m), (0, m), (1, 1), (-1, 2)]))
    out.append(("square4", [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (1.0, 1.0)]))
    out.append(("quad", [(0.0, 0.0), (4.0, 0.0), (3.0, 1.0), (1.0, 1.0)]))
    return out


def small_cases():
    """(name, (n, 2) float64 array) pairs, each a few thousand points at most."""
    cases = []
    for name, pts in _structured():
        base = np.array(pts, dtype=np.float64).reshape(-1, 2)
        for s in range(5):
            p = base.copy()
            if s:
                p = p[np.random.default_rng(77 + s).permutation(p.shape[0])]
            cases.append(("%s_s%d" % (name, s), p))

    ranges = [2, 3, 4, 6, 10, 30, 100, 10000, 1 << 20]
    for s in range(40):
        rng = np.random.default_rng(1000 + s)
        n = int(rng.integers(0, 70))
        R = ranges[int(rng.integers(0, len(ranges)))]
        cases.append(("batch_%d" % s, rng.integers(-R, R + 1, size=(n, 2)).astype(np.float64)))

    levels = [0, 2, 5, 9, 14, 20, 26, 28]
    for s in range(30):
        rng = np.random.default_rng(41000 + s)
        mode = s % 3
        n = 4 + int(rng.integers(0, 60))
        offx = (1 if rng.integers(0, 2) else -1) * (1 << 27)
        offy = (1 if rng.integers(0, 2) else -1) * (1 << 27)
        pts = []
        for i in range(n):
            far = mode == 1 or (mode == 2 and (i & 1))
            if far:
                b = 1 << int(rng.integers(0, 9))
                pts.append((offx + int(rng.integers(-b, b + 1)), offy + int(rng.integers(-b, b + 1))))
            else:
                b = 1 << levels[int(rng.integers(0, len(levels)))]
                pts.append((int(rng.integers(-b, b + 1)), int(rng.integers(-b, b + 1))))
        cases.append(("magnitudes_%d" % s, np.array(pts, dtype=np.float64)))

    for k in (-1000, -600, -300, -64, 64, 300, 600, 900):
        for s in range(6):
            rng = np.random.default_rng(31000 + s)
            R = 6 if rng.integers(0, 2) else 1000
            n = 3 + int(rng.integers(0, 40))
            p = rng.integers(-R, R + 1, size=(n, 2)).astype(np.float64) * np.ldexp(1.0, k)
            cases.append(("scale_%d_%d" % (k, s), p))

    for s in range(20):
        rng = np.random.default_rng(55000 + s)
        n = 8 + int(rng.integers(0, 120))
        Rr = 1 << (20 + int(rng.integers(0, 8)))
        a = 2 * np.pi * rng.integers(0, 100000, size=n) / 100000.0
        cases.append(("circle_%d" % s, np.stack([np.round(Rr * np.cos(a)), np.round(Rr * np.sin(a))], axis=1)))

    cases.append(("uniform_2000", W.uniform(2000, 101)))
    cases.append(("lattice_32_dups", W.lattice_with_duplicates(32, 0.05, 102)))
    cases.append(("gauss_2000", W.gaussian_mixture(2000, 8, 103)))
    cases.append(("unit_circle_500", W.unit_circle(500, 104)))
    cases.append(("noisy_line_1000", W.noisy_line(1000, 105)))
    cases.append(("bench_uniform_100", W.bench_uniform(100, W.BENCH_SEED + 100)))
    return cases


def large_specs():
    specs = []
    for n in sorted(W.BENCH_KNOWN_COUNTS):
        specs.append({"name": "bench_uniform_%d" % n, "gen": "bench_uniform", "n": n,
                      "seed": W.BENCH_SEED + n, "known_ntri": W.BENCH_KNOWN_COUNTS[n]})
    specs.append({"name": "uniform_100k", "gen": "uniform", "n": 100000, "seed": 12345})
    specs.append({"name": "uniform_1m", "gen": "uniform", "n": 1048576, "seed": 1})
    specs.append({"name": "uniform_2p6m", "gen": "uniform", "n": 2600000, "seed": 2})
    specs.append({"name": "lattice_1024_dups", "gen": "lattice", "n": 1024, "seed": 7})
    specs.append({"name": "gauss_4m", "gen": "gauss", "n": 4000000, "seed": 11})
    specs.append({"name": "circle_100k", "gen": "circle", "n": 100000, "seed": 13})
    specs.append({"name": "line_1m", "gen": "line", "n": 1000000, "seed": 17})
    specs.append({"name": "uniform_16m", "gen": "uniform", "n": 1 << 24, "seed": 3})
    return specs


def limit_spec():
    """The reference's size limit (kMaxPoints = 1e8, libqdt/wrapper.hxx:15):
    uniform points, one call."""
    return {"name": "uniform_100m", "gen": "uniform", "n": 100_000_000, "seed": 5}


def canonical_digest32(tris: np.ndarray, chunk: int = 1 << 24) -> str:
    """SHA-256 of oracle.canonical(tris) as int64 rows, computed with 32-bit
    columns and a lexicographic sort of them (indices below 2^31), hashed in
    chunks: the same digest with a fraction of the memory at 1e8 points."""
    import hashlib
    t = np.asarray(tris).reshape(-1, 3)
    h = hashlib.sha256()
    if t.shape[0] == 0:
        return h.hexdigest()
    t = t.astype(np.int32, copy=False)
    k = np.argmin(t, axis=1).astype(np.int8)
    r = np.empty_like(t)
    for j in range(3):
        r[:, j] = np.choose((k + j) % 3, (t[:, 0], t[:, 1], t[:, 2]))
    del k
    if int(r.max()) < (1 << 27):
        # the first two indices identify a triangle of a triangulation (a
        # directed edge bounds one triangle): one 54-bit key, the same order
        order = np.argsort((r[:, 0].astype(np.uint64) << np.uint64(27)) | r[:, 1].astype(np.uint64), kind="stable")
    else:
        order = np.lexsort((r[:, 2], r[:, 1], r[:, 0]))
    for s in range(0, order.shape[0], chunk):
        h.update(r[order[s:s + chunk]].astype(np.int64).tobytes())
    return h.hexdigest()


# The many-set workload at its stated size: 4,096 sets, sizes log-uniform in
# [16, 65,536], square or disk, 10 % snapped to a 256 x 256 grid.
CONFIG_B = {"count": 4096, "lo": 16, "hi": 65536, "seed": 23}


def config_b_sets():
    return W.many_sets(**CONFIG_B)


def canonical_small(tris: np.ndarray) -> np.ndarray:
    """The canonical form of oracle.canonical (each triangle rotated to its
    smallest index, rows sorted) for indices below 2^16, by one sort of
    packed 48-bit keys: the same array, faster on the 4,096 sets."""
    t = np.asarray(tris, dtype=np.int64).reshape(-1, 3)
    if t.shape[0] == 0:
        return t
    assert t.max() < (1 << 16) and t.min() >= 0
    k = np.argmin(t, axis=1)
    idx = (k[:, None] + np.arange(3)[None, :]) % 3
    r = np.take_along_axis(t, idx, axis=1).astype(np.uint64)
    key = np.sort((r[:, 0] << np.uint64(32)) | (r[:, 1] << np.uint64(16)) | r[:, 2])
    out = np.empty((key.shape[0], 3), dtype=np.int64)
    out[:, 0] = (key >> np.uint64(32)).astype(np.int64)
    out[:, 1] = ((key >> np.uint64(16)) & np.uint64(0xFFFF)).astype(np.int64)
    out[:, 2] = (key & np.uint64(0xFFFF)).astype(np.int64)
    return out


def digest64(a: np.ndarray) -> int:
    """The first 8 bytes of the SHA-256 of an array's bytes, as an integer."""
    import hashlib
    return int.from_bytes(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest()[:8], "little")


def set_record(status: int, tris: np.ndarray, used: np.ndarray):
    """(status, triangle count, digest of the canonical triangles, digest of
    the used-point flags) of one set: what the config-B fixture keeps."""
    ct = canonical_small(tris)
    return int(status), int(ct.shape[0]), digest64(ct), digest64(np.asarray(used, dtype=np.uint8))


def make_large(spec) -> np.ndarray:
    g = spec["gen"]
    if g == "bench_uniform":
        return W.bench_uniform(spec["n"], spec["seed"])
    if g == "uniform":
        return W.uniform(spec["n"], spec["seed"])
    if g == "lattice":
        return W.lattice_with_duplicates(spec["n"], 0.01, spec["seed"])
    if g == "gauss":
        return W.gaussian_mixture(spec["n"], 64, spec["seed"])
    if g == "circle":
        return W.unit_circle(spec["n"], spec["seed"])
    if g == "line":
        return W.noisy_line(spec["n"], spec["seed"])
    raise ValueError(g)


def mesh_cases():
    """Handle operations after a batch call (qdt_verify.cpp's `examples`,
    `insert` and `constraint` scenarios in spirit): (name, points, ops) with
    ops a list of ("insert", x, y) and ("constraint", i, j)."""
    out = []
    sq = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0]])
    out.append(("six_point_example", sq, [("insert", 0.5, 0.5), ("insert", 0.25, 0.75)]))
    quad = np.array([[0.0, 0.0], [4.0, 0.0], [3.0, 1.0], [1.0, 1.0]])
    out.append(("quad_constraint", quad, [("constraint", 0, 2), ("constraint", 0, 9), ("constraint", 1, 1),
                                          ("constraint", 2, 0)]))
    for s in range(12):
        rng = np.random.default_rng(7000 + s)
        n = int(rng.integers(5, 300))
        if s % 3 == 0:
            p = rng.random((n, 2))
        elif s % 3 == 1:
            p = rng.integers(0, 50, size=(n, 2)).astype(np.float64)
        else:
            p = np.round(rng.random((n, 2)) * 1000) / 8.0
        ops = []
        for _ in range(int(rng.integers(1, 40))):
            if rng.random() < 0.5:
                if s % 3 == 0:
                    ops.append(("insert", float(rng.random() * 1.4 - 0.2), float(rng.random() * 1.4 - 0.2)))
                else:
                    q = p[int(rng.integers(0, n))] if rng.random() < 0.2 else rng.integers(-5, 55, size=2)
                    ops.append(("insert", float(q[0]), float(q[1])))
            else:
                ops.append(("constraint", int(rng.integers(0, n + 5)), int(rng.integers(0, n + 5))))
        out.append(("mixed_%d" % s, p, ops))
    # long runs of single insertions: enough walk steps that the host's seed
    # grid of walk starts is built part-way through (uniform points with
    # insertions partly outside the hull; an integer lattice with insertions
    # on its vertices, on its edges and outside)
    rng = np.random.default_rng(7100)
    p = rng.random((4000, 2))
    ops = [("insert", float(x), float(y)) for x, y in rng.random((300, 2)) * 1.2 - 0.1]
    out.append(("long_uniform", p, ops))
    g = np.stack(np.meshgrid(np.arange(40.0), np.arange(40.0)), axis=-1).reshape(-1, 2)
    ops = []
    for k in range(300):
        i, j = (float(v) for v in rng.integers(0, 40, size=2))
        kind = k % 4
        q = (i, j) if kind == 0 else ((i + 0.5, j) if kind == 1 else ((i + 0.25, j + 0.75) if kind == 2 else
                                                                      (i * 1.5 - 10.0, j - 45.0)))
        ops.append(("insert", q[0], q[1]))
    out.append(("long_lattice", g, ops))
    return out
