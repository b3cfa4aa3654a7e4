"""Parity of the GPU batch path with the reference, through the C ABI.

* small structured and random cases: the canonical triangle set and the
  used-point flags equal the reference's own outputs (tests/golden);
* the large workloads (up to 4M points): SHA-256 of the canonical set and of
  the used flags equal the reference's, and the README's published counts;
* random sets of many shapes: equal to the CPU oracle, triangles and
  representatives;
* the exact Delaunay checker finds zero violations on the stress workloads;
* errors: NaN/inf input gives QDT_ERR_NOT_FINITE and an empty context.
Integer/index outputs, so every comparison is bit-exact.
"""
import hashlib
import json
import os
import threading

import numpy as np
import pytest

import libqdt_gb300 as G
from libqdt_gb300 import qdt_api as Q
from libqdt_gb300 import workloads as W
from oracle import delaunay_check as D
from oracle import oracle as O
from tests.golden import cases as C

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def lib():
    return G.load()


def run(lib, pts, parallel=False):
    with G.Triangulation(lib) as t:
        st = t.execute(pts, parallel=parallel)
        return st, t.triangles_array().astype(np.int64), t.rep_array(), t.points_size()


def used_flags(tris, n):
    u = np.zeros(n, dtype=np.uint8)
    if tris.shape[0]:
        u[np.unique(tris.ravel())] = 1
    return u


def test_small_cases_equal_reference(lib):
    d = np.load(os.path.join(GOLDEN, "small_cases.npz"))
    names = sorted({k.split("/")[0] for k in d.files})
    for name in names:
        pts = d[name + "/pts"]
        for par in (False, True):
            st, tris, rep, npts = run(lib, pts, par)
            assert st == 0, name
            assert npts == pts.shape[0]
            assert np.array_equal(O.canonical(tris), d[name + "/tris"]), name
            assert np.array_equal(used_flags(tris, pts.shape[0]), d[name + "/used"]), name
            with G.Triangulation(lib) as t:
                t.execute(pts)
                flags = np.array([t.point_is_used(i) for i in range(pts.shape[0])], dtype=np.uint8)
            assert np.array_equal(flags, d[name + "/used"]), name


with open(os.path.join(GOLDEN, "digests.json")) as _f:
    _DIGESTS = json.load(_f)["cases"]


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("spec", _DIGESTS, ids=[s["name"] for s in _DIGESTS])
def test_large_workloads_equal_reference(lib, spec):
    pts = C.make_large(spec)
    st, tris, rep, npts = run(lib, pts)
    assert st == 0
    ct = O.canonical(tris).astype(np.int64)
    assert ct.shape[0] == spec["serial"]["ntri"]
    if "known_ntri" in spec:
        assert ct.shape[0] == spec["known_ntri"]
    assert _digest(ct) == spec["serial"]["tri_digest"]
    used = (rep == np.arange(npts)).astype(np.uint8) if ct.shape[0] else np.zeros(npts, np.uint8)
    assert _digest(used) == spec["serial"]["used_digest"]


def _canonical_digest_on_gpu(tris):
    """tests/golden/cases.canonical_digest32 (the SHA-256 of oracle.canonical
    as int64 rows) with the rotation and the sort done by torch on the GPU:
    the same bytes hashed, in seconds at 2e8 triangles."""
    torch = pytest.importorskip("torch")
    t = torch.from_numpy(np.ascontiguousarray(tris).astype(np.int64)).cuda()
    k = torch.argmin(t, dim=1)
    idx = (k[:, None] + torch.arange(3, device=t.device)[None, :]) % 3
    r = torch.gather(t, 1, idx)
    del t, k, idx
    assert int(r.max()) < (1 << 27)
    order = torch.argsort(r[:, 0] * (1 << 27) + r[:, 1], stable=True)
    r = r[order]
    del order
    h = hashlib.sha256()
    step = 1 << 24
    for i in range(0, r.shape[0], step):
        h.update(r[i:i + step].cpu().numpy().tobytes())
    del r
    torch.cuda.empty_cache()
    return h.hexdigest()


def test_reference_size_limit(lib):
    """At the reference's own size limit (kMaxPoints = 1e8 points,
    libqdt/wrapper.hxx:15) one call gives the reference's triangles and
    used points: digests made by the reference itself, serial call
    (tests/golden/limit.json, make_limit.py)."""
    with open(os.path.join(GOLDEN, "limit.json")) as f:
        spec = json.load(f)["case"]
    pts = C.make_large(spec)
    assert pts.shape[0] == 100_000_000
    with G.Triangulation(lib) as t:
        assert t.execute(pts) == 0
        tris = t.triangles_array()
        rep = t.rep_array()
    del pts
    assert tris.shape[0] == spec["serial"]["ntri"]
    assert _canonical_digest_on_gpu(tris) == spec["serial"]["tri_digest"]
    del tris
    used = (rep == np.arange(rep.shape[0], dtype=rep.dtype)).astype(np.uint8)
    assert _digest(used) == spec["serial"]["used_digest"]


def _random_sets():
    rng = np.random.default_rng(2024)
    out = []
    for i in range(120):
        n = int(rng.integers(0, 3000)) if i % 3 else int(rng.integers(0, 40))
        kind = i % 6
        if kind == 0:
            R = int(rng.choice([1, 2, 3, 5, 10, 100, 1 << 20]))
            p = rng.integers(-R, R + 1, size=(n, 2)).astype(np.float64)
        elif kind == 1:
            p = rng.random((n, 2))
        elif kind == 2:
            p = np.round(rng.random((n, 2)) * 64) / 64
        elif kind == 3:
            a = rng.integers(0, 360, size=n) * (np.pi / 180)
            p = np.stack([np.round(1000 * np.cos(a)), np.round(1000 * np.sin(a))], axis=1)
        elif kind == 4:
            p = rng.random((n, 2)) * np.ldexp(1.0, int(rng.integers(-900, 900)))
        else:
            x = rng.random(n)
            p = np.stack([x, 0.5 * x + rng.uniform(-1, 1, size=n) * 2.0 ** -40], axis=1)
        out.append(p)
    return out


def test_random_sets_equal_oracle(lib):
    for p in _random_sets():
        st, tris, rep, _ = run(lib, p)
        o = O.triangulate(p)
        assert st == 0
        assert np.array_equal(O.canonical(tris), O.canonical(o.tris))
        assert np.array_equal(rep, o.rep)


def test_cell_sizes_same_result(lib):
    """The shared-memory cells are a schedule, not a different algorithm: the
    triangulation is the same for every cell size, none included."""
    inputs = [W.uniform(60000, 31), W.lattice_with_duplicates(128, 0.02, 32), W.unit_circle(5000, 33),
              W.noisy_line(20000, 34), W.gaussian_mixture(30000, 8, 35), W.uniform(5, 36), W.uniform(1100, 37)]
    for p in inputs:
        want = O.canonical(O.triangulate(p).tris)
        with G.Triangulation(lib) as t:
            for c in (0, 4, 5, 17, 64, 256, 1024):
                assert t.set_cell_points(c)
                assert t.execute(p) == 0
                assert np.array_equal(O.canonical(t.triangles_array()), want), (p.shape, c)
            assert not t.set_cell_points(3) and not t.set_cell_points(1025)
            assert t.set_cell_points(0)
            for nodes in (1, 64, 1 << 20):       # warp merges from the fewest depths to every depth
                assert t.set_warp_nodes(nodes)
                assert t.execute(p) == 0
                assert np.array_equal(O.canonical(t.triangles_array()), want), (p.shape, nodes)
            assert not t.set_warp_nodes(0)


def test_graphs_same_result(lib):
    """The stages after the distinct-point count replay from a CUDA graph per
    (count, knobs): sizes that come and go, knob changes between calls and
    the launch-by-launch form all give the oracle's triangles and the same
    launch count."""
    inputs = [W.uniform(70000, 51), W.lattice_with_duplicates(100, 0.02, 52), W.uniform(70000, 53),
              W.uniform(5000, 54), W.uniform(70000, 51)]
    with G.Triangulation(lib) as t:
        for p in inputs:
            want = O.canonical(O.triangulate(p).tris)
            got = {}
            for graphs in (True, False, True):
                assert t.set_graphs(graphs)
                for cells, nodes in ((0, 4096), (64, 64)):
                    assert t.set_cell_points(cells) and t.set_warp_nodes(nodes)
                    assert t.execute(p) == 0
                    assert np.array_equal(O.canonical(t.triangles_array()), want), (p.shape, graphs, cells)
                    got.setdefault((cells, nodes), set()).add(t.run_info()["kernel_launches"])
            assert all(len(v) == 1 for v in got.values()), got
        assert t.set_cell_points(0) and t.set_warp_nodes(4096)


def test_split_tail_same_result(lib):
    """The split depths of nodes of at most 4,096 points run in one
    shared-memory launch or one level at a time: the same triangles (the
    oracle's), sizes on both sides of the block limit, degenerate inputs."""
    rng = np.random.default_rng(81)
    inputs = [W.uniform(n, 80 + n) for n in (4, 5, 7, 8, 100, 4095, 4096, 4097, 8192, 8193, 12289, 70000)]
    inputs += [W.lattice_with_duplicates(90, 0.05, 82), W.unit_circle(9000, 83), W.noisy_line(20000, 84),
               np.round(rng.random((30000, 2)) * 64) / 64]
    with G.Triangulation(lib) as t:
        for p in inputs:
            want = O.canonical(O.triangulate(p).tris)
            launches = {}
            for tail in (True, False, True):
                assert t.set_split_tail(tail)
                assert t.execute(p) == 0
                assert np.array_equal(O.canonical(t.triangles_array()), want), (p.shape, tail)
                launches.setdefault(tail, set()).add(t.run_info()["kernel_launches"])
            assert len(launches[True]) == 1
            if p.shape[0] > 4:
                assert min(launches[True]) < min(launches[False]), (p.shape, launches)


def test_side_prefetch_same_result(lib):
    """The seam prefetch of the next depth runs on a side stream while the
    current depth's merges edit the records it scans (a read-only hint: it
    selects record numbers below the pool size and never writes a record).
    On and off give bit-identical triangle and representative arrays, and on
    the 1M uniform workload the reference's digest."""
    spec = next(s for s in _DIGESTS if s["name"] == "uniform_1m")
    inputs = [("uniform_1m", C.make_large(spec)), ("lattice", W.lattice_with_duplicates(400, 0.01, 91)),
              ("gauss", W.gaussian_mixture(300000, 64, 92)), ("circle", W.unit_circle(70000, 93))]
    for name, p in inputs:
        got = {}
        for side in (False, True, False, True):
            with G.Triangulation(lib) as t:
                assert t.set_side_prefetch(side)
                assert t.execute(p) == 0
                got.setdefault(side, []).append((t.triangles_array().copy(), t.rep_array().copy()))
        ref_tris, ref_rep = got[False][0]
        for side in (False, True):
            for tris, rep in got[side]:
                assert np.array_equal(tris, ref_tris), (name, side)
                assert np.array_equal(rep, ref_rep), (name, side)
        if name == "uniform_1m":
            assert _digest(O.canonical(ref_tris).astype(np.int64)) == spec["serial"]["tri_digest"]


def _split_inputs():
    """Workloads for the two-walker merges: general position, clusters,
    heavy ties (lattice, snapped grid), cocircular and near-collinear points,
    and long seams (points on two lines parallel to the root's cut)."""
    rng = np.random.default_rng(97)
    n = 300000
    yield "gauss", W.gaussian_mixture(400000, 64, 94)
    yield "lattice", W.lattice_with_duplicates(400, 0.01, 95)
    yield "circle", W.unit_circle(70000, 96)
    yield "line", W.noisy_line(n, 97)
    yield "skewed", np.column_stack([rng.exponential(1.0, n) ** 3, rng.standard_normal(n)])
    yield "snapped", np.round(rng.random((n, 2)) * 256.0) / 256.0
    centers = rng.random((40, 2))
    yield "blobs", centers[rng.integers(0, 40, n)] + 1e-6 * rng.standard_normal((n, 2))
    y = rng.random(n)
    yield "two_lines", np.column_stack([np.where(np.arange(n) % 2 == 0, 0.25, 0.75) + 1e-9 * rng.random(n), y])


def test_split_merges_same_result(lib):
    """The top merges with two walkers (rising and mirrored falling, meeting
    on the seam) give the canonical triangle set and representatives of the
    one-walker build on every kind of input, without falling back (the
    fallback would hide a wrong walk); two runs give identical arrays; the
    1M uniform workload keeps the reference's digest. The merge window is
    fixed at 2, so that lattice-like input (where a call leaves the split
    merges off by default) runs them too. One seam segment a merge here;
    test_split_segments_same_result covers more."""
    spec = next(s for s in _DIGESTS if s["name"] == "uniform_1m")
    inputs = [("uniform_1m", C.make_large(spec))] + list(_split_inputs())
    for name, p in inputs:
        out = {}
        for split in (True, False, True):
            with G.Triangulation(lib) as t:
                assert t.set_merge_window(2)
                assert t.set_split_segments(1)
                if not split:
                    assert t.set_split_merges(-1)
                assert t.execute(p) == 0, name
                info = t.run_info()
                if split:
                    assert info["split_depth"] >= 0, name
                    assert info["split_rerun"] == 0, name
                else:
                    assert info["split_depth"] == -1, name
                out.setdefault(split, []).append((t.triangles_array().copy(), t.rep_array().copy()))
        (t1, r1), (t2, r2) = out[True]
        assert np.array_equal(t1, t2) and np.array_equal(r1, r2), name
        t0, r0 = out[False][0]
        assert np.array_equal(O.canonical(t1), O.canonical(t0)), name
        assert np.array_equal(r1, r0), name
        if name == "uniform_1m":
            assert _digest(O.canonical(t1).astype(np.int64)) == spec["serial"]["tri_digest"]


# inputs in general position whose seams are not much longer than 3 sqrt(n)
# steps: their split merges must run with more than one seam segment and
# without falling back (the heavy-tailed "skewed" input has seams several
# times longer, where a segment's walkers can run out of spare records and
# the call runs again with one segment)
_GENERAL = ("uniform_1m", "uniform_2p6m", "gauss", "blobs", "line")


def test_split_segments_same_result(lib):
    """Seams cut into segments at boundary edges (mutually nearest vertices
    of the two halves, the children's edges that cross them deleted first),
    two walkers a segment: for 1, 2 and 5 segments the canonical triangles
    and representatives of the one-walker build, on every kind of input, and
    identical arrays on a second run. On input in general position the
    merges use the segments without falling back; on degenerate input (a
    walker above the first segment meets a zero) or very long seams (a
    segment's walkers run out of spare records) the call runs again with one
    segment, with the same result."""
    spec = next(s for s in _DIGESTS if s["name"] == "uniform_1m")
    inputs = [("uniform_1m", C.make_large(spec)), ("uniform_2p6m", W.uniform(2600000, 7))] + list(_split_inputs())
    for name, p in inputs:
        with G.Triangulation(lib) as t:
            assert t.set_merge_window(2)
            assert t.set_split_merges(-1)
            assert t.execute(p) == 0, name
            want_t = O.canonical(t.triangles_array())
            want_r = t.rep_array().copy()
        for segs in (1, 2, 5):
            runs = []
            for _ in range(2):
                with G.Triangulation(lib) as t:
                    assert t.set_merge_window(2)
                    assert t.set_split_segments(segs)
                    assert t.execute(p) == 0, (name, segs)
                    info = t.run_info()
                    runs.append((t.triangles_array().copy(), t.rep_array().copy(), info))
            (t1, r1, i1), (t2, r2, _) = runs
            assert np.array_equal(t1, t2) and np.array_equal(r1, r2), (name, segs)
            assert np.array_equal(O.canonical(t1), want_t), (name, segs)
            assert np.array_equal(r1, want_r), (name, segs)
            assert i1["split_segments"] <= segs, (name, segs)
            if name in _GENERAL:
                assert i1["split_rerun"] == 0, (name, segs)
                assert i1["split_segments"] == segs, (name, segs)
        if name == "uniform_1m":
            assert _digest(O.canonical(t1).astype(np.int64)) == spec["serial"]["tri_digest"]


def test_split_segments_knob(lib):
    with G.Triangulation(lib) as t:
        assert not t.set_split_segments(0)
        assert not t.set_split_segments(6)
        assert not t.set_split_segments(2, 1023)
        for segs in (1, 2, 3, 4, 5):
            assert t.set_split_segments(segs)


def test_split_merges_off_on_lattice_like_input(lib):
    """On lattice-like input (most points share their x with another) a call
    runs every merge with one walker, unless the merge window is fixed."""
    p = W.lattice_with_duplicates(400, 0.01, 99)
    with G.Triangulation(lib) as t:
        assert t.execute(p) == 0
        assert t.run_info()["split_depth"] == -1
        ref = O.canonical(t.triangles_array())
        assert t.set_merge_window(2)
        assert t.execute(p) == 0
        assert t.run_info()["split_depth"] >= 0
        assert np.array_equal(O.canonical(t.triangles_array()), ref)


def test_split_merges_knob(lib):
    """qdtg_set_split_merges: depth -1..9 and at least 256 points accepted,
    anything else refused; deeper splits and smaller nodes give the same
    triangles."""
    p = W.uniform(200000, 98)
    with G.Triangulation(lib) as t:
        assert not t.set_split_merges(10)
        assert not t.set_split_merges(-2)
        assert not t.set_split_merges(3, 255)
        assert t.set_split_merges(-1)
        assert t.execute(p) == 0
        ref = O.canonical(t.triangles_array())
        for depth, mn in ((0, 4096), (5, 4096), (9, 4096), (8, 65536), (9, 256)):
            assert t.set_split_merges(depth, mn)
            assert t.execute(p) == 0
            info = t.run_info()
            assert info["split_rerun"] == 0
            assert info["split_depth"] == min(depth, int(np.floor(np.log2(200000 / mn))), 9), (depth, mn)
            assert np.array_equal(O.canonical(t.triangles_array()), ref), (depth, mn)


def test_filter_stats_per_stage(lib):
    """Counting the predicates (per stage: leaves, thread merges, warp
    merges, extraction) leaves the result unchanged; every stage is counted;
    undecided counts nest (exact <= float-undecided <= calls); the totals
    equal run_info's; uniform points never need the exact in-circle, the
    lattice with duplicates does."""
    cases = [("uniform", W.uniform(300000, 61), False), ("lattice", W.lattice_with_duplicates(300, 0.01, 62), True)]
    for name, p, degenerate in cases:
        with G.Triangulation(lib) as t:
            assert t.execute(p) == 0
            plain = O.canonical(t.triangles_array())
            t.set_options(count_filter_failures=True)
            assert t.execute(p) == 0
            assert np.array_equal(O.canonical(t.triangles_array()), plain), name
            fs = t.filter_stats()
            info = t.run_info()
        tot = {"orient2d": 0, "incircle": 0}
        for stage in ("leaf", "thread", "warp", "extract"):
            for pred in ("orient2d", "incircle"):
                c = fs[stage][pred]
                assert c["exact"] <= c["f32_undecided"] <= c["calls"], (name, stage, pred, c)
                tot[pred] += c["exact"]
            assert fs[stage]["orient2d"]["calls"] > 0, (name, stage)
        assert fs["extract"]["incircle"]["calls"] == 0 and fs["leaf"]["incircle"]["calls"] == 0
        assert fs["warp"]["incircle"]["calls"] > 0 and fs["thread"]["incircle"]["calls"] > 0
        assert tot["orient2d"] == info["orient_exact"] and tot["incircle"] == info["incircle_exact"]
        if degenerate:
            assert tot["incircle"] > 0 and tot["orient2d"] > 0
        else:
            assert tot["incircle"] == 0


def test_wide_exact_rerun(lib):
    """Coordinates that span more than 95 bits inside one predicate need the
    widest exact tier, which the default build kernels leave out: such a
    call runs its build again with the kernels that have it (run_info
    wide_exact), and its triangles are the oracle's. Ordinary inputs never
    take the second run."""
    rng = np.random.default_rng(71)
    base = rng.integers(0, 40, size=(3000, 2)).astype(np.float64)
    tiny = base.copy()
    tiny[::7] += np.ldexp(rng.integers(1, 8, size=(tiny[::7].shape[0], 2)).astype(np.float64), -90)
    for p, wide in ((tiny, 1), (W.uniform(20000, 72), 0), (W.lattice_with_duplicates(60, 0.02, 73), 0)):
        with G.Triangulation(lib) as t:
            assert t.execute(p) == 0
            assert t.run_info()["wide_exact"] == wide
            assert np.array_equal(O.canonical(t.triangles_array()), O.canonical(O.triangulate(p).tris))


def test_merge_window_same_result(lib):
    """The warp merges' candidate window (1 or 2) is a schedule: the same
    triangulation either way; the automatic choice takes 1 on lattice-like
    input and 2 on points in general position."""
    grid = np.round(np.random.default_rng(41).random((40000, 2)) * 96) / 96
    inputs = [("uniform", W.uniform(80000, 41), 2), ("lattice", W.lattice_with_duplicates(160, 0.02, 42), 1),
              ("grid", grid, 1), ("circle", W.unit_circle(6000, 43), 2), ("line", W.noisy_line(30000, 44), 2)]
    for name, p, auto in inputs:
        want = O.canonical(O.triangulate(p).tris)
        with G.Triangulation(lib) as t:
            assert t.set_warp_nodes(1 << 20)   # every depth merges with warps
            t.set_options(stage_timing=False)
            for w in (1, 2, 0):
                assert t.set_merge_window(w)
                assert t.execute(p) == 0
                assert np.array_equal(O.canonical(t.triangles_array()), want), (name, w)
                assert t.run_info()["merge_window"] == (w or auto), (name, w)
            assert not t.set_merge_window(3)


@pytest.mark.parametrize("name", ["gauss_300k", "circle_100k", "line_1m", "lattice_512"])
def test_exact_checker_zero_violations(lib, name):
    pts = {"gauss_300k": lambda: W.gaussian_mixture(300000, 64, 5),
           "circle_100k": lambda: W.unit_circle(100000, 6),
           "line_1m": lambda: W.noisy_line(1000000, 7),
           "lattice_512": lambda: W.lattice_with_duplicates(512, 0.01, 8)}[name]()
    st, tris, rep, _ = run(lib, pts)
    assert st == 0
    res = D.check(pts, tris, rep)
    assert D.ok(res), res


def test_not_finite_and_recovery(lib):
    p = W.uniform(1000, 1)
    bad = p.copy()
    bad[517, 0] = np.nan
    with G.Triangulation(lib) as t:
        assert t.execute(p) == 0 and t.triangles_size() > 0
        assert t.execute(bad) == Q.QDT_ERR_NOT_FINITE
        assert t.points_size() == 0 and t.triangles_size() == 0
        bad[517, 0] = np.inf
        assert t.execute(bad, parallel=True) == Q.QDT_ERR_NOT_FINITE
        assert t.execute(p) == 0
        assert np.array_equal(O.canonical(t.triangles_array()), O.canonical(O.triangulate(p).tris))


def test_workspace_limit_out_of_memory(lib):
    """Allocation failure driven from the host: a workspace cap below what a
    call needs gives QDT_ERR_OUT_OF_MEMORY and an empty context, calls that
    fit still run, and lifting the cap recovers."""
    big, small = W.uniform(100000, 61), W.uniform(1000, 62)
    need = lib.qdtg_workspace_bytes(100000)
    want_big = O.canonical(O.triangulate(big).tris)
    want_small = O.canonical(O.triangulate(small).tris)
    with G.Triangulation(lib) as t:
        assert t.set_workspace_limit(need - 1)
        assert t.execute(big) == Q.QDT_ERR_OUT_OF_MEMORY
        assert t.points_size() == 0 and t.triangles_size() == 0
        assert t.execute(small) == 0
        assert np.array_equal(O.canonical(t.triangles_array()), want_small)
        assert 0 < t.workspace_bytes() < need
        assert t.execute(big, parallel=True) == Q.QDT_ERR_OUT_OF_MEMORY
        assert t.set_workspace_limit(need)          # exactly enough: no growth margin
        assert t.execute(big) == 0 and t.workspace_bytes() == need
        assert np.array_equal(O.canonical(t.triangles_array()), want_big)
        assert t.set_workspace_limit(lib.qdtg_workspace_bytes(2000))   # frees the larger workspace
        assert t.workspace_bytes() == 0
        assert t.execute(small) == 0
        assert np.array_equal(O.canonical(t.triangles_array()), want_small)
        assert t.set_workspace_limit(0)
        assert t.execute(big) == 0
        assert np.array_equal(O.canonical(t.triangles_array()), want_big)


def test_input_is_copied(lib):
    p = np.array([[0.0, 0.0], [4.0, 0.0], [3.0, 1.0], [1.0, 1.0]])
    keep = p.copy()
    with G.Triangulation(lib) as t:
        assert t.execute(p) == 0
        assert np.array_equal(p, keep)
        p[:] = -999.0
        assert t.triangles_size() == 2
        for i in range(4):
            ok, xy = t.point(i)
            assert ok == 1 and xy == tuple(keep[i])


def test_reuse_and_sizes(lib):
    # one context, growing and shrinking inputs
    with G.Triangulation(lib) as t:
        for n in (10, 100000, 3, 5000, 250000, 0, 7):
            p = W.uniform(n, n)
            assert t.execute(p) == 0
            assert np.array_equal(O.canonical(t.triangles_array()), O.canonical(O.triangulate(p).tris))


def test_concurrent_contexts(lib):
    inputs = [W.uniform(20000 + 1000 * i, 300 + i) for i in range(8)]
    expect = [O.canonical(O.triangulate(p).tris) for p in inputs]
    got = [None] * 8

    def work(i):
        with G.Triangulation(lib) as t:
            for _ in range(3):
                assert t.execute(inputs[i], parallel=(i % 2 == 1)) == 0
            got[i] = O.canonical(t.triangles_array())

    th = [threading.Thread(target=work, args=(i,)) for i in range(8)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    for i in range(8):
        assert np.array_equal(got[i], expect[i])


def test_device_resident_path(lib):
    torch = pytest.importorskip("torch")
    p = W.uniform(200000, 77)
    d = torch.from_numpy(p).cuda().contiguous()
    torch.cuda.synchronize()
    with G.Triangulation(lib) as t:
        assert t.execute_device(d.data_ptr(), p.shape[0]) == 0
        assert t.triangles_size() == 0   # the host side is left empty
        host = t.download_device_triangles()
    assert np.array_equal(O.canonical(host), O.canonical(O.triangulate(p).tris))


def test_device_arrays_of_one_size(lib):
    """The device path reads the caller's array in place and the first stages
    replay from a graph per (size, array): two arrays of one size, each
    triangulated twice in turn, with host calls of the same size between."""
    torch = pytest.importorskip("torch")
    ps = [W.uniform(50000, 91), W.gaussian_mixture(50000, 4, 92)]
    want = [O.canonical(O.triangulate(p).tris) for p in ps]
    ds = [torch.from_numpy(p).cuda().contiguous() for p in ps]
    torch.cuda.synchronize()
    with G.Triangulation(lib) as t:
        for i in (0, 1, 0, 1):
            assert t.execute_device(ds[i].data_ptr(), ps[i].shape[0]) == 0
            assert np.array_equal(O.canonical(t.download_device_triangles()), want[i]), i
            assert t.execute(ps[1 - i]) == 0
            assert np.array_equal(O.canonical(t.triangles_array()), want[1 - i]), i


def test_filter_failure_counts(lib):
    with G.Triangulation(lib) as t:
        t.set_options(count_filter_failures=True, stage_timing=True)
        assert t.execute(W.lattice_with_duplicates(256, 0.01, 3)) == 0
        info = t.run_info()
        assert info["orient_exact"] > 0 and info["incircle_exact"] > 0
        assert info["ms_total"] > 0
        assert t.execute(W.uniform(100000, 4)) == 0
        info = t.run_info()
        assert info["incircle_exact"] == 0
        # stage times come from events inside the replayed graphs too
        for graphs in (True, False):
            assert t.set_graphs(graphs)
            for _ in range(2):
                assert t.execute(W.uniform(100000, 4)) == 0
                info = t.run_info()
                for k in ("ms_sort", "ms_unique", "ms_split", "ms_build", "ms_extract"):
                    assert info[k] > 0, (graphs, k, info[k])
