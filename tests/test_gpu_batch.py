"""The many-set engine (qdtg_batch_*): every set of a batch gets exactly the
result that the reference's batch call (qdt_execute) gives for that set
alone -- the canonical triangle set, the representatives and the distinct
count -- checked against the CPU oracle set by set. Covers uneven sizes,
empty and tiny sets, duplicates, -0.0, collinear and cocircular sets, a set
with a NaN among good ones, repeated calls (CUDA graph replay), changing
shapes and the device-resident entry point. Index outputs: bit-exact.
"""
import os

import numpy as np
import pytest

import libqdt_gb300 as G
from libqdt_gb300 import qdt_api as Q
from libqdt_gb300 import workloads as W
from oracle import oracle as O
from tests.golden import cases as C

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def lib():
    return G.load()


def special_sets():
    rng = np.random.default_rng(77)
    s = []
    s.append(np.zeros((0, 2)))                                            # empty
    s.append(np.array([[0.25, 0.5]]))                                     # one point
    s.append(np.array([[0.0, 0.0], [1.0, 1.0]]))                         # two points
    s.append(np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 2.0]]))             # three collinear
    s.append(np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]]))             # one triangle
    s.append(np.array([[0.5, 0.5]] * 9))                                  # one distinct point
    s.append(np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 0.0], [1.0, 0.0], [0.0, 1.0]]))   # 3 distinct of 5
    s.append(np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]]))  # cocircular square
    z = rng.random((200, 2))
    z[10] = (-0.0, z[10, 1])
    z = np.concatenate([z, [[0.0, z[10, 1]]], z[:30]])                   # -0.0 and exact duplicates
    s.append(z)
    s.append(W.lattice_with_duplicates(64, 0.01, 5))                     # collinear/cocircular lattice
    s.append(W.unit_circle(3000, 6))                                     # all cocircular
    s.append(W.noisy_line(5000, 7))                                      # near-collinear
    s.append(rng.random((4, 2)))
    s.append(rng.random((7, 2)))
    return s


def check_batch(b, sets):
    assert b.set_count() == len(sets)
    for i, p in enumerate(sets):
        o = O.triangulate(p)
        assert b.status(i) == o.status, i
        if o.status != Q.QDT_OK:
            assert b.triangles(i).shape[0] == 0
            continue
        tris = b.triangles(i)
        assert np.array_equal(O.canonical(tris), O.canonical(o.tris)), i
        assert b.unique_points(i) == o.unique_points, i
        assert np.array_equal(b.rep(i), o.rep), i


def test_special_sets_equal_oracle(lib):
    sets = special_sets()
    with G.Batch(lib) as b:
        assert b.execute_sets(sets) == Q.QDT_OK
        check_batch(b, sets)


def test_uneven_sets_equal_oracle_and_replay(lib):
    sets = W.many_sets(count=300, lo=16, hi=20000, seed=5)
    sets[17] = np.concatenate([sets[17], sets[17][:50]])                 # duplicates inside one set
    mixed = special_sets() + sets
    with G.Batch(lib) as b:
        for _ in range(3):                                                # capture, then graph replays
            assert b.execute_sets(mixed) == Q.QDT_OK
            check_batch(b, mixed)
        info = b.run_info()
        assert info["kernel_launches"] > 0
        assert info["n"] == sum(len(s) for s in mixed)
        # another shape in the same batch object, then the first again
        few = W.many_sets(count=40, lo=16, hi=3000, seed=6)
        assert b.execute_sets(few) == Q.QDT_OK
        check_batch(b, few)
        assert b.execute_sets(mixed) == Q.QDT_OK
        check_batch(b, mixed)


def test_graphs_off_and_timing_same_result(lib):
    sets = W.many_sets(count=64, lo=16, hi=8000, seed=8)
    with G.Batch(lib) as b:
        b.set_options(count_filter_failures=True, stage_timing=True, use_graphs=False, warp_min_points=64)
        assert b.execute_sets(sets) == Q.QDT_OK
        check_batch(b, sets)
        info = b.run_info()
        assert info["ms_build"] > 0 and info["ms_total"] > 0
        # warp merges at every height, then at none
        for points, nodes in ((1 << 30, 1 << 30), (1 << 30, 0)):
            b.set_options(use_graphs=True, warp_min_points=points)
            assert b.set_warp_nodes(nodes)
            assert b.execute_sets(sets) == Q.QDT_OK
            check_batch(b, sets)


@pytest.mark.parametrize("cells", [0, 4, 33, 128, 1024])
def test_cell_sizes_same_result(lib, cells):
    sets = special_sets() + W.many_sets(count=80, lo=16, hi=9000, seed=12)
    with G.Batch(lib) as b:
        assert b.set_cell_points(cells)
        assert b.execute_sets(sets) == Q.QDT_OK
        check_batch(b, sets)
        assert not b.set_cell_points(2000)


def test_not_finite_set_leaves_others_intact(lib):
    sets = W.many_sets(count=20, lo=16, hi=2000, seed=9)
    bad = sets[4].copy()
    bad[3, 0] = np.nan
    sets[4] = bad
    inf = sets[11].copy()
    inf[0, 1] = -np.inf
    sets[11] = inf
    with G.Batch(lib) as b:
        assert b.execute_sets(sets) == Q.QDT_OK
        assert b.status(4) == Q.QDT_ERR_NOT_FINITE
        assert b.status(11) == Q.QDT_ERR_NOT_FINITE
        check_batch(b, sets)


def test_matches_plain_path_set_by_set(lib):
    sets = W.many_sets(count=24, lo=1000, hi=60000, seed=10)
    with G.Batch(lib) as b:
        assert b.execute_sets(sets) == Q.QDT_OK
        for i, p in enumerate(sets):
            with G.Triangulation(lib) as t:
                assert t.execute(p) == Q.QDT_OK
                assert np.array_equal(O.canonical(b.triangles(i)), O.canonical(t.triangles_array())), i


def test_device_resident_batch(lib):
    torch = pytest.importorskip("torch")
    sets = W.many_sets(count=50, lo=16, hi=5000, seed=11)
    off = G.Batch.offsets_of(sets)
    d = torch.from_numpy(np.concatenate(sets)).cuda()
    torch.cuda.synchronize()
    with G.Batch(lib) as b:
        assert b.execute_device(d.data_ptr(), off) == Q.QDT_OK
        total, d_tris, d_off = b.device_triangles()
        assert total > 0 and d_tris and d_off
        tri, toff = b.download_device_triangles()
        assert toff.shape[0] == len(sets) + 1 and toff[-1] == total
        for i, p in enumerate(sets):
            t = tri[toff[i]: toff[i + 1]]
            assert np.array_equal(O.canonical(t), O.canonical(O.triangulate(p).tris)), i


def test_config_b_every_set_equals_reference(lib):
    """The many-set workload at its stated size -- 4,096 sets, sizes
    log-uniform in [16, 65,536], square or disk, 10 % snapped to a 256 grid
    -- in one qdtg_batch_execute call (then a graph replay): every set's
    status, triangle count and digests of its canonical triangles and
    used-point flags equal what the reference's qdt_execute gave for that set
    alone (tests/golden/config_b.npz, made by the reference)."""
    ref = np.load(os.path.join(GOLDEN, "config_b.npz"))
    sets = C.config_b_sets()
    assert np.array_equal(np.array([p.shape[0] for p in sets]), ref["sizes"])
    with G.Batch(lib) as b:
        for rep_call in range(2):
            assert b.execute_sets(sets) == Q.QDT_OK
            bad = []
            for i, p in enumerate(sets):
                st = b.status(i)
                tris = b.triangles(i)
                rep = b.rep(i)
                used = (rep == np.arange(p.shape[0])).astype(np.uint8) if tris.shape[0] else \
                    np.zeros(p.shape[0], np.uint8)
                got = C.set_record(st, tris, used)
                want = (int(ref["status"][i]), int(ref["ntri"][i]), int(ref["tri_digest"][i]),
                        int(ref["used_digest"][i]))
                if got != want:
                    bad.append(i)
            assert not bad, (rep_call, bad[:10], len(bad))


def test_persistent_build_same_result(lib):
    """The build as one persistent launch (qdtg_batch_set_persistent: warps
    take node units from a counter and wait for their children's done flags)
    gives every set the oracle's result, like the launch per height: special
    and uneven sets, graph replay, the thread form at every height and the
    warp form at every height, a failing set among good ones, and back to the
    launch per height in the same batch object."""
    sets = special_sets() + W.many_sets(count=200, lo=16, hi=40000, seed=31)
    with G.Batch(lib) as b:
        assert b.execute_sets(sets) == Q.QDT_OK
        per_height = b.run_info()["kernel_launches"]
        assert b.set_persistent(True)
        for _ in range(2):                                                # capture, then graph replay
            assert b.execute_sets(sets) == Q.QDT_OK
            check_batch(b, sets)
            assert b.run_info()["device_flags"] == 0
        assert b.run_info()["kernel_launches"] < per_height
        for points, nodes in ((1 << 30, 0), (1 << 30, 1 << 30), (4, 0)):
            b.set_options(warp_min_points=points)
            assert b.set_warp_nodes(nodes)
            assert b.execute_sets(sets) == Q.QDT_OK
            check_batch(b, sets)
        bad = [s.copy() for s in sets[-30:]]
        bad[5][2, 1] = np.nan
        assert b.execute_sets(bad) == Q.QDT_OK
        assert b.status(5) == Q.QDT_ERR_NOT_FINITE
        check_batch(b, bad)
        assert b.set_persistent(False)
        assert b.execute_sets(sets) == Q.QDT_OK
        check_batch(b, sets)


def test_persistent_build_one_large_set(lib):
    """One set of 300,000 points and a few small ones in the persistent
    form: the chain of waits runs from the leaves to a root that is merged
    by one warp while most other warps have run out of work."""
    sets = [W.uniform(300000, 33), W.uniform(100, 34), W.lattice_with_duplicates(40, 0.02, 35)]
    with G.Batch(lib) as b:
        assert b.set_persistent(True)
        assert b.execute_sets(sets) == Q.QDT_OK
        check_batch(b, sets)


def test_batch_wide_exact_rerun(lib):
    """A set whose coordinates span more than 95 bits inside one predicate
    needs the widest exact tier. The batch's thread-per-node merges (and its
    persistent build) come from the build that has it; its leaves, warp
    merges and extraction come from the build without it, where such a
    predicate flags the batch, which then runs its stages after the
    synchronisation again with the kernels that have the tier (run_info
    wide_exact). Every set -- that one and the ordinary ones beside it --
    gets the oracle's result either way; ordinary batches never take the
    second run."""
    rng = np.random.default_rng(71)
    base = rng.integers(0, 40, size=(3000, 2)).astype(np.float64)
    tiny = base.copy()
    tiny[::7] += np.ldexp(rng.integers(1, 8, size=(tiny[::7].shape[0], 2)).astype(np.float64), -90)
    ordinary = W.many_sets(count=30, lo=16, hi=5000, seed=36)
    mixed = ordinary[:10] + [tiny] + ordinary[10:]
    with G.Batch(lib) as b:
        assert b.execute_sets(ordinary) == Q.QDT_OK
        assert b.run_info()["wide_exact"] == 0
        check_batch(b, ordinary)
        assert b.execute_sets(mixed) == Q.QDT_OK
        check_batch(b, mixed)
        # a warp per node at every height: the merges meet the tier in the
        # build without it
        b.set_options(warp_min_points=4)
        assert b.execute_sets(mixed) == Q.QDT_OK
        assert b.run_info()["wide_exact"] == 1
        check_batch(b, mixed)
        assert b.set_persistent(True)
        assert b.execute_sets(mixed) == Q.QDT_OK
        check_batch(b, mixed)
