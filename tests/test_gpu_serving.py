"""The serving loop (qdtg_server_*): requests of mixed sizes and
distributions, submitted open-loop so that they overlap on the device and the
small ones are coalesced into many-set batches, each give exactly the result
of the same request run alone through qdt_execute (triangles, representatives,
distinct count; index outputs, compared bit for bit). Admission keeps the
device pools within the HBM budget, rejects what cannot fit, and bounds the
queue.
"""
import numpy as np
import pytest

import libqdt_gb300 as G
from libqdt_gb300 import qdt_api as Q
from libqdt_gb300 import serving as S
from libqdt_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    return G.load()


def alone(lib, pts):
    with G.Triangulation(lib) as t:
        st = t.execute(pts)
        if st != Q.QDT_OK:
            return st, None, None, 0
        return st, O.canonical(t.triangles_array()), t.rep_array(), t.run_info()["unique_points"]


def test_alone_vs_in_mix_identical(lib):
    reqs = W.request_stream(80, rate_per_s=400.0, lo=100, hi=300_000, seed=41)
    bad = reqs[5][1].copy()
    bad[7, 1] = np.nan
    reqs[5] = (reqs[5][0], bad)
    reqs[9] = (reqs[9][0], np.zeros((0, 2)))
    reqs[12] = (reqs[12][0], np.concatenate([reqs[12][1], reqs[12][1][:40]]))   # duplicates
    with S.Server(lib, large_workers=3, small_threshold=20000) as srv:
        out = S.run_open_loop(srv, reqs, keep_results=True)
        stats = srv.stats()
    assert out["completed"] == len(reqs)              # the NaN request is accepted; its result has the error
    assert stats["rejected"] == 0
    assert out["coalesced"] > 0 and out["coalesced"] < out["completed"]
    assert stats["batches"] > 0
    for i, (_, p) in enumerate(reqs):
        st, tris, rep, uniq = out["results"][i]
        want = alone(lib, p)
        assert st == want[0], i
        if st != Q.QDT_OK:
            continue
        assert np.array_equal(O.canonical(tris), want[1]), i
        assert np.array_equal(rep, want[2]), i
        assert uniq == want[3], i
    # and the coalesced small ones against the oracle directly
    for i, (_, p) in enumerate(reqs[:15]):
        st, tris, rep, _ = out["results"][i]
        if st == Q.QDT_OK and p.shape[0]:
            assert np.array_equal(O.canonical(tris), O.canonical(O.triangulate(p).tris)), i


def test_large_requests_alone_vs_in_mix_identical(lib):
    """Requests of 0.5 to 2 million points (the top of the serving
    workload's size range; uniform, Gaussian mixture and snapped grid)
    arriving while others run on the large engines, with small requests
    coalesced beside them: each result equals the same request run alone
    through qdt_execute."""
    big = W.request_stream(10, rate_per_s=40.0, lo=500_000, hi=2_000_000, seed=43)
    small = W.request_stream(40, rate_per_s=160.0, lo=100, hi=20_000, seed=44)
    reqs = sorted(big + small, key=lambda r: r[0])
    with S.Server(lib, large_workers=4, small_threshold=65536) as srv:
        out = S.run_open_loop(srv, reqs, keep_results=True)
        stats = srv.stats()
    assert out["completed"] == len(reqs)
    assert stats["rejected"] == 0
    assert out["coalesced"] > 0
    for i, (_, p) in enumerate(reqs):
        st, tris, rep, uniq = out["results"][i]
        want = alone(lib, p)
        assert st == want[0] == Q.QDT_OK, i
        assert np.array_equal(O.canonical(tris), want[1]), (i, p.shape[0])
        assert np.array_equal(rep, want[2]), i
        assert uniq == want[3], i


def test_budget_admission_and_queue_limit(lib):
    with S.Server(lib, large_workers=3, small_threshold=1000, batch_max_points=100_000) as srv:
        batch_pool = srv.stats()["resident_bytes"]
    assert batch_pool > 0
    n_big = 200_000
    budget = batch_pool + int(1.3 * lib.qdtg_workspace_bytes(n_big))
    reqs = [W.uniform(n_big - 1000 * k, 50 + k) for k in range(6)]
    with S.Server(lib, large_workers=3, small_threshold=1000, batch_max_points=100_000,
                  hbm_budget_bytes=budget) as srv:
        tickets = [srv.submit(p) for p in reqs]
        assert all(st == Q.QDT_OK for st, _ in tickets)
        too_big = W.uniform(2 * n_big, 60)
        st, tk = srv.submit(too_big)
        assert st == Q.QDT_ERR_OUT_OF_MEMORY and tk
        for (st, tk), p in zip(tickets, reqs):
            assert srv.wait(tk, 120.0)
            r = srv.result(tk)
            want = alone(lib, p)
            assert r[0] == Q.QDT_OK
            assert np.array_equal(O.canonical(r[1]), want[1])
        s = srv.stats()
        assert s["peak_resident_bytes"] <= budget
        assert s["rejected"] == 1 and s["queued"] >= 1
    with S.Server(lib, large_workers=1, small_threshold=1000, batch_max_points=100_000, max_queue=2) as srv:
        res = [srv.submit(p) for p in reqs]
        rejected = [st for st, _ in res if st == Q.QDT_ERR_OUT_OF_MEMORY]
        assert len(rejected) >= 1
        for st, tk in res:
            assert srv.wait(tk, 120.0)
            srv.release(tk)
        assert srv.stats()["rejected"] == len(rejected)
