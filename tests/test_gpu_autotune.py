"""The autotuner on the GPU: the knobs it installs as the library's defaults
are the ones it reports (and that bench.py copies into config.tuning), they
survive a reload from the cache, and a call made with them gives the
oracle's triangles (the knobs change speed, never the result)."""
import ctypes

import numpy as np
import pytest

import libqdt_gb300 as G
from libqdt_gb300 import autotune as A
from libqdt_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    return G.load()


def defaults(lib):
    vals = [ctypes.c_int() for _ in A.KNOBS]
    lib.qdtg_get_defaults(*[ctypes.byref(v) for v in vals])
    return {k: v.value for k, v in zip(A.KNOBS, vals)}


def test_installed_knobs_are_the_reported_ones(lib):
    cfg = A.ensure(lib)
    reported = {k: int(cfg[k]) for k in A.KNOBS}
    assert defaults(lib) == reported
    assert cfg["gpu"] == A.gpu_name(lib)
    assert cfg["library"] == lib.qdtg_version().decode()
    # the cache holds the same choice, and applying it installs it again
    cached = A.load_cached(lib)
    assert cached is not None
    assert {k: int(cached[k]) for k in A.KNOBS} == reported
    assert A.apply(lib, cached)
    assert defaults(lib) == reported
    # every candidate the tuner measured is one of its candidate values
    assert reported["single_warp_nodes"] in A.SINGLE_WARP_NODES
    assert reported["cell_points"] in A.CELLS and reported["batch_cell_points"] in A.CELLS
    assert reported["batch_warp_min_points"] in A.BATCH_WARP_POINTS
    assert reported["batch_warp_nodes"] in A.BATCH_WARP_NODES
    assert reported["server_large_workers"] in A.WORKERS


def test_apply_round_trip_and_results_unchanged(lib):
    saved = defaults(lib)
    p = W.uniform(120000, 17)
    ref = O.triangulate(p)
    try:
        other = dict(saved)
        other["single_warp_nodes"] = 1024 if saved["single_warp_nodes"] != 1024 else 8192
        other["cell_points"] = 128 if saved["cell_points"] == 0 else 0
        assert A.apply(lib, other)
        assert defaults(lib) == other
        for cfg in (other, saved):
            assert A.apply(lib, cfg)
            with G.Triangulation(lib) as t:
                assert t.execute(p) == 0
                assert np.array_equal(O.canonical(t.triangles_array()), O.canonical(ref.tris))
                assert np.array_equal(t.rep_array(), ref.rep)
    finally:
        A.apply(lib, saved)
    assert defaults(lib) == saved
