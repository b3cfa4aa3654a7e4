"""qdtg_unique_points_noalloc: the batch path's first stage for callers that
cannot allocate device memory (hosts that own every allocation, real-time
loops that may not take the allocator's locks). Called through the C ABI on
device arrays the test owns, twice in a row on different inputs, and
compared with the representatives and distinct count that the regular entry
point (qdt_execute) produces for the same points. Integer outputs: the
comparison is exact. One more case runs on a stream of its own and checks
that a warm call changes neither torch's allocation count nor the device's
free memory.

This file is collected last on purpose, so a run that stops at the first
failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

import libqdt_gb300 as G
from libqdt_gb300 import qdt_api as Q
from libqdt_gb300 import workloads as W

pytestmark = pytest.mark.gpu

LIMIT = 1 << 16


def regular(lib, pts):
    with G.Triangulation(lib) as t:
        assert t.execute(pts) == 0
        return t.rep_array(), t.run_info()["unique_points"]


def noalloc(lib, torch, pts, stream=None):
    d = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    rep = torch.full((pts.shape[0],), 0xFFFFFFFF, dtype=torch.int64, device="cuda").to(torch.int32)
    torch.cuda.synchronize()
    uniq = ctypes.c_size_t(12345)
    handle = None if stream is None else stream.cuda_stream
    st = lib.qdtg_unique_points_noalloc(d.data_ptr(), pts.shape[0], rep.data_ptr(), ctypes.byref(uniq), handle)
    torch.cuda.synchronize()
    return st, rep.cpu().numpy().astype(np.uint32), uniq.value


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    lib = G.load()
    rng = np.random.default_rng(3)
    a = W.uniform(40000, 8)
    a = np.concatenate([a, a[rng.integers(0, 40000, size=5000)]])          # exact duplicates
    a[7] = (-0.0, a[7, 1])
    a = np.concatenate([a, [[0.0, a[7, 1]]]])                              # -0.0 equals +0.0
    a = a[rng.permutation(a.shape[0])]
    b = W.lattice_with_duplicates(255, 0.008, 9)[:LIMIT]                   # exactly at the limit
    assert b.shape[0] == LIMIT
    for pts in (a, b):
        st, rep, uniq = noalloc(lib, torch, pts)
        want_rep, want_uniq = regular(lib, pts)
        assert st == Q.QDT_OK
        assert uniq == want_uniq
        assert np.array_equal(rep, want_rep)


def test_noalloc_limits_and_errors():
    torch = pytest.importorskip("torch")
    lib = G.load()
    big = W.uniform(LIMIT + 1, 1)
    st, _, _ = noalloc(lib, torch, big)
    assert st == Q.QDT_ERR_TOO_MANY_POINTS
    bad = W.uniform(100, 2)
    bad[50, 1] = np.inf
    st, _, _ = noalloc(lib, torch, bad)
    assert st == Q.QDT_ERR_NOT_FINITE
    uniq = ctypes.c_size_t(7)
    assert lib.qdtg_unique_points_noalloc(None, 0, None, ctypes.byref(uniq), None) == Q.QDT_OK and uniq.value == 0
    assert lib.qdtg_unique_points_noalloc(None, 5, None, ctypes.byref(uniq), None) == Q.QDT_ERR_NULL_ARGUMENT


def test_noalloc_on_own_stream_allocates_nothing():
    torch = pytest.importorskip("torch")
    lib = G.load()
    pts = W.lattice_with_duplicates(120, 0.05, 4)
    want_rep, want_uniq = regular(lib, pts)
    stream = torch.cuda.Stream()
    d = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    rep = torch.zeros(pts.shape[0], dtype=torch.int32, device="cuda")
    uniq = ctypes.c_size_t(0)
    torch.cuda.synchronize()
    # warm call: the first call on a device looks up the array's address
    assert lib.qdtg_unique_points_noalloc(d.data_ptr(), pts.shape[0], rep.data_ptr(), ctypes.byref(uniq),
                                          stream.cuda_stream) == Q.QDT_OK
    torch.cuda.synchronize()
    rep.fill_(-1)
    torch.cuda.synchronize()
    used = torch.cuda.memory_allocated()
    free_before, _ = torch.cuda.mem_get_info()
    uniq = ctypes.c_size_t(0)
    st = lib.qdtg_unique_points_noalloc(d.data_ptr(), pts.shape[0], rep.data_ptr(), ctypes.byref(uniq),
                                        stream.cuda_stream)
    free_after, _ = torch.cuda.mem_get_info()
    assert st == Q.QDT_OK
    assert torch.cuda.memory_allocated() == used
    assert free_after == free_before
    assert uniq.value == want_uniq
    assert np.array_equal(rep.cpu().numpy().astype(np.uint32), want_rep)
