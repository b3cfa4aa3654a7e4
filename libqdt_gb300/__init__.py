"""libqdt_gb300 -- GPU (GB300, sm_103a) implementation of libqdt's batch
Delaunay triangulation behind the unchanged qdt.h C ABI.

The product is the shared library ``_build/libqdt_gb300.so`` (built from
``csrc/`` by ``libqdt_gb300.build``). This module loads it and offers a thin
Python mirror of the handle API (qdt.h) plus the GPU additions (qdt_gpu.h).
There is no CPU fallback: without the library, or without a GPU, batch calls
fail (QDT_ERR_INTERNAL from the C ABI, an exception here).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import qdt_api
from .qdt_api import (QDT_OK, QDT_ERR_NULL_CONTEXT, QDT_ERR_NULL_ARGUMENT, QDT_ERR_TOO_MANY_POINTS,  # noqa: F401
                      QDT_ERR_NOT_FINITE, QDT_ERR_INVALID_INDEX, QDT_ERR_SAME_POINT, QDT_ERR_NO_TRIANGLES,
                      QDT_ERR_CROSSES_CONSTRAINT, QDT_ERR_THROUGH_POINT, QDT_ERR_OUT_OF_MEMORY, QDT_ERR_INTERNAL)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqdt_gb300.so")

GPU_SYMBOLS = ("qdtg_set_options", "qdtg_set_cell_points", "qdtg_set_merge_window", "qdtg_set_graphs", "qdtg_set_warp_nodes",
               "qdtg_set_defaults",
               "qdtg_batch_set_warp_nodes", "qdtg_batch_set_persistent", "qdtg_set_mesh_on_gpu", "qdtg_locate_points", "qdtg_insert_points",
               "qdtg_trace_constraints", "qdtg_set_workspace_limit", "qdtg_context_workspace_bytes",
               "qdtg_set_split_tail", "qdtg_get_filter_stats", "qdtg_batch_get_filter_stats", "qdtg_set_side_prefetch", "qdtg_set_triangulation", "qdtg_set_split_merges", "qdtg_set_split_segments",
               "qdtg_get_defaults", "qdtg_device_name", "qdtg_get_run_info", "qdtg_execute_device", "qdtg_device_triangles",
               "qdtg_download_device_triangles",
               "qdtg_copy_triangles", "qdtg_copy_rep", "qdtg_stream", "qdtg_last_cuda_error", "qdtg_orient2d",
               "qdtg_incircle", "qdtg_eval_predicates", "qdtg_unique_points_noalloc", "qdtg_version",
               "qdtg_batch_create", "qdtg_batch_destroy", "qdtg_batch_execute", "qdtg_batch_execute_device",
               "qdtg_batch_set_count", "qdtg_batch_set_status", "qdtg_batch_triangles", "qdtg_batch_unique_points",
               "qdtg_batch_rep", "qdtg_batch_device_triangles", "qdtg_batch_download_device_triangles",
               "qdtg_batch_set_options", "qdtg_batch_set_cell_points", "qdtg_batch_get_run_info",
               "qdtg_batch_stream", "qdtg_batch_reserve", "qdtg_batch_workspace_bytes", "qdtg_workspace_bytes",
               "qdtg_server_default_config", "qdtg_server_create", "qdtg_server_destroy", "qdtg_server_submit",
               "qdtg_server_wait", "qdtg_server_result", "qdtg_server_timing", "qdtg_server_release",
               "qdtg_server_get_stats")


class RunInfo(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_size_t),
        ("unique_points", ctypes.c_size_t),
        ("triangles", ctypes.c_size_t),
        ("orient_exact", ctypes.c_ulonglong),
        ("incircle_exact", ctypes.c_ulonglong),
        ("ms_h2d", ctypes.c_float),
        ("ms_sort", ctypes.c_float),
        ("ms_unique", ctypes.c_float),
        ("ms_split", ctypes.c_float),
        ("ms_build", ctypes.c_float),
        ("ms_extract", ctypes.c_float),
        ("ms_d2h", ctypes.c_float),
        ("ms_total", ctypes.c_float),
        ("device_flags", ctypes.c_int),
        ("kernel_launches", ctypes.c_int),
        ("merge_window", ctypes.c_int),
        ("wide_exact", ctypes.c_int),
        ("split_depth", ctypes.c_int),
        ("split_rerun", ctypes.c_int),
        ("split_segments", ctypes.c_int),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


STAGES = ("leaf", "thread", "warp", "extract")


def filter_stats_dict(raw: np.ndarray) -> dict:
    """qdtg_filter_stats (3 x 4 x 2 unsigned 64-bit) as per-stage dicts of
    calls, float-undecided and exact counts per predicate."""
    out = {}
    for s, name in enumerate(STAGES):
        out[name] = {p: {"calls": int(raw[0, s, k]), "f32_undecided": int(raw[1, s, k]), "exact": int(raw[2, s, k])}
                     for k, p in enumerate(("orient2d", "incircle"))}
    return out


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads the GB300 library (building it first when it is missing or
    older than its sources)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libqdt_gb300.so is not built; run python -m libqdt_gb300.build")
    lib = qdt_api.bind(ctypes.CDLL(LIB_PATH))
    P = ctypes.c_void_p
    lib.qdtg_set_options.argtypes = [P, ctypes.c_int, ctypes.c_int]
    lib.qdtg_set_options.restype = None
    lib.qdtg_set_cell_points.argtypes = [P, ctypes.c_int]
    lib.qdtg_set_cell_points.restype = ctypes.c_int
    lib.qdtg_set_merge_window.argtypes = [P, ctypes.c_int]
    lib.qdtg_set_merge_window.restype = ctypes.c_int
    lib.qdtg_set_graphs.argtypes = [P, ctypes.c_int]
    lib.qdtg_set_graphs.restype = ctypes.c_int
    lib.qdtg_get_filter_stats.argtypes = [P, ctypes.c_void_p]
    lib.qdtg_get_filter_stats.restype = ctypes.c_int
    lib.qdtg_batch_get_filter_stats.argtypes = [P, ctypes.c_void_p]
    lib.qdtg_batch_get_filter_stats.restype = ctypes.c_int
    lib.qdtg_set_split_tail.argtypes = [P, ctypes.c_int]
    lib.qdtg_set_split_tail.restype = ctypes.c_int
    lib.qdtg_set_triangulation.argtypes = [P, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_size_t]
    lib.qdtg_set_triangulation.restype = ctypes.c_int
    lib.qdtg_set_side_prefetch.argtypes = [P, ctypes.c_int]
    lib.qdtg_set_side_prefetch.restype = ctypes.c_int
    lib.qdtg_set_split_merges.argtypes = [P, ctypes.c_int, ctypes.c_int]
    lib.qdtg_set_split_merges.restype = ctypes.c_int
    lib.qdtg_set_split_segments.argtypes = [P, ctypes.c_int, ctypes.c_int]
    lib.qdtg_set_split_segments.restype = ctypes.c_int
    lib.qdtg_set_workspace_limit.argtypes = [P, ctypes.c_size_t]
    lib.qdtg_set_workspace_limit.restype = ctypes.c_int
    lib.qdtg_context_workspace_bytes.argtypes = [P]
    lib.qdtg_context_workspace_bytes.restype = ctypes.c_size_t
    lib.qdtg_workspace_bytes.argtypes = [ctypes.c_size_t]
    lib.qdtg_workspace_bytes.restype = ctypes.c_size_t
    lib.qdtg_set_warp_nodes.argtypes = [P, ctypes.c_int]
    lib.qdtg_set_warp_nodes.restype = ctypes.c_int
    lib.qdtg_set_mesh_on_gpu.argtypes = [P, ctypes.c_int]
    lib.qdtg_set_mesh_on_gpu.restype = ctypes.c_int
    lib.qdtg_locate_points.argtypes = [P, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    lib.qdtg_locate_points.restype = ctypes.c_int
    lib.qdtg_insert_points.argtypes = [P, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    lib.qdtg_insert_points.restype = ctypes.c_int
    lib.qdtg_trace_constraints.argtypes = [P, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    lib.qdtg_trace_constraints.restype = ctypes.c_int
    lib.qdtg_set_defaults.argtypes = [ctypes.c_int] * 6
    lib.qdtg_set_defaults.restype = ctypes.c_int
    lib.qdtg_device_name.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    lib.qdtg_device_name.restype = ctypes.c_int
    lib.qdtg_get_defaults.argtypes = [ctypes.POINTER(ctypes.c_int)] * 6
    lib.qdtg_get_defaults.restype = None
    lib.qdtg_get_run_info.argtypes = [P, ctypes.POINTER(RunInfo)]
    lib.qdtg_get_run_info.restype = ctypes.c_int
    lib.qdtg_execute_device.argtypes = [P, P, ctypes.c_size_t, P]
    lib.qdtg_execute_device.restype = ctypes.c_int
    lib.qdtg_device_triangles.argtypes = [P, ctypes.POINTER(ctypes.c_void_p)]
    lib.qdtg_device_triangles.restype = ctypes.c_size_t
    lib.qdtg_download_device_triangles.argtypes = [P, P, ctypes.c_size_t]
    lib.qdtg_download_device_triangles.restype = ctypes.c_size_t
    lib.qdtg_copy_triangles.argtypes = [P, P, ctypes.c_size_t]
    lib.qdtg_copy_triangles.restype = ctypes.c_size_t
    lib.qdtg_copy_rep.argtypes = [P, P, ctypes.c_size_t]
    lib.qdtg_copy_rep.restype = ctypes.c_size_t
    lib.qdtg_stream.argtypes = [P]
    lib.qdtg_stream.restype = ctypes.c_void_p
    lib.qdtg_last_cuda_error.argtypes = [P]
    lib.qdtg_last_cuda_error.restype = ctypes.c_int
    lib.qdtg_orient2d.argtypes = [P, P, P]
    lib.qdtg_orient2d.restype = ctypes.c_int
    lib.qdtg_incircle.argtypes = [P, P, P, P]
    lib.qdtg_incircle.restype = ctypes.c_int
    lib.qdtg_eval_predicates.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, ctypes.c_size_t, P]
    lib.qdtg_eval_predicates.restype = ctypes.c_int
    lib.qdtg_unique_points_noalloc.argtypes = [P, ctypes.c_size_t, P, ctypes.POINTER(ctypes.c_size_t), P]
    lib.qdtg_unique_points_noalloc.restype = ctypes.c_int
    lib.qdtg_version.argtypes = []
    lib.qdtg_version.restype = ctypes.c_char_p
    S = ctypes.c_size_t
    PP = ctypes.POINTER(ctypes.c_void_p)
    for name, args, res in (
            ("qdtg_batch_create", [], P),
            ("qdtg_batch_destroy", [P], None),
            ("qdtg_batch_execute", [P, P, P, S], ctypes.c_int),
            ("qdtg_batch_execute_device", [P, P, P, S, P], ctypes.c_int),
            ("qdtg_batch_set_count", [P], S),
            ("qdtg_batch_set_status", [P, S], ctypes.c_int),
            ("qdtg_batch_triangles", [P, S, PP], S),
            ("qdtg_batch_unique_points", [P, S], S),
            ("qdtg_batch_rep", [P, S], P),
            ("qdtg_batch_device_triangles", [P, PP, PP], S),
            ("qdtg_batch_download_device_triangles", [P, P, S, P], S),
            ("qdtg_batch_set_options", [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int], None),
            ("qdtg_batch_set_cell_points", [P, ctypes.c_int], ctypes.c_int),
            ("qdtg_batch_set_warp_nodes", [P, ctypes.c_int], ctypes.c_int),
            ("qdtg_batch_set_persistent", [P, ctypes.c_int], ctypes.c_int),
            ("qdtg_batch_reserve", [P, S, S], ctypes.c_int),
            ("qdtg_batch_workspace_bytes", [P], S),
            ("qdtg_batch_get_run_info", [P, ctypes.POINTER(RunInfo)], ctypes.c_int),
            ("qdtg_batch_stream", [P], P)):
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    # the autotuner's choice for this GPU, when one is cached (it changes the
    # schedule, not the results)
    from . import autotune
    autotune.load_cached(lib)
    return lib


class Triangulation(qdt_api.Context):
    """A qdt_t handle of the GB300 library with bulk result access."""

    def __init__(self, lib: ctypes.CDLL | None = None):
        super().__init__(lib or load())

    def execute(self, pts, parallel: bool = False) -> int:
        st = super().execute(pts, parallel)
        return st

    def check(self, st: int):
        if st != QDT_OK:
            raise RuntimeError("qdt call failed: %s (cuda error %d)" % (
                self.lib.qdt_status_string(st).decode(), self.lib.qdtg_last_cuda_error(self.ptr)))

    def triangles_array(self) -> np.ndarray:
        n = self.triangles_size()
        out = np.zeros((n, 3), dtype=np.uint32)
        if n:
            self.lib.qdtg_copy_triangles(self.ptr, out.ctypes.data, n)
        return out

    def rep_array(self) -> np.ndarray:
        n = self.points_size()
        out = np.zeros(n, dtype=np.uint32)
        if n:
            self.lib.qdtg_copy_rep(self.ptr, out.ctypes.data, n)
        return out

    def set_options(self, count_filter_failures: bool = False, stage_timing: bool = False):
        self.lib.qdtg_set_options(self.ptr, int(count_filter_failures), int(stage_timing))

    def run_info(self) -> dict:
        ri = RunInfo()
        self.lib.qdtg_get_run_info(self.ptr, ctypes.byref(ri))
        return ri.as_dict()

    def set_cell_points(self, cell_points: int) -> bool:
        return self.lib.qdtg_set_cell_points(self.ptr, int(cell_points)) == 1

    def set_merge_window(self, window: int) -> bool:
        return self.lib.qdtg_set_merge_window(self.ptr, int(window)) == 1

    def set_graphs(self, on: bool) -> bool:
        return self.lib.qdtg_set_graphs(self.ptr, int(bool(on))) == 1

    def set_split_tail(self, on: bool) -> bool:
        return self.lib.qdtg_set_split_tail(self.ptr, int(bool(on))) == 1

    def set_triangulation(self, pts, tris, rep=None) -> int:
        """Loads a triangulation made earlier (points, triangles and
        representatives as triangles_array / rep_array gave them) in place of
        a batch call; works without a GPU."""
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)
        t = np.ascontiguousarray(tris, dtype=np.uint32).reshape(-1, 3)
        r = None if rep is None else np.ascontiguousarray(rep, dtype=np.uint32)
        return self.lib.qdtg_set_triangulation(self.ptr, p.ctypes.data if p.size else None, p.shape[0],
                                               None if r is None else r.ctypes.data,
                                               t.ctypes.data if t.size else None, t.shape[0])

    def set_side_prefetch(self, on: bool) -> bool:
        return self.lib.qdtg_set_side_prefetch(self.ptr, int(bool(on))) == 1

    def set_split_merges(self, max_depth: int, min_points: int = 1024) -> bool:
        """Split merges (seam segments, two walkers each) at depths
        0..max_depth, nodes of at least min_points points (the library's
        defaults: 7 and 1,024); max_depth -1: one walker per merge."""
        return self.lib.qdtg_set_split_merges(self.ptr, int(max_depth), int(min_points)) == 1

    def set_split_segments(self, max_segments: int, segment_points: int = 16384) -> bool:
        """Seam segments of one split merge at most (1..5), one more per
        segment_points points of the node: segments beyond the first begin
        at cross edges found before the merge."""
        return self.lib.qdtg_set_split_segments(self.ptr, int(max_segments), int(segment_points)) == 1

    def filter_stats(self) -> dict:
        """Per-stage predicate statistics of the last batch call (counted
        when set_options(count_filter_failures=True))."""
        raw = np.zeros((3, 4, 2), dtype=np.uint64)
        self.lib.qdtg_get_filter_stats(self.ptr, raw.ctypes.data)
        return filter_stats_dict(raw)

    def set_workspace_limit(self, nbytes: int) -> bool:
        """Caps the device workspace (0: no cap); calls that need more
        return QDT_ERR_OUT_OF_MEMORY."""
        return self.lib.qdtg_set_workspace_limit(self.ptr, int(nbytes)) == 1

    def workspace_bytes(self) -> int:
        return int(self.lib.qdtg_context_workspace_bytes(self.ptr))

    def set_warp_nodes(self, nodes: int) -> bool:
        return self.lib.qdtg_set_warp_nodes(self.ptr, int(nodes)) == 1

    def set_mesh_on_gpu(self, on_gpu: bool) -> bool:
        return self.lib.qdtg_set_mesh_on_gpu(self.ptr, int(bool(on_gpu))) == 1

    def locate(self, pts):
        """(status, tri, where) for an (k, 2) array of query points: the
        smallest index of a triangle containing each point (-1 outside) and
        its class (-1 outside, 0 inside, 1 on an edge, 2 on a vertex)."""
        q = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)
        k = q.shape[0]
        tri = np.full(k, -1, dtype=np.int64)
        where = np.full(k, -1, dtype=np.int32)
        st = self.lib.qdtg_locate_points(self.ptr, q.ctypes.data if k else None, k,
                                         tri.ctypes.data if k else None, where.ctypes.data if k else None)
        return st, tri, where

    def insert_points(self, pts):
        """(status, results, indices): qdt_insert_point for each row in order,
        the points located on the GPU first."""
        q = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)
        k = q.shape[0]
        res = np.zeros(k, dtype=np.int32)
        idx = np.zeros(k, dtype=np.uint64)
        st = self.lib.qdtg_insert_points(self.ptr, q.ctypes.data if k else None, k,
                                         idx.ctypes.data if k else None, res.ctypes.data if k else None)
        return st, res, idx

    def trace_constraints(self, edges):
        """(status, per-edge statuses, crossed): what qdt_insert_constraint
        would return for each edge on its own now, and the edges its segment
        crosses; nothing is inserted."""
        e = np.ascontiguousarray(edges, dtype=np.uint64).reshape(-1, 2)
        k = e.shape[0]
        res = np.zeros(k, dtype=np.int32)
        crossed = np.zeros(k, dtype=np.int64)
        st = self.lib.qdtg_trace_constraints(self.ptr, e.ctypes.data if k else None, k,
                                             res.ctypes.data if k else None, crossed.ctypes.data if k else None)
        return st, res, crossed

    def execute_device(self, d_ptr: int, n: int, stream: int = 0) -> int:
        return self.lib.qdtg_execute_device(self.ptr, d_ptr, n, stream or None)

    def stream(self) -> int:
        return self.lib.qdtg_stream(self.ptr) or 0

    def device_triangles(self):
        p = ctypes.c_void_p(0)
        n = self.lib.qdtg_device_triangles(self.ptr, ctypes.byref(p))
        return n, p.value

    def download_device_triangles(self) -> np.ndarray:
        n, _ = self.device_triangles()
        out = np.zeros((n, 3), dtype=np.uint32)
        if n:
            self.lib.qdtg_download_device_triangles(self.ptr, out.ctypes.data, n)
        return out


class Batch:
    """Many independent point sets triangulated by one GPU pipeline
    (qdtg_batch_* of qdt_gpu.h). Set i of a call is points
    offsets[i]:offsets[i+1]; its result equals qdt_execute() on those points
    alone."""

    def __init__(self, lib: ctypes.CDLL | None = None):
        self.lib = lib or load()
        self.ptr = self.lib.qdtg_batch_create()
        if not self.ptr:
            raise RuntimeError("qdtg_batch_create failed (no usable GPU)")
        self._offsets = None

    def close(self):
        if self.ptr:
            self.lib.qdtg_batch_destroy(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def offsets_of(sets) -> np.ndarray:
        off = np.zeros(len(sets) + 1, dtype=np.uint64)
        off[1:] = np.cumsum([len(s) for s in sets])
        return off

    def execute(self, pts, offsets) -> int:
        """pts: (N, 2) float64 host array of all sets back to back."""
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        self._offsets = off
        return self.lib.qdtg_batch_execute(self.ptr, p.ctypes.data if p.size else None, off.ctypes.data,
                                           len(off) - 1)

    def execute_sets(self, sets) -> int:
        off = self.offsets_of(sets)
        pts = np.concatenate([np.asarray(s, dtype=np.float64).reshape(-1, 2) for s in sets]) if len(sets) else \
            np.zeros((0, 2))
        return self.execute(pts, off)

    def execute_device(self, d_ptr: int, offsets, stream: int = 0) -> int:
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        self._offsets = off
        return self.lib.qdtg_batch_execute_device(self.ptr, d_ptr or None, off.ctypes.data, len(off) - 1,
                                                  stream or None)

    def set_count(self) -> int:
        return self.lib.qdtg_batch_set_count(self.ptr)

    def status(self, i: int) -> int:
        return self.lib.qdtg_batch_set_status(self.ptr, i)

    def triangles(self, i: int) -> np.ndarray:
        p = ctypes.c_void_p(0)
        n = self.lib.qdtg_batch_triangles(self.ptr, i, ctypes.byref(p))
        if n == 0 or not p.value:
            return np.zeros((0, 3), dtype=np.uint32)
        return np.ctypeslib.as_array((ctypes.c_uint32 * (3 * n)).from_address(p.value)).reshape(n, 3).copy()

    def unique_points(self, i: int) -> int:
        return self.lib.qdtg_batch_unique_points(self.ptr, i)

    def rep(self, i: int) -> np.ndarray:
        p = self.lib.qdtg_batch_rep(self.ptr, i)
        n = int(self._offsets[i + 1] - self._offsets[i])
        if not p or n == 0:
            return np.zeros(0, dtype=np.uint32)
        return np.ctypeslib.as_array((ctypes.c_uint32 * n).from_address(p)).copy()

    def device_triangles(self):
        t, o = ctypes.c_void_p(0), ctypes.c_void_p(0)
        n = self.lib.qdtg_batch_device_triangles(self.ptr, ctypes.byref(t), ctypes.byref(o))
        return n, t.value, o.value

    def download_device_triangles(self):
        """All triangles (total, 3) and the per-set triangle offsets."""
        total, _, _ = self.device_triangles()
        tri = np.zeros((total, 3), dtype=np.uint32)
        off = np.zeros(self.set_count() + 1, dtype=np.uint32)
        self.lib.qdtg_batch_download_device_triangles(self.ptr, tri.ctypes.data if total else None, total,
                                                      off.ctypes.data)
        return tri, off

    def set_options(self, count_filter_failures=False, stage_timing=False, use_graphs=True, warp_min_points=0):
        self.lib.qdtg_batch_set_options(self.ptr, int(count_filter_failures), int(stage_timing), int(use_graphs),
                                        int(warp_min_points))

    def run_info(self) -> dict:
        ri = RunInfo()
        self.lib.qdtg_batch_get_run_info(self.ptr, ctypes.byref(ri))
        return ri.as_dict()

    def set_cell_points(self, cell_points: int) -> bool:
        return self.lib.qdtg_batch_set_cell_points(self.ptr, int(cell_points)) == 1

    def filter_stats(self) -> dict:
        raw = np.zeros((3, 4, 2), dtype=np.uint64)
        self.lib.qdtg_batch_get_filter_stats(self.ptr, raw.ctypes.data)
        return filter_stats_dict(raw)

    def set_warp_nodes(self, nodes: int) -> bool:
        return self.lib.qdtg_batch_set_warp_nodes(self.ptr, int(nodes)) == 1

    def set_persistent(self, on: bool) -> bool:
        """The build of every set's tree as one persistent launch (on) or one
        launch per node height (off, the default)."""
        return self.lib.qdtg_batch_set_persistent(self.ptr, int(bool(on))) == 1

    def stream(self) -> int:
        return self.lib.qdtg_batch_stream(self.ptr) or 0


def eval_predicates(kind: str, coords, mode: str = "full", device: bool = False) -> np.ndarray:
    """Signs of orient2d (kind "orient", coords (k, 6)) or incircle (kind
    "incircle", coords (k, 8)); mode "full", "f32" (pre-filter only, 0 when
    undecided) or "exact"."""
    lib = load()
    c = np.ascontiguousarray(coords, dtype=np.float64)
    k = c.shape[0]
    out = np.zeros(k, dtype=np.int8)
    rc = lib.qdtg_eval_predicates(0 if kind == "orient" else 1, {"full": 0, "f32": 1, "exact": 2}[mode],
                                  1 if device else 0, c.ctypes.data, k, out.ctypes.data)
    if rc != 0:
        raise RuntimeError("qdtg_eval_predicates failed: %d" % rc)
    return out


def triangulate(pts) -> np.ndarray:
    """Convenience: the triangles (k, 3) uint32 of one point set."""
    with Triangulation() as t:
        t.check(t.execute(pts))
        return t.triangles_array()
