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

GPU_SYMBOLS = ("qdtg_set_options", "qdtg_get_run_info", "qdtg_execute_device", "qdtg_device_triangles",
               "qdtg_download_device_triangles",
               "qdtg_copy_triangles", "qdtg_copy_rep", "qdtg_stream", "qdtg_last_cuda_error", "qdtg_orient2d",
               "qdtg_incircle", "qdtg_eval_predicates", "qdtg_unique_points_noalloc", "qdtg_version")


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
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


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
    _lib = lib
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
