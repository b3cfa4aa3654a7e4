"""ctypes binding of the qdt.h C ABI.

This is the binding a Python caller of libqdt would write against qdt.h
(qdt.h:102-401 of the reference); it works for any shared library that
exports those 14 functions -- the GB300 library of this package, or the
reference compiled as a shared object. The status codes and argument
meanings are those of qdt.h.
"""
from __future__ import annotations

import ctypes

import numpy as np

QDT_OK = 0
QDT_ERR_NULL_CONTEXT = -1
QDT_ERR_NULL_ARGUMENT = -2
QDT_ERR_TOO_MANY_POINTS = -3
QDT_ERR_NOT_FINITE = -4
QDT_ERR_INVALID_INDEX = -5
QDT_ERR_SAME_POINT = -6
QDT_ERR_NO_TRIANGLES = -7
QDT_ERR_CROSSES_CONSTRAINT = -8
QDT_ERR_THROUGH_POINT = -9
QDT_ERR_OUT_OF_MEMORY = -10
QDT_ERR_INTERNAL = -11

QDT_SYMBOLS = (
    "qdt_status_string", "qdt_create", "qdt_execute", "qdt_execute_parallel",
    "qdt_insert_point", "qdt_insert_point_parallel", "qdt_insert_constraint",
    "qdt_insert_constraints_batch", "qdt_triangles_size", "qdt_get_triangle",
    "qdt_points_size", "qdt_get_point", "qdt_point_is_used", "qdt_destroy",
)


class Vec2d(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double)]


class Edge(ctypes.Structure):
    _fields_ = [("v0", ctypes.c_size_t), ("v1", ctypes.c_size_t)]


def bind(lib: ctypes.CDLL) -> ctypes.CDLL:
    """Declares the qdt.h prototypes on a loaded library."""
    P = ctypes.c_void_p
    lib.qdt_status_string.argtypes = [ctypes.c_int]
    lib.qdt_status_string.restype = ctypes.c_char_p
    lib.qdt_create.argtypes = []
    lib.qdt_create.restype = P
    for name in ("qdt_execute", "qdt_execute_parallel"):
        f = getattr(lib, name)
        f.argtypes = [P, P, ctypes.c_size_t]
        f.restype = ctypes.c_int
    for name in ("qdt_insert_point", "qdt_insert_point_parallel"):
        f = getattr(lib, name)
        f.argtypes = [P, Vec2d, ctypes.POINTER(ctypes.c_size_t)]
        f.restype = ctypes.c_int
    lib.qdt_insert_constraint.argtypes = [P, ctypes.c_size_t, ctypes.c_size_t]
    lib.qdt_insert_constraint.restype = ctypes.c_int
    lib.qdt_insert_constraints_batch.argtypes = [P, P, ctypes.c_size_t, P]
    lib.qdt_insert_constraints_batch.restype = ctypes.c_int
    lib.qdt_triangles_size.argtypes = [P]
    lib.qdt_triangles_size.restype = ctypes.c_size_t
    lib.qdt_get_triangle.argtypes = [P, ctypes.POINTER(ctypes.c_size_t), ctypes.c_size_t]
    lib.qdt_get_triangle.restype = ctypes.c_size_t
    lib.qdt_points_size.argtypes = [P]
    lib.qdt_points_size.restype = ctypes.c_size_t
    lib.qdt_get_point.argtypes = [P, ctypes.POINTER(Vec2d), ctypes.c_size_t]
    lib.qdt_get_point.restype = ctypes.c_size_t
    lib.qdt_point_is_used.argtypes = [P, ctypes.c_size_t]
    lib.qdt_point_is_used.restype = ctypes.c_size_t
    lib.qdt_destroy.argtypes = [P]
    lib.qdt_destroy.restype = None
    return lib


class Context:
    """One qdt_t handle of a bound library (qdt.h:125)."""

    def __init__(self, lib: ctypes.CDLL):
        self.lib = lib
        self.ptr = lib.qdt_create()
        if not self.ptr:
            raise MemoryError("qdt_create returned NULL")

    def close(self):
        if self.ptr:
            self.lib.qdt_destroy(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def execute(self, pts, parallel: bool = False) -> int:
        if pts is None:
            return self.execute_raw(None, 0, parallel)
        a = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)
        return self.execute_raw(a.ctypes.data if a.shape[0] else None, a.shape[0], parallel, keep=a)

    def execute_raw(self, ptr, n, parallel=False, keep=None) -> int:
        f = self.lib.qdt_execute_parallel if parallel else self.lib.qdt_execute
        return f(self.ptr, ptr, n)

    def insert_point(self, x: float, y: float, parallel: bool = False):
        idx = ctypes.c_size_t(0)
        f = self.lib.qdt_insert_point_parallel if parallel else self.lib.qdt_insert_point
        st = f(self.ptr, Vec2d(x, y), ctypes.byref(idx))
        return st, idx.value

    def insert_constraint(self, v0: int, v1: int) -> int:
        return self.lib.qdt_insert_constraint(self.ptr, v0, v1)

    def insert_constraints_batch(self, edges):
        e = np.ascontiguousarray(edges, dtype=np.uint64).reshape(-1, 2)
        res = np.zeros(e.shape[0], dtype=np.int32)
        st = self.lib.qdt_insert_constraints_batch(self.ptr, e.ctypes.data if e.shape[0] else None,
                                                   e.shape[0], res.ctypes.data if e.shape[0] else None)
        return st, res

    def triangles_size(self) -> int:
        return self.lib.qdt_triangles_size(self.ptr)

    def points_size(self) -> int:
        return self.lib.qdt_points_size(self.ptr)

    def triangles(self) -> np.ndarray:
        """All triangles via qdt_get_triangle (the query path of the ABI)."""
        n = self.triangles_size()
        out = np.zeros((n, 3), dtype=np.int64)
        T = (ctypes.c_size_t * 3)()
        for i in range(n):
            if not self.lib.qdt_get_triangle(self.ptr, T, i):
                raise RuntimeError("qdt_get_triangle failed for a valid id")
            out[i] = (T[0], T[1], T[2])
        return out

    def point(self, i: int):
        p = Vec2d()
        ok = self.lib.qdt_get_point(self.ptr, ctypes.byref(p), i)
        return ok, (p.x, p.y)

    def point_is_used(self, i: int) -> int:
        return self.lib.qdt_point_is_used(self.ptr, i)


def load(path: str) -> ctypes.CDLL:
    return bind(ctypes.CDLL(path))
