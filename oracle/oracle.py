"""CPU oracle for the batch Delaunay path -- TEST INFRASTRUCTURE ONLY.

Python binding of oracle/qdt_oracle.c, the plain-C restatement of the
reference's batch triangulation (serial and threaded drivers), and of the
reference library itself when it was compiled here into oracle/_ref.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker or the timed
baseline. The product path (``libqdt_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libqdt_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB_PATH = os.path.join(REF_DIR, "libqdt_ref.so")

CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


def build(force: bool = False) -> str:
    """Compiles the C restatement (seconds). Returns the library path."""
    src = os.path.join(HERE, "qdt_oracle.c")
    hdr = os.path.join(HERE, "qdt_oracle.h")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", *CFLAGS, "-o", tmp, src, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_reference() -> bool:
    """Compiles the reference from its own sources into oracle/_ref when the
    reference tree is present (this container only). Returns True when
    oracle/_ref/libqdt_ref.so is usable afterwards."""
    script = os.path.join(HERE, "build_ref.sh")
    if not os.path.exists(REF_LIB_PATH):
        subprocess.call(["sh", script])
    return reference_available()


def reference_available() -> bool:
    if not os.path.exists(REF_LIB_PATH):
        return False
    try:
        ctypes.CDLL(REF_LIB_PATH)
        return True
    except OSError:
        return False


class _Stats(ctypes.Structure):
    _fields_ = [
        ("orient_calls", ctypes.c_uint64),
        ("orient_exact", ctypes.c_uint64),
        ("incircle_calls", ctypes.c_uint64),
        ("incircle_exact", ctypes.c_uint64),
        ("records_used", ctypes.c_uint64),
        ("threaded_used", ctypes.c_int),
        ("fell_back", ctypes.c_int),
    ]


class _Result(ctypes.Structure):
    _fields_ = [
        ("tris", ctypes.POINTER(ctypes.c_uint32)),
        ("ntri", ctypes.c_size_t),
        ("rep", ctypes.POINTER(ctypes.c_uint32)),
        ("n", ctypes.c_size_t),
        ("unique_points", ctypes.c_size_t),
        ("stats", _Stats),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.qdo_triangulate.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(_Result)]
        _lib.qdo_triangulate.restype = ctypes.c_int
        _lib.qdo_result_free.argtypes = [ctypes.POINTER(_Result)]
        _lib.qdo_check_input.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        _lib.qdo_check_input.restype = ctypes.c_int
        for name in ("qdo_orient2d", "qdo_orient2d_exact"):
            f = getattr(_lib, name)
            f.argtypes = [ctypes.c_void_p] * 3
            f.restype = ctypes.c_int
        for name in ("qdo_incircle", "qdo_incircle_exact"):
            f = getattr(_lib, name)
            f.argtypes = [ctypes.c_void_p] * 4
            f.restype = ctypes.c_int
    return _lib


class OracleResult:
    def __init__(self, status, tris, rep, unique, stats):
        self.status = status
        self.tris = tris
        self.rep = rep
        self.unique_points = unique
        self.stats = stats


def triangulate(pts: np.ndarray, threaded: bool = False, nthreads: int = 0) -> OracleResult:
    """Triangulates an (n, 2) float64 array; returns status, triangles
    (k, 3) uint32 in input indices, rep (n,) uint32, unique count, stats."""
    L = lib()
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)
    n = pts.shape[0]
    res = _Result()
    st = L.qdo_triangulate(pts.ctypes.data if n else None, n, 1 if threaded else 0, nthreads, ctypes.byref(res))
    if st != 0:
        return OracleResult(st, np.zeros((0, 3), np.uint32), np.zeros(0, np.uint32), 0, {})
    tris = np.ctypeslib.as_array(res.tris, shape=(res.ntri * 3,)).reshape(-1, 3).copy() if res.ntri else \
        np.zeros((0, 3), np.uint32)
    rep = np.ctypeslib.as_array(res.rep, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
    stats = {f: getattr(res.stats, f) for f, _ in _Stats._fields_}
    uniq = res.unique_points
    L.qdo_result_free(ctypes.byref(res))
    return OracleResult(st, tris, rep, uniq, stats)


def check_input(pts) -> int:
    L = lib()
    if pts is None:
        return L.qdo_check_input(None, 1)
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)
    return L.qdo_check_input(pts.ctypes.data if pts.shape[0] else None, pts.shape[0])


def orient2d(a, b, c, exact: bool = False) -> int:
    L = lib()
    arr = [np.ascontiguousarray(p, dtype=np.float64) for p in (a, b, c)]
    f = L.qdo_orient2d_exact if exact else L.qdo_orient2d
    return f(*[x.ctypes.data for x in arr])


def incircle(a, b, c, d, exact: bool = False) -> int:
    L = lib()
    arr = [np.ascontiguousarray(p, dtype=np.float64) for p in (a, b, c, d)]
    f = L.qdo_incircle_exact if exact else L.qdo_incircle
    return f(*[x.ctypes.data for x in arr])


def canonical(tris: np.ndarray) -> np.ndarray:
    """The reference harness's canonical form (qdt_verify.cpp:408-427): every
    triangle rotated so that its smallest index comes first, orientation
    kept; rows sorted."""
    t = np.asarray(tris, dtype=np.int64).reshape(-1, 3)
    if t.shape[0] == 0:
        return t
    k = np.argmin(t, axis=1)
    idx = (k[:, None] + np.arange(3)[None, :]) % 3
    r = np.take_along_axis(t, idx, axis=1)
    order = np.lexsort((r[:, 2], r[:, 1], r[:, 0]))
    return r[order]


def canonical_digest(tris: np.ndarray) -> str:
    import hashlib
    c = canonical(tris).astype(np.int64)
    return hashlib.sha256(c.tobytes()).hexdigest()
