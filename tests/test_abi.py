"""The C-ABI library without a GPU: it builds for sm_103a, loads, exports
every function that include/*.h declares, and its host logic (input checks,
NULL handling, status strings, the empty context) behaves like the
reference shim (libqdt/qdt.cpp). Nothing here launches a kernel.
"""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import libqdt_gb300 as G
from libqdt_gb300 import qdt_api as Q

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    return G.load()


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        names += re.findall(r"QDT_API\s+[\w\s\*]+?\b(\w+)\s*\(", src)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 14 + len(G.GPU_SYMBOLS)
    for name in names:
        assert hasattr(lib, name), name
    for name in Q.QDT_SYMBOLS:
        assert name in names


def test_status_strings(lib):
    assert lib.qdt_status_string(0) == b"success"
    assert lib.qdt_status_string(-1) == b"the context is NULL"
    assert lib.qdt_status_string(-11) == b"internal error"
    assert lib.qdt_status_string(5) == b"unknown status"
    assert lib.qdt_status_string(-12) == b"unknown status"


def test_null_context(lib):
    assert lib.qdt_execute(None, None, 0) == Q.QDT_ERR_NULL_CONTEXT
    assert lib.qdt_execute_parallel(None, None, 0) == Q.QDT_ERR_NULL_CONTEXT
    idx = ctypes.c_size_t(777)
    assert lib.qdt_insert_point(None, Q.Vec2d(1, 2), ctypes.byref(idx)) == Q.QDT_ERR_NULL_CONTEXT
    assert idx.value == 777
    assert lib.qdt_insert_point_parallel(None, Q.Vec2d(1, 2), None) == Q.QDT_ERR_NULL_CONTEXT
    assert lib.qdt_insert_constraint(None, 0, 1) == Q.QDT_ERR_NULL_CONTEXT
    res = (ctypes.c_int * 2)(5, 5)
    edges = (Q.Edge * 2)()
    assert lib.qdt_insert_constraints_batch(None, edges, 2, res) == Q.QDT_ERR_NULL_CONTEXT
    assert list(res) == [Q.QDT_ERR_NULL_CONTEXT] * 2
    T = (ctypes.c_size_t * 3)(7, 8, 9)
    assert lib.qdt_triangles_size(None) == 0
    assert lib.qdt_get_triangle(None, T, 0) == 0 and list(T) == [7, 8, 9]
    assert lib.qdt_points_size(None) == 0
    p = Q.Vec2d(3, 4)
    assert lib.qdt_get_point(None, ctypes.byref(p), 0) == 0 and (p.x, p.y) == (3, 4)
    assert lib.qdt_point_is_used(None, 0) == 0
    lib.qdt_destroy(None)


def test_host_side_checks_without_gpu(lib):
    with G.Triangulation(lib) as t:
        # order of checks: TOO_MANY, then NULL (qdt.cpp:29-43)
        assert t.execute_raw(None, 100000001) == Q.QDT_ERR_TOO_MANY_POINTS
        assert t.execute_raw(None, 5) == Q.QDT_ERR_NULL_ARGUMENT
        assert t.execute_raw(None, 0) == Q.QDT_OK
        assert t.points_size() == 0 and t.triangles_size() == 0
        # rejected points and constraints change nothing
        assert t.insert_point(float("nan"), 0.0)[0] == Q.QDT_ERR_NOT_FINITE
        assert t.insert_point(0.0, float("inf"))[0] == Q.QDT_ERR_NOT_FINITE
        assert t.insert_constraint(0, 1) == Q.QDT_ERR_INVALID_INDEX
        st, res = t.insert_constraints_batch(np.zeros((0, 2)))
        assert st == Q.QDT_OK
        assert lib.qdt_insert_constraints_batch(t.ptr, None, 3, None) == Q.QDT_ERR_NULL_ARGUMENT
        T = (ctypes.c_size_t * 3)(7, 8, 9)
        assert lib.qdt_get_triangle(t.ptr, T, 0) == 0 and list(T) == [7, 8, 9]
        assert lib.qdt_get_triangle(t.ptr, None, 0) == 0
        assert lib.qdt_get_point(t.ptr, None, 0) == 0
        assert t.point_is_used(0) == 0


def test_version(lib):
    assert b"sm_103a" in lib.qdtg_version()


def test_schedule_defaults(lib):
    """qdtg_set_defaults / qdtg_get_defaults: the autotuner's interface."""
    def get():
        a = [ctypes.c_int() for _ in range(6)]
        lib.qdtg_get_defaults(*[ctypes.byref(x) for x in a])
        return [x.value for x in a]
    old = get()
    want = [64, 128, 1024, 256, 8192, 2]
    try:
        assert lib.qdtg_set_defaults(*want) == 1
        assert get() == want
        assert lib.qdtg_set_defaults(-1, -1, 0, 0, 0, 0) == 1 and get() == want    # keep
        assert lib.qdtg_set_defaults(3, -1, 0, 0, 0, 0) == 0 and get() == want     # cells < 4
        assert lib.qdtg_set_defaults(-1, 2048, 0, 0, 0, 0) == 0                    # cells > 1024
        assert lib.qdtg_set_defaults(-1, -1, 0, 0, 0, 65) == 0                     # > 64 engines
        assert lib.qdtg_set_defaults(0, 0, 0, 0, 0, 0) == 1 and get()[:2] == [0, 0]   # cells off
    finally:
        lib.qdtg_set_defaults(*old)
    assert get() == old
    buf = ctypes.create_string_buffer(64)
    lib.qdtg_device_name(buf, 64)    # no device here: empty, no crash
    assert lib.qdtg_device_name(None, 0) == 0


def test_batch_and_server_host_checks(lib):
    """Argument checks of the many-set and serving entry points that return
    before any GPU work, and the workspace sizing used by admission."""
    from libqdt_gb300 import serving as S
    S.bind(lib)
    assert lib.qdtg_batch_execute(None, None, None, 0) == Q.QDT_ERR_NULL_CONTEXT
    assert lib.qdtg_batch_set_count(None) == 0
    assert lib.qdtg_batch_triangles(None, 0, None) == 0
    assert lib.qdtg_batch_set_cell_points(None, 64) == 0
    w1, w2 = lib.qdtg_workspace_bytes(1_000_000), lib.qdtg_workspace_bytes(2_000_000)
    assert 250 * 1_000_000 < w1 < 600 * 1_000_000 and w2 > w1
    c = S.default_config(lib)
    assert c.hbm_budget_bytes == 150 << 30 and c.large_workers == 4 and c.small_threshold == 65536
    t = ctypes.c_uint64(5)
    assert lib.qdtg_server_submit(None, None, 0, ctypes.byref(t)) == Q.QDT_ERR_NULL_CONTEXT
    bad = S.default_config(lib)
    bad.large_workers = 0
    assert not lib.qdtg_server_create(ctypes.byref(bad))
    bad = S.default_config(lib)
    bad.small_threshold = bad.batch_max_points + 1
    assert not lib.qdtg_server_create(ctypes.byref(bad))
    assert lib.qdtg_server_wait(None, 1, 0.0) == -1
    assert lib.qdtg_server_release(None, 1) == 0


def test_locate_and_batch_insert_host_checks(lib):
    """Batch location and batch insertion: argument checks, NaN queries, and
    the context without triangles (every point outside), none of which needs
    the GPU."""
    assert lib.qdtg_locate_points(None, None, 0, None, None) == Q.QDT_ERR_NULL_CONTEXT
    res = np.zeros(3, dtype=np.int32)
    idx = np.zeros(3, dtype=np.uint64)
    assert lib.qdtg_insert_points(None, None, 3, idx.ctypes.data, res.ctypes.data) == Q.QDT_ERR_NULL_CONTEXT
    assert (res == Q.QDT_ERR_NULL_CONTEXT).all() and (idx == np.iinfo(np.uint64).max).all()
    with G.Triangulation(lib) as t:
        assert lib.qdtg_locate_points(t.ptr, None, 2, None, None) == Q.QDT_ERR_NULL_ARGUMENT
        assert lib.qdtg_insert_points(t.ptr, None, 2, None, None) == Q.QDT_ERR_NULL_ARGUMENT
        assert lib.qdtg_insert_points(t.ptr, None, 0, None, None) == Q.QDT_OK
        st, tri, where = t.locate(np.array([[0.5, 0.5], [np.inf, 0.0]]))
        assert st == Q.QDT_ERR_NOT_FINITE and (tri == -1).all()
        st, tri, where = t.locate(np.array([[0.5, 0.5], [3.0, -1.0]]))
        assert st == Q.QDT_OK and (tri == -1).all() and (where == -1).all()
        assert t.points_size() == 0
        assert lib.qdtg_trace_constraints(None, None, 0, None, None) == Q.QDT_ERR_NULL_CONTEXT
        assert lib.qdtg_trace_constraints(t.ptr, None, 1, None, None) == Q.QDT_ERR_NULL_ARGUMENT
        st, s, c = t.trace_constraints(np.array([[0, 1], [2, 2]]))
        assert st == Q.QDT_OK and (s == Q.QDT_ERR_INVALID_INDEX).all() and (c == 0).all()


def _c_layout(tmp_path, struct, fields):
    """sizeof and offsetof of a header struct, printed by a C program built
    against include/qdt.h and include/qdt_gpu.h."""
    import shutil
    import subprocess
    cc = shutil.which("cc") or shutil.which("gcc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    body = "".join(f'    printf("%zu\\n", offsetof({struct}, {f}));\n' for f in fields)
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"qdt.h\"\n#include \"qdt_gpu.h\"\n"
                   f"int main(void)\n{{\n    printf(\"%zu\\n\", sizeof({struct}));\n{body}    return 0;\n}}\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    return int(out[0]), [int(x) for x in out[1:]]


@pytest.mark.parametrize("name", ["run_info", "server_config", "server_stats", "vec2d", "edge"])
def test_ctypes_structs_match_the_headers(tmp_path, name):
    """Every struct the Python binding passes through the C ABI has the
    header's size and field offsets."""
    from libqdt_gb300 import serving as S
    py, c = {"run_info": (G.RunInfo, "qdtg_run_info"), "server_config": (S.ServerConfig, "qdtg_server_config"),
             "server_stats": (S.ServerStats, "qdtg_server_stats"), "vec2d": (Q.Vec2d, "qdt_vec2d"),
             "edge": (Q.Edge, "qdt_edge")}[name]
    fields = [f for f, _ in py._fields_]
    size, offsets = _c_layout(tmp_path, c, fields)
    assert ctypes.sizeof(py) == size
    assert [getattr(py, f).offset for f in fields] == offsets


def test_filter_stats_size_matches_the_header(tmp_path):
    size, _ = _c_layout(tmp_path, "qdtg_filter_stats", [])
    assert size == 3 * 4 * 2 * 8


def test_split_knob_argument_checks(lib):
    """qdtg_set_split_merges and qdtg_set_split_segments reject a NULL
    context and out-of-range values before they touch the GPU."""
    assert lib.qdtg_set_split_merges(None, 7, 1024) == 0
    assert lib.qdtg_set_split_segments(None, 2, 16384) == 0
    with G.Triangulation(lib) as t:
        assert lib.qdtg_set_split_merges(t.ptr, -2, 1024) == 0
        assert lib.qdtg_set_split_merges(t.ptr, 10, 1024) == 0     # deepest split depth is 9
        assert lib.qdtg_set_split_merges(t.ptr, 7, 255) == 0       # at least 256 points a node
        assert lib.qdtg_set_split_segments(t.ptr, 0, 16384) == 0
        assert lib.qdtg_set_split_segments(t.ptr, 6, 16384) == 0   # at most 5 segments a merge
        assert lib.qdtg_set_split_segments(t.ptr, 2, 1023) == 0    # at least 1024 points a segment
        info = G.RunInfo()
        assert lib.qdtg_get_run_info(t.ptr, ctypes.byref(info)) == 1
        assert info.n == 0 and info.triangles == 0 and info.split_segments == 0
        assert lib.qdtg_get_run_info(t.ptr, None) == 0
    assert lib.qdtg_get_run_info(None, ctypes.byref(G.RunInfo())) == 0
