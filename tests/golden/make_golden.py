"""Generates the golden fixtures of the batch path from the reference itself.

Run in a container that has the reference tree (it is compiled from its own
sources into oracle/_ref by oracle/build_ref.sh):

    python tests/golden/make_golden.py

It feeds seeded inputs to the reference library through its C ABI
(qdt_execute and qdt_execute_parallel), reads the triangles back with
qdt_get_triangle and the used-point flags with qdt_point_is_used, and
writes:

* small_cases.npz -- points, canonical triangles and used flags of small
  structured and random cases (full arrays);
* digests.json    -- for the large workloads: counts and SHA-256 digests of
  the canonical triangle list and of the used flags;
* config_b.npz    -- the many-set workload at its stated size (4,096 sets):
  per set the status, the triangle count and 64-bit digests of the
  canonical triangles and of the used flags (`--config-b-only` makes this
  file alone).

The canonical form is the reference harness's (qdt_verify.cpp:408-427).
Nothing at test time reads the reference; the tests read only these files.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from libqdt_gb300 import qdt_api as Q  # noqa: E402
from libqdt_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.golden import cases as C  # noqa: E402


_dump = None


def load_dump():
    """The bulk readers of a reference context (oracle/qdt_dump.c)."""
    global _dump
    import ctypes
    if _dump is None:
        _dump = ctypes.CDLL(os.path.join(O.REF_DIR, "libqdt_dump_ref.so"))
        _dump.qdt_dump_triangles.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        _dump.qdt_dump_triangles.restype = ctypes.c_size_t
        _dump.qdt_dump_used.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        _dump.qdt_dump_used.restype = ctypes.c_size_t
    return _dump


def run_ref(lib, pts, parallel):
    """Runs the reference's batch call and reads the context back through its
    query functions (in bulk, via oracle/qdt_dump.c)."""
    load_dump()
    with Q.Context(lib) as c:
        st = c.execute(pts, parallel=parallel)
        tris = np.zeros((c.triangles_size(), 3), dtype=np.int64)
        used = np.zeros(c.points_size(), dtype=np.uint8)
        _dump.qdt_dump_triangles(c.ptr, tris.ctypes.data)
        _dump.qdt_dump_used(c.ptr, used.ctypes.data)
    return st, tris, used


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    if not O.build_reference():
        print("reference not available; nothing generated")
        return 1
    lib = Q.load(O.REF_LIB_PATH)
    mesh_only = "--mesh-only" in sys.argv   # regenerate mesh_cases.npz alone
    if "--config-b-only" in sys.argv:
        return make_config_b(lib)
    if "--large-only" in sys.argv:
        return make_large(lib)

    small = {}
    for name, pts in ([] if mesh_only else C.small_cases()):
        st, tris, used = run_ref(lib, pts, False)
        st2, tris2, used2 = run_ref(lib, pts, True)
        ct = O.canonical(tris)
        assert st == 0 and st2 == 0, name
        assert np.array_equal(ct, O.canonical(tris2)), name
        assert np.array_equal(used, used2), name
        small[name + "/pts"] = pts
        small[name + "/tris"] = ct.astype(np.int64)
        small[name + "/used"] = used
    if not mesh_only:
        np.savez_compressed(os.path.join(HERE, "small_cases.npz"), **small)
        print("small cases:", len(small) // 3)

    mesh = {}
    load_dump()
    for name, pts, ops in C.mesh_cases():
        for par in (False, True):
            with Q.Context(lib) as c:
                st = c.execute(pts, parallel=par)
                statuses = []
                for op in ops:
                    if op[0] == "insert":
                        sti, idx = c.insert_point(op[1], op[2], parallel=par)
                        statuses.append(int(sti))
                        statuses.append(int(idx))
                    else:
                        statuses.append(int(c.insert_constraint(op[1], op[2])))
                n = c.points_size()
                tris = np.zeros((c.triangles_size(), 3), dtype=np.int64)
                _ = run_ref  # bulk reader bound below
                import ctypes as _ct
                _dump.qdt_dump_triangles(c.ptr, tris.ctypes.data)
                used = np.zeros(n, dtype=np.uint8)
                _dump.qdt_dump_used(c.ptr, used.ctypes.data)
            key = "%s/%s" % (name, "par" if par else "ser")
            mesh[key + "/tris"] = O.canonical(tris).astype(np.int64)
            mesh[key + "/status"] = np.array(statuses, dtype=np.int64)
            mesh[key + "/used"] = used
    np.savez_compressed(os.path.join(HERE, "mesh_cases.npz"), **mesh)
    print("mesh cases:", len(mesh) // 3)
    if mesh_only:
        return 0

    make_large(lib)
    return make_config_b(lib)


def make_config_b(lib):
    """Every set of the many-set workload through the reference's
    qdt_execute, one call per set (the serial batch path)."""
    t0 = time.time()
    sets = C.config_b_sets()
    rec = np.zeros((len(sets), 4), dtype=np.uint64)
    sizes = np.array([p.shape[0] for p in sets], dtype=np.int64)
    for i, p in enumerate(sets):
        st, tris, used = run_ref(lib, p, False)
        r = C.set_record(st, tris, used)
        rec[i] = [np.uint64(r[0] & 0xFFFFFFFFFFFFFFFF), r[1], r[2], r[3]]
    np.savez_compressed(os.path.join(HERE, "config_b.npz"), sizes=sizes, status=rec[:, 0].astype(np.int64),
                        ntri=rec[:, 1].astype(np.int64), tri_digest=rec[:, 2], used_digest=rec[:, 3])
    print("config B: %d sets, %d points, %.1fs" % (len(sets), int(sizes.sum()), time.time() - t0))
    return 0


def make_large(lib):
    out = {"canonical_form": "qdt_verify.cpp:408-427", "cases": []}
    for spec in C.large_specs():
        pts = C.make_large(spec)
        rec = dict(spec)
        for par in (False, True):
            t0 = time.time()
            st, tris, used = run_ref(lib, pts, par)
            ct = O.canonical(tris)
            key = "threaded" if par else "serial"
            rec[key] = {
                "status": int(st),
                "ntri": int(ct.shape[0]),
                "tri_digest": digest(ct.astype(np.int64)),
                "used_digest": digest(used),
                "used_count": int(used.sum()),
            }
            print(spec["name"], key, ct.shape[0], "%.1fs" % (time.time() - t0), flush=True)
        rec["npts"] = int(pts.shape[0])
        out["cases"].append(rec)
    with open(os.path.join(HERE, "digests.json"), "w") as f:
        json.dump(out, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
