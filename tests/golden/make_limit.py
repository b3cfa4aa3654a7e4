"""Generates tests/golden/limit.json: the reference's result at its own
size limit (1e8 points, libqdt/wrapper.hxx:15), uniform points in the unit
square (seed 5), from the reference itself, serial and threaded calls.

Run in a container that has the reference tree (compiled from its own
sources into oracle/_ref by oracle/build_ref.sh; about 30 GB of host memory
and a few minutes):

    python tests/golden/make_limit.py

The digests are those of digests.json (SHA-256 of the canonical triangle
list as int64 rows, qdt_verify.cpp:408-427, and of the used-point flags),
computed here with 32-bit keys to keep the memory in bounds; the bytes
hashed are the same.
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
from tests.golden import make_golden as MG  # noqa: E402


def main():
    if not O.build_reference():
        print("reference not available; nothing generated")
        return 1
    lib = Q.load(O.REF_LIB_PATH)
    spec = C.limit_spec()
    pts = C.make_large(spec)
    rec = dict(spec)
    for par in (False, True):
        t0 = time.time()
        st, tris, used = MG.run_ref(lib, pts, par)
        key = "threaded" if par else "serial"
        rec[key] = {"status": int(st), "ntri": int(tris.shape[0]), "tri_digest": C.canonical_digest32(tris),
                    "used_digest": hashlib.sha256(np.ascontiguousarray(used).tobytes()).hexdigest(),
                    "used_count": int(used.sum())}
        del tris, used
        print(key, rec[key]["ntri"], "%.1fs" % (time.time() - t0), flush=True)
    rec["npts"] = int(pts.shape[0])
    with open(os.path.join(HERE, "limit.json"), "w") as f:
        json.dump({"canonical_form": "qdt_verify.cpp:408-427", "case": rec}, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
