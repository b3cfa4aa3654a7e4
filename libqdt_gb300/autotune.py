"""Autotuner of the build schedule.

The schedule has knobs that change the speed, never the result (the parity
tests run every setting): the node size from which a merge runs on a whole
warp instead of one thread (single-set and many-set builds), the size of the
shared-memory cells (0 = none), and the number of serving engines. The best
values depend on the GPU and its clocks, so they are measured: `tune()` times
candidate values on seeded synthetic workloads with CUDA events (the build
stage, best of three calls), keeps the fastest, writes them to a JSON cache
per GPU model and library version (in the package's build folder) and sets
them as the library's process-wide defaults (qdtg_set_defaults). `load()` of
the package applies a cached tuning when one exists; `ensure()` tunes when
none does.

    python -m libqdt_gb300.autotune [--force]
"""
from __future__ import annotations

import json
import os
import re
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE_DIR = os.path.join(HERE, "_build")

SINGLE_WARP_NODES = (1024, 2048, 4096, 8192)
BATCH_WARP_POINTS = (256, 512, 1024)
BATCH_WARP_NODES = (1024, 4096, 16384)
CELLS = (0, 128)
WORKERS = (2, 4, 8)


def gpu_name(lib) -> str:
    import ctypes
    buf = ctypes.create_string_buffer(256)
    return buf.value.decode() if lib.qdtg_device_name(buf, 256) == 1 else ""


def cache_path(name: str) -> str:
    return os.path.join(CACHE_DIR, "tuning_%s.json" % re.sub(r"[^A-Za-z0-9]+", "_", name).strip("_"))


def _version(lib) -> str:
    return lib.qdtg_version().decode()


KNOBS = ("cell_points", "batch_cell_points", "single_warp_nodes", "batch_warp_min_points", "batch_warp_nodes",
         "server_large_workers")


def apply(lib, cfg: dict) -> bool:
    return lib.qdtg_set_defaults(*[int(cfg[k]) for k in KNOBS]) == 1


def load_cached(lib) -> dict | None:
    name = gpu_name(lib)
    if not name:
        return None
    path = cache_path(name)
    if not os.path.exists(path):
        return None
    try:
        cfg = json.load(open(path))
    except (OSError, ValueError):
        return None
    if cfg.get("library") != _version(lib) or any(k not in cfg for k in KNOBS):
        return None
    return cfg if apply(lib, cfg) else None


def _best_build_ms(run, calls: int = 3) -> float:
    run()   # warm-up (workspace allocation, first-touch)
    best = min(run() for _ in range(calls))
    if not best > 0:
        # a zero build time means the stage events did not record: choosing
        # by it would pick an arbitrary candidate
        raise RuntimeError("autotune: the build stage timed at %r ms" % best)
    return best


def tune(lib, verbose: bool = False) -> dict:
    import numpy as np

    import libqdt_gb300 as G
    from libqdt_gb300 import serving as S
    from libqdt_gb300 import workloads as W

    t_start = time.time()
    meas = {"single": {}, "batch": {}, "serving": {}}

    def log(*a):
        if verbose:
            print("autotune:", *a, flush=True)

    # single set: one large set (1,048,576 uniform points, throughput) and
    # 16 small ones (2,000 points, latency); the cost is the sum of builds
    singles = [W.uniform(1 << 20, 101)] + [W.uniform(2000, 200 + i) for i in range(16)]

    def single(nodes, cells):
        with G.Triangulation(lib) as t:
            t.set_options(stage_timing=True)
            t.set_warp_nodes(nodes)
            t.set_cell_points(cells)

            def run():
                total = 0.0
                for p in singles:
                    if t.execute(p) != 0:
                        raise RuntimeError("qdt_execute failed during tuning")
                    total += t.run_info()["ms_build"]
                return total
            return _best_build_ms(run)

    for w in SINGLE_WARP_NODES:
        meas["single"]["nodes%d_cells0" % w] = single(w, 0)
        log("single warp nodes", w, meas["single"]["nodes%d_cells0" % w])
    best_w = min(SINGLE_WARP_NODES, key=lambda w: meas["single"]["nodes%d_cells0" % w])
    for c in CELLS[1:]:
        meas["single"]["nodes%d_cells%d" % (best_w, c)] = single(best_w, c)
        log("single cells", c, meas["single"]["nodes%d_cells%d" % (best_w, c)])
    best_c = min(CELLS, key=lambda c: meas["single"]["nodes%d_cells%d" % (best_w, c)])

    # many sets: 1,024 sets of the batched workload's distribution
    # (throughput) and 16 sets of 4,000 points (latency, like a coalesced
    # serving batch)
    batches = []
    for sets in (W.many_sets(count=1024, lo=16, hi=65536, seed=102),
                 [W.uniform(4000, 300 + i) for i in range(16)]):
        batches.append((np.concatenate(sets), G.Batch.offsets_of(sets)))

    def batch(points, nodes, cells):
        with G.Batch(lib) as b:
            b.set_options(stage_timing=True, use_graphs=False, warp_min_points=points)
            b.set_warp_nodes(nodes)
            b.set_cell_points(cells)

            def run():
                total = 0.0
                for allpts, off in batches:
                    if b.execute(allpts, off) != 0:
                        raise RuntimeError("qdtg_batch_execute failed during tuning")
                    total += b.run_info()["ms_build"]
                return total
            return _best_build_ms(run)

    for pw in BATCH_WARP_POINTS:
        for nw in BATCH_WARP_NODES:
            key = "points%d_nodes%d_cells0" % (pw, nw)
            meas["batch"][key] = batch(pw, nw, 0)
            log("batch", key, meas["batch"][key])
    best_bw, best_bn = min(((pw, nw) for pw in BATCH_WARP_POINTS for nw in BATCH_WARP_NODES),
                           key=lambda x: meas["batch"]["points%d_nodes%d_cells0" % x])
    for c in CELLS[1:]:
        key = "points%d_nodes%d_cells%d" % (best_bw, best_bn, c)
        meas["batch"][key] = batch(best_bw, best_bn, c)
        log("batch", key, meas["batch"][key])
    best_bc = min(CELLS, key=lambda c: meas["batch"]["points%d_nodes%d_cells%d" % (best_bw, best_bn, c)])

    # serving engines: throughput of a saturating request stream
    reqs = W.request_stream(48, rate_per_s=2000.0, lo=20_000, hi=1_000_000, seed=103)
    for k in WORKERS:
        with S.Server(lib, large_workers=k, small_threshold=20_000) as srv:
            S.run_open_loop(srv, reqs[:8])
            r = S.run_open_loop(srv, reqs)
        meas["serving"]["workers%d" % k] = r["mpts_per_s"]
        log("serving workers", k, r["mpts_per_s"])
    best_k = max(WORKERS, key=lambda k: meas["serving"]["workers%d" % k])

    cfg = {
        "gpu": gpu_name(lib), "library": _version(lib), "date": time.strftime("%Y-%m-%d %H:%M:%S"),
        "cell_points": best_c, "batch_cell_points": best_bc, "single_warp_nodes": best_w,
        "batch_warp_min_points": best_bw, "batch_warp_nodes": best_bn,
        "server_large_workers": best_k, "seconds": round(time.time() - t_start, 1),
        "measured": {k: {kk: round(vv, 3) for kk, vv in v.items()} for k, v in meas.items()},
        "units": {"single": "ms build, 1,048,576 uniform + 16 x 2,000",
                  "batch": "ms build, 1,024 sets + 16 sets of 4,000",
                  "serving": "Mpts/s, 48 requests 2e4..1e6 points"},
    }
    os.makedirs(CACHE_DIR, exist_ok=True)
    path = cache_path(gpu_name(lib))
    tmp = "%s.%d" % (path, os.getpid())
    with open(tmp, "w") as f:
        json.dump(cfg, f, indent=1)
    os.replace(tmp, path)
    apply(lib, cfg)
    return cfg


def ensure(lib=None, force: bool = False, verbose: bool = False) -> dict:
    import libqdt_gb300 as G
    lib = lib or G.load()
    if not force:
        cfg = load_cached(lib)
        if cfg:
            return cfg
    return tune(lib, verbose=verbose)


if __name__ == "__main__":
    cfg = ensure(force="--force" in sys.argv, verbose=True)
    print(json.dumps({k: v for k, v in cfg.items() if k != "measured"}))
