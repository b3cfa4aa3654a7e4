#!/usr/bin/env python3
"""Benchmark of the batch Delaunay triangulation path.

Metric: Mpoints/s triangulated, with 0 exact-predicate violations (checked
once per run, outside the timed region, by the oracle's exact checker).
Workload (default): 2,600,000 float64 points uniform in [0,1)^2 -- the
single-GPU plain-path configuration the target is quoted on. Data are
synthetic (seeded), as the reference's own benchmark is.

GB300 arm (default):
  value -- device-resident: the points are in HBM when the timed region
           starts; one step = qdtg_execute_device() (all stages, result in
           HBM). Timed with CUDA events on the library's stream; L2 flushed
           (256 MiB write) between steps, outside the events.
  e2e   -- through qdt_execute() with host buffers: host copy into the
           context, H2D, all stages, D2H of triangles and representatives;
           wall-clock per call.
Reference arm (--impl reference): the CPU restatement of the reference's
threaded batch driver (oracle/, pthreads, all host cores) on the same
workload -- the reference's own sources are not available on this machine.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path has no exchange step); value = all ranks' points / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpoints/s triangulated (0 exact violations), single+batched; p50/p99 latency"
UNIT = "Mpoints/s"

PROFILES = os.path.join(ROOT, "profiles")


def profile_traffic(workload, stage="build"):
    """DRAM bytes (read + written) of one call's launches of a stage, from the
    `traffic-record:` line of a committed ncu summary under profiles/ (one
    capture of the workload; the line names the commit it measured). Returns
    (bytes or None, source dict)."""
    import glob
    import re
    for path in sorted(glob.glob(os.path.join(PROFILES, "*.md"))):
        with open(path) as f:
            for line in f:
                m = re.match(r"\s*traffic-record:\s*(.*)$", line)
                if not m:
                    continue
                kv = dict(t.split("=", 1) for t in m.group(1).split() if "=" in t)
                if kv.get("workload") == workload and kv.get("stage") == stage:
                    total = int(kv["dram_read"]) + int(kv["dram_write"])
                    return total, {"profile": os.path.relpath(path, ROOT), "commit": kv.get("commit"),
                                   "date": kv.get("date"), "launches": int(kv.get("launches", 0))}
    return None, {"reason": "no committed ncu capture of this workload's %s stage" % stage}

WORKLOADS = {
    "uniform_2p6m": ("uniform", 2600000, 2),
    "uniform_1m": ("uniform", 1048576, 1),
    "lattice_1024_dups": ("lattice", 1024, 7),
    "gauss_4m": ("gauss", 4000000, 11),
    "uniform_100k": ("uniform", 100000, 12345),
    "circle_100k": ("circle", 100000, 13),
    "line_1m": ("line", 1000000, 17),
}


def make_points(name):
    from libqdt_gb300 import workloads as W
    kind, n, seed = WORKLOADS[name]
    if kind == "uniform":
        return W.uniform(n, seed)
    if kind == "lattice":
        return W.lattice_with_duplicates(n, 0.01, seed)
    if kind == "gauss":
        return W.gaussian_mixture(n, 64, seed)
    if kind == "circle":
        return W.unit_circle(n, seed)
    if kind == "line":
        return W.noisy_line(n, seed)
    raise ValueError(name)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", "qdt_clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out["sm_mhz"] = statistics.median(sm)
            out["sm_max_mhz"] = max(mx)
            out["samples"] = len(sm)
        out["reasons"] = sorted(reasons)
        return out


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_threads():
    return max(1, min(64, os.cpu_count() or 1))


def max_over_ranks(value, dist, device="cuda"):
    """The slowest rank's value (replicas: the job ends when the last one
    does). dist is torch.distributed or None."""
    if dist is None:
        return value
    import torch
    x = torch.tensor([float(value)], device=device, dtype=torch.float64)
    dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return float(x.item())


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's threaded
    batch driver, all host threads, on the same workload."""
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    from oracle import oracle as O
    pts = make_points(args.workload)
    n = pts.shape[0]
    nt = cpu_threads()
    for _ in range(args.warmup):
        O.triangulate(pts, threaded=True, nthreads=nt)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = O.triangulate(pts, threaded=True, nthreads=nt)
        times.append(time.perf_counter() - t0)
        assert r.status == 0
    ms = 1e3 * statistics.mean(times)
    value = n / (ms / 1e3) / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "points": n, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": nt, "kind": "port",
                         "sample": "full workload (%d points) per step, threaded driver" % n},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import numpy as np
    import torch

    import libqdt_gb300 as G
    from oracle import delaunay_check as D
    from oracle import oracle as O

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    pts = make_points(args.workload)
    n = pts.shape[0]
    lib = G.load()
    # the schedule knobs for this GPU: cached, or measured now (outside every
    # timed region; they change the speed, not the results)
    from libqdt_gb300 import autotune
    tuning = autotune.ensure(lib) if not args.no_tune else None
    t = G.Triangulation(lib)
    t.set_options(count_filter_failures=False, stage_timing=True)
    d_pts = torch.from_numpy(pts).cuda().contiguous()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    # correctness once, outside the timed region: exact checker on the result
    st = t.execute_device(d_pts.data_ptr(), n)
    if st != 0:
        raise RuntimeError("qdtg_execute_device failed: %d" % st)
    tris = t.download_device_triangles()
    viol = None
    if not args.no_check:
        rep = O.triangulate(pts).rep if n <= 4_000_000 else None
        res = D.check(pts, tris, rep)
        viol = int(sum(res.values()))
    ntri = tris.shape[0]
    m = t.run_info()["unique_points"]

    stream = torch.cuda.ExternalStream(t.stream())
    for _ in range(max(0, args.warmup - 1)):
        t.execute_device(d_pts.data_ptr(), n)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    step_ms, stage = [], {}
    launches = 0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = t.execute_device(d_pts.data_ptr(), n)
        e1.record(stream)
        e1.synchronize()
        if st != 0:
            raise RuntimeError("qdtg_execute_device failed: %d" % st)
        step_ms.append(e0.elapsed_time(e1))
        info = t.run_info()
        launches += info["kernel_launches"]
        for k in ("ms_sort", "ms_unique", "ms_split", "ms_build", "ms_extract"):
            stage.setdefault(k, []).append(info[k])
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ck = clocks.stop()
    ms = max_over_ranks(statistics.mean(step_ms), dist)
    value = ws * n / (ms / 1e3) / 1e6

    # end to end through qdt_execute with host buffers
    e2e_ms = []
    for _ in range(max(1, args.warmup)):
        t.execute(pts)
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = t.execute(pts)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
        if st != 0:
            raise RuntimeError("qdt_execute failed: %d" % st)
    e2e = max_over_ranks(statistics.mean(e2e_ms), dist)
    e2e_value = ws * n / (e2e / 1e3) / 1e6
    h2d = 16 * n
    d2h = 4 * 3 * 2 * m + 4 * n + 64

    # roofline of the dominant stage
    stage_ms = {k: statistics.mean(v) for k, v in stage.items()}
    peak, peak_kind = peaks()
    # algorithmic bytes of each stage: the build reads each distinct point
    # (16 B) and writes the links of its 3 records (32 B each)
    nrec = 3 * m
    alg = {
        "ms_sort": 16 * n + 20 * n + 16 * (16 * n + 40 * n),   # keys + 16 radix passes (hist read, scatter r+w)
        "ms_unique": 16 * n + 4 * n + 16 * m + 8 * m + 4 * n,
        "ms_split": 0,
        "ms_build": 16 * m + 32 * nrec,
        "ms_extract": 32 * nrec + 12 * ntri,
    }
    top = max(stage_ms, key=lambda k: stage_ms[k])
    achieved = (alg[top] or 1) / (stage_ms[top] / 1e3) / 1e9 if stage_ms[top] > 0 else 0.0
    traffic, traffic_src = profile_traffic(args.workload, top[3:])
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded uniform [0,1)^2)",
        "config": {"workload": args.workload, "points": n, "distinct": m, "triangles": ntri,
                   "l2": "flushed between steps (256 MiB write)", "parallelism": "replicas" if ws > 1 else "single",
                   "tuning": ({k: tuning[k] for k in autotune.KNOBS} if tuning else "defaults")},
        "exact_violations": viol,
        "stage_ms": {k[3:]: round(v, 4) for k, v in stage_ms.items()},
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(e2e, 3)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "stage": top[3:], "achieved": round(achieved, 2), "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 5),
                     "traffic": traffic,
                     "traffic_per": "one call's %s launches, ncu dram bytes read + written" % top[3:],
                     "traffic_source": traffic_src,
                     "algorithmic_bytes": alg[top]},
        "clocks": ck,
    }
    if rank == 0 and not args.no_cpu_baseline:
        nt = cpu_threads()
        times = []
        t0 = time.perf_counter()
        while len(times) < 5 and time.perf_counter() - t0 < 20:
            a = time.perf_counter()
            O.triangulate(pts, threaded=True, nthreads=nt)
            times.append(time.perf_counter() - a)
        cb = n / statistics.median(times) / 1e6
        line["cpu_baseline"] = {"value": round(cb, 4), "unit": UNIT, "cores": nt, "kind": "port",
                                "sample": "%d full runs of the workload, threaded driver" % len(times)}
    t.close()
    del d_pts
    torch.cuda.empty_cache()
    if rank == 0 and ws == 1:
        legs = [x for x in args.legs.split(",") if x]
        if "batched" in legs:
            line["batched"] = run_batched_leg(lib, args, flush)
        if "serving" in legs:
            line["serving"] = run_serving_leg(lib, args)
        if "handle" in legs:
            line["handle"] = run_handle_leg(lib, pts, args)
        if "stress" in legs:
            line["stress"] = run_stress_leg(lib, args, flush)
        line["summary"] = summarize(line)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def summarize(line):
    """The legs' headline figures in one small object at the end of the line
    (the line's tail is what a log keeps): single device and e2e Mpts/s, the
    batched ones, serving p50/p99 per rate, the stress rows' Mpts/s."""
    out = {"single": line.get("value"), "single_e2e": (line.get("e2e") or {}).get("value")}
    b = line.get("batched")
    if b:
        out["batched"] = b.get("value")
        out["batched_e2e"] = (b.get("e2e") or {}).get("value")
        out["batched_vs_plain"] = b.get("speedup_e2e_vs_plain")
    sv = line.get("serving")
    if sv:
        out["serving_p50_p99_ms"] = {str(int(r["rate_per_s"])): [r["p50_ms"], r["p99_ms"]] for r in sv.get("rates", [])}
    st = line.get("stress")
    if st:
        out["stress"] = {r["workload"]: r["value"] for r in st}
    return out


def run_batched_leg(lib, args, flush):
    """Config B: 4,096 independent sets (sizes log-uniform in [16, 65536],
    unit square or disk, 10% snapped to a 256 grid) in one many-set call,
    against the plain path called once per set. Device-resident timing with
    CUDA events on the batch's stream (L2 flushed between steps), end to end
    through qdtg_batch_execute with host buffers, and the plain qdt_execute
    loop over the sets (wall clock, one pass)."""
    import numpy as np
    import torch

    import libqdt_gb300 as G
    from libqdt_gb300 import workloads as W
    from oracle import delaunay_check as D

    sets = W.many_sets(count=4096, lo=16, hi=65536, seed=23)
    off = G.Batch.offsets_of(sets)
    pts = np.concatenate(sets)
    n = pts.shape[0]
    d_pts = torch.from_numpy(pts).cuda()
    b = G.Batch(lib)
    stream = torch.cuda.ExternalStream(b.stream())
    torch.cuda.synchronize()
    for _ in range(max(3, args.warmup)):
        if b.execute_device(d_pts.data_ptr(), off) != 0:
            raise RuntimeError("qdtg_batch_execute_device failed")
    steps_ms, launches = [], 0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = b.execute_device(d_pts.data_ptr(), off)
        e1.record(stream)
        e1.synchronize()
        if st != 0:
            raise RuntimeError("qdtg_batch_execute_device failed")
        steps_ms.append(e0.elapsed_time(e1))
        launches += b.run_info()["kernel_launches"]
    ms = statistics.mean(steps_ms)
    info = b.run_info()
    # end to end with host buffers
    e2e_ms = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        if b.execute(pts, off) != 0:
            raise RuntimeError("qdtg_batch_execute failed")
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e = statistics.mean(e2e_ms)
    # exactness on a sample of sets (exact checker, outside the timings)
    viol = None
    if not args.no_check:
        viol = 0
        for i in range(0, len(sets), 64):
            viol += int(sum(D.check(sets[i], b.triangles(i), b.rep(i)).values()))
    b.close()
    del d_pts
    torch.cuda.empty_cache()
    # the plain path, once per set
    t = G.Triangulation(lib)
    for s in sets[:16]:
        t.execute(s)
    t0 = time.perf_counter()
    for s in sets:
        if t.execute(s) != 0:
            raise RuntimeError("qdt_execute failed")
    plain_s = time.perf_counter() - t0
    t.close()
    plain = n / plain_s / 1e6
    # the CPU port over the same sets: one serial triangulation per set, as
    # many threads as host cores, each with its own sets (independent
    # contexts); the oracle releases the GIL inside the C call
    cpu = None
    if not args.no_cpu_baseline:
        from concurrent.futures import ThreadPoolExecutor

        from oracle import oracle as O
        nt = os.cpu_count() or 1
        O.lib()   # load once before the threads share it
        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=nt) as ex:
            list(ex.map(lambda s: O.triangulate(s).status, sets, chunksize=16))
        cpu_s = time.perf_counter() - t0
        cpu = {"value": round(n / cpu_s / 1e6, 3), "s": round(cpu_s, 3), "unit": UNIT, "cores": nt,
               "kind": "port", "how": "serial port once per set, %d threads with their own sets" % nt}
    return {
        "workload": "4096 sets, log-uniform 16..65536 points, square/disk, 10% on a 256 grid (seed 23)",
        "points": n, "distinct": info["unique_points"], "triangles": info["triangles"],
        "value": round(n / (ms / 1e3) / 1e6, 3), "ms_per_step": round(ms, 3), "unit": UNIT,
        "e2e": {"value": round(n / (e2e / 1e3) / 1e6, 3), "ms_per_step": round(e2e, 3),
                "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": 24 * info["unique_points"] + 4 * n},
        "plain_set_by_set": {"value": round(plain, 3), "s": round(plain_s, 3), "unit": UNIT,
                             "how": "qdt_execute once per set, host buffers"},
        "speedup_e2e_vs_plain": round((n / (e2e / 1e3) / 1e6) / plain, 2),
        "cpu_port_contexts": cpu,
        "gpu_launches": launches, "exact_violations_sampled": viol, "sampled_sets": len(range(0, len(sets), 64)),
    }


def run_serving_leg(lib, args):
    """Config V: an open-loop Poisson stream of requests (sizes log-uniform in
    [100, 2,000,000], each uniform, Gaussian-mixture or snapped to a 256
    grid) at three arrival rates, served by qdtg_server under a 150 GB HBM
    budget. Latency from scheduled arrival to result in host memory."""
    from libqdt_gb300 import serving as S
    from libqdt_gb300 import workloads as W

    base = W.request_stream(args.serve_requests, rate_per_s=1.0, lo=100, hi=2_000_000, seed=29)
    out = {"workload": "%d requests, log-uniform 100..2e6 points, uniform/gauss/grid (seed 29)" % len(base),
           "points_per_stream": int(sum(p.shape[0] for _, p in base)), "budget_bytes": 150 << 30, "rates": []}
    with S.Server(lib) as srv:
        # warm the engines' pools and the batching path
        S.run_open_loop(srv, [(0.0, p) for _, p in base[:24]])
        for rate in (50.0, 200.0, 800.0):
            reqs = [(at / rate, p) for at, p in base]
            s0 = srv.stats()
            r = S.run_open_loop(srv, reqs)
            s1 = r["stats"]
            out["rates"].append({"rate_per_s": rate, "p50_ms": round(r["p50_ms"], 3), "p99_ms": round(r["p99_ms"], 3),
                                 "mpts_per_s": round(r["mpts_per_s"], 3), "completed": r["completed"],
                                 "coalesced": r["coalesced"], "span_s": round(r["span_s"], 3),
                                 "rejected": s1["rejected"] - s0["rejected"], "queued": s1["queued"] - s0["queued"],
                                 "batches": s1["batches"] - s0["batches"]})
        st = srv.stats()
        out["rejected"] = st["rejected"]
        out["queued"] = st["queued"]
        out["batches"] = st["batches"]
        out["peak_resident_bytes"] = st["peak_resident_bytes"]
    return out


STRESS = ("uniform_100k", "uniform_1m", "lattice_1024_dups", "gauss_4m", "circle_100k", "line_1m")


def run_stress_leg(lib, args, flush):
    """The single-set path on the degenerate and skewed distributions:
    1,048,576 uniform; the 1024^2 lattice with 1% exact duplicates; 4,000,000
    points from 64 Gaussians; 100,000 points on the unit circle; 1,000,000
    points on a line with 2^-40 noise. Per workload: device-resident
    Mpoints/s (CUDA events on the engine's stream, L2 flushed between steps),
    violations under the exact checker, and the predicate evaluations that
    took the exact path on the device (counted in a separate run, per 1,000
    points), beside the reference algorithm's filter-failure rate per call
    (the oracle's serial builder, which restates it)."""
    import numpy as np
    import torch

    import libqdt_gb300 as G
    from oracle import delaunay_check as D
    from oracle import oracle as O

    out = []
    for name in STRESS:
        pts = make_points(name)
        n = pts.shape[0]
        d_pts = torch.from_numpy(pts).cuda()
        t = G.Triangulation(lib)
        stream = torch.cuda.ExternalStream(t.stream())
        for _ in range(2):
            t.execute_device(d_pts.data_ptr(), n)
        ms = []
        for _ in range(max(1, min(args.steps, 5))):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st = t.execute_device(d_pts.data_ptr(), n)
            e1.record(stream)
            e1.synchronize()
            if st != 0:
                raise RuntimeError("%s: qdtg_execute_device failed: %d" % (name, st))
            ms.append(e0.elapsed_time(e1))
        t.set_options(count_filter_failures=True)
        t.execute_device(d_pts.data_ptr(), n)
        info = t.run_info()
        fstats = t.filter_stats()
        t.set_options(count_filter_failures=False)
        tris = t.download_device_triangles()
        row = {"workload": name, "points": n, "distinct": info["unique_points"], "triangles": int(tris.shape[0]),
               "value": round(n / (statistics.median(ms) / 1e3) / 1e6, 3), "unit": UNIT,
               "ms_per_step": round(statistics.median(ms), 3),
               "exact_per_1000_points": {"orient2d": round(1e3 * info["orient_exact"] / n, 4),
                                         "incircle": round(1e3 * info["incircle_exact"] / n, 4)},
               "filter_by_stage": stage_rates(fstats, n)}
        if not args.no_check:
            ref = O.triangulate(pts)
            s = ref.stats
            nt = os.cpu_count() or 1
            a = time.perf_counter()
            O.triangulate(pts, threaded=True, nthreads=nt)
            cpu_s = time.perf_counter() - a
            row["cpu_port_threaded"] = {"value": round(n / cpu_s / 1e6, 3), "unit": UNIT, "cores": nt,
                                        "ms": round(1e3 * cpu_s, 1)}
            res = D.check(pts, tris, ref.rep)
            row["exact_violations"] = int(sum(res.values()))
            row["same_triangle_count_as_oracle"] = bool(ref.tris.shape[0] == tris.shape[0])
            row["reference_filter_failure_rate"] = {
                "orient2d": round(s["orient_exact"] / max(1, s["orient_calls"]), 6),
                "incircle": round(s["incircle_exact"] / max(1, s["incircle_calls"]), 6),
                "exact_per_1000_points": {"orient2d": round(1e3 * s["orient_exact"] / n, 4),
                                          "incircle": round(1e3 * s["incircle_exact"] / n, 4)}}
        out.append(row)
        t.close()
        del d_pts
        torch.cuda.empty_cache()
    return out


def stage_rates(fstats, n):
    """Per build stage and predicate: the call count, the fraction the float
    pre-filter left undecided (f32_fail_rate), the fraction the double
    filter left undecided too (fp64_fail_rate: the exact evaluation ran) and
    exact evaluations per 1,000 points."""
    out = {}
    for stage, preds in fstats.items():
        row = {}
        for p, c in preds.items():
            calls = c["calls"]
            row[p] = {"calls": calls,
                      "f32_fail_rate": round(c["f32_undecided"] / calls, 6) if calls else 0.0,
                      "fp64_fail_rate": round(c["exact"] / calls, 6) if calls else 0.0,
                      "exact_per_1000_points": round(1e3 * c["exact"] / n, 4)}
        out[stage] = row
    return out


def run_handle_leg(lib, pts, args):
    """Handle operations after a batch call on the workload's points: the
    first insertion (the half-edge mesh built on the GPU from the resident
    result), batch location of 1,000,000 random points (qdtg_locate_points),
    and 20,000 random insertions through qdtg_insert_points against
    qdt_insert_point called point by point (2,000 points; per-point cost
    compared). Wall clock through the C ABI with host buffers."""
    import numpy as np

    import libqdt_gb300 as G

    rng = np.random.default_rng(31)
    lo, hi = pts.min(0), pts.max(0)
    q = lo + rng.random((1_000_000, 2)) * (hi - lo)
    ins = lo + rng.random((20_000, 2)) * (hi - lo)
    seq = lo + rng.random((2_000, 2)) * (hi - lo)
    out = {"workload": "the bench points; 1e6 random queries, 2e4 batch + 2e3 single insertions (seed 31)"}
    with G.Triangulation(lib) as t:
        ms = []
        for _ in range(3):
            t.execute(pts)
            a = time.perf_counter()
            st, _ = t.insert_point(float(ins[0, 0]), float(ins[0, 1]))
            ms.append(1e3 * (time.perf_counter() - a))
            if st != 0:
                raise RuntimeError("qdt_insert_point failed: %d" % st)
        out["first_insert_ms"] = round(statistics.median(ms), 2)
        t.execute(pts)
        a = time.perf_counter()
        st, _, _ = t.locate(q[:1])
        out["mesh_build_and_index_ms"] = round(1e3 * (time.perf_counter() - a), 2)
        ms = []
        for _ in range(3):
            a = time.perf_counter()
            st, tri, where = t.locate(q)
            ms.append(1e3 * (time.perf_counter() - a))
            if st != 0:
                raise RuntimeError("qdtg_locate_points failed: %d" % st)
        out["locate_1e6_ms"] = round(statistics.median(ms), 2)
        out["locate_mqueries_per_s"] = round(1.0 / statistics.median(ms) * 1e3, 2)
        out["outside"] = int((where < 0).sum())
        a = time.perf_counter()
        st, res, _ = t.insert_points(ins)
        b = time.perf_counter()
        if st != 0:
            raise RuntimeError("qdtg_insert_points failed: %d" % st)
        out["insert_points_us_per_point"] = round(1e6 * (b - a) / len(ins), 3)
        a = time.perf_counter()
        for x, y in seq:
            t.insert_point(float(x), float(y))
        b = time.perf_counter()
        out["insert_point_us_per_point"] = round(1e6 * (b - a) / len(seq), 3)
        out["speedup_batch_insert"] = round(out["insert_point_us_per_point"] / out["insert_points_us_per_point"], 2)
        a = time.perf_counter()
        t.locate(q)
        out["locate_1e6_after_edits_ms"] = round(1e3 * (time.perf_counter() - a), 2)
        # constraint tracing: 10,000 segments between random points (long:
        # each crosses on the order of sqrt(n) edges)
        segs = rng.integers(0, pts.shape[0], size=(10_000, 2))
        t.trace_constraints(segs[:10])
        a = time.perf_counter()
        st, status, crossed = t.trace_constraints(segs)
        out["trace_1e4_ms"] = round(1e3 * (time.perf_counter() - a), 2)
        out["trace_mean_crossed"] = round(float(crossed.mean()), 1)
        out["trace_ok"] = int((status == 0).sum())
    return out


def run_profile_target(args):
    """Runs one form of the path (warmup + steps calls, device-resident input,
    no timing, no L2 flush, no checks) for a profiler to capture: 'single'
    (the --workload points) or 'batched' (config B's 4,096 sets)."""
    import numpy as np
    import torch

    import libqdt_gb300 as G
    from libqdt_gb300 import workloads as W

    lib = G.load()
    if args.profile_run == "single":
        pts = make_points(args.workload)
        d = torch.from_numpy(pts).cuda()
        t = G.Triangulation(lib)
        for _ in range(args.warmup + args.steps):
            if t.execute_device(d.data_ptr(), pts.shape[0]) != 0:
                raise RuntimeError("qdtg_execute_device failed")
        torch.cuda.synchronize()
        print("profile run: single %s, %d calls" % (args.workload, args.warmup + args.steps))
        t.close()
    else:
        sets = W.many_sets(count=args.sets, lo=16, hi=65536, seed=23)
        off = G.Batch.offsets_of(sets)
        d = torch.from_numpy(np.concatenate(sets)).cuda()
        b = G.Batch(lib)
        b.set_options(use_graphs=False)
        for _ in range(args.warmup + args.steps):
            if b.execute_device(d.data_ptr(), off) != 0:
                raise RuntimeError("qdtg_batch_execute_device failed")
        torch.cuda.synchronize()
        print("profile run: batched %d sets, %d calls" % (args.sets, args.warmup + args.steps))
        b.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="uniform_2p6m", choices=sorted(WORKLOADS))
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--legs", default="batched,serving,handle,stress",
                    help="extra legs in the same line (rank 0, one GPU): batched, serving, handle, stress; "
                         "'' for none")
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--no-tune", action="store_true", help="library defaults instead of the autotuner's choice")
    ap.add_argument("--profile-run", choices=["single", "batched"],
                    help="only run the path (no timing) for a profiler; see profiles/")
    ap.add_argument("--sets", type=int, default=4096, help="sets of --profile-run batched")
    args = ap.parse_args()
    if args.profile_run:
        return run_profile_target(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
