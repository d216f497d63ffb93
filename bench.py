"""Benchmark: harmonic-mean GTEPS over 64 seeded roots on a Graph500 Kronecker
graph (scale 26, edgefactor 16) on one GB300, plain vs batched BFS.

A step is one pass of the hot path over the 64-root batch:
  plain   -- 64 one-root searches (the drop-in, g5_bfs_run), device-resident
  batched -- one batched level loop over the same 64 roots (g5_batch_run)
TEPS per root = Graph500 edge count of the search (generated edges with a
visited endpoint, self loops and duplicates included) / search time; the
headline value is the harmonic mean over roots of the plain form, as the
reference driver reports (cpu_2d/main.cpp:524-529,944-950).

Inputs: the Kronecker graph is generated and built on the GPU with the
reference generator's seeds (1, 2); synthetic data standing in for the
Graph500 benchmark input.  The CSR (8.6 GB at scale 26) is far larger than
L2, so no flush is needed between searches.

Prints one JSON line (rank 0).  --impl reference times the reference's CPU
path (the oracle port of CPUBFS_bin) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "harmonic-mean GTEPS @scale 26, 64 roots: batched vs plain BFS; p99 query ms"
UNIT = "GTEPS"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=26)
    ap.add_argument("--roots", type=int, default=64)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep Beamer's alpha=14, beta=24")
    ap.add_argument("--alpha", type=float, default=None)
    ap.add_argument("--beta", type=float, default=None)
    ap.add_argument("--tile-edges", type=int, default=None, help="fixed top-down tile size (skips the sizes tuner)")
    ap.add_argument("--bu-serial", type=int, default=None, help="fixed bottom-up serial length (skips the sizes tuner)")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-codec", action="store_true")
    ap.add_argument("--no-c2", action="store_true", help="skip the search with the codec in the level loop")
    ap.add_argument("--c2-scale", type=int, default=-1,
                    help="scale of the search with the codec in the level loop (default: 22 when --scale is 26, "
                         "else none; 0: none)")
    ap.add_argument("--big-scale", type=int, default=-1,
                    help="also compare plain and batched search on a second, larger graph (default: 28 when "
                         "--scale is 26, else none; 0: none)")
    ap.add_argument("--serve-rates", default="1000,5000,20000")
    ap.add_argument("--serve-modes", default="streams,cohorts",
                    help="comma list of server slot kinds to measure: streams, levels, auto, cohorts")
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--profile-batch", action="store_true",
                    help="only the batched search, host-driven with per-kernel CUDA events (for ncu)")
    ap.add_argument("--profile-codec", action="store_true",
                    help="only the codec: the largest level queue of one search at --scale, encoded and "
                         "decoded three times (for ncu)")
    ap.add_argument("--host-loop", action="store_true",
                    help="host-driven level loop (same kernels, one launch each; for ncu, which "
                         "cannot profile kernels inside graphs with conditional nodes)")
    return ap.parse_args()


def hmean(xs):
    xs = [x for x in xs if x > 0]
    return len(xs) / sum(1.0 / x for x in xs) if xs else 0.0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
                for name, val in zip(names, f[5:9]):
                    if val.lower() == "active":
                        reasons.add(name)
            os.unlink(self.path)
        except Exception:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return rank, ws, dist


def barrier_sync(dist):
    from gpugraph500_gb300 import replicas
    replicas.barrier(dist)


def max_over_ranks(x, dist):
    from gpugraph500_gb300 import replicas
    return replicas.reduce_max(x, dist)


def sum_over_ranks(x, dist):
    from gpugraph500_gb300 import replicas
    return replicas.reduce_sum(x, dist)


# ---------------------------------------------------------------------------
# CPU side (oracle port of the reference CPU BFS)
# ---------------------------------------------------------------------------

def cpu_bfs_sample(ro, col, roots, nedges, seconds, threads):
    """Times the oracle's CPUBFS_bin restatement on host cores over a bounded
    sample of the roots; returns (harmonic-mean GTEPS, roots run, threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    lib = orc.lib()
    n = len(ro) - 1
    res = []
    lock = threading.Lock()
    t_end = time.time() + seconds
    idx = [0]

    def worker():
        pred = np.empty(n, np.int64)
        while True:
            with lock:
                if idx[0] >= len(roots) or (time.time() > t_end and res):
                    return
                i = idx[0]
                idx[0] += 1
            t0 = time.perf_counter()
            lib.g5o_bfs(n, ro.ctypes.data, col.ctypes.data, int(roots[i]), pred.ctypes.data, None)
            dt = time.perf_counter() - t0
            with lock:
                res.append(nedges[i] / dt / 1e9)

    ts = [threading.Thread(target=worker) for _ in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return hmean(res), len(res)


def workload_name(scale, roots):
    """config.workload of both arms: the same string for the same workload."""
    return f"plain BFS, kronecker scale {scale} edgefactor 16, {roots} roots"


def cpu_throughput_windows(lib, ro, col, roots, end_deg, threads, win_s, warm, steps):
    """The oracle's CPUBFS_bin restatement on `threads` host threads, each
    running one serial search after another over the roots, for warm + steps
    windows of win_s seconds.  A search's Graph500 edges are credited to each
    window in proportion to the part of its run inside the window (its edges
    per second times the overlap), so a window's value is the threads'
    aggregate edges per second whether or not a search ends inside it.
    Returns per timed window GTEPS, the per-search GTEPS of every search that
    overlapped the timed windows, and the searches run."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    n = len(ro) - 1
    lock = threading.Lock()
    runs = []  # (t_start, t_end, edges)
    nxt = [0]
    t0 = time.perf_counter()
    t_stop = t0 + (warm + steps) * win_s

    def worker():
        pred = np.empty(n, np.int64)
        while True:
            with lock:
                if time.perf_counter() >= t_stop:
                    return
                i = nxt[0] % len(roots)
                nxt[0] += 1
            a = time.perf_counter()
            lib.g5o_bfs(n, ro.ctypes.data, col.ctypes.data, int(roots[i]), pred.ctypes.data, None)
            b = time.perf_counter()
            ne = orc.teps_edges(end_deg, pred)
            with lock:
                runs.append((a, b, ne))

    ts = [threading.Thread(target=worker) for _ in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    vals = []
    for k in range(warm, warm + steps):
        w0, w1 = t0 + k * win_s, t0 + (k + 1) * win_s
        e = sum(ne * max(0.0, min(b, w1) - max(a, w0)) / (b - a) for a, b, ne in runs if b > a)
        vals.append(e / win_s / 1e9)
    lo, hi = t0 + warm * win_s, t_stop
    per = [ne / (b - a) / 1e9 for a, b, ne in runs if b > lo and a < hi and b > a]
    return vals, per, len(runs)


def reference_arm(args):
    """The reference's CPU path (the oracle's restatement of CPUBFS_bin,
    cpu_2d/cpubfs_bin.cpp:116-180, in the level order of
    cpu_2d/globalbfs.hh:657-1128) on the host cores, on the same workload:
    the Kronecker graph generated, built and searched by the oracle on the
    host (generator cpu_2d/generator/graph_generator.c:157-187, CSR
    cpu_2d/distmatrix2d.hh:745-1166, roots cpu_2d/main.cpp:351-392), TEPS
    edge counts as the validator counts them (validate.h:440-443,485).  No
    part of the GPU library is loaded.  Under torchrun only rank 0 runs."""
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    threads = orc.host_threads()
    n = 1 << args.scale
    t0 = time.perf_counter()
    edges = orc.kronecker(args.scale, threads=threads)
    end_deg = orc.endpoint_counts(n, edges, threads)
    ro, col = orc.build_csr(n, edges, threads=threads)
    del edges
    build_s = time.perf_counter() - t0
    roots = orc.select_roots(ro, args.roots)
    lib = orc.lib()
    # one search alone on one core: the reference loop is serial
    # (cpu_2d/cpubfs_bin.cpp:147,168)
    pred = np.empty(n, np.int64)
    for _ in range(2):  # the first run also faults in the output's pages
        a = time.perf_counter()
        lib.g5o_bfs(n, ro.ctypes.data, col.ctypes.data, int(roots[0]), pred.ctypes.data, None)
        serial_s = time.perf_counter() - a
    serial = orc.teps_edges(end_deg, pred) / serial_s / 1e9
    del pred
    # aggregate over the host threads, one serial search per thread
    win = max(args.cpu_seconds / max(args.steps + args.warmup, 1), 0.5)
    vals, per, nrun = cpu_throughput_windows(lib, ro, col, roots, end_deg, threads, win, args.warmup, args.steps)
    value = sum(vals) / len(vals) if vals else 0.0
    sample = (f"oracle CPUBFS_bin restatement on the oracle-built graph, scale {args.scale}: {threads} host "
              f"threads each running serial searches over the {len(roots)} roots, {nrun} searches; each step is "
              f"a {win:.2f} s window credited with the edges per second of the searches running in it")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * win,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic (Graph500 Kronecker, seeds 1,2, generated on the host by the oracle)",
            "config": {"workload": workload_name(args.scale, len(roots)), "graph_build_s": round(build_s, 1),
                       "nnz": int(ro[-1])},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "serial_one_core_gteps": serial,
                             "per_search_hmean_gteps_under_load": hmean(per)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------

def main():
    args = parse()
    # the default workload (scale 26) also runs the scale-28 plain-vs-batched
    # leg and the scale-22 codec-in-loop leg; other scales only when asked
    if args.big_scale < 0:
        args.big_scale = 28 if args.scale == 26 else 0
    if args.c2_scale < 0:
        args.c2_scale = 22 if args.scale == 26 else 0
    if args.impl == "reference":
        return reference_arm(args)
    rank, ws, dist = dist_init(args)
    import torch
    import gpugraph500_gb300 as g5

    dev = torch.cuda.current_device()
    t0 = time.time()
    g = g5.Graph.kronecker(args.scale)
    gen_s = time.time() - t0
    # every rank holds the graph and searches its own block of roots
    from gpugraph500_gb300 import replicas
    roots = replicas.shard_roots(g5.select_roots(g, args.roots * ws), args.roots, rank, ws)
    nr = len(roots)
    if args.profile_codec:
        print(json.dumps(profile_codec(g5, torch, g, roots)))
        return 0
    if args.profile_batch:
        bt = g5.Batch([g])
        out = torch.empty(nr * g.n, dtype=torch.int32, device="cuda")
        bt.profile(roots, [nr], out)  # warm-up (host-driven: no graph launch, so ncu sees every kernel)
        prof = bt.profile(roots, [nr], out)
        print(json.dumps({"profile_batch": prof, "scale": args.scale, "roots": nr}))
        return 0
    # Graph500 edge counts (untimed)
    probe = g5.CudaBFS(g, use_graph=not args.host_loop)
    nedges = []
    for r in roots:
        probe.runBFS(int(r))
        nedges.append(probe.teps_edges())
    probe.close()

    # direction thresholds: autotuned on a sample of the roots (untimed)
    from gpugraph500_gb300 import tune
    tuned = None
    alpha, beta = 14.0, 24.0
    if args.alpha is not None or args.beta is not None:
        alpha = args.alpha if args.alpha is not None else alpha
        beta = args.beta if args.beta is not None else beta
    elif not args.no_tune:
        k = min(16, nr)
        tuned = tune.tune_plain(g5, g, roots[:k], nedges[:k])
        alpha, beta = tuned["alpha"], tuned["beta"]
    sizes = {}
    if args.tile_edges is not None or args.bu_serial is not None:
        sizes = {k: v for k, v in (("tile_edges", args.tile_edges), ("bu_serial", args.bu_serial)) if v is not None}
        tuned_sizes = None
    elif not args.no_tune:
        st = tune.tune_sizes(g5, g, roots[:min(16, nr)], nedges[:min(16, nr)], alpha, beta)
        sizes = {"tile_edges": st["tile_edges"], "bu_serial": st["bu_serial"]}
        tuned_sizes = st["grid"][:6]
    else:
        tuned_sizes = None
    bfs = g5.CudaBFS(g, alpha=alpha, beta=beta, use_graph=not args.host_loop, **sizes)

    # Graph500 validation of every root on the device (untimed)
    all_valid, all_minpar = True, True
    for r in roots:
        bfs.runBFS(int(r))
        v, mp = bfs.validate(int(r))
        all_valid &= v
        all_minpar &= mp

    def plain_step(stats_out):
        for i, r in enumerate(roots):
            code = bfs.run(int(r), None, None, stats=True)
            if code != 0:
                raise g5.G5Error(code, "g5_bfs_run")
            s = bfs.stats
            stats_out.append((i, s.device_ms, s.alg_bytes, s.levels, s.bottom_up_levels))

    for _ in range(args.warmup):
        plain_step([])
    recs = []
    with Clocks(dev) as clk:
        barrier_sync(dist)
        t_start = time.perf_counter()
        for _ in range(args.steps):
            plain_step(recs)
        barrier_sync(dist)
        wall = time.perf_counter() - t_start
    clocks = clk.summary()
    wall = max_over_ranks(wall, dist)
    teps = [nedges[i] / (ms * 1e-3) / 1e9 for (i, ms, _, _, _) in recs]
    value_rank = hmean(teps)
    dev_ms = [ms for (_, ms, _, _, _) in recs]
    alg = [b for (_, _, b, _, _) in recs]
    achieved = sum(alg) / (sum(dev_ms) * 1e-3) / 1e9
    peak, peak_kind = peaks()

    # dominant kernel: one untimed pass in profile mode (host-driven, CUDA
    # events around every launch) over the same roots
    kern = kernel_roofline(g5, g, roots, alpha, beta, peak, sizes)

    # end to end through the C ABI with host (pinned) output buffers: one
    # g5_bfs_run_many call per step over the 64 roots (each search's 8n-byte
    # parent array copied to the host while the next search runs), and the
    # one-call-per-root form beside it
    pinned = [torch.empty(g.n, dtype=torch.int64, pin_memory=True) for _ in range(2)]
    outs = [pinned[i & 1] for i in range(nr)]
    bfs.run_many(roots[:2], outs[:2])  # first use builds the second buffer's graph
    e2e_steps = []
    for _ in range(max(args.steps, 1)):
        t1 = time.perf_counter()
        bfs.run_many(roots, outs)
        e2e_steps.append(sum(nedges) / (time.perf_counter() - t1) / 1e9)
    e2e_value = hmean(e2e_steps)
    e2e_seq = []
    for i, r in enumerate(roots):
        t1 = time.perf_counter()
        code = bfs.run(int(r), pinned[0].data_ptr(), None, stats=False)
        dt = time.perf_counter() - t1
        if code != 0:
            raise g5.G5Error(code, "g5_bfs_run")
        e2e_seq.append(nedges[i] / dt / 1e9)

    # batched form
    batched = None
    if not args.no_batch and hasattr(g5.lib(), "g5_batch_run"):
        try:
            batched = bench_batched(g5, torch, g, roots, nedges, args, tune if not args.no_tune else None, bfs)
        except g5.G5Error as e:
            batched = {"error": str(e)}

    serve = mixed = codec = c2 = None
    torch.cuda.empty_cache()  # the batched leg's output goes back to the device
    if rank == 0 and not args.no_c2 and args.c2_scale:
        c2 = bench_c2(g5, args)
    if rank == 0 and not args.no_serve:
        serve = bench_serve(g5, g, args)
    if rank == 0 and not args.no_mixed:
        mixed = bench_mixed(g5, torch, args)
    if rank == 0 and not args.no_codec:
        codec = bench_codec(g5, torch, args)

    cpu = None
    if rank == 0 and not args.no_cpu:
        ro, col = g.csr()
        cores = 1
        v, k = cpu_bfs_sample(ro, col, roots, nedges, args.cpu_seconds, cores)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"oracle CPUBFS_bin port on {k} of the {nr} roots, serial like the reference "
                         f"(cpu_2d/cpubfs_bin.cpp:147,168), ~{args.cpu_seconds:.0f} s budget"}
        del ro, col

    big = None
    if rank == 0 and args.big_scale:
        # the main graph and workspace go first: the larger graph needs the room
        bfs.close()
        g.close()
        torch.cuda.empty_cache()
        big = bench_big(g5, torch, args, tune if not args.no_tune else None, (alpha, beta))

    value = sum_over_ranks(value_rank, dist) if ws > 1 else value_rank
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic (Graph500 Kronecker generated on the GPU, seeds 1,2)",
            "config": {"workload": workload_name(args.scale, nr),
                       "n": g.n, "nnz": g.nnz, "roots": nr, "parallelism": "replicas" if ws > 1 else "1 GPU",
                       "l2": "inputs larger than L2 (CSR %.1f GB)" % ((g.nnz * 4 + g.n * 8) / 1e9),
                       "graph_build_s": round(gen_s, 2), "alpha": alpha, "beta": beta,
                       "tuner": tuned["grid"][:6] if tuned else None, "sizes": sizes or "defaults (256, 8)",
                       "sizes_tuner": tuned_sizes},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * nr,
                    "d2h_bytes_per_step": 8 * g.n * nr,
                    "how": "g5_bfs_run_many over the roots, int64 parents of every search copied to pinned host "
                           "memory inside the timed call; GTEPS = Graph500 edges of all searches / wall time",
                    "one_call_per_root_hmean": hmean(e2e_seq)},
            "gpu_launches": None,
            "roofline": {"bound": "hbm", "achieved": kern["achieved"], "peak": peak, "unit": "GB/s",
                         "frac": kern["achieved"] / peak, "traffic": kern["traffic"],
                         "peak_kind": peak_kind + " (copy, burst)", "kernel": kern,
                         "search": {"achieved": achieved, "frac": achieved / peak,
                                    "scope": "whole search (every kernel of the level loop), algorithmic bytes"},
                         "dram_measured": dram_measured(g.scale, peak),
                         # the headline traffic comes from the per-kind capture
                         "traffic_settings": capture_settings("k_bu_kinds", g.scale, alpha, beta, sizes or {})},
            "clocks": clocks,
            "validation": {"all_valid": all_valid, "all_min_parent": all_minpar},
            "plain": {"hmean_gteps": value_rank, "mean_ms": statistics.mean(dev_ms),
                      "p99_ms": float(np.percentile(dev_ms, 99)), "levels": recs[0][3] if recs else None},
            "batched": batched,
            "serve": serve,
            "mixed_batch": mixed,
            "codec": codec,
            "codec_in_loop": c2,
            "big_scale": big,
            "cpu_baseline": cpu,
        }
        if batched and "aggregate_gteps" in batched:
            line["batched_over_plain"] = batched["aggregate_gteps"] / value_rank if value_rank else None
        if serve:
            # headline: the lowest offered rate, from the serving mode with the lower p99 there
            modes = [m for m in ("streams", "levels", "auto", "cohorts") if m in serve]
            best = min(modes, key=lambda m: serve[m]["rates"][0]["p99_ms"])
            line["p99_query_ms"] = serve[best]["rates"][0]["p99_ms"]
            line["p50_query_ms"] = serve[best]["rates"][0]["p50_ms"]
            line["serve_mode"] = best
            # p99 and GTEPS of every mode at every offered rate
            line["p99_query_ms_by_rate"] = {m: {str(int(r["rate_qps"])): {"p99_ms": r["p99_ms"], "gteps": r["gteps"]}
                                                for r in serve[m]["rates"]} for m in modes}
        # per search: k_init + (k_td, k_bu, k_count, k_write) per level
        line["gpu_launches"] = sum(1 + 4 * rec[3] for rec in recs)
        print(json.dumps(line))
    bfs.close()
    g.close()
    return 0


BU_KERNEL = "k_bu"
# graphs of at least this many vertices sweep the unvisited list from their
# first bottom-up level on (the library's rule; smaller ones sweep the words)
LIST_FIRST = 1 << 21
TD_KERNEL = "k_td"


def ncu_summary(kernel, scale):
    """The 'key: value' lines of the committed ncu summary
    profiles/<kernel>_scale<scale>.txt (DRAM bytes per launch and mean launch
    time per launch kind, the capture's settings), as floats; {} when
    absent."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_scale{scale}.txt")
    out = {}
    try:
        with open(path) as f:
            for ln in f:
                k, sep, v = ln.partition(":")
                if sep and k in ("first_dram_bytes_per_launch", "list_dram_bytes_per_launch",
                                 "first_ncu_us_scale24",
                                 "first_dram_bytes_scale24", "list_ncu_us_scale24", "list_dram_bytes_scale24"):
                    out[k] = float(v)
                elif sep and k == "settings":
                    # "alpha=14 beta=2000 tile_edges=128 bu_serial=8"
                    out["settings"] = {kv.split("=")[0]: float(kv.split("=")[1]) for kv in v.split() if "=" in kv}
    except (OSError, ValueError, IndexError):
        pass
    return out


def kind_traffic(kind, scale):
    """DRAM bytes per launch of one k_bu launch kind ("bu_first" or
    "bu_list") from the committed summary profiles/k_bu_kinds_scale<s>.txt,
    or None."""
    key = {"bu_first": "first_dram_bytes_per_launch", "bu_list": "list_dram_bytes_per_launch"}.get(kind)
    return ncu_summary("k_bu_kinds", scale).get(key) if key else None


def capture_settings(kernel, scale, alpha, beta, sizes):
    """The thresholds and sizes of the committed capture, and whether they are
    this run's (the per-launch traffic depends on the launch mix they give)."""
    cap = ncu_summary(kernel, scale).get("settings")
    if cap is None:
        return None
    run = {"alpha": float(alpha), "beta": float(beta),
           "tile_edges": float(sizes.get("tile_edges", 256)), "bu_serial": float(sizes.get("bu_serial", 8))}
    return {"capture": cap, "run": run, "match": all(cap.get(k) == v for k, v in run.items())}


def dram_measured(scale, peak):
    """Measured DRAM throughput of the bottom-up expansion from the committed
    single-kernel ncu capture at scale 24, summarised in
    profiles/k_bu_kinds_scale<s>.txt: each launch kind's DRAM bytes over its
    own ncu durations (one capture for both, so cold-cache and serialised).
    Reported beside the algorithmic roofline, not instead of it."""
    s = ncu_summary("k_bu_kinds", scale)
    out = {}
    for kind, key in (("bu_first", "first"), ("bu_list", "list")):
        b, us = s.get(f"{key}_dram_bytes_scale24"), s.get(f"{key}_ncu_us_scale24")
        if b and us:
            gbs = b / (us * 1e-6) / 1e9
            out[kind] = {"gbs": gbs, "frac": gbs / peak, "bytes_per_launch": b, "ncu_us": us}
    if not out:
        return None
    out["source"] = (f"ncu, k_bu alone at scale 24, profiles/k_bu_kinds_scale{scale}.txt "
                     "(bytes and durations of one capture)")
    return out


def kernel_roofline(g5, g, roots, alpha, beta, peak, sizes=None):
    """Per-kernel times of the plain search (profile mode) and the
    algorithmic-bytes roofline of each expansion launch kind, the dominant
    one as the headline.  C = candidates of a bottom-up level (vertices with
    edges not yet visited), off = bytes of a row offset (4 while nnz < 2^32).
    Per launch:
      k_bu over the list of unvisited vertices: 4 C (the list) + (2 off + 4) C
        (row bounds and first neighbour of each listed vertex) + 4 E_bu
        (adjacency read until the first hit) + N/8 frontier probes
      k_bu over the bitmap words (the library's first bottom-up level of a run
        on graphs of fewer than 2^21 vertices): N/8 visited words + (off + 4) C
        (row start and dense first neighbour) + 4 E_bu + N/8 frontier probes +
        N/8 next words
      the first bottom-up level of a run ("bu_first", the largest C) is
      reported apart from the later ones ("bu_list")
      k_td: 20 |F| (queue entry, edge offset, row base) + 4 E_td + N/8 visited."""
    pb = g5.CudaBFS(g, alpha=alpha, beta=beta, use_graph=False, profile=True, **(sizes or {}))
    n = g.n
    off = 4 if g.nnz < (1 << 32) - 64 else 8
    ro = g.row_offsets()
    with_edges = int(np.count_nonzero(np.diff(ro)))
    del ro
    tot = {}
    acc = {k: [0.0, 0.0, 0] for k in ("bu_first", "bu_list", "td")}  # bytes, ms, launches
    for r in roots:
        code = pb.run(int(r), None, None, stats=True)
        if code != 0:
            raise g5.G5Error(code, "g5_bfs_run (profile)")
        log = pb.profile_log()
        for k, ms in log:
            tot[k] = tot.get(k, 0.0) + ms
        exp = [ms for k, ms in log if k == "expand"]
        seen = 0      # vertices visited up to and including the level
        prev_bu = False
        for lvl, row in enumerate(pb.level_log()):
            if lvl >= len(exp):
                break
            d, nf, _, read = (int(x) for x in row)
            seen += nf
            cand = max(with_edges - seen, 0)
            if d == 1 and not prev_bu and n < LIST_FIRST:
                b = 3 * n / 8 + (off + 4) * cand + 4 * read
                key = "bu_first"
            elif d == 1:
                b = (4 + 2 * off + 4) * cand + 4 * read + n / 8
                key = "bu_list" if prev_bu else "bu_first"
            else:
                b = 20 * nf + 4 * read + n / 8
                key = "td"
            prev_bu = d == 1
            acc[key][0] += b
            acc[key][1] += exp[lvl]
            acc[key][2] += 1
    pb.close()
    # the search's kernel time (not the host loop's gap after each level)
    total_ms = sum(v for k, v in tot.items() if k != "host")
    kinds = {}
    for key, (b, ms, cnt) in acc.items():
        if cnt:
            kinds[key] = {"launches": cnt, "ms_per_launch": ms / cnt, "bytes_per_launch": b / cnt,
                          "achieved": b / (ms * 1e-3) / 1e9 if ms > 0 else 0.0,
                          "frac": (b / (ms * 1e-3) / 1e9 / peak) if ms > 0 else 0.0,
                          "share_of_search": ms / total_ms if total_ms else None,
                          "traffic": kind_traffic(key, g.scale)}
    key = max(kinds, key=lambda k: acc[k][1])
    name = TD_KERNEL if key == "td" else BU_KERNEL
    head = kinds[key]
    return {"name": name, "kind": key, "launches": head["launches"], "ms_per_launch": head["ms_per_launch"],
            "bytes_per_launch": head["bytes_per_launch"], "achieved": head["achieved"],
            "share_of_search": head["share_of_search"],
            "traffic": kind_traffic(key, g.scale),
            "traffic_source": f"profiles/k_bu_kinds_scale{g.scale}.txt (DRAM bytes per launch of this kind)",
            "kinds": kinds, "offset_bytes": off, "vertices_with_edges": with_edges,
            "kernel_ms_per_search": {k: v / len(roots) for k, v in tot.items()}}


class _DevArray:
    """A device array handed to torch through __cuda_array_interface__."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3}


def bench_batched(g5, torch, g, roots, nedges, args, tune=None, bfs=None):
    nr = len(roots)
    tuned = tune.tune_batch(g5, torch, [g], [roots]) if tune is not None else None
    bt = g5.Batch([g])
    if tuned:
        bt.set_direction(tuned["alpha"], tuned["beta"])
    out = torch.empty(nr * g.n, dtype=torch.int32, device="cuda")

    def one():
        if args.host_loop:  # host-driven loop, same kernels (profilable by ncu)
            return sum(bt.profile(roots, [nr], out)["kernel_ms"].values())
        return bt.run(roots, [nr], out)

    for _ in range(args.warmup):
        one()
    ms = []
    for _ in range(args.steps):
        ms.append(one())
    total = sum(nedges)
    agg = [total / (m * 1e-3) / 1e9 for m in ms]
    bt.close()
    # every root's parents from the batch equal the plain search's (untimed)
    same = None
    if bfs is not None:
        same = True
        dst = torch.empty(g.n, dtype=torch.int32, device="cuda")
        for j, r in enumerate(roots):
            bfs.runBFS(int(r))
            plain = torch.as_tensor(_DevArray(bfs.device_pred_ptr(), g.n, "<i8"), device="cuda")
            g5.batch_root_parents(out, g.n, nr, j, dst)
            same &= bool(torch.equal(plain.to(torch.int32), dst))
        del dst
    del out
    return {"aggregate_gteps": hmean(agg), "ms_per_batch": statistics.mean(ms), "parents_equal_plain": same,
            "alpha": tuned["alpha"] if tuned else 14.0, "beta": tuned["beta"] if tuned else 24.0}


def bench_serve(g5, big, args):
    """Continuous-batching server over resident Kronecker graphs (the big one
    is the bench graph); seeded Poisson arrivals, graph chosen uniformly."""
    scales = [s for s in (20, 22, 24) if s < args.scale] + [args.scale]
    graphs = [g5.Graph.kronecker(s) for s in scales[:-1]] + [big]
    pools, nedge = [], []
    for gr in graphs:
        roots = g5.select_roots(gr, 64)
        b = g5.CudaBFS(gr)
        ne = {}
        for r in roots:
            b.runBFS(int(r))
            ne[int(r)] = b.teps_edges()
        b.close()
        pools.append(roots)
        nedge.append(ne)
    budget = 96 << 30
    res = {"graphs_scales": scales, "mem_budget_bytes": budget}
    kinds = {"streams": g5.Server.STREAMS, "levels": g5.Server.LEVELS, "auto": g5.Server.AUTO,
             "cohorts": g5.Server.COHORTS}
    for name in args.serve_modes.split(","):
        sv = g5.Server(graphs, mem_budget=budget, keep_results=False, mode=kinds[name])
        res[name] = {"slots": sv.slots(), "rates": serve_rates(sv, args, pools, nedge, len(graphs))}
        sv.close()
    for gr in graphs[:-1]:
        gr.close()
    res["mode_note"] = ("streams: one-root workspaces for every graph; levels: root slots of the bit-sliced "
                        "batch; auto: level slots for graphs of >= 2^25 vertices, workspaces for the rest; "
                        "cohorts: the queued queries of a graph of >= 2^21 vertices start together as one "
                        "batched search whenever one of its two batch workspaces is free, workspaces for the rest")
    return res


def serve_rates(sv, args, pools, nedge, ngraphs):
    """Seeded Poisson arrivals at each rate (graph chosen uniformly); p50/p99
    latency from submission to completion, and GTEPS over the run."""
    rng = np.random.default_rng(12345)
    out = []
    for rate in [float(x) for x in args.serve_rates.split(",")]:
        n = int(rate * args.serve_seconds)
        gaps = rng.exponential(1.0 / rate, n)
        which = rng.integers(0, ngraphs, n)
        picks = [int(pools[w][rng.integers(0, len(pools[w]))]) for w in which]
        st0 = sv.stats()
        t0 = time.perf_counter()
        due = t0
        tickets = []
        for k in range(n):
            due += gaps[k]
            while time.perf_counter() < due:
                pass
            tickets.append((sv.submit(int(which[k]), picks[k]), int(which[k]), picks[k]))
        lat, edges = [], 0
        for t, w, r in tickets:
            sv.wait(t, 600.0)
            _, l, _ = sv.result(t, with_pred=False)
            lat.append(l)
            edges += nedge[w][r]
        wall = time.perf_counter() - t0
        st1 = sv.stats()
        out.append({"rate_qps": rate, "queries": n, "p50_ms": float(np.percentile(lat, 50)),
                    "p99_ms": float(np.percentile(lat, 99)), "gteps": edges / wall / 1e9,
                    "wall_s": wall, "level_steps": st1["steps"] - st0["steps"]})
    return out


def bench_big(g5, torch, args, tune, ab):
    """Plain vs batched search, 64 roots, on a second graph of scale
    args.big_scale (built after the main graph is released)."""
    t0 = time.time()
    g = g5.Graph.kronecker(args.big_scale)
    build_s = time.time() - t0
    res = plain_vs_batched(g5, torch, g, args, tune, ab)
    g.close()
    res.update({"scale": args.big_scale, "graph_build_s": round(build_s, 2)})
    return res


def plain_vs_batched(g5, torch, g, args, tune, ab):
    """64 roots on graph g: harmonic-mean GTEPS of the plain search, then the
    batched search over the same roots (parents checked against plain)."""
    roots = g5.select_roots(g, 64)
    bfs = g5.CudaBFS(g, alpha=ab[0], beta=ab[1], use_graph=not args.host_loop)
    nedges, ms = [], []
    for r in roots:  # warm-up pass, also the TEPS edge counts
        bfs.runBFS(int(r))
        nedges.append(bfs.teps_edges())
    for r in roots:
        code = bfs.run(int(r), None, None, stats=True)
        if code != 0:
            raise g5.G5Error(code, "g5_bfs_run")
        ms.append(bfs.stats.device_ms)
    plain = hmean([ne / (t * 1e-3) / 1e9 for ne, t in zip(nedges, ms)])
    batched = bench_batched(g5, torch, g, roots, nedges, args, tune, bfs)
    bfs.close()
    return {"plain_hmean_gteps": plain, "plain_mean_ms": statistics.mean(ms), "batched": batched,
            "batched_over_plain": batched["aggregate_gteps"] / plain if plain else None}


def profile_codec(g5, torch, g, roots):
    """The largest level queue of the first root's search, encoded and decoded
    three times with s4-bp128-d4 (one-stream calls); checks the round trip."""
    b = g5.CudaBFS(g, want_levels=True)
    b.runBFS(int(roots[0]))
    lev = b.getLevels()
    b.close()
    L = int(np.bincount(lev[lev >= 0]).argmax())
    q = np.nonzero(lev == L)[0].astype(np.uint32)
    n = len(q)
    c = g5.Codec(n + 256)
    din = torch.from_numpy(q.view(np.int32)).cuda()
    dout = torch.zeros(g5.Codec.bound(n) + 64, dtype=torch.int32, device="cuda")
    back = torch.zeros(n + 256, dtype=torch.int32, device="cuda")
    w = m = 0
    for _ in range(3):
        w = c.encode(din, n, dout, g5.CODEC_D4)
        m = c.decode(dout, w, back, n + 256, g5.CODEC_D4)
    ok = m == n and bool(torch.equal(back[:n], din))
    c.close()
    return {"profile_codec": {"level": L, "values": n, "words": w, "round_trip": ok}}


def bench_c2(g5, args):
    """Plain search with every level's sorted queue encoded and decoded by the
    s4-bp128-d4 codec inside the level loop (the decoded queue feeds the next
    top-down level; a device-side compare of the round trip turns any
    difference into G5_ERR_MISMATCH): 64 roots on a Kronecker graph of scale
    --c2-scale, harmonic-mean GTEPS with and without the codec, and the codec's
    share of the search (what it adds in the CUDA graph), with a profile-mode
    pass's split by kernel."""
    g = g5.Graph.kronecker(args.c2_scale)
    roots = g5.select_roots(g, 64)
    res = {"scale": args.c2_scale, "roots": len(roots), "codec": "s4-bp128-d4", "threshold": 64}
    nedges = None
    for name, codec in (("no_codec", g5.CODEC_NONE), ("codec", g5.CODEC_D4)):
        b = g5.CudaBFS(g, codec=codec, codec_threshold=64)
        if nedges is None:
            nedges = []
            for r in roots:
                b.runBFS(int(r))
                nedges.append(b.teps_edges())
        ms, vals, words = [], 0, 0
        for rep in range(2):
            for r in roots:
                code = b.run(int(r), None, None, stats=True)
                if code != 0:
                    raise g5.G5Error(code, "g5_bfs_run (codec in loop)")
                if rep:
                    ms.append(b.stats.device_ms)
                    vals += b.stats.codec_values
                    words += b.stats.codec_words
        b.close()
        res[name] = {"hmean_gteps": hmean([ne / (t * 1e-3) / 1e9 for ne, t in zip(nedges, ms)]),
                     "mean_ms": statistics.mean(ms)}
        if codec:
            res[name]["values_through_codec"] = vals
            res[name]["ratio_words_per_value"] = words / vals if vals else None
    pb = g5.CudaBFS(g, codec=g5.CODEC_D4, codec_threshold=64, use_graph=False, profile=True)
    tot = {}
    for r in roots[:16]:
        pb.run(int(r), None, None, stats=True)
        for k, t in pb.profile_log():
            tot[k] = tot.get(k, 0.0) + t
    pb.close()
    g.close()
    # the codec's cost is what it adds to the search in the CUDA graph; the
    # profile pass (one launch at a time, events between kernel groups) splits
    # the search by kernel, with the host loop's gap after each level apart
    added = res["codec"]["mean_ms"] - res["no_codec"]["mean_ms"]
    res["codec_ms_per_search"] = added
    res["codec_share_of_search"] = added / res["codec"]["mean_ms"] if res["codec"]["mean_ms"] else None
    res["profile_ms_per_search"] = {k: v / 16 for k, v in tot.items()}
    res["round_trip"] = "device compare of every level's decoded queue with the encoded one (no mismatch)"
    return res


def bench_mixed(g5, torch, args):
    """One batched launch over 8 graphs of uneven scale, 16 roots each."""
    scales = [s for s in (18, 19, 20, 21, 22, 22, 23, 24) if s <= args.scale]
    graphs = [g5.Graph.kronecker(s) for s in scales]
    roots = [g5.select_roots(gr, 16) for gr in graphs]
    total_edges = 0
    for gr, rs in zip(graphs, roots):
        b = g5.CudaBFS(gr)
        for r in rs:
            b.runBFS(int(r))
            total_edges += b.teps_edges()
        b.close()
    bt = g5.Batch(graphs)
    out = torch.empty(sum(16 * gr.n for gr in graphs), dtype=torch.int32, device="cuda")
    allroots = np.concatenate(roots)
    counts = [len(r) for r in roots]
    for _ in range(2):
        bt.run(allroots, counts, out)
    ms = [bt.run(allroots, counts, out) for _ in range(3)]
    bt.close()
    del out
    # the single-graph batched case: 64 roots on the largest graph of the set
    single = plain_vs_batched(g5, torch, graphs[-1], args, None, (14.0, 200.0))
    single["scale"] = scales[-1]
    for gr in graphs:
        gr.close()
    return {"scales": scales, "roots_per_graph": 16, "ms": float(np.median(ms)),
            "aggregate_gteps": total_edges / (np.median(ms) * 1e-3) / 1e9,
            "single_graph_64_roots": single}


CODEC_BUCKETS = ((0, 4096, "<=4K"), (4096, 1 << 18, "4K-256K"), (1 << 18, 1 << 20, "256K-1M"),
                 (1 << 20, 1 << 40, ">1M"))


def codec_device_times(g5, torch, c, queues, mode):
    """Device time of one-stream encode and decode per queue, from CUDA events
    around a captured CUDA graph of the asynchronous entry points (lengths in
    device memory, nothing read back), so the time is the kernels' alone.  A
    queue of 1M values or more is copied round-robin over enough buffers to
    exceed L2 (256 MB), so its bytes come from HBM.  Per size bucket:
    uncompressed GB/s (4n / t) and the roofline fraction of the algorithmic
    bytes 4n + 4w (values and stream words, read once and written once)."""
    peak = peaks()[0]
    reps = 6
    acc = {}
    words_total = vals_total = 0
    st = torch.cuda.Stream()
    for q in queues:
        n = len(q)
        copies = 1 if n < (1 << 20) else min(64, -(-(256 << 20) // (4 * n)))
        bound = g5.Codec.bound(n) + 64
        ins = [torch.from_numpy(q.view(np.int32)).cuda() for _ in range(copies)]
        streams = [torch.zeros(bound, dtype=torch.int32, device="cuda") for _ in range(copies)]
        backs = [torch.zeros(n + 256, dtype=torch.int32, device="cuda") for _ in range(copies)]
        lens = torch.tensor([n, 0, 0], dtype=torch.int64, device="cuda")  # n, words, decoded n
        st.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(st):  # warm-up and the word count
            for i in range(copies):
                c.encode_async(ins[i], lens[0:1], streams[i], lens[1:2], mode, stream=st.cuda_stream)
                c.decode_async(streams[i], lens[1:2], backs[i], n + 256, lens[2:3], mode, stream=st.cuda_stream)
        torch.cuda.current_stream().wait_stream(st)
        torch.cuda.synchronize()
        if c.status() != 0 or int(lens[2]) != n or not torch.equal(backs[0][:n].cpu(), ins[0].cpu()):
            raise RuntimeError(f"codec round trip failed on a queue of {n}")
        w = int(lens[1])
        t = {}
        for kind in ("enc", "dec"):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=st):
                for r in range(reps):
                    i = r % copies
                    if kind == "enc":
                        c.encode_async(ins[i], lens[0:1], streams[i], lens[1:2], mode, stream=st.cuda_stream)
                    else:
                        c.decode_async(streams[i], lens[1:2], backs[i], n + 256, lens[2:3], mode, stream=st.cuda_stream)
            g.replay()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            g.replay()
            e1.record()
            torch.cuda.synchronize()
            t[kind] = e0.elapsed_time(e1) * 1e-3 / reps
            del g
        for lo, hi, name in CODEC_BUCKETS:
            if lo < n <= hi or (lo == 0 and n <= hi):
                b = acc.setdefault(name, {"queues": 0, "values": 0, "words": 0, "enc_s": 0.0, "dec_s": 0.0})
                b["queues"] += 1
                b["values"] += n
                b["words"] += w
                b["enc_s"] += t["enc"]
                b["dec_s"] += t["dec"]
                break
        words_total += w
        vals_total += n
        del ins, streams, backs
    out = {"ratio_words_per_value": words_total / vals_total if vals_total else None,
           "timing": f"device time: {reps} calls captured in a CUDA graph, CUDA events around its replay; "
                     f"queues of >= 1M values round-robin over buffers larger than L2", "buckets": {}}
    for name, b in acc.items():
        alg = 4 * (b["values"] + b["words"])
        out["buckets"][name] = {
            "queues": b["queues"], "values": b["values"],
            "encode_GBps": 4 * b["values"] / b["enc_s"] / 1e9, "decode_GBps": 4 * b["values"] / b["dec_s"] / 1e9,
            "encode_us_per_queue": 1e6 * b["enc_s"] / b["queues"], "decode_us_per_queue": 1e6 * b["dec_s"] / b["queues"],
            "encode_frac": alg / b["enc_s"] / 1e9 / peak, "decode_frac": alg / b["dec_s"] / 1e9 / peak}
    allv = sum(b["values"] for b in acc.values())
    out["encode_GBps"] = 4 * allv / sum(b["enc_s"] for b in acc.values()) / 1e9
    out["decode_GBps"] = 4 * allv / sum(b["dec_s"] for b in acc.values()) / 1e9
    return out


def bench_codec(g5, torch, args):
    """s4-bp128 encode/decode on every level queue of 16 roots of a scale-24
    graph, and the 8-way frontier-bitmap OR on 2^24-bit bitmaps."""
    scale = min(24, args.scale)
    gr = g5.Graph.kronecker(scale)
    roots = g5.select_roots(gr, 16)
    b = g5.CudaBFS(gr, want_levels=True)
    queues = []
    lev = np.empty(gr.n, np.int32)
    for r in roots:
        b.run(int(r), None, lev)
        order = np.argsort(lev, kind="stable")
        ls = lev[order]
        for L in range(1, int(lev.max()) + 1):
            lo, hi = np.searchsorted(ls, L), np.searchsorted(ls, L + 1)
            if hi > lo:
                queues.append(np.sort(order[lo:hi]).astype(np.uint32))
    b.close()
    maxn = max(len(q) for q in queues)
    c = g5.Codec(maxn + 256)
    din = torch.empty(maxn + 256, dtype=torch.int32, device="cuda")
    dout = torch.empty(g5.Codec.bound(maxn) + 64, dtype=torch.int32, device="cuda")
    back = torch.empty(maxn + 256, dtype=torch.int32, device="cuda")
    stats = {}
    # all queues concatenated, for the batched calls
    cat = np.concatenate(queues)
    in_off = np.zeros(len(queues) + 1, np.uint64)
    in_off[1:] = np.cumsum([len(q) for q in queues])
    bin_ = torch.from_numpy(cat.view(np.int32)).cuda()
    bout = torch.empty(g5.Codec.batch_bound(in_off) + 64, dtype=torch.int32, device="cuda")
    bback = torch.empty(len(cat) + 256, dtype=torch.int32, device="cuda")
    for mode, name in ((g5.CODEC_D4, "d4"), (g5.CODEC_DM, "dm")):
        stats[name] = codec_device_times(g5, torch, c, queues, mode)
        # the same queues in one batched call each way (host set-up included)
        cs = torch.cuda.current_stream().cuda_stream
        times = {"enc": [], "dec": []}
        singles = []
        for q in queues:
            din[: len(q)] = torch.from_numpy(q.view(np.int32)).cuda()
            w = c.encode(din, len(q), dout, mode)
            singles.append(dout[:w].cpu().numpy())
        vals = sum(len(q) for q in queues)
        for rep in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out_off, bw = c.encode_batch(bin_, in_off, bout, mode=mode, stream=cs)
            times["enc"].append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            c.decode_batch(bout, out_off[:-1], bw, np.diff(in_off), bback, mode=mode, stream=cs)
            times["dec"].append(time.perf_counter() - t0)
        hb = bout.cpu().numpy()
        same = all(np.array_equal(hb[int(o):int(o) + int(w)], sg) for o, w, sg in zip(out_off[:-1], bw, singles))
        same &= bool(torch.equal(bback[:len(cat)].cpu(), torch.from_numpy(cat.view(np.int32))))
        stats[name]["batched"] = {"encode_GBps": 4 * vals / min(times["enc"]) / 1e9,
                                  "decode_GBps": 4 * vals / min(times["dec"]) / 1e9,
                                  "streams_equal_single_calls": bool(same),
                                  "timing": "one call for all queues, wall time incl. host set-up, best of 3"}
    c.close()
    gr.close()
    # bitmap OR: 8 sources of 2^24 bits, densities 1..60 %, 12 independent sets
    # round-robin so the footprint (12 x 9 x 2 MB = 216 MB) exceeds L2
    words64 = (1 << 24) // 64
    rng = np.random.default_rng(7)
    res = {}
    for dens in (0.01, 0.05, 0.1, 0.2, 0.4, 0.6):
        sets = []
        for _ in range(12):
            srcs = []
            for _ in range(8):
                bits = rng.random(1 << 24) < dens
                srcs.append(torch.from_numpy(np.packbits(bits, bitorder="little").view(np.int64)).cuda())
            sets.append((torch.zeros(words64, dtype=torch.int64, device="cuda"), srcs))
        # the calls are captured once in a CUDA graph and replayed, so the
        # events time the kernels back to back, not the host's launch rate
        reps = 24
        st = torch.cuda.Stream()
        st.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(st):
            for k in range(len(sets)):
                g5.bitmap_or(sets[k][0], sets[k][1], words64, stream=st.cuda_stream)
        torch.cuda.current_stream().wait_stream(st)
        cg = torch.cuda.CUDAGraph()
        with torch.cuda.graph(cg, stream=st):
            for k in range(reps):
                dst, srcs = sets[k % len(sets)]
                g5.bitmap_or(dst, srcs, words64, stream=st.cuda_stream)
        cg.replay()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        cg.replay()
        e1.record(); torch.cuda.synchronize()
        t = e0.elapsed_time(e1) * 1e-3 / reps
        res[str(dens)] = {"GBps": 10 * words64 * 8 / t / 1e9, "us": t * 1e6, "frac": 10 * words64 * 8 / t / 1e9 / peaks()[0]}
        del cg
    return {"queues": len(queues), "values": vals, "max_queue": maxn, "codecs": stats,
            "bitmap_or_8x2^24": res, "bitmap_or_bytes_per_call": 10 * words64 * 8,
            "bitmap_or_timing": "24 calls captured in one CUDA graph, CUDA events around its replay",
            "l2": "12 bitmap sets used round-robin (216 MB > L2)"}


if __name__ == "__main__":
    sys.exit(main())
