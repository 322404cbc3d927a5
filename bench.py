"""Benchmark: radix-scale PK-FK hash join, 16M build x 256M probe, on one GB300,
followed by every other configuration of the operator path.

Headline step = build the hash table over |R| = 16,777,216 (int64 key, int64
payload) tuples and probe it with |S| = 268,435,456 foreign-key tuples,
materialising every (probe payload, build payload) output row. Keys of R are
a random permutation of 1..|R|; probe keys are uniform over R's keys (seeded
synthetic data).

  value   join tuples/s = (|R| + |S|) / step time, inputs resident in HBM,
          CUDA events on the operator's stream, max over ranks.
  e2e     the same metric through pg_hashjoin_host with pinned HOST buffers:
          host->device copies of R and S and the device->host copy of every
          output row are inside the timed region.
  parity  a whole-row digest (row count, column sums, sum of a row hash) of
          the rows the timed kernel wrote, against the oracle join's.
  roofline  the dominant kernel (the probe) against the measured HBM copy
          bandwidth: algorithmic bytes per launch = 16|S| + 16|out|.
  cpu_baseline  the oracle's port of the reference HashJoinOp (chained
          buckets, per-bucket spinlocks, rows into 1 MiB output pages, all
          host threads) on a bounded sample.
  configs  (one GPU, unless --headline-only) the line of every other
          configuration, measured in this run at full size: the 1M x 16M
          join into aggregate_count + aggregate_sum, the 16M x 256M join
          with Zipf s=1.0 probes and with sparse keys (hashed table), the
          256M-row group-by, the 64M x 64M MPSM join (count/sum and
          materialised), the page sorts, the partition, the 10,000-instance
          batch and the serving loop.

--impl reference times the reference algorithm on the host cores instead:
the oracle port of HashJoinOp over the whole workload every step.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NR = 1 << 24            # overridable with --build-log2 / --probe-log2 (smaller configs)
NS = 1 << 28
TUPLE = 16
# DRAM bytes per probe tuple of the materialising probe against the 16M-key
# (64 MB) dense table, measured by ncu on a 32M-tuple probe of the same table;
# traffic scales with the probe tuples.
PROBE_DRAM_BYTES_PER_TUPLE = (1.054382e9 + 0.514778e9) / (1 << 25)
# DRAM bytes per 24-byte line of the staged probe against a 4M-part table, measured
# by ncu on 16M lines; traffic scales with the lines.
WIDE_DRAM_BYTES_PER_LINE = (419.517440e6 + 358.811904e6) / (1 << 24)


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def dist_setup(n):
    ws = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    local = env_int("LOCAL_RANK", 0)
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """Samples SM clocks and throttle reasons while the timed region runs."""

    def __init__(self, index):
        self.index, self.proc, self.lines = index, None, []
        self.first = threading.Event()

    def start(self):
        """Starts nvidia-smi and returns once its first sample arrived (at most
        5 s): its start-up holds driver calls for up to a second, which must
        not fall into a timed region."""
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(5.0)
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())
            self.first.set()
        self.first.set()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                mhz.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(mhz)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def host_threads():
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count())


# ---------------------------------------------------------------------------
# Hash joins: the 16M x 256M headline (uniform probe), its Zipf s=1.0 and
# sparse-key (hashed table) runs, and the 1M x 16M join feeding
# aggregate_count + aggregate_sum. One step = build + probe over inputs
# resident in HBM.
# ---------------------------------------------------------------------------
PROJ = (("P", 8, 8), ("B", 8, 8))
SPARSE_MUL = 0x9E3779B97F4A7C15 - (1 << 64)      # odd: a bijection on int64 keys


def join_spec(nr, ns, dist="uniform", zipf_s=1.0, key_domain="dense", mode="materialise"):
    what = {"materialise": "output (P$1,B$1) rows materialised",
            "count_sum": "aggregate_count + aggregate_sum(B$1) over the join output, fused into the probe"}[mode]
    probe = "uniform FK" if dist == "uniform" else f"Zipf s={zipf_s} FK (hot ranks scattered over R's keys)"
    keys = ("keys 1..|R| (random permutation)" if key_domain == "dense"
            else "keys 1..|R| times an odd 64-bit constant (hashed table)")
    return {"nr": nr, "ns": ns, "dist": dist, "zipf_s": zipf_s, "key_domain": key_domain, "mode": mode,
            "workload": f"PK-FK hash join: |R|={nr} unique int64 {keys}, |S|={ns} {probe}, 16-byte tuples, {what}"}


def _count(n):
    return f"{n >> 20}M" if n >= 1 << 20 and n % (1 << 20) == 0 else f"{n >> 10}K" if n % 1024 == 0 else str(n)


def join_metric(sp):
    size = f"{_count(sp['nr'])} build x {_count(sp['ns'])} probe"
    if sp["mode"] == "count_sum":
        return f"join tuples/s ({size}, PK-FK, int64 keys, count+sum)"
    tail = "" if sp["dist"] == "uniform" else f", Zipf s={sp['zipf_s']}"
    tail += "" if sp["key_domain"] == "dense" else ", sparse keys"
    return f"join tuples/s ({size}, PK-FK, int64 keys, materialised{tail})"


def join_config(sp, ws):
    """The config dict both arms print for a join workload."""
    return {"workload": sp["workload"], "build_tuples": sp["nr"], "probe_tuples": sp["ns"],
            "probe_dist": sp["dist"] if sp["dist"] == "uniform" else f"zipf s={sp['zipf_s']}",
            "key_domain": sp["key_domain"], "output": sp["mode"],
            "l2": (f"probe side ({16 * sp['ns'] >> 20} MiB) larger than L2 (129 MB); no flush"
                   if 16 * sp["ns"] > 129_000_000 else "probe side fits in L2 (small case; not a bench config)"),
            "parallelism": f"replicas x{ws}"}


def make_join_inputs(sp, R, S, threads):
    from pythia_gb300 import datagen as dg
    dg.build_relation(sp["nr"], dg.seed_for(101), out=R, threads=threads)
    if sp["dist"] == "zipf":
        dg.probe_zipf(sp["ns"], sp["zipf_s"], R, dg.seed_for(103), out=S, threads=threads)
    else:
        dg.probe_uniform(sp["ns"], R, dg.seed_for(102), out=S, threads=threads)
    if sp["key_domain"] == "sparse":
        R[:, 0] *= SPARSE_MUL
        S[:, 0] *= SPARSE_MUL


def cpu_join(sp, R, S, threads, sample=None):
    """Times the oracle port of HashJoinOp (chained buckets, fn=modulo with
    |R| buckets, 4 tuples per bucket, all host threads), every output row
    written into the thread's 1 MiB output page as HashJoinOp::getNext does.
    sample=None: one timed build + probe of the whole workload. Else the
    build alone, then the build with the first `sample` probe tuples, and the
    probe time scaled linearly to |S|. Returns (tuples/s, info)."""
    from oracle import oracle as orc
    nr, ns = sp["nr"], sp["ns"]
    cfg = orc.hashcfg("modulo", nr)
    sc = 1 if sp["mode"] == "count_sum" else -1
    if sample is None or sample >= ns:
        t0 = time.perf_counter()
        n, _ = orc.hashjoin_paged(R, S, hash=cfg, threads=threads, sum_col=sc)
        t = time.perf_counter() - t0
        return (nr + ns) / t, {"build_probe_s": t, "probe_tuples_timed": ns, "rows": int(n), "scaled": False}
    Ssub = np.ascontiguousarray(S[:sample])
    t0 = time.perf_counter()
    orc.hashjoin_paged(R, Ssub[:1], hash=cfg, threads=threads)
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    n, _ = orc.hashjoin_paged(R, Ssub, hash=cfg, threads=threads, sum_col=sc)
    t_all = time.perf_counter() - t0
    t_est = t_build + max(t_all - t_build, 1e-9) * (ns / sample)
    return (nr + ns) / t_est, {"build_s": t_build, "build_probe_s": t_all, "probe_tuples_timed": sample,
                               "rows": int(n), "scaled": True}


def run_reference(args, ws, rank):
    """The reference algorithm on the host cores, on the GPU arm's workload:
    every step builds the table and probes all |S| tuples (rows written into
    1 MiB output pages), all host threads."""
    if rank != 0:
        return
    threads = host_threads()
    sp = headline_spec(args)
    R = np.empty((sp["nr"], 2), dtype=np.int64)
    S = np.empty((sp["ns"], 2), dtype=np.int64)
    make_join_inputs(sp, R, S, threads)
    vals, infos = [], []
    for i in range(args.warmup + args.steps):
        v, info = cpu_join(sp, R, S, threads)
        if i >= args.warmup:
            vals.append(v); infos.append(info)
    value = statistics.median(vals)
    ms = (sp["nr"] + sp["ns"]) / value * 1e3
    line = {"impl": "reference", "metric": join_metric(sp), "value": value, "unit": "tuples/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic (seeded generator)", "config": join_config(sp, ws),
            "cpu_baseline": {"value": value, "unit": "tuples/s", "cores": threads, "kind": "port",
                             "sample": f"whole workload every step: {sp['nr']}-tuple build + all {sp['ns']} probe "
                                       f"tuples (oracle port of HashJoinOp, modulo {sp['nr']} buckets, 4 tuples "
                                       f"per bucket, rows into 1 MiB pages)",
                             "detail": infos[len(infos) // 2]},
            "e2e": {"value": value, "unit": "tuples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def headline_spec(args):
    return join_spec(NR, NS, args.probe_dist, args.zipf_s, args.key_domain, "materialise")


def make_ctx(args, local):
    """GPU context with the --tune knobs applied (name=value,...)."""
    from pythia_gb300 import gpu
    ctx = gpu.Context(local)
    if args.tune:
        ctx.tune(**{k: int(v) for k, v in (kv.split("=") for kv in args.tune.split(","))})
    return ctx


def run_join(args, ws, rank, local, sp, steps, warmup, e2e_steps=3, cpu_sample=None, want_cpu=True):
    """One join workload on the GPU: device-resident steps (value), the probe
    kernel alone (roofline), the host-buffer entry point (e2e), a whole-row
    digest of the timed kernel's output against the oracle's (parity) and
    the CPU port (cpu_baseline). Returns the JSON dict (rank 0) or None."""
    import torch
    from oracle import oracle as orc
    from pythia_gb300 import gpu
    torch.cuda.set_device(local)
    threads = host_threads()
    nr, ns, mode = sp["nr"], sp["ns"], sp["mode"]
    mat = mode == "materialise"
    ctx = make_ctx(args, local)
    L = gpu.lib()

    def pinned(nbytes):
        p = ctypes.c_void_p()
        ctx._check(L.pg_host_alloc(ctx.h, max(nbytes, 16), ctypes.byref(p)))
        return p.value
    hR, hS = pinned(nr * TUPLE), pinned(ns * TUPLE)
    hO = pinned(ns * TUPLE) if mat else pinned(64)
    R = np.ctypeslib.as_array((ctypes.c_int64 * (nr * 2)).from_address(hR)).reshape(nr, 2)
    S = np.ctypeslib.as_array((ctypes.c_int64 * (ns * 2)).from_address(hS)).reshape(ns, 2)
    make_join_inputs(sp, R, S, threads)
    # Expected results from the oracle (the same rows whatever the key domain).
    cfg = orc.hashcfg("modulo", nr)
    if mat:
        want = orc.hashjoin_digest(R, S, proj=PROJ, hash=cfg, threads=threads)
    else:
        _, wn, wsum = orc.hashjoin(R, S, proj=PROJ, hash=cfg, threads=threads, materialise=False, sum_col=1)
        want = {"rows": int(wn), "sum_B1": int(wsum)}

    dR, dS = ctx.alloc(nr * TUPLE), ctx.alloc(ns * TUPLE)
    dO = ctx.alloc(ns * TUPLE) if mat else None
    ctx._check(L.pg_h2d(ctx.h, ctx.stream, dR.ptr, hR, nr * TUPLE))
    ctx._check(L.pg_h2d(ctx.h, ctx.stream, dS.ptr, hS, ns * TUPLE))
    ctx.sync()
    rR = gpu.Rel(dR.ptr, nr, TUPLE, 0, 8)
    rS = gpu.Rel(dS.ptr, ns, TUPLE, 0, 8)
    proj, nproj = gpu.cols(PROJ)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flags = gpu.JOIN_MATERIALIZE if mat else gpu.JOIN_COUNT | gpu.JOIN_SUM
    sum_col = -1 if mat else 1
    probe_ms = []
    last = gpu.JoinResult()

    def step(timed_probe=False):
        ht = ctypes.c_void_p()
        ctx._check(L.pg_hashjoin_build(ctx.h, ctx.stream, ctypes.byref(rR), proj, nproj, ctypes.byref(ht)))
        if timed_probe:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        ctx._check(L.pg_hashjoin_probe(ctx.h, ctx.stream, ht.value, ctypes.byref(rS), proj, nproj,
                                       dO.ptr if mat else None, ns if mat else 0, flags, sum_col,
                                       ctypes.byref(last)))
        if timed_probe:
            e1.record(stream)
            e1.synchronize()
            probe_ms.append(e0.elapsed_time(e1))
        L.pg_hashtable_free(ctx.h, ht.value)

    for _ in range(warmup):
        step()
    clocks = Clocks(local)
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    k0 = gpu.kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        step()
    ev1.record(stream)
    ev1.synchronize()
    launches = gpu.kernel_launches() - k0
    torch.cuda.synchronize()
    barrier(ws)
    clk = clocks.stop()
    ms = max_over_ranks(ws, ev0.elapsed_time(ev1) / steps)
    value = ws * (nr + ns) / (ms / 1e3)
    # Parity of the timed kernel's own output (the last timed step's rows).
    if mat:
        ctx._check(L.pg_d2h(ctx.h, ctx.stream, hO, dO.ptr, last.n_out * TUPLE))
        ctx.sync()
        O = np.ctypeslib.as_array((ctypes.c_int64 * (last.n_out * 2)).from_address(hO)).reshape(-1, 2) \
            if last.n_out else np.zeros((0, 2), dtype=np.int64)
        got = orc.rows_digest(O, threads=threads)
    else:
        got = {"rows": int(last.n_out), "sum_B1": int(last.sum)}
    parity = {"check": "whole-row digest of the timed step's output rows vs the oracle join's"
              if mat else "count and wrapping int64 sum of B$1 vs the oracle join's",
              "expected": want, "got": got, "ok": got == want}

    # Dominant kernel (probe) timed alone with events on its stream.
    for _ in range(max(3, min(steps, 5))):
        step(timed_probe=True)
    probe = statistics.median(probe_ms)
    peak, peak_kind = measured_peak()
    alg_probe = TUPLE * ns + (TUPLE * last.n_out if mat else 0)
    achieved = alg_probe / (probe / 1e3) / 1e9
    alg_step = TUPLE * (nr + ns) + (TUPLE * last.n_out if mat else 0)

    # End to end through the host-buffer entry point.
    e2e_ms = []
    hres = gpu.JoinResult()
    for i in range(max(1, e2e_steps) + 1):
        rRh = gpu.Rel(hR, nr, TUPLE, 0, 8)
        rSh = gpu.Rel(hS, ns, TUPLE, 0, 8)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx._check(L.pg_hashjoin_host(ctx.h, ctypes.byref(rRh), ctypes.byref(rSh), proj, nproj,
                                      hO if mat else None, ns if mat else 0, flags, sum_col, ctypes.byref(hres)))
        t1 = time.perf_counter()
        if i:
            e2e_ms.append((t1 - t0) * 1e3)
    if mat:
        O = np.ctypeslib.as_array((ctypes.c_int64 * (hres.n_out * 2)).from_address(hO)).reshape(-1, 2) \
            if hres.n_out else np.zeros((0, 2), dtype=np.int64)
        e2e_ok = orc.rows_digest(O, threads=threads) == want
    else:
        e2e_ok = {"rows": int(hres.n_out), "sum_B1": int(hres.sum)} == want
    parity["e2e_ok"] = bool(e2e_ok)
    e2e = max_over_ranks(ws, statistics.median(e2e_ms))

    cpu = None
    if rank == 0 and ws == 1 and want_cpu:
        v, info = cpu_join(sp, R, S, threads, cpu_sample)
        m = info["probe_tuples_timed"]
        cpu = {"value": v, "unit": "tuples/s", "cores": threads, "kind": "port",
               "sample": (f"full {nr}-tuple build + " + (f"first {m} probe tuples, probe time scaled to {ns}"
                          if m != ns else f"all {ns} probe tuples")) +
                         f" (oracle port of HashJoinOp, modulo {nr} buckets, 4 tuples/bucket, rows into 1 MiB pages)",
               "detail": info}
    line = None
    if rank == 0:
        kern = ("k_probe16_deep (materialise)" if mat else "k_probe16_direct (count + sum)") \
            if sp["key_domain"] == "dense" else "hashed-table probe"
        line = {"metric": join_metric(sp), "value": value, "unit": "tuples/s", "n_gpus": ws,
                "steps": steps, "warmup": warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
                "data": "synthetic (seeded generator, resident in HBM)",
                "config": join_config(sp, ws),
                "parity": parity,
                "e2e": {"value": ws * (nr + ns) / (e2e / 1e3), "unit": "tuples/s",
                        "h2d_bytes_per_step": (nr + ns) * TUPLE,
                        "d2h_bytes_per_step": (int(hres.n_out) * TUPLE) if mat else 16,
                        "ms_per_step": e2e},
                "roofline": {"bound": "hbm", "kernel": kern, "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak,
                             "traffic": PROBE_DRAM_BYTES_PER_TUPLE * ns
                             if (mat and sp["key_domain"] == "dense" and sp["dist"] == "uniform" and nr == 1 << 24)
                             else None,
                             "peak_source": peak_kind, "probe_ms": probe,
                             "algorithmic_bytes_per_launch": alg_probe,
                             "step_frac": alg_step / (ms / 1e3) / 1e9 / peak,
                             "step_algorithmic_bytes": alg_step},
                "gpu_launches": int(launches), "clocks": clk}
        if cpu:
            line["cpu_baseline"] = cpu
    for h in (hR, hS, hO):
        L.pg_host_free(ctx.h, h)
    ctx.close()
    return line


# ---------------------------------------------------------------------------
# Other operators of the path (bench.py --op ...): one JSON line each, same
# keys as the headline. Sizes are the configurations' full sizes.
# ---------------------------------------------------------------------------
OPS = {
    "partition": dict(n=1 << 28, metric="partition tuples/s (256M int64 tuples, 256-way radix, stable)",
                      workload="radix partition of 256M 16-byte tuples on the low 8 key bits (parammodulo)"),
    "groupby": dict(n=1 << 28, metric="group-by rows/s (256M rows, 1M groups, exact FP64 sum)",
                    workload="aggregate_sum over (long key U[0,1M), dec value U[0,1e4)), 256M rows"),
    "sort": dict(n=1 << 26, metric="page sort tuples/s (64M int64-keyed 16-byte tuples)",
                 workload="page sort of 64M (long key U[0,16M), long payload) tuples"),
    "mpsm": dict(n=1 << 26, metric="MPSM join tuples/s (64M x 64M, keys U[0,16M), fused count+sum)",
                 workload="sort-merge join of two 64M-tuple relations, keys U[0,16M) (~4 duplicates per side)"),
    "mpsmmat": dict(n=1 << 26, metric="MPSM join tuples/s (64M x 64M, keys U[0,16M), output rows materialised)",
                    workload="sort-merge join of two 64M-tuple relations, keys U[0,16M) (~4 duplicates per side), "
                             "every (P$1,B$1) pair written (~268M rows): page sort, then run matching and the "
                             "per-key cartesian write"),
    "sortwide": dict(n=1 << 26, metric="page sort tuples/s (64M int64-keyed 16-byte tuples, keys over 2^40)",
                     workload="page sort of 64M (long key U[0,2^40), long payload) tuples: LSD radix over the 40 "
                              "bits of key - min, five 8-bit passes"),
    "sortbitonic": dict(n=1 << 26, metric="page sort tuples/s (64M int64-keyed 16-byte tuples, keys over 2^40, "
                                          "bitonic)",
                        workload="page sort of 64M (long key U[0,2^40), long payload) tuples as 4096-tuple bitonic "
                                 "tiles in shared memory then merge-path merges (sort path 2)"),
    "groupjoin": dict(n=1 << 28, metric="join + group-by tuples/s (16M build x 256M probe, 1% groups, one pass)",
                      workload="hash join of 16M unique keys (group column = payload mod 167,772) with 256M FK "
                               "probes carrying dec values U[0,1e4), then aggregate_sum per group, one pass"),
}
SORT_OPS = ("sort", "sortwide", "sortbitonic")
GJ_BUILD = 1 << 24
GJ_GROUPS = GJ_BUILD // 100


def _pinned_array(ctx, L, n, cols=2):
    p = ctypes.c_void_p()
    ctx._check(L.pg_host_alloc(ctx.h, n * 8 * cols, ctypes.byref(p)))
    return p.value, np.ctypeslib.as_array((ctypes.c_int64 * (n * cols)).from_address(p.value)).reshape(n, cols)


def _op_inputs(op, n, threads):
    from pythia_gb300 import datagen as dg
    if op == "partition":
        return [dg.uniform_keys(n, 1 << 40, dg.seed_for(111), threads=threads)]
    if op == "groupby":
        return [dg.groupby_rows(n, 1 << 20, 1e4, dg.seed_for(112), threads=threads)]
    if op == "sort":
        return [dg.uniform_keys(n, 1 << 24, dg.seed_for(113), threads=threads)]
    if op in ("sortwide", "sortbitonic"):
        return [dg.uniform_keys(n, 1 << 40, dg.seed_for(118), threads=threads)]
    if op == "groupjoin":
        nb = min(GJ_BUILD, max(n // 16, 1024))
        R = dg.build_relation(nb, dg.seed_for(116), threads=threads)
        R[:, 1] = (dg.raw_words(dg.seed_for(116), 3, nb) % np.uint64(max(nb // 100, 1))).astype(np.int64)
        S = dg.probe_uniform(n, R, dg.seed_for(117), threads=threads)
        S[:, 1] = ((dg.raw_words(dg.seed_for(117), 4, n) >> np.uint64(11)).astype(np.float64)
                   * (1e4 / 2.0 ** 53)).view(np.int64)
        return [R, S]
    return [dg.uniform_keys(n, 1 << 24, dg.seed_for(114), threads=threads),
            dg.uniform_keys(n, 1 << 24, dg.seed_for(115), threads=threads)]


def _op_parity(op, ins, out, extra):
    """Size-independent checks at full size (integer ones exact)."""
    if op == "partition":
        keys = ins[0][:, 0]
        hist = np.bincount((keys & 255).astype(np.int64), minlength=256).astype(np.uint64)
        offs = extra
        ok = np.array_equal(np.diff(offs), hist)
        o = out.reshape(-1, 2)
        for b in (0, 17, 255):
            part = o[int(offs[b]):int(offs[b + 1]), 0]
            ok &= bool(np.all((part & 255) == b))
        ok &= int(o.astype(np.uint64).sum(dtype=np.uint64)) == int(ins[0].astype(np.uint64).sum(dtype=np.uint64))
        return {"offsets_equal_histogram": bool(ok)}
    if op == "groupby":
        rows = ins[0]
        from oracle import oracle as orc
        g = out.view(np.int64).reshape(-1, 2)
        ngroups_ok = g.shape[0] == int((np.bincount(rows[:, 0], minlength=1 << 20) > 0).sum())
        total = orc.fsum(rows[:, 1].view(np.float64))
        got_total = orc.fsum(g[:, 1].view(np.float64))
        rng = np.random.default_rng(7)
        pick = rng.choice(1 << 20, 16, replace=False)
        sel = np.isin(rows[:, 0], pick)
        sub = rows[sel]
        d = {int(k): float(v) for k, v in zip(g[:, 0], g[:, 1].view(np.float64))}
        worst = 0.0
        for k in pick:
            ex = orc.fsum(sub[sub[:, 0] == k, 1].view(np.float64))
            worst = max(worst, abs(d[int(k)] - ex) / abs(ex))
        return {"groups_ok": bool(ngroups_ok), "total_rel_err": abs(got_total - total) / total,
                "sampled_group_max_rel_err": worst, "tolerance": 1e-12,
                "ok": bool(ngroups_ok and worst <= 1e-12)}
    if op in SORT_OPS:
        o = out.reshape(-1, 2)
        ok = bool(np.all(np.diff(o[:, 0]) >= 0))
        ok &= int(o.astype(np.uint64).sum(dtype=np.uint64)) == int(ins[0].astype(np.uint64).sum(dtype=np.uint64))
        return {"sorted_and_same_multiset_checksum": ok}
    if op == "groupjoin":
        from oracle import oracle as orc
        R, S = ins
        g = out.view(np.int64).reshape(-1, 2)
        gk_by_key = np.zeros(int(R[:, 0].max()) + 1, dtype=np.int64)
        gk_by_key[R[:, 0]] = R[:, 1]
        gk = gk_by_key[S[:, 0]]
        ngroups_ok = g.shape[0] == int(np.unique(gk).shape[0])
        total = orc.fsum(S[:, 1].view(np.float64))
        got_total = orc.fsum(g[:, 1].view(np.float64))
        pick = np.random.default_rng(9).choice(np.unique(gk), 16, replace=False)
        sel = np.isin(gk, pick)
        sk, sv = gk[sel], S[sel, 1].view(np.float64)
        d = {int(k): float(v) for k, v in zip(g[:, 0], g[:, 1].view(np.float64))}
        worst = 0.0
        for k in pick:
            ex = orc.fsum(sv[sk == k])
            worst = max(worst, abs(d[int(k)] - ex) / abs(ex))
        return {"groups_ok": bool(ngroups_ok), "total_rel_err": abs(got_total - total) / total,
                "sampled_group_max_rel_err": worst, "tolerance": 1e-12,
                "ok": bool(ngroups_ok and worst <= 1e-12)}
    if op == "mpsmmat":
        got, want = extra
        return {"check": "whole-row digest of the timed step's output rows vs the oracle join's",
                "expected": want, "got": got, "ok": got == want}
    R, S = ins
    cr = np.bincount(R[:, 0], minlength=1 << 24).astype(np.int64)
    cs = np.bincount(S[:, 0], minlength=1 << 24).astype(np.int64)
    pr = np.bincount(R[:, 0], weights=R[:, 1].astype(np.float64), minlength=1 << 24).astype(np.int64)
    count = int((cr * cs).sum())
    sum_build = int((pr * cs).astype(np.uint64).sum(dtype=np.uint64).astype(np.int64))
    return {"count_ok": extra[0] == count, "build_payload_sum_ok": extra[1] == sum_build,
            "count": count}


def run_op(args, ws, rank, local, op):
    import torch
    from pythia_gb300 import gpu
    torch.cuda.set_device(local)
    spec = OPS[op]
    n = spec["n"] >> args.scale_down
    threads = host_threads()
    ctx = make_ctx(args, local)
    if op == "sortbitonic":
        ctx.tune(sort_path=2)
    L = gpu.lib()
    ins = _op_inputs(op, n, threads)
    d_in = [ctx.upload(a) for a in ins]
    stream = torch.cuda.ExternalStream(ctx.stream)
    c, nc = gpu.cols((("P", 8, 8), ("B", 8, 8)))
    nb = ins[0].shape[0]
    rel = [gpu.Rel(d.ptr, a.shape[0], 16, 0, 8) for d, a in zip(d_in, ins)]
    n_pairs = 0
    if op == "mpsmmat":
        # Output room from a counting pass (not timed).
        r0 = gpu.JoinResult()
        ctx._check(L.pg_mpsm_join(ctx.h, ctx.stream, ctypes.byref(rel[0]), ctypes.byref(rel[1]), c, nc,
                                  None, 0, gpu.JOIN_COUNT, -1, ctypes.byref(r0)))
        n_pairs = int(r0.n_out)
    out_bytes = {"partition": n * 16, "groupby": (1 << 20) * 16 + 16, "sort": n * 16, "sortwide": n * 16, "sortbitonic": n * 16,
                 "mpsm": 16, "mpsmmat": max(n_pairs, 1) * 16, "groupjoin": (nb // 100 + 1) * 16}[op]
    d_out = ctx.alloc(out_bytes)
    offs = ctx.alloc(8 * 257)
    ng = ctypes.c_uint64()
    res = gpu.JoinResult()
    gcols, gnc = gpu.cols((("B", 8, 8), ("P", 8, 8)))

    def step():
        if op == "partition":
            cfg = gpu.hashcfg("parammodulo", 256)
            ctx._check(L.pg_partition(ctx.h, ctx.stream, ctypes.byref(rel[0]), ctypes.byref(cfg), d_out.ptr, offs.ptr))
        elif op == "groupby":
            ctx._check(L.pg_groupby(ctx.h, ctx.stream, ctypes.byref(rel[0]), 8, 2, 0, 1 << 20, d_out.ptr,
                                    1 << 20, ctypes.byref(ng)))
        elif op in SORT_OPS:
            ctx._check(L.pg_sort_pages(ctx.h, ctx.stream, ctypes.byref(rel[0]), d_out.ptr))
        elif op == "mpsmmat":
            ctx._check(L.pg_mpsm_join(ctx.h, ctx.stream, ctypes.byref(rel[0]), ctypes.byref(rel[1]), c, nc,
                                      d_out.ptr, n_pairs, gpu.JOIN_MATERIALIZE, -1, ctypes.byref(res)))
        elif op == "groupjoin":
            ht = ctypes.c_void_p()
            ctx._check(L.pg_hashjoin_build(ctx.h, ctx.stream, ctypes.byref(rel[0]), gcols, gnc, ctypes.byref(ht)))
            try:
                ctx._check(L.pg_hashjoin_groupby(ctx.h, ctx.stream, ht.value, ctypes.byref(rel[1]), 8, 2, 0,
                                                 d_out.ptr, nb // 100 + 1, ctypes.byref(ng)))
            finally:
                L.pg_hashtable_free(ctx.h, ht.value)
        else:
            ctx._check(L.pg_mpsm_join(ctx.h, ctx.stream, ctypes.byref(rel[0]), ctypes.byref(rel[1]), c, nc,
                                      None, 0, gpu.JOIN_COUNT | gpu.JOIN_SUM, 1, ctypes.byref(res)))

    for _ in range(args.warmup):
        step()
    ctx.sync()
    k0 = gpu.kernel_launches()
    clocks = Clocks(local)
    barrier(ws)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    launches = gpu.kernel_launches() - k0
    ms = max_over_ranks(ws, e0.elapsed_time(e1) / args.steps)
    units = 2 * n if op in ("mpsm", "mpsmmat") else (n + nb if op == "groupjoin" else n)
    value = ws * units / (ms / 1e3)
    alg = {"partition": 32 * n, "groupby": 16 * n + 16 * (1 << 20), "sort": 32 * n, "sortwide": 32 * n, "sortbitonic": 32 * n,
           "mpsm": 16 * 2 * n, "mpsmmat": 16 * 2 * n + 16 * n_pairs,
           "groupjoin": 16 * (n + nb) + 16 * (nb // 100)}[op]
    peak, peak_kind = measured_peak()
    achieved = alg / (ms / 1e3) / 1e9
    # Parity at full size.
    if op == "partition":
        out = ctx.download(d_out, n * 16).view(np.int64)
        parity = _op_parity(op, ins, out, ctx.download(offs, 8 * 257, np.uint64))
    elif op == "groupby":
        parity = _op_parity(op, ins, ctx.download(d_out, ng.value * 16), None)
    elif op in SORT_OPS:
        parity = _op_parity(op, ins, ctx.download(d_out, n * 16).view(np.int64), None)
    elif op == "mpsmmat":
        from oracle import oracle as orc
        got = orc.rows_digest(ctx.download(d_out, int(res.n_out) * 16).view(np.int64).reshape(-1, 2),
                              threads=threads)
        want = orc.hashjoin_digest(ins[0], ins[1], proj=PROJ, hash=orc.hashcfg("modulo", 1 << 24),
                                   threads=threads)
        parity = _op_parity(op, ins, None, (got, want))
    elif op == "groupjoin":
        parity = _op_parity(op, ins, ctx.download(d_out, ng.value * 16), None)
    else:
        parity = _op_parity(op, ins, None, (res.n_out, res.sum))
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_op_sample(op, ins, threads)
    if rank == 0:
        line = {"metric": spec["metric"], "value": value, "unit": "tuples/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64" if op in ("groupby", "groupjoin") else "int64",
                "data": "synthetic (seeded generator, resident in HBM)",
                "config": {"workload": spec["workload"], "op": op, "tuples": n,
                           "l2": "inputs larger than L2; no flush"} | ({"output_rows": n_pairs} if n_pairs else {}),
                "parity": parity,
                "roofline": {"bound": "hbm", "kernel": f"pg_{op} (whole operator)", "achieved": achieved,
                             "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                             "peak_source": peak_kind, "algorithmic_bytes": alg},
                "gpu_launches": int(launches), "clocks": clk}
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    ctx.close()


def cpu_op_sample(op, ins, threads):
    """Times the oracle port of the reference operator on a bounded sample and
    scales linearly in tuples (n log n for the sort) to the full size."""
    from oracle import oracle as orc
    n = ins[0].shape[0]
    m = min(n, 1 << 24)
    a = np.ascontiguousarray(ins[0][:m])
    t0 = time.perf_counter()
    if op == "partition":
        orc.partition(a, orc.hashcfg("parammodulo", 256), threads=threads)
        scale, kind = n / m, "linear"
    elif op == "groupby":
        orc.groupby(a, val=(8, "dec"), agg="sum", hash=orc.hashcfg("modulo", 1 << 20), threads=threads)
        scale, kind = n / m, "linear"
    elif op in SORT_OPS:
        m = min(n, 1 << 22)
        a = np.ascontiguousarray(ins[0][:m])
        t0 = time.perf_counter()
        orc.sort(a)
        scale, kind = (n * np.log2(n)) / (m * np.log2(m)), "n log n"
    elif op == "groupjoin":
        R = ins[0]
        n = ins[1].shape[0]
        m = min(n, 1 << 22)
        S = np.ascontiguousarray(ins[1][:m])
        cfg = orc.hashcfg("modulo", R.shape[0])
        t0 = time.perf_counter()
        orc.hashjoin(R, S[:1], hash=cfg, threads=threads, materialise=False)
        t_build = time.perf_counter() - t0
        t0 = time.perf_counter()
        joined, _, _ = orc.hashjoin(R, S, proj=(("B", 8, 8), ("P", 8, 8)), hash=cfg, threads=threads, out_cap=m)
        orc.groupby(joined.view(np.int64).reshape(-1, 2), val=(8, "dec"), agg="sum",
                    hash=orc.hashcfg("modulo", 1 << 18), threads=threads)
        t_rest = max(time.perf_counter() - t0 - t_build, 1e-9)
        t = t_build + t_rest * n / m
        units = n + R.shape[0]
        return {"value": units / t, "unit": "tuples/s", "cores": threads, "kind": "port",
                "sample": f"full {R.shape[0]}-tuple build + {m} probe tuples joined and grouped (oracle port), "
                          f"probe and group-by time scaled linearly to {n}"}
    else:
        m = min(n, 1 << 22)
        R = np.ascontiguousarray(ins[0][:m]); S = np.ascontiguousarray(ins[1][:m])
        R[:, 0] >>= 4; S[:, 0] >>= 4      # same ~4 duplicates per key at 1/16 of the size
        t0 = time.perf_counter()
        orc.mergejoin(R, S, materialise=False, sum_col=1, threads=threads)
        scale, kind = n / m, "linear"
    t = (time.perf_counter() - t0) * scale
    units = 2 * n if op in ("mpsm", "mpsmmat") else (n + ins[0].shape[0] if op == "groupjoin" else n)
    one = op in SORT_OPS
    return {"value": units / t, "unit": "tuples/s", "cores": 1 if one else threads,
            "kind": "port", "sample": f"{m} tuples (oracle port{', one thread' if one else ''}), "
                                      f"time scaled {kind} to {n}"}


# ---------------------------------------------------------------------------
# Batched uneven joins (bench.py --op batch): 10,000 join + aggregate_count
# instances, |R_i| log-uniform in [1K, 4M] unique keys, |S_i| = 8|R_i| FK.
# ---------------------------------------------------------------------------
BATCH_N = 10_000
BATCH_POOL = 1 << 22


def batch_sizes(n):
    from pythia_gb300 import datagen as dg
    u = dg.raw_words(dg.seed_for(120), 0, n).astype(np.float64) * (1.0 / 2.0 ** 64)
    lo, hi = np.log(1000.0), np.log(float(BATCH_POOL))
    return np.clip(np.rint(np.exp(lo + u * (hi - lo))).astype(np.int64), 1000, BATCH_POOL)


def fk_host(R, seed, n):
    """Host replica of pg_generate_fk (k_generate_fk), for the CPU sample."""
    M = (1 << 64) - 1
    j = np.arange(1, n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + j * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
        nR = np.uint64(R.shape[0])
        # multiply-high of z * nR (nR < 2^32): split z into 32-bit halves
        zh, zl = z >> np.uint64(32), z & np.uint64(0xFFFFFFFF)
        idx = (zh * nR + ((zl * nR) >> np.uint64(32))) >> np.uint64(32)
        pay = ((z * np.uint64(0xD1B54A32D192ED03)) >> np.uint64(33)).astype(np.int64)
    del M
    out = np.empty((n, 2), dtype=np.int64)
    out[:, 0] = R[idx.astype(np.int64), 0]
    out[:, 1] = pay
    return out


def run_batch(args, ws, rank, local):
    import torch
    from pythia_gb300 import autotune, datagen as dg, gpu
    torch.cuda.set_device(local)
    threads = host_threads()
    ctx = make_ctx(args, local)
    L = gpu.lib()
    n_inst = BATCH_N >> args.scale_down
    sizes = batch_sizes(n_inst)
    pool = dg.build_relation(BATCH_POOL, dg.seed_for(121), threads=threads)
    d_pool = ctx.upload(pool)
    wave_cap = (1 << 30) >> args.scale_down          # probe tuples per wave
    waves, cur, tot = [], [], 0
    for i, r in enumerate(sizes):
        if cur and tot + 8 * r > wave_cap:
            waves.append(cur); cur, tot = [], 0
        cur.append(i); tot += 8 * r
    if cur:
        waves.append(cur)
    d_S = ctx.alloc(16 * max(sum(8 * int(sizes[i]) for i in w) for w in waves))
    gpu_name = torch.cuda.get_device_name(local)

    def gen_wave(w):
        items, off = [], 0
        for i in w:
            r = int(sizes[i]); s = 8 * r
            Sp = d_S.ptr + 16 * off
            ctx._check(L.pg_generate_fk(ctx.h, ctx.stream, d_pool.ptr, r, dg.seed_for(1000 + i), Sp, s))
            items.append((i, (d_pool.ptr, r, Sp, s)))
            off += s
        ctx.sync()
        return items

    # Autotune per size class on the first wave (cached per GPU).
    cached = autotune.load(gpu_name) or {}
    shapes = cached.get("batch")
    sweep = None
    items0 = gen_wave(waves[0])
    if shapes is None or args.retune:
        by_cls = {}
        for i, it in items0:
            by_cls.setdefault(autotune.size_class(int(sizes[i])), []).append(it)
        shapes, sweep = autotune.tune_batch(ctx, by_cls, repeats=2)
        cached["batch"] = shapes
        autotune.save(gpu_name, cached)
    default = autotune.BATCH_SHAPES[0]

    counts = np.zeros(n_inst, dtype=np.uint64)
    loop_counts = np.zeros(n_inst, dtype=np.uint64)
    t_batch = 0.0
    t_loop = 0.0
    launches = 0
    c, nc = gpu.cols((("P", 8, 8), ("B", 8, 8)))
    for wi, w in enumerate(waves):
        items = items0 if wi == 0 else gen_wave(w)
        by_cls = {}
        for i, it in items:
            by_cls.setdefault(autotune.size_class(int(sizes[i])), []).append((i, it))
        batches = []
        for cls, lst in by_cls.items():
            b = autotune.prepare(ctx, [it for _, it in lst], shapes.get(cls, default))
            batches.append((b, [i for i, _ in lst]))
        for b, _ in batches:
            autotune.run(ctx, b)           # warm-up replay
        ctx.sync()
        k0 = gpu.kernel_launches()
        best = float("inf")
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            for b, _ in batches:
                autotune.run(ctx, b)
            best = min(best, time.perf_counter() - t0)
        launches += (gpu.kernel_launches() - k0) // max(1, args.steps)
        t_batch += best
        for b, idx in batches:
            cc = np.zeros(len(idx), dtype=np.uint64)
            autotune.run(ctx, b, cc)
            counts[idx] = cc
            autotune.free(ctx, b)
        # The same instances through the plain entry points, one by one.
        t0 = time.perf_counter()
        for i, (Rp, r, Sp, s) in items:
            rR = gpu.Rel(Rp, r, 16, 0, 8)
            rS = gpu.Rel(Sp, s, 16, 0, 8)
            ht = ctypes.c_void_p()
            ctx._check(L.pg_hashjoin_build(ctx.h, ctx.stream, ctypes.byref(rR), c, nc, ctypes.byref(ht)))
            res = gpu.JoinResult()
            ctx._check(L.pg_hashjoin_probe(ctx.h, ctx.stream, ht.value, ctypes.byref(rS), c, nc, None, 0,
                                           gpu.JOIN_COUNT, -1, ctypes.byref(res)))
            L.pg_hashtable_free(ctx.h, ht.value)
            loop_counts[i] = res.n_out
        t_loop += time.perf_counter() - t0
    want = (8 * sizes).astype(np.uint64)
    parity = {"counts_equal_probe_sizes": bool(np.array_equal(counts, want)),
              "batched_equals_loop": bool(np.array_equal(counts, loop_counts))}
    alg = int(16 * (sizes.sum() + 8 * sizes.sum()))
    value = n_inst / t_batch
    peak, peak_kind = measured_peak()
    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as orc
        pick = [i for i in range(n_inst) if sizes[i] <= 65536][:40]
        t0 = time.perf_counter()
        tuples = 0
        for i in pick:
            r = int(sizes[i])
            S = fk_host(pool[:r], dg.seed_for(1000 + i), 8 * r)
            _, n_out, _ = orc.hashjoin(pool[:r], S, hash=orc.hashcfg("modulo", r), tuplesperbucket=4,
                                       threads=threads, materialise=False)
            assert n_out == 8 * r
            tuples += 9 * r
        t = time.perf_counter() - t0
        total_tuples = int(9 * sizes.sum())
        cpu = {"value": n_inst / (t * total_tuples / tuples), "unit": "instances/s", "cores": threads,
               "kind": "port", "sample": f"{len(pick)} instances with |R| <= 64K (oracle port, join + count), "
                                        f"time scaled by tuples to all {n_inst}"}
    if rank == 0:
        line = {"metric": "batched join+count instances/s (10,000 uneven PK-FK instances)", "value": value,
                "unit": "instances/s", "n_gpus": ws, "steps": args.steps, "warmup": 1,
                "ms_per_step": t_batch * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "int64", "data": "synthetic (build pool + device FK generator)",
                "config": {"workload": f"{n_inst} instances, |R| log-uniform [1K, 4M], |S| = 8|R|, "
                                       f"join + aggregate_count", "waves": len(waves),
                           "total_build": int(sizes.sum()), "total_probe": int(8 * sizes.sum()),
                           "shapes": shapes},
                "loop_baseline": {"value": n_inst / t_loop, "unit": "instances/s", "ms": t_loop * 1e3,
                                  "what": "pg_hashjoin_build + pg_hashjoin_probe(COUNT) per instance"},
                "speedup_vs_loop": t_loop / t_batch,
                "parity": parity,
                "roofline": {"bound": "hbm", "kernel": "k_batch_build + k_batch_probe_count",
                             "achieved": alg / t_batch / 1e9, "peak": peak, "unit": "GB/s",
                             "frac": alg / t_batch / 1e9 / peak, "traffic": None, "peak_source": peak_kind},
                "gpu_launches": int(launches)}
        if sweep:
            line["autotune"] = sweep
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    ctx.close()


# ---------------------------------------------------------------------------
# Serving (bench.py --op serve): join + group-by plans on resident tables,
# continuous batching vs one at a time.
# ---------------------------------------------------------------------------
def run_serve(args, ws, rank, local):
    import torch
    from pythia_gb300 import datagen as dg, gpu, serving
    torch.cuda.set_device(local)
    ctx = make_ctx(args, local)
    ntab = 24 >> min(args.scale_down, 3)
    u = dg.raw_words(dg.seed_for(130), 0, ntab).astype(np.float64) * (1.0 / 2.0 ** 64)
    lo, hi = np.log(10_000.0), np.log(float((64 << 20) >> args.scale_down))
    sizes = np.rint(np.exp(lo + u * (hi - lo))).astype(np.int64)
    t0 = time.perf_counter()
    cat = serving.Catalog(ctx, sizes, threads=host_threads())
    build_s = time.perf_counter() - t0
    nq = 200 >> min(args.scale_down, 2)
    rng_t = dg.raw_words(dg.seed_for(131), 0, nq) % np.uint64(ntab)
    rng_z = dg.raw_words(dg.seed_for(131), 1, nq) & np.uint64(1)

    def queries(arrivals):
        return [serving.Query(i, int(rng_t[i]), 0.8 if rng_z[i] else 0.0, float(arrivals[i])) for i in range(nq)]

    budget = 150 << 30
    one = serving.Server(ctx, cat, 1, budget)
    many = serving.Server(ctx, cat, args.slots, budget)
    short = serving.Server(ctx, cat, args.slots, budget, policy="short-first")
    for srv in (one, many, short):                    # warm-up
        srv.run(queries(np.zeros(nq))[: min(nq, 8)])
    sat_one = serving.summarize(one.run(queries(np.zeros(nq))))
    qs_many = many.run(queries(np.zeros(nq)))
    sat_many = serving.summarize(qs_many)
    sat_short = serving.summarize(short.run(queries(np.zeros(nq))))
    # Same results alone (one slot) and in the mix.
    qs_one = one.run(queries(np.zeros(nq)))
    same = True
    worst = 0.0
    for a, b in zip(qs_one, qs_many):
        ka, va = serving.canonical(a.result)
        kb, vb = serving.canonical(b.result)
        same &= bool(np.array_equal(ka, kb))
        if len(va):
            worst = max(worst, float(np.max(np.abs(va - vb) / np.maximum(np.abs(va), 1e-300))))
    sweep = []
    for frac in (0.5, 0.9, 2.0):
        lam = frac * sat_one["queries_per_s"]
        arr = serving.poisson_arrivals(nq, lam, dg.seed_for(132))
        sweep.append({"rate_qps": lam,
                      "one_at_a_time": serving.summarize(one.run(queries(arr))),
                      "continuous_batching": serving.summarize(many.run(queries(arr))),
                      "continuous_batching_short_first": serving.summarize(short.run(queries(arr)))})
    one.close(); many.close(); short.close()
    # Warm start: the tables written as images, the catalog dropped, and a new
    # catalog loaded from the images (probe pools regenerated, not timed).
    import gc
    import shutil
    import tempfile
    img_dir = tempfile.mkdtemp(prefix="pg_tables_")
    try:
        cat.save(img_dir)
        build_tables_s = cat.table_seconds
        resident = cat.resident_bytes
        cat.close()
        del cat
        gc.collect()
        warm = serving.Catalog(ctx, sizes, threads=host_threads(), images=img_dir)
        warm_same = True
        for a in qs_one[: min(nq, 32)]:
            kw, vw = serving.canonical(serving.execute(ctx, ctx.stream, warm, serving.Query(a.qid, a.table, a.zipf)))
            ka, va = serving.canonical(a.result)
            warm_same &= bool(np.array_equal(ka, kw)) and bool(np.all(np.abs(va - vw) <= 1e-12 * np.abs(va)))
        load_tables_s = warm.table_seconds
        warm.close()
    finally:
        shutil.rmtree(img_dir, ignore_errors=True)
    if rank == 0:
        line = {"metric": "served join+group-by queries/s (continuous batching) and p50/p99 latency",
                "value": sat_many["queries_per_s"], "unit": "queries/s", "n_gpus": ws, "steps": 1, "warmup": 1,
                "ms_per_step": sat_many["makespan_s"] * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic resident catalog (device generator)",
                "config": {"workload": f"{nq} plans: hash join on a resident table (|R| log-uniform "
                                       f"[10K, 64M], {ntab} tables), |S| = 10|R| uniform or Zipf 0.8, then "
                                       f"aggregate_sum over |R|/100 groups (one-pass plan: probe folds into "
                                       f"the group table)", "slots": args.slots,
                           "hbm_budget_bytes": budget, "resident_bytes": resident,
                           "catalog_build_s": build_s},
                "warm_start": {"tables_built_s": build_tables_s, "tables_loaded_from_images_s": load_tables_s,
                               "same_results_after_load": warm_same},
                "saturation": {"one_at_a_time": sat_one, "continuous_batching": sat_many,
                               "continuous_batching_short_first": sat_short,
                               "throughput_ratio": sat_many["queries_per_s"] / sat_one["queries_per_s"]},
                "poisson_sweep": sweep,
                "parity": {"same_results_alone_and_mixed": same, "max_rel_diff": worst, "tolerance": 1e-12}}
        print(json.dumps(line), flush=True)
    ctx.close()


# ---------------------------------------------------------------------------
# Join-table images (bench.py --op tableimage): the 16M-key build side of the
# headline join written to pinned host memory and loaded back, against
# rebuilding the table from its host relation (the warm start an image
# replaces) and against a plain pinned copy of the same bytes (the link).
# ---------------------------------------------------------------------------
def run_tableimage(args, ws, rank, local):
    import torch
    from pythia_gb300 import datagen as dg
    from pythia_gb300 import gpu
    torch.cuda.set_device(local)
    nb = GJ_BUILD >> args.scale_down
    threads = host_threads()
    ctx = make_ctx(args, local)
    L = gpu.lib()
    R = dg.build_relation(nb, dg.seed_for(118), threads=threads)
    rp, Rh = _pinned_array(ctx, L, nb)
    Rh[:] = R
    dR = ctx.upload(R)
    dR2 = ctx.alloc(R.nbytes)
    c, nc = gpu.cols((("P", 8, 8), ("B", 8, 8)))
    rel = gpu.Rel(dR.ptr, nb, 16, 0, 8)
    rel2 = gpu.Rel(dR2.ptr, nb, 16, 0, 8)
    ht = ctypes.c_void_p()
    ctx._check(L.pg_hashjoin_build(ctx.h, ctx.stream, ctypes.byref(rel), c, nc, ctypes.byref(ht)))
    size = ctypes.c_uint64()
    ctx._check(L.pg_hashtable_image_size(ctx.h, ht.value, ctypes.byref(size)))
    nbytes = size.value
    ip = ctypes.c_void_p()
    ctx._check(L.pg_host_alloc(ctx.h, nbytes, ctypes.byref(ip)))
    dcopy = ctx.alloc(nbytes)
    stream = torch.cuda.ExternalStream(ctx.stream)
    got = ctypes.c_uint64()

    def save():
        ctx._check(L.pg_hashtable_serialize(ctx.h, ctx.stream, ht.value, ip.value, nbytes, ctypes.byref(got)))

    def load():
        t = ctypes.c_void_p()
        ctx._check(L.pg_hashtable_deserialize(ctx.h, ctx.stream, ip.value, nbytes, ctypes.byref(t)))
        L.pg_hashtable_free(ctx.h, t.value)

    def rebuild():
        t = ctypes.c_void_p()
        ctx._check(L.pg_h2d(ctx.h, ctx.stream, dR2.ptr, rp, R.nbytes))
        ctx._check(L.pg_hashjoin_build(ctx.h, ctx.stream, ctypes.byref(rel2), c, nc, ctypes.byref(t)))
        L.pg_hashtable_free(ctx.h, t.value)

    def copy():
        ctx._check(L.pg_h2d(ctx.h, ctx.stream, dcopy.ptr, ip.value, nbytes))

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return max_over_ranks(ws, e0.elapsed_time(e1) / args.steps)

    save()
    k0 = gpu.kernel_launches()
    clocks = Clocks(local)
    barrier(ws)
    clocks.start()
    ms_load = timed(load)
    clk = clocks.stop()
    launches = (gpu.kernel_launches() - k0) * args.steps // (args.steps + args.warmup)
    ms_save = timed(save)
    ms_rebuild = timed(rebuild)
    ms_copy = timed(copy)
    # Parity: the loaded table probes a 4M-tuple FK sample exactly like the
    # built one, and its own image is the same bytes.
    S = dg.probe_uniform(1 << 22, R, dg.seed_for(119), threads=threads)
    S[::97, 0] += 2 * nb
    dS = ctx.upload(S)
    relS = gpu.Rel(dS.ptr, S.shape[0], 16, 0, 8)
    t2 = ctypes.c_void_p()
    ctx._check(L.pg_hashtable_deserialize(ctx.h, ctx.stream, ip.value, nbytes, ctypes.byref(t2)))
    r1, r2 = gpu.JoinResult(), gpu.JoinResult()
    fl = gpu.JOIN_COUNT | gpu.JOIN_SUM
    ctx._check(L.pg_hashjoin_probe(ctx.h, ctx.stream, ht.value, ctypes.byref(relS), c, nc, None, 0, fl, 1,
                                   ctypes.byref(r1)))
    ctx._check(L.pg_hashjoin_probe(ctx.h, ctx.stream, t2.value, ctypes.byref(relS), c, nc, None, 0, fl, 1,
                                   ctypes.byref(r2)))
    img1 = np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(ip.value)).copy()
    ctx._check(L.pg_hashtable_serialize(ctx.h, ctx.stream, t2.value, ip.value, nbytes, ctypes.byref(got)))
    img2 = np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(ip.value))
    hit = S[:, 0] <= nb
    parity = {"probe_count_equal": r1.n_out == r2.n_out == int(hit.sum()),
              "probe_sum_equal": r1.sum == r2.sum, "reserialized_image_identical": bool(np.array_equal(img1, img2))}
    L.pg_hashtable_free(ctx.h, t2.value)
    L.pg_hashtable_free(ctx.h, ht.value)
    link = nbytes / (ms_copy / 1e3) / 1e9
    achieved = nbytes / (ms_load / 1e3) / 1e9
    cpu = None
    if rank == 0 and not args.no_cpu:
        # The reference's deserialize copies the table partition out of its
        # mapped segment with memcpy (util/hashtable.cpp:180-201): the same
        # bytes copied host to host.
        src = np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(ip.value))
        dst = np.empty(nbytes, dtype=np.uint8)
        np.copyto(dst, src)
        t0 = time.perf_counter()
        reps = 5
        for _ in range(reps):
            np.copyto(dst, src)
        t = (time.perf_counter() - t0) / reps
        cpu = {"value": nbytes / t / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
               "sample": f"memcpy of the {nbytes}-byte image, host to host, as the reference's deserialize "
                         f"copies a mapped segment into the table (mean of {reps})"}
    if rank == 0:
        line = {"metric": "join-table image load GB/s (16M-key narrow dense table from pinned host memory)",
                "value": ws * achieved, "unit": "GB/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms_load, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "u32", "data": "synthetic (seeded generator; image in pinned host memory)",
                "config": {"workload": f"load (H2D + device checksum + allocation) of the {nbytes}-byte image of "
                                       f"a {nb}-key join table; rebuild = H2D of the {R.nbytes}-byte relation + "
                                       "build", "op": "tableimage", "build_tuples": nb, "image_bytes": nbytes,
                           "l2": "copies are link-bound; no flush"},
                "save_ms": ms_save, "save_gbs": nbytes / (ms_save / 1e3) / 1e9, "load_ms": ms_load,
                "rebuild_from_host_relation_ms": ms_rebuild, "load_speedup_vs_rebuild": ms_rebuild / ms_load,
                "parity": parity,
                "roofline": {"bound": "host link", "kernel": "pg_hashtable_deserialize (copy + k_image_sum)",
                             "achieved": achieved, "peak": link, "unit": "GB/s", "frac": achieved / link,
                             "traffic": None, "peak_source": "pinned H2D copy of the same bytes, same run"},
                "e2e": {"value": ws * achieved, "unit": "GB/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": 8},
                "gpu_launches": int(launches), "clocks": clk}
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    L.pg_host_free(ctx.h, ip.value)
    L.pg_host_free(ctx.h, rp)
    ctx.close()


# ---------------------------------------------------------------------------
# A q1-shaped plan through the operator layer (bench.py --op plan): the
# reference's join -> join -> aggregate shape (q1/query1.conf:115-166) as
# gpuhashjoin(orders, gpuhashjoin(parts, lines)) under gpuaggregate_sum,
# memscan leaves over host relations, 16 threads; timed with the device
# exchange between the GPU operators on and off (host pages in between).
# ---------------------------------------------------------------------------
PLAN_Q1 = """
buffsize = 1048576;
treeroot = { name = "sum"; input = { name = "joinO"; build = { name = "scanO"; };
             probe = { name = "joinP"; build = { name = "scanP"; }; probe = { name = "scanL"; }; }; }; };
scanO = { type = "memscan"; relation = "O"; schema = ("long", "long"); };
scanP = { type = "memscan"; relation = "P"; schema = ("long", "long"); };
scanL = { type = "memscan"; relation = "L"; schema = ("long", "long", "dec"); };
joinP = { type = "gpuhashjoin"; buildjattr = 0; probejattr = 1; projection = ("P$0", "P$2", "B$1");
          threadgroups = (%(all)s); hash = { fn = "modulo"; buckets = 1024; }; tuplesperbucket = 4; };
joinO = { type = "gpuhashjoin"; buildjattr = 0; probejattr = 0; projection = ("B$1", "P$1");
          threadgroups = (%(all)s); hash = { fn = "modulo"; buckets = 1024; }; tuplesperbucket = 4; };
sum = { type = "gpuaggregate_sum"; field = 0; sumfield = 1; global = true; threads = %(t)d; };
"""
PLAN_L, PLAN_O, PLAN_P, PLAN_GROUPS = 1 << 26, 1 << 24, 1 << 22, 1000


def _plan_inputs(nL, nO, nP, threads):
    from pythia_gb300 import datagen as dg
    O = dg.build_relation(nO, dg.seed_for(120), threads=threads)
    O[:, 1] = O[:, 0] % PLAN_GROUPS
    P = dg.build_relation(nP, dg.seed_for(121), threads=threads)
    lo = dg.probe_uniform(nL, O, dg.seed_for(122), threads=threads)
    lp = dg.probe_uniform(nL, P, dg.seed_for(123), threads=threads)
    L = np.empty((nL, 3), np.int64)
    L[:, 0] = lo[:, 0]
    L[:, 1] = lp[:, 0]
    L[:, 2] = ((lo[:, 1] & 0xFFFF).astype(np.float64) * 0.01).view(np.int64)
    return O, P, L


def run_plan(args, ws, rank, local):
    import torch
    from pythia_gb300 import plans
    torch.cuda.set_device(local)
    threads = min(16, host_threads())
    nL, nO, nP = PLAN_L >> args.scale_down, PLAN_O >> args.scale_down, PLAN_P >> args.scale_down
    O, P, L = _plan_inputs(nL, nO, nP, host_threads())
    plans.register("O", O); plans.register("P", P); plans.register("L", L)
    plan = PLAN_Q1 % {"all": "(" + ", ".join(str(t) for t in range(threads)) + ")", "t": threads}

    def timed(on):
        plans.set_device_exchange(on)
        for _ in range(args.warmup):
            plans.run(plan, threads=threads)
        plans.transfer_stats(reset=True)
        torch.cuda.synchronize()
        barrier(ws)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            rows, _ = plans.run(plan, threads=threads)
        torch.cuda.synchronize()
        ms = max_over_ranks(ws, (time.perf_counter() - t0) * 1e3 / args.steps)
        st = plans.transfer_stats(reset=True)
        return ms, rows, {k: v // args.steps for k, v in st.items()}

    from pythia_gb300 import gpu
    k0 = gpu.kernel_launches()
    clocks = Clocks(local)
    clocks.start()
    ms_on, rows_on, st_on = timed(True)
    clk = clocks.stop()
    launches = (gpu.kernel_launches() - k0) * args.steps // (args.steps + args.warmup)
    ms_off, rows_off, st_off = timed(False)
    # Leaves in registered memory (a loader reading into pinned memory): their
    # pages go to the device without the staging copy.
    plans.register("O", O, pin=True); plans.register("P", P, pin=True); plans.register("L", L, pin=True)
    ms_pin, rows_pin, st_pin = timed(True)
    plans.register("O", O); plans.register("P", P); plans.register("L", L)
    plans.set_device_exchange(True)
    # Parity at full size: every line's price lands in its order's group.
    from oracle import oracle as orc
    g_on = orc.canonical(rows_on).view(np.int64).reshape(-1, 2)
    g_off = orc.canonical(rows_off).view(np.int64).reshape(-1, 2)
    grp = L[:, 0] % PLAN_GROUPS
    price = L[:, 2].view(np.float64)
    pick = np.random.default_rng(5).choice(PLAN_GROUPS, 8, replace=False)
    worst = 0.0
    d = {int(k): float(v) for k, v in zip(g_on[:, 0], g_on[:, 1].view(np.float64))}
    for k in pick:
        ex = orc.fsum(price[grp == k])
        worst = max(worst, abs(d[int(k)] - ex) / abs(ex))
    parity = {"groups": int(g_on.shape[0]), "groups_ok": int(g_on.shape[0]) == PLAN_GROUPS,
              "same_groups_on_and_off": bool(np.array_equal(g_on[:, 0], g_off[:, 0])),
              "same_groups_pinned_leaves": bool(np.array_equal(
                  orc.canonical(rows_pin).view(np.int64).reshape(-1, 2)[:, 0], g_on[:, 0])),
              "sampled_group_max_rel_err": worst, "tolerance": 1e-12, "ok": worst <= 1e-12}
    cpu = None
    if rank == 0 and not args.no_cpu:
        m = min(nL, 1 << 22)
        t0 = time.perf_counter()
        jp, _, _ = orc.hashjoin(P, L[:m], proj=(("P", 0, 8), ("P", 16, 8), ("B", 8, 8)), pkey=(8, 8),
                                hash=orc.hashcfg("modulo", nP), threads=host_threads())
        jo, _, _ = orc.hashjoin(O, jp.view(np.int64).reshape(-1, 3), proj=(("B", 8, 8), ("P", 8, 8)),
                                hash=orc.hashcfg("modulo", nO), threads=host_threads())
        orc.groupby(jo.view(np.int64).reshape(-1, 2), val=(8, "dec"), hash=orc.hashcfg("modulo", 1 << 10),
                    threads=host_threads())
        t = (time.perf_counter() - t0) * nL / m
        cpu = {"value": nL / t, "unit": "lines/s", "cores": host_threads(), "kind": "port",
               "sample": f"{m} lines through the oracle port's join, join and group-by (full order and part "
                         f"builds), time scaled linearly to {nL}"}
    value = ws * nL / (ms_on / 1e3)
    if rank == 0:
        line = {"metric": "q1-shaped plan lines/s through the GPU operator layer (join -> join -> aggregate_sum)",
                "value": value, "unit": "lines/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms_on, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "int64/f64", "data": "synthetic (seeded generator, host relations read by memscan)",
                "config": {"workload": f"{nL} lines (long, long, dec) joined with {nP} parts and {nO} orders, "
                                       f"summed into {PLAN_GROUPS} groups; {threads} plan threads, one thread group",
                           "op": "plan", "timing": "wall clock per plan run, host relations in and host rows out",
                           "l2": "inputs larger than L2; no flush"},
                "exchange_off_ms": ms_off, "exchange_speedup": ms_off / ms_on,
                "pinned_leaves_ms": ms_pin, "pinned_leaves_lines_per_s": ws * nL / (ms_pin / 1e3),
                "transfer_bytes_per_run": {"exchange_on": st_on, "exchange_off": st_off,
                                           "exchange_on_pinned_leaves": st_pin},
                "parity": parity,
                "e2e": {"value": value, "unit": "lines/s", "h2d_bytes_per_step": st_on["h2d"],
                        "d2h_bytes_per_step": st_on["d2h"]},
                "gpu_launches": int(launches), "clocks": clk}
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Filter fused into the probe (bench.py --op filterjoin): the headline 16M x
# 256M join with a Filter on the probe side (payload < 2^30, half the probe
# tuples pass). Timed: the fused probe (pg_hashjoin_probe_where), the same
# work as filter then probe, and pg_filter / pg_project alone.
# ---------------------------------------------------------------------------
def run_filterjoin(args, ws, rank, local):
    import torch
    from pythia_gb300 import gpu
    torch.cuda.set_device(local)
    threads = host_threads()
    ctx = make_ctx(args, local)
    L = gpu.lib()
    hR, R = _pinned_array(ctx, L, NR)
    hS, S = _pinned_array(ctx, L, NS)
    make_join_inputs(join_spec(NR, NS), R, S, threads)
    dR, dS = ctx.alloc(NR * TUPLE), ctx.alloc(NS * TUPLE)
    dT, dO = ctx.alloc(NS * TUPLE), ctx.alloc(NS * TUPLE)
    ctx._check(L.pg_h2d(ctx.h, ctx.stream, dR.ptr, hR, NR * TUPLE))
    ctx._check(L.pg_h2d(ctx.h, ctx.stream, dS.ptr, hS, NS * TUPLE))
    ctx.sync()
    rR = gpu.Rel(dR.ptr, NR, TUPLE, 0, 8)
    rS = gpu.Rel(dS.ptr, NS, TUPLE, 0, 8)
    proj, nproj = gpu.cols((("P", 8, 8), ("B", 8, 8)))
    where, nwhere = gpu.preds([("long", "<", 8, 1 << 30)])
    pcols = (gpu.Col * 2)(gpu.Col(0, 8, 8), gpu.Col(0, 0, 8))
    ht = ctypes.c_void_p()
    ctx._check(L.pg_hashjoin_build(ctx.h, ctx.stream, ctypes.byref(rR), proj, nproj, ctypes.byref(ht)))
    stream = torch.cuda.ExternalStream(ctx.stream)
    res = gpu.JoinResult()
    m = ctypes.c_uint64()
    MAT = gpu.JOIN_MATERIALIZE

    def fused():
        ctx._check(L.pg_hashjoin_probe_where(ctx.h, ctx.stream, ht.value, ctypes.byref(rS), where, nwhere, proj, nproj,
                                             dO.ptr, NS, MAT, -1, ctypes.byref(res)))

    def unfused():
        ctx._check(L.pg_filter(ctx.h, ctx.stream, ctypes.byref(rS), where, nwhere, dT.ptr, ctypes.byref(m)))
        rT = gpu.Rel(dT.ptr, m.value, TUPLE, 0, 8)
        ctx._check(L.pg_hashjoin_probe(ctx.h, ctx.stream, ht.value, ctypes.byref(rT), proj, nproj,
                                       dO.ptr, NS, MAT, -1, ctypes.byref(res)))

    def filter_only():
        ctx._check(L.pg_filter(ctx.h, ctx.stream, ctypes.byref(rS), where, nwhere, dT.ptr, ctypes.byref(m)))

    def project_only():
        ctx._check(L.pg_project(ctx.h, ctx.stream, ctypes.byref(rS), pcols, 2, dT.ptr))

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ctx.sync()
        barrier(ws)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return max_over_ranks(ws, e0.elapsed_time(e1) / args.steps)

    k0 = gpu.kernel_launches()
    clocks = Clocks(local)
    clocks.start()
    ms_fused = timed(fused)
    clk = clocks.stop()
    launches = (gpu.kernel_launches() - k0) * args.steps // (args.steps + args.warmup)
    n_fused = res.n_out
    ms_unfused = timed(unfused)
    n_unfused = res.n_out
    ms_filter = timed(filter_only)
    n_filter = m.value
    ms_project = timed(project_only)
    # Parity: every probe key is in R (keys 1..|R|), so the rows are exactly
    # the probe tuples passing the filter; count and build-payload sums of
    # both paths agree with the host's count.
    want = int((S[:, 1] < (1 << 30)).sum())
    fl = gpu.JOIN_COUNT | gpu.JOIN_SUM
    r1, r2 = gpu.JoinResult(), gpu.JoinResult()
    ctx._check(L.pg_hashjoin_probe_where(ctx.h, ctx.stream, ht.value, ctypes.byref(rS), where, nwhere, proj, nproj,
                                         None, 0, fl, 1, ctypes.byref(r1)))
    ctx._check(L.pg_filter(ctx.h, ctx.stream, ctypes.byref(rS), where, nwhere, dT.ptr, ctypes.byref(m)))
    rT = gpu.Rel(dT.ptr, m.value, TUPLE, 0, 8)
    ctx._check(L.pg_hashjoin_probe(ctx.h, ctx.stream, ht.value, ctypes.byref(rT), proj, nproj, None, 0, fl, 1,
                                   ctypes.byref(r2)))
    L.pg_hashtable_free(ctx.h, ht.value)
    cpu = None
    if rank == 0 and not args.no_cpu:
        # The reference's plan on the host: Filter over the probe scan, then
        # HashJoinOp (oracle port), full build + a probe sample scaled to |S|.
        from oracle import oracle as orc
        m_s = min(NS, 1 << 22)
        Rc = np.array(R, copy=True)
        Ssub = np.array(S[:m_s], copy=True)
        cfg = orc.hashcfg("modulo", NR)
        t0 = time.perf_counter()
        orc.hashjoin(Rc, Ssub[:1], hash=cfg, threads=threads, materialise=False)
        t_build = time.perf_counter() - t0
        t0 = time.perf_counter()
        Sf = orc.filter(Ssub, [("long", "<", 8, 1 << 30)])
        orc.hashjoin(Rc, Sf, hash=cfg, threads=threads, out_cap=Sf.shape[0])
        # The oracle's join builds its table inside the call: its build time,
        # measured above, is taken out.
        t_rest = max(time.perf_counter() - t0 - t_build, 1e-9)
        cpu = {"value": NS / (t_rest * NS / m_s), "unit": "tuples/s", "cores": threads, "kind": "port",
               "sample": f"Filter + probe of the first {m_s} probe tuples against the full {NR}-tuple table "
                         f"(oracle port; build {t_build:.2f} s not counted, as the GPU line probes a prebuilt table), "
                         f"time scaled linearly to {NS}"}
    parity = {"rows": int(n_fused), "rows_ok": n_fused == n_unfused == n_filter == want,
              "count_and_sum_equal": (r1.n_out, r1.sum) == (r2.n_out, r2.sum)}
    peak, peak_kind = measured_peak()
    alg_probe = NS * 16 + want * 16                      # read the probe, write passing rows
    alg_filter = NS * 16 + want * 16
    alg_project = NS * 16 + NS * 16
    gbs = lambda b, ms: b / (ms / 1e3) / 1e9
    if rank == 0:
        line = {"metric": "filtered probe tuples/s (16M build x 256M probe, Filter payload < 2^30 fused into the probe)",
                "value": ws * NS / (ms_fused / 1e3), "unit": "tuples/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_fused, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "int64", "data": "synthetic (seeded generator, resident in HBM)",
                "config": {"workload": "probe of a prebuilt 16M-key table by 256M FK tuples through a Filter on "
                                       "the probe payload (half pass)", "op": "filterjoin", "probe_tuples": NS,
                           "l2": "inputs larger than L2; no flush"},
                "unfused_filter_then_probe_ms": ms_unfused, "fused_speedup": ms_unfused / ms_fused,
                "pg_filter": {"ms": ms_filter, "gbs": gbs(alg_filter, ms_filter), "frac": gbs(alg_filter, ms_filter) / peak,
                              "algorithmic_bytes": alg_filter},
                "pg_project": {"ms": ms_project, "gbs": gbs(alg_project, ms_project),
                               "frac": gbs(alg_project, ms_project) / peak, "algorithmic_bytes": alg_project},
                "parity": parity,
                "roofline": {"bound": "hbm", "kernel": "k_probe16_stage<true, true> (filter fused, compacting stages)",
                             "achieved": gbs(alg_probe, ms_fused), "peak": peak, "unit": "GB/s",
                             "frac": gbs(alg_probe, ms_fused) / peak, "traffic": None, "peak_source": peak_kind,
                             "algorithmic_bytes": alg_probe},
                "gpu_launches": int(launches), "clocks": clk}
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    L.pg_host_free(ctx.h, hR)
    L.pg_host_free(ctx.h, hS)
    ctx.close()


def run_wideprobe(args, ws, rank, local):
    """The q1-shaped plan's first join as one probe: 64M 24-byte lines (order,
    part, price) against a prebuilt 4M-part dense table, 24-byte rows (order,
    price, part payload). Tuples and rows other than 16 bytes take the probe
    staged through shared memory; the per-thread-load probe is timed beside it."""
    import torch
    from pythia_gb300 import gpu
    torch.cuda.set_device(local)
    threads = host_threads()
    ctx = make_ctx(args, local)
    L = gpu.lib()
    nL, nP = 1 << (args.probe_log2 - 2), 1 << (args.build_log2 - 2)
    _, P, Ln = _plan_inputs(nL, 1 << 10, nP, threads)
    dP, dL, dO = ctx.upload(P), ctx.upload(Ln), ctx.alloc(nL * 24)
    rP = gpu.Rel(dP.ptr, nP, 16, 0, 8)
    rL = gpu.Rel(dL.ptr, nL, 24, 8, 8)
    proj, nproj = gpu.cols((("P", 0, 8), ("P", 16, 8), ("B", 8, 8)))
    ht = ctypes.c_void_p()
    ctx._check(L.pg_hashjoin_build(ctx.h, ctx.stream, ctypes.byref(rP), proj, nproj, ctypes.byref(ht)))
    stream = torch.cuda.ExternalStream(ctx.stream)
    res = gpu.JoinResult()

    def probe():
        ctx._check(L.pg_hashjoin_probe(ctx.h, ctx.stream, ht.value, ctypes.byref(rL), proj, nproj, dO.ptr, nL,
                                       gpu.JOIN_MATERIALIZE, -1, ctypes.byref(res)))

    def timed():
        for _ in range(args.warmup):
            probe()
        ctx.sync()
        barrier(ws)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            probe()
        e1.record(stream)
        e1.synchronize()
        return max_over_ranks(ws, e0.elapsed_time(e1) / args.steps)

    k0 = gpu.kernel_launches()
    clocks = Clocks(local)
    clocks.start()
    ms = timed()
    clk = clocks.stop()
    launches = (gpu.kernel_launches() - k0) * args.steps // (args.steps + args.warmup)
    n_rows = res.n_out
    # Parity at full size: every line finds its part, so the rows' columns sum
    # (wrapping) to the lines' orders, the lines' prices and the parts'
    # payloads looked up by each line's part key.
    out = ctx.download(dO, n_rows * 24, np.int64).reshape(-1, 3)
    by_key = np.zeros(nP + 1, np.int64)
    by_key[P[:, 0]] = P[:, 1]
    with np.errstate(over="ignore"):
        want = [int(Ln[:, 0].sum()), int(Ln[:, 2].sum()), int(by_key[Ln[:, 1]].sum())]
        got = [int(out[:, 0].sum()), int(out[:, 1].sum()), int(out[:, 2].sum())]
    del out
    ctx.tune(probe_wide=1)
    ms_plain = timed()
    ctx.tune(probe_wide=0)
    L.pg_hashtable_free(ctx.h, ht.value)
    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as orc
        m = min(nL, 1 << 22)
        cfg = orc.hashcfg("modulo", nP)
        Lsub = np.array(Ln[:m], copy=True)
        t0 = time.perf_counter()
        orc.hashjoin(P, Lsub[:1], proj=(("P", 0, 8), ("P", 16, 8), ("B", 8, 8)), pkey=(8, 8), hash=cfg,
                     threads=threads, materialise=False)
        t_build = time.perf_counter() - t0
        t0 = time.perf_counter()
        orc.hashjoin(P, Lsub, proj=(("P", 0, 8), ("P", 16, 8), ("B", 8, 8)), pkey=(8, 8), hash=cfg,
                     threads=threads, out_cap=m)
        t = max(time.perf_counter() - t0 - t_build, 1e-9) * nL / m
        cpu = {"value": nL / t, "unit": "tuples/s", "cores": threads, "kind": "port",
               "sample": f"probe of the first {m} lines against the full {nP}-part table (oracle port; its build, "
                         f"{t_build:.2f} s, not counted), time scaled linearly to {nL}"}
    peak, peak_kind = measured_peak()
    alg = nL * 24 + n_rows * 24
    gbs = alg / (ms / 1e3) / 1e9
    if rank == 0:
        line = {"metric": "probe tuples/s, 24-byte lines into 24-byte rows (64M lines x 4M-part dense table)",
                "value": ws * nL / (ms / 1e3), "unit": "tuples/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "int64", "data": "synthetic (seeded generator, resident in HBM)",
                "config": {"workload": f"{nL} lines (order, part, price) probing a prebuilt {nP}-part table, rows "
                                       "(order, price, part payload): the q1-shaped plan's first join",
                           "op": "wideprobe", "l2": "inputs larger than L2; no flush"},
                "per_thread_load_probe_ms": ms_plain, "staged_speedup": ms_plain / ms,
                "parity": {"rows": int(n_rows), "rows_ok": int(n_rows) == nL, "column_sums_ok": got == want},
                "roofline": {"bound": "hbm", "kernel": "k_probe_staged<true, 2, 2>", "achieved": gbs, "peak": peak,
                             "unit": "GB/s", "frac": gbs / peak,
                             "traffic": WIDE_DRAM_BYTES_PER_LINE * nL if nP == 1 << 22 else None,
                             "peak_source": peak_kind, "algorithmic_bytes": alg},
                "gpu_launches": int(launches), "clocks": clk}
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    ctx.close()


# ---------------------------------------------------------------------------
# The default run: the headline line carries every other configuration's
# line under "configs", each measured in this same process.
# ---------------------------------------------------------------------------
def _captured(fn, *a):
    """Runs a bench function that prints one JSON line; returns that line."""
    import contextlib
    import io
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        fn(*a)
    for ln in reversed(buf.getvalue().strip().splitlines()):
        try:
            return json.loads(ln)
        except ValueError:
            continue
    return None


def suite(args, ws, rank, local):
    """The configurations other than the headline, at their full sizes, with
    fewer steps (warm-up 3, timed 5) to keep the whole run within minutes."""
    import copy
    import gc
    import torch
    sub = copy.copy(args)
    sub.steps, sub.warmup = min(args.steps, 5), max(3, min(args.warmup, 3))
    jobs = [
        ("cfg1_join_1Mx16M_count_sum",
         lambda: run_join(sub, ws, rank, local, join_spec(1 << 20, 1 << 24, mode="count_sum"),
                          max(sub.steps, 10), sub.warmup, cpu_sample=None, want_cpu=not args.no_cpu)),
        ("cfg2a_join_16Mx256M_zipf1.0",
         lambda: run_join(sub, ws, rank, local, join_spec(1 << 24, 1 << 28, "zipf", 1.0), sub.steps, sub.warmup,
                          e2e_steps=3, cpu_sample=1 << 23, want_cpu=not args.no_cpu)),
        ("cfg2a_join_16Mx256M_sparse_keys",
         lambda: run_join(sub, ws, rank, local, join_spec(1 << 24, 1 << 28, key_domain="sparse"), sub.steps,
                          sub.warmup, e2e_steps=3, cpu_sample=1 << 23, want_cpu=not args.no_cpu)),
        ("cfg2b_groupby_256M_1M_groups", lambda: _captured(run_op, sub, ws, rank, local, "groupby")),
        ("cfg3_mpsm_64Mx64M_count_sum", lambda: _captured(run_op, sub, ws, rank, local, "mpsm")),
        ("cfg3_mpsm_64Mx64M_materialised", lambda: _captured(run_op, sub, ws, rank, local, "mpsmmat")),
        ("sort_64M_keys_over_2e32_radix", lambda: _captured(run_op, sub, ws, rank, local, "sortwide")),
        ("sort_64M_keys_over_2e32_bitonic", lambda: _captured(run_op, sub, ws, rank, local, "sortbitonic")),
        ("sort_64M_keys_16M_radix", lambda: _captured(run_op, sub, ws, rank, local, "sort")),
        ("partition_256M_256way", lambda: _captured(run_op, sub, ws, rank, local, "partition")),
        ("cfg4_batch_10000", lambda: _captured(run_batch, sub, ws, rank, local)),
        ("cfg5_serve", lambda: _captured(run_serve, sub, ws, rank, local)),
    ]
    only = set(args.suite.split(",")) if args.suite else None
    out = {}
    for name, fn in jobs:
        if only and name not in only:
            continue
        t0 = time.perf_counter()
        try:
            r = fn()
        except Exception as e:  # one configuration failing must not take the others down
            r = {"error": f"{type(e).__name__}: {e}"}
        if r is not None:
            r["wall_s"] = time.perf_counter() - t0
            out[name] = r
        print(f"[suite] {name}: {r.get('value') if r else None} ({time.perf_counter() - t0:.1f} s)",
              file=sys.stderr, flush=True)
        gc.collect()
        torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--key-domain", default="dense", choices=["dense", "sparse"],
                    help="dense: keys 1..|R| (direct-mapped table); sparse: the same keys "
                         "multiplied by an odd constant (hashed table)")
    ap.add_argument("--probe-dist", default="uniform", choices=["uniform", "zipf"],
                    help="probe foreign keys: uniform over R's keys, or Zipf ranks (--zipf-s)")
    ap.add_argument("--zipf-s", type=float, default=1.0)
    ap.add_argument("--op", default="hashjoin", choices=["hashjoin", "join1m", "batch", "serve", "tableimage", "plan",
                                                      "filterjoin", "wideprobe"] + sorted(OPS))
    ap.add_argument("--headline-only", action="store_true",
                    help="the headline join alone, without the other configurations")
    ap.add_argument("--suite", default="", help="comma-separated subset of the other configurations")
    ap.add_argument("--slots", type=int, default=8, help="worker slots for --op serve")
    ap.add_argument("--retune", action="store_true", help="rerun the autotuner for --op batch")
    ap.add_argument("--scale-down", type=int, default=0, help="divide --op sizes by 2^k")
    ap.add_argument("--tune", default="", help="tuning knobs, e.g. probe_items=8,build_spec=2")
    ap.add_argument("--build-log2", type=int, default=24)
    ap.add_argument("--probe-log2", type=int, default=28)
    args = ap.parse_args()
    global NR, NS
    NR, NS = 1 << args.build_log2, 1 << args.probe_log2
    ws, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, ws, rank)
    elif args.op == "batch":
        run_batch(args, ws, rank, local)
    elif args.op == "serve":
        run_serve(args, ws, rank, local)
    elif args.op == "tableimage":
        run_tableimage(args, ws, rank, local)
    elif args.op == "plan":
        run_plan(args, ws, rank, local)
    elif args.op == "filterjoin":
        run_filterjoin(args, ws, rank, local)
    elif args.op == "wideprobe":
        run_wideprobe(args, ws, rank, local)
    elif args.op == "join1m":
        line = run_join(args, ws, rank, local, join_spec(1 << 20, 1 << 24, mode="count_sum"), args.steps,
                        args.warmup, args.e2e_steps, None, not args.no_cpu)
        if line:
            print(json.dumps(line), flush=True)
    elif args.op != "hashjoin":
        run_op(args, ws, rank, local, args.op)
    else:
        line = run_join(args, ws, rank, local, headline_spec(args), args.steps, args.warmup, args.e2e_steps,
                        max(1, NS // 32), not args.no_cpu)
        if ws == 1 and not args.headline_only:
            configs = suite(args, ws, rank, local)
            if line is not None:
                line["configs"] = configs
        if line is not None:
            print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
