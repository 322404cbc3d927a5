"""Serving loop for join + group-by query plans on one GPU.

A query plan is the reference's join-then-aggregate pipeline (HashJoinOp ->
AggregateSum over a dec column, operators/join.cpp:273-675,
genericaggregate.cpp:240-487): probe a resident build table with the query's
probe relation, materialise (group key, value) rows, and sum the values per
group key.

* Resident state: the build tables' hash tables and the probe relations stay
  in HBM across queries (the catalog); only per-query working memory is
  allocated, stream-ordered, while a query runs.
* Admission: a query enters when a worker slot is free and its working-memory
  footprint fits in the remaining HBM budget; a query that does not fit lets
  smaller ones behind it in (no head-of-line blocking by size).
* Continuous batching: every slot runs on its own CUDA stream, so queries
  admitted while others run overlap on the device; a finished query frees its
  slot and memory for the next admission immediately.
* One-at-a-time execution is the same server with one slot.

Host-side failures (an exception in one query's execution) are recorded for
that query and the loop continues.
"""
import collections
import ctypes
import threading
import time

import numpy as np

from pythia_gb300 import datagen as dg
from pythia_gb300 import gpu

PROJ = (("B", 8, 8), ("P", 8, 8))          # output (group key, value)


class Table:
    def __init__(self, tid, n, groups, R_dev, ht, pools):
        self.tid, self.n, self.groups = tid, n, groups
        self.R_dev, self.ht, self.pools = R_dev, ht, pools   # pools: {zipf s: device buffer}


class Catalog:
    """Resident build tables (hash tables built once) and probe pools."""

    def __init__(self, ctx, sizes, zipf=(0.0, 0.8), probe_factor=10, seed_base=500, threads=None):
        self.ctx, self.tables, self.resident_bytes = ctx, [], 0
        L = gpu.lib()
        c, nc = gpu.cols(PROJ)
        self._cols = (c, nc)
        for t, r in enumerate(sizes):
            r = int(r)
            groups = max(1, r // 100)
            R = dg.build_relation(r, dg.seed_for(seed_base + t), threads=threads)
            R[:, 1] = dg.raw_words(dg.seed_for(seed_base + t), 7, r) % np.uint64(groups)
            dR = ctx.upload(R)
            rel = gpu.Rel(dR.ptr, r, 16, 0, 8)
            ht = ctypes.c_void_p()
            ctx._check(L.pg_hashjoin_build(ctx.h, ctx.stream, ctypes.byref(rel), c, nc, ctypes.byref(ht)))
            pools = {}
            for s in zipf:
                buf = ctx.alloc(16 * probe_factor * r)
                ctx._check(L.pg_generate_zipf_fk(ctx.h, ctx.stream, dR.ptr, r, float(s),
                                                 dg.seed_for(seed_base + 1000 + t) ^ int(s * 1000),
                                                 buf.ptr, probe_factor * r, 1e4))
                pools[s] = buf
                self.resident_bytes += 16 * probe_factor * r
            self.resident_bytes += 16 * r * 3
            self.tables.append(Table(t, r, groups, dR, ht.value, pools))
        self.probe_factor = probe_factor
        ctx.sync()

    def close(self):
        for t in self.tables:
            gpu.lib().pg_hashtable_free(self.ctx.h, t.ht)
        self.tables = []


class Query:
    __slots__ = ("qid", "table", "zipf", "arrival", "start", "end", "result", "error", "fail")

    def __init__(self, qid, table, zipf, arrival=0.0, fail=False):
        self.qid, self.table, self.zipf, self.arrival = qid, table, zipf, arrival
        self.start = self.end = None
        self.result = self.error = None
        self.fail = fail


def footprint(cat, q):
    t = cat.tables[q.table]
    ns = cat.probe_factor * t.n
    return 32 * ns + 64 * t.groups + (1 << 20)


def execute(ctx, stream, cat, q):
    """Runs one query on `stream`; returns (group keys, sums) sorted by key."""
    if q.fail:
        raise RuntimeError(f"query {q.qid}: injected host failure")
    L = gpu.lib()
    t = cat.tables[q.table]
    ns = cat.probe_factor * t.n
    c, nc = cat._cols
    w1, w2 = ctypes.c_void_p(), ctypes.c_void_p()
    ctx._check(L.pg_buffer_alloc_async(ctx.h, stream, 16 * ns, ctypes.byref(w1)))
    ctx._check(L.pg_buffer_alloc_async(ctx.h, stream, 16 * (t.groups + 1), ctypes.byref(w2)))
    try:
        rS = gpu.Rel(t.pools[q.zipf].ptr, ns, 16, 0, 8)
        res = gpu.JoinResult()
        ctx._check(L.pg_hashjoin_probe(ctx.h, stream, t.ht, ctypes.byref(rS), c, nc, w1.value, ns,
                                       gpu.JOIN_MATERIALIZE, -1, ctypes.byref(res)))
        rJ = gpu.Rel(w1.value, res.n_out, 16, 0, 8)
        ng = ctypes.c_uint64()
        ctx._check(L.pg_groupby(ctx.h, stream, ctypes.byref(rJ), 8, gpu.VAL["dec"], gpu.AGG["sum"],
                                t.groups, w2.value, t.groups + 1, ctypes.byref(ng)))
        out = np.empty(ng.value * 2, dtype=np.int64)
        if ng.value:
            ctx._check(L.pg_d2h(ctx.h, stream, out.ctypes.data, w2.value, 16 * ng.value))
            ctx._check(L.pg_sync(ctx.h, stream))
    finally:
        L.pg_buffer_free_async(ctx.h, stream, w1.value)
        L.pg_buffer_free_async(ctx.h, stream, w2.value)
    rows = out.reshape(-1, 2)
    order = np.argsort(rows[:, 0], kind="stable")
    return rows[order, 0].copy(), rows[order, 1].view(np.float64).copy(), int(res.n_out)


class Server:
    def __init__(self, ctx, cat, slots, budget_bytes):
        self.ctx, self.cat, self.slots, self.budget = ctx, cat, slots, budget_bytes
        self.streams = []
        for _ in range(slots):
            s = ctypes.c_void_p()
            ctx._check(gpu.lib().pg_stream_create(ctx.h, ctypes.byref(s)))
            self.streams.append(s.value)

    def close(self):
        for s in self.streams:
            gpu.lib().pg_stream_destroy(self.ctx.h, s)

    def run(self, queries):
        """Serves `queries` (arrival = seconds after start). Returns them with
        start/end times (seconds after start), results or errors."""
        pending = collections.deque()
        cv = threading.Condition()
        state = {"used": 0, "arrived": 0, "t0": time.perf_counter()}
        n = len(queries)

        def now():
            return time.perf_counter() - state["t0"]

        def dispatcher():
            for q in sorted(queries, key=lambda q: q.arrival):
                d = q.arrival - now()
                if d > 0:
                    time.sleep(d)
                with cv:
                    pending.append(q)
                    state["arrived"] += 1
                    cv.notify_all()

        def take():
            # First pending query whose footprint fits; None when none fits.
            for i, q in enumerate(pending):
                fp = footprint(self.cat, q)
                if state["used"] + fp <= self.budget or state["used"] == 0:
                    del pending[i]
                    state["used"] += fp
                    return q, fp
            return None, 0

        def worker(stream):
            while True:
                with cv:
                    while True:
                        q, fp = take()
                        if q is not None:
                            break
                        if state["arrived"] == n and not pending:
                            return
                        cv.wait(0.05)
                q.start = now()
                try:
                    q.result = execute(self.ctx, stream, self.cat, q)
                except Exception as e:            # host-side failure: record, keep serving
                    q.error = str(e)
                q.end = now()
                with cv:
                    state["used"] -= fp
                    cv.notify_all()

        threads = [threading.Thread(target=worker, args=(s,), daemon=True) for s in self.streams]
        disp = threading.Thread(target=dispatcher, daemon=True)
        state["t0"] = time.perf_counter()
        disp.start()
        for t in threads:
            t.start()
        disp.join()
        for t in threads:
            t.join()
        return queries


def poisson_arrivals(n, rate, seed):
    u = dg.raw_words(seed, 3, n).astype(np.float64) * (1.0 / 2.0 ** 64)
    gaps = -np.log1p(-u) / rate
    return np.cumsum(gaps)


def summarize(queries):
    ok = [q for q in queries if q.error is None]
    lat = np.array([q.end - q.arrival for q in ok]) * 1e3
    span = max(q.end for q in queries) - min(q.arrival for q in queries)
    return {"queries": len(queries), "errors": len(queries) - len(ok),
            "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "queries_per_s": len(ok) / span if span > 0 else None, "makespan_s": span}
