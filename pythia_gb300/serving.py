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
import ctypes
import os
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
    """Resident build tables (hash tables built once) and probe pools.

    With `images` (a directory written by save()), every table is loaded from
    its table image (pg_hashtable_load) instead of being built: the warm start
    of a server that keeps its tables across restarts. `table_seconds` is the
    time spent building or loading the tables."""

    def __init__(self, ctx, sizes, zipf=(0.0, 0.8), probe_factor=10, seed_base=500, threads=None, images=None):
        self.ctx, self.tables, self.resident_bytes = ctx, [], 0
        self.table_seconds = 0.0
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
            t0 = time.perf_counter()
            if images:
                ctx._check(L.pg_hashtable_load(ctx.h, ctx.stream, os.fsencode(self.image_path(images, t)),
                                               ctypes.byref(ht)))
            else:
                ctx._check(L.pg_hashjoin_build(ctx.h, ctx.stream, ctypes.byref(rel), c, nc, ctypes.byref(ht)))
            ctx.sync()
            self.table_seconds += time.perf_counter() - t0
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

    @staticmethod
    def image_path(directory, tid):
        return os.path.join(directory, f"table_{tid}.img")

    def save(self, directory):
        """Writes every table's image (pg_hashtable_save) into `directory`."""
        os.makedirs(directory, exist_ok=True)
        for t in self.tables:
            self.ctx._check(gpu.lib().pg_hashtable_save(self.ctx.h, self.ctx.stream, t.ht,
                                                        os.fsencode(self.image_path(directory, t.tid))))

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


def execute(ctx, stream, cat, q, fused=True):
    """Runs one query on `stream`; returns (group keys, sums, join rows) with
    groups in unspecified order. The plan runs as one pass (probe folding
    straight into the group table, pg_hashjoin_groupby) when the table allows
    it, else as a materialised probe followed by a group-by."""
    if q.fail:
        raise RuntimeError(f"query {q.qid}: injected host failure")
    L = gpu.lib()
    t = cat.tables[q.table]
    ns = cat.probe_factor * t.n
    c, nc = cat._cols
    rS = gpu.Rel(t.pools[q.zipf].ptr, ns, 16, 0, 8)
    w2 = ctypes.c_void_p()
    ctx._check(L.pg_buffer_alloc_async(ctx.h, stream, 16 * (t.groups + 1), ctypes.byref(w2)))
    w1 = ctypes.c_void_p()
    try:
        ng = ctypes.c_uint64()
        rc = L.pg_hashjoin_groupby(ctx.h, stream, t.ht, ctypes.byref(rS), 8, gpu.VAL["dec"], gpu.AGG["sum"],
                                   w2.value, t.groups + 1, ctypes.byref(ng)) if fused else gpu.PG_ERR_UNSUPPORTED
        if rc == gpu.PG_ERR_UNSUPPORTED:
            ctx._check(L.pg_buffer_alloc_async(ctx.h, stream, 16 * ns, ctypes.byref(w1)))
            res = gpu.JoinResult()
            ctx._check(L.pg_hashjoin_probe(ctx.h, stream, t.ht, ctypes.byref(rS), c, nc, w1.value, ns,
                                           gpu.JOIN_MATERIALIZE, -1, ctypes.byref(res)))
            rJ = gpu.Rel(w1.value, res.n_out, 16, 0, 8)
            ctx._check(L.pg_groupby(ctx.h, stream, ctypes.byref(rJ), 8, gpu.VAL["dec"], gpu.AGG["sum"],
                                    t.groups, w2.value, t.groups + 1, ctypes.byref(ng)))
        else:
            ctx._check(rc)
        out = np.empty(ng.value * 2, dtype=np.int64)
        if ng.value:
            ctx._check(L.pg_d2h(ctx.h, stream, out.ctypes.data, w2.value, 16 * ng.value))
        ctx._check(L.pg_sync(ctx.h, stream))
    finally:
        if w1.value:
            L.pg_buffer_free_async(ctx.h, stream, w1.value)
        L.pg_buffer_free_async(ctx.h, stream, w2.value)
    rows = out.reshape(-1, 2)
    return rows[:, 0], rows[:, 1].view(np.float64)


def canonical(result):
    """A query result sorted by group key (results are unordered)."""
    keys, sums = result
    order = np.argsort(keys, kind="stable")
    return keys[order], sums[order]


def work(cat, q):
    """Estimated work of a query: tuples it reads (probe + build)."""
    t = cat.tables[q.table]
    return (cat.probe_factor + 1) * t.n


class Server:
    """Worker slots over one GPU context.

    policy "fifo": a free slot takes the first pending query (arrival order)
    whose footprint fits. policy "short-first": it takes the fitting query of
    least estimated work, except that a query pending longer than `max_wait`
    seconds goes first (no starvation); queries below `urgent_below` tuples
    run on high-priority streams, so their kernels are scheduled ahead of the
    long queries' kernels already on the GPU."""

    def __init__(self, ctx, cat, slots, budget_bytes, policy="fifo", max_wait=0.25, urgent_below=32 << 20):
        self.ctx, self.cat, self.slots, self.budget = ctx, cat, slots, budget_bytes
        self.policy, self.max_wait, self.urgent_below = policy, max_wait, urgent_below
        self.streams, self.urgent = [], []
        L = gpu.lib()
        for _ in range(slots):
            s = ctypes.c_void_p()
            ctx._check(L.pg_stream_create(ctx.h, ctypes.byref(s)))
            self.streams.append(s.value)
            u = ctypes.c_void_p()
            ctx._check(L.pg_stream_create_urgent(ctx.h, ctypes.byref(u)))
            self.urgent.append(u.value)

    def close(self):
        for s in self.streams + self.urgent:
            gpu.lib().pg_stream_destroy(self.ctx.h, s)
        self.streams, self.urgent = [], []

    def run(self, queries):
        """Serves `queries` (arrival = seconds after start). Returns them with
        start/end times (seconds after start), results or errors."""
        pending = []
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

        def fits(q):
            fp = footprint(self.cat, q)
            return (state["used"] + fp <= self.budget or state["used"] == 0), fp

        def take():
            # The next query to admit, or None when none fits.
            order = range(len(pending))
            if self.policy == "short-first" and pending:
                t = now()
                overdue = [i for i in order if t - pending[i].arrival > self.max_wait]
                order = overdue + sorted((i for i in order if i not in set(overdue)),
                                         key=lambda i: work(self.cat, pending[i]))
            for i in order:
                ok, fp = fits(pending[i])
                if ok:
                    q = pending.pop(i)
                    state["used"] += fp
                    return q, fp
            return None, 0

        def worker(slot):
            while True:
                with cv:
                    while True:
                        q, fp = take()
                        if q is not None:
                            break
                        if state["arrived"] == n and not pending:
                            return
                        cv.wait(0.05)
                urgent = self.policy == "short-first" and work(self.cat, q) < self.urgent_below
                stream = self.urgent[slot] if urgent else self.streams[slot]
                q.start = now()
                try:
                    q.result = execute(self.ctx, stream, self.cat, q)
                except Exception as e:            # host-side failure: record, keep serving
                    q.error = str(e)
                q.end = now()
                with cv:
                    state["used"] -= fp
                    cv.notify_all()

        threads = [threading.Thread(target=worker, args=(k,), daemon=True) for k in range(self.slots)]
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
