"""The allocation-free join count/sum (pg_hashjoin_agg_noalloc).

Callers that may not allocate device memory while a query runs (a host whose
own pool holds the device's memory, a sandbox with a fixed budget) use this
entry point; its hash table is a fixed array the library declares. The tests
call it through the C ABI, several times in a row on the same array, and check
each result against the oracle's join (counts and wrapping integer sums must
be equal) and against the allocating entry points (pg_hashjoin_build +
pg_hashjoin_probe with PG_JOIN_COUNT | PG_JOIN_SUM). They cover 8- and 4-byte
keys, a 4-byte summed column (sign-extended), keys equal to -1 (the table's
empty marker) on both sides, the limits (a build side above 524,288 tuples,
more than 1024 build keys equal to -1), and that calls after the first one on
the device allocate no device memory. This file runs last in the suite (its
name) and also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as orc
from pythia_gb300 import datagen as dg
from pythia_gb300 import gpu
from tests.golden import inputs as gin

pytestmark = pytest.mark.gpu

MAX_BUILD = 524_288
PG_ERR_UNSUPPORTED = 7


class _Dev:
    """Inputs uploaded once, so that the calls themselves are all that runs."""

    def __init__(self, ctx, R, S, key_bytes):
        self.keep = (ctx.upload(R), ctx.upload(S))
        self.rR = ctx.rel(self.keep[0], R.shape[0], gpu.row_width(R), 0, key_bytes)
        self.rS = ctx.rel(self.keep[1], S.shape[0], gpu.row_width(S), 0, key_bytes)


def _call(ctx, d, proj, sum_col):
    c, nc = gpu.cols(proj)
    res = gpu.JoinResult()
    rc = gpu.lib().pg_hashjoin_agg_noalloc(ctx.h, ctx.stream, ctypes.byref(d.rR), ctypes.byref(d.rS),
                                            c, nc, sum_col, ctypes.byref(res))
    return rc, res.n_out, res.sum


def _cases():
    long_proj = (("P", 8, 8), ("B", 8, 8))
    R1 = dg.build_relation(MAX_BUILD, dg.seed_for(201))             # PK-FK at the size limit
    S1 = dg.probe_uniform(2_000_000, R1, dg.seed_for(202))
    R2 = dg.uniform_keys(100_000, 30_000, dg.seed_for(203))          # repeated keys on both sides,
    S2 = dg.uniform_keys(400_000, 40_000, dg.seed_for(204))          # probe keys without a partner
    R3 = dg.build_relation(50_000, dg.seed_for(206))                 # keys equal to the empty marker
    R3[::5000, 0] = -1
    S3 = dg.probe_uniform(300_000, R3, dg.seed_for(207))
    S3[::333, 0] = -1
    I = gin.make({"gen": "formula", "name": "int_pairs", "n": 40_000})   # 4-byte keys and columns
    I[:, 0] %= 5000
    I[::1000, 0] = -1
    int_proj = (("P", 4, 4), ("B", 4, 4))
    return [("pkfk_at_limit", R1, S1, long_proj, 1, 8), ("repeated_keys", R2, S2, long_proj, 0, 8),
            ("empty_marker_keys", R3, S3, long_proj, 1, 8), ("int_keys", I, I[::-1].copy(), int_proj, 1, 4),
            ("no_sum", R2, S2, long_proj, -1, 8)]


def _oracle(R, S, proj, sum_col, kb):
    _, n, s = orc.hashjoin(R, S, proj=proj, bkey=(0, kb), pkey=(0, kb), materialise=False,
                           sum_col=sum_col, hash=orc.hashcfg("modulo", 1 << 16), threads=8)
    return n, (s if sum_col >= 0 else 0)


def test_noalloc_join_matches_oracle_and_allocating_entry_points():
    ctx = gpu.Context(0)
    try:
        for name, R, S, proj, sum_col, kb in _cases():
            d = _Dev(ctx, R, S, kb)
            want = _oracle(R, S, proj, sum_col, kb)
            for _ in range(2):                       # the array keeps the previous call's contents
                rc, n, s = _call(ctx, d, proj, sum_col)
                assert rc == gpu.PG_OK, (name, gpu.lib().pg_last_error(ctx.h))
                assert (n, s) == want, name
            _, wn, ws = ctx.hashjoin(R, S, proj=proj, bkey=(0, kb), pkey=(0, kb),
                                     flags=gpu.JOIN_COUNT | (gpu.JOIN_SUM if sum_col >= 0 else 0), sum_col=sum_col)
            assert (wn, ws if sum_col >= 0 else 0) == want, name
    finally:
        ctx.close()


def test_noalloc_limits_are_refused():
    ctx = gpu.Context(0)
    try:
        proj = (("P", 8, 8), ("B", 8, 8))
        too_big = dg.build_relation(MAX_BUILD + 1, dg.seed_for(205))
        rc, _, _ = _call(ctx, _Dev(ctx, too_big, too_big[:10], 8), proj, 1)
        assert rc == gpu.PG_ERR_ARG
        assert b"524288" in gpu.lib().pg_last_error(ctx.h)
        marks = dg.build_relation(3000, dg.seed_for(208))
        marks[:1025, 0] = -1                          # 1025 build keys equal to the empty marker
        rc, _, _ = _call(ctx, _Dev(ctx, marks, marks, 8), proj, 1)
        assert rc == PG_ERR_UNSUPPORTED
        # The array is fine afterwards.
        R = dg.build_relation(1000, dg.seed_for(209))
        S = dg.probe_uniform(10_000, R, dg.seed_for(210))
        rc, n, s = _call(ctx, _Dev(ctx, R, S, 8), proj, 1)
        assert rc == gpu.PG_OK and (n, s) == _oracle(R, S, proj, 1, 8)
    finally:
        ctx.close()


def test_noalloc_calls_after_the_first_allocate_nothing():
    torch = pytest.importorskip("torch")
    ctx = gpu.Context(0)
    torch.cuda.mem_get_info(0)                   # torch's own CUDA set-up happens here, not below
    try:
        proj = (("P", 8, 8), ("B", 8, 8))
        R = dg.build_relation(200_000, dg.seed_for(211))
        S = dg.probe_uniform(1_000_000, R, dg.seed_for(212))
        d = _Dev(ctx, R, S, 8)
        empty = _Dev(ctx, R[:0], S[:0], 8)
        assert _call(ctx, empty, proj, 1)[0] == gpu.PG_OK        # the first call on the device sets up
        ctx.sync()
        free0, _ = torch.cuda.mem_get_info(0)
        results = [_call(ctx, d, proj, 1) for _ in range(3)]
        ctx.sync()
        free1, _ = torch.cuda.mem_get_info(0)
        assert free1 == free0, f"device memory changed by {free0 - free1} bytes"
        want = _oracle(R, S, proj, 1, 8)
        assert all(r == (gpu.PG_OK,) + want for r in results)
    finally:
        ctx.close()
