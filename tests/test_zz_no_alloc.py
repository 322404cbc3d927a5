"""The allocation-free join count/sum (pg_hashjoin_agg_noalloc).

Callers that may not allocate device memory while a query runs use this entry
point; its hash table is a fixed array the library declares. This test calls it
through the C ABI twice in a row, on different inputs, and checks each result
against the allocating entry points (pg_hashjoin_build + pg_hashjoin_probe with
PG_JOIN_COUNT | PG_JOIN_SUM): counts and integer sums must be equal. It also
checks that a build side above the stated limit is refused. It runs last in
the suite (file name) and also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from pythia_gb300 import datagen as dg
from pythia_gb300 import gpu

pytestmark = pytest.mark.gpu

MAX_BUILD = 524_288


def _noalloc(ctx, R, S, proj, sum_col):
    dR, dS = ctx.upload(R), ctx.upload(S)
    rR = ctx.rel(dR, R.shape[0], gpu.row_width(R), 0, 8)
    rS = ctx.rel(dS, S.shape[0], gpu.row_width(S), 0, 8)
    c, nc = gpu.cols(proj)
    res = gpu.JoinResult()
    rc = gpu.lib().pg_hashjoin_agg_noalloc(ctx.h, ctx.stream, ctypes.byref(rR), ctypes.byref(rS),
                                            c, nc, sum_col, ctypes.byref(res))
    return rc, res.n_out, res.sum


def test_noalloc_join_matches_allocating_entry_points():
    ctx = gpu.Context(0)
    try:
        proj = (("P", 8, 8), ("B", 8, 8))
        cases = [
            # PK-FK at the size limit, build payload summed.
            (dg.build_relation(MAX_BUILD, dg.seed_for(201)), None, 1),
            # Duplicate keys on both sides and probe keys with no partner,
            # probe payload summed: the array still holds the previous call.
            (dg.uniform_keys(100_000, 30_000, dg.seed_for(203)),
             dg.uniform_keys(400_000, 40_000, dg.seed_for(204)), 0),
        ]
        for R, S, sum_col in cases:
            if S is None:
                S = dg.probe_uniform(2_000_000, R, dg.seed_for(202))
            rc, n, s = _noalloc(ctx, R, S, proj, sum_col)
            assert rc == gpu.PG_OK, gpu.lib().pg_last_error(ctx.h)
            _, wn, ws = ctx.hashjoin(R, S, proj=proj, flags=gpu.JOIN_COUNT | gpu.JOIN_SUM, sum_col=sum_col)
            assert (n, s) == (wn, ws)
        too_big = dg.build_relation(MAX_BUILD + 1, dg.seed_for(205))
        rc, _, _ = _noalloc(ctx, too_big, too_big[:10], proj, 1)
        assert rc == gpu.PG_ERR_ARG
        assert b"524288" in gpu.lib().pg_last_error(ctx.h)
    finally:
        ctx.close()
