"""Serving loop: results are the same alone and in the mix, a host-side
failure in one query leaves the others served, and a sample of results matches
the oracle (join -> exactly rounded per-group sums). The dec sums are exact
fixed-point sums, so "the same" is bit for bit; the contract's 1e-12 relative
bound is checked too."""
import numpy as np
import pytest

from oracle import oracle as orc
from pythia_gb300 import gpu, serving

pytestmark = pytest.mark.gpu
RTOL = 1e-12


@pytest.fixture(scope="module")
def catalog(ctx):
    cat = serving.Catalog(ctx, [10_000, 31_000, 100_000, 320_000, 1_000_000])
    yield cat
    cat.close()


def _queries(n, fail_at=None):
    rng = np.random.default_rng(11)
    return [serving.Query(i, int(rng.integers(0, 5)), float(rng.choice([0.0, 0.8])), 0.0, fail=(i == fail_at))
            for i in range(n)]


def _same(a, b):
    ka, va = serving.canonical(a)
    kb, vb = serving.canonical(b)
    assert np.array_equal(ka, kb)
    assert np.all(np.abs(va - vb) <= RTOL * np.abs(vb))
    assert np.array_equal(va.view(np.int64), vb.view(np.int64))


def test_results_identical_alone_and_mixed(ctx, catalog):
    alone = serving.Server(ctx, catalog, slots=1, budget_bytes=150 << 30)
    mixed = serving.Server(ctx, catalog, slots=8, budget_bytes=150 << 30)
    try:
        qa = alone.run(_queries(24, fail_at=5))
        qb = mixed.run(_queries(24, fail_at=5))
    finally:
        alone.close(); mixed.close()
    for a, b in zip(qa, qb):
        if a.qid == 5:
            assert a.error and b.error and a.result is None and b.result is None
            continue
        assert a.error is None and b.error is None
        _same(a.result, b.result)


def test_admission_budget_serialises_large_queries(ctx, catalog):
    # A budget that fits one query of the largest table at a time still serves
    # everything (a query that alone exceeds the budget runs alone).
    srv = serving.Server(ctx, catalog, slots=4, budget_bytes=1 << 20)
    try:
        qs = srv.run(_queries(8))
    finally:
        srv.close()
    assert all(q.error is None for q in qs)
    spans = sorted((q.start, q.end) for q in qs)
    assert all(spans[i][1] <= spans[i + 1][0] + 1e-6 for i in range(len(spans) - 1))


def test_results_match_oracle(ctx, catalog):
    srv = serving.Server(ctx, catalog, slots=2, budget_bytes=150 << 30)
    try:
        qs = srv.run([serving.Query(0, 0, 0.0), serving.Query(1, 1, 0.8)])
    finally:
        srv.close()
    for q in qs:
        t = catalog.tables[q.table]
        R = ctx.download(t.R_dev, 16 * t.n).view(np.int64).reshape(-1, 2)
        ns = catalog.probe_factor * t.n
        S = ctx.download(t.pools[q.zipf], 16 * ns).view(np.int64).reshape(-1, 2)
        joined, n, _ = orc.hashjoin(R, S, proj=(("B", 8, 8), ("P", 8, 8)), hash=orc.hashcfg("modulo", 1 << 16))
        exact = orc.groupby_exact(joined.view(np.int64).reshape(-1, 2)).view(np.int64).reshape(-1, 2)
        keys, sums = serving.canonical(q.result)
        assert np.array_equal(keys, exact[:, 0])
        ev = exact[:, 1].view(np.float64)
        assert np.all(np.abs(sums - ev) <= RTOL * np.abs(ev))
        assert np.array_equal(np.ascontiguousarray(sums).view(np.int64), exact[:, 1])


def test_one_pass_plan_matches_two_step_plan(ctx, catalog):
    # The fused join+group-by and the materialised probe + group-by give the
    # same groups and the same sums, bit for bit.
    stream = ctx.stream
    for table in range(len(catalog.tables)):
        for z in (0.0, 0.8):
            q = serving.Query(0, table, z)
            _same(serving.execute(ctx, stream, catalog, q, fused=True),
                  serving.execute(ctx, stream, catalog, q, fused=False))


def test_short_first_policy_serves_everything_with_same_results(ctx, catalog):
    fifo = serving.Server(ctx, catalog, slots=1, budget_bytes=150 << 30)
    short = serving.Server(ctx, catalog, slots=4, budget_bytes=150 << 30, policy="short-first",
                           max_wait=0.01, urgent_below=1 << 22)
    try:
        qa = fifo.run(_queries(24))
        qb = short.run(_queries(24))
    finally:
        fifo.close(); short.close()
    assert all(q.error is None and q.end is not None for q in qb)
    for a, b in zip(qa, qb):
        _same(a.result, b.result)


def test_warm_start_from_table_images(ctx, catalog, tmp_path):
    # The catalog's tables written as images and a second catalog loaded from
    # them (no builds): every query gives the same groups and sums.
    catalog.save(str(tmp_path))
    warm = serving.Catalog(ctx, [10_000, 31_000, 100_000, 320_000, 1_000_000], images=str(tmp_path))
    try:
        for q in _queries(10):
            _same(serving.execute(ctx, ctx.stream, warm, q), serving.execute(ctx, ctx.stream, catalog, q))
    finally:
        warm.close()
    with pytest.raises(gpu.PgError):
        serving.Catalog(ctx, [10_000], images=str(tmp_path / "missing"))
