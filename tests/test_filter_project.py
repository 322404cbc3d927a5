"""Filter and Project on the GPU against the oracle (filter.cpp:37-85,
project.cpp:37-104), and the filter fused into the join probe as its
prologue (pg_hashjoin_probe_where) against filter-then-join.

Every filter output must equal the oracle's byte for byte, in input order
(the reference Filter keeps the order of each thread's input). The mixed
relation covers int, long (4-byte aligned), dec with NaN / signed zeros /
infinities, char with shared prefixes and bytes above 0x7f, and packed dates;
the oracle itself is pinned to the reference's Filter and Project by the
golden cases (tests/golden/golden.json, op filter / project).
"""
import numpy as np
import pytest

from oracle import oracle as orc
from pythia_gb300 import datagen as dg
from pythia_gb300 import gpu
from pythia_gb300 import plans
from tests.golden import inputs as gin

pytestmark = pytest.mark.gpu
SCHEMA = gin.MIXED_SCHEMA
W = gin.MIXED_WIDTH


def canon(a):
    return orc.canonical(np.ascontiguousarray(a))


def mixed(n):
    return gin.make({"gen": "formula", "name": "mixed_cols", "n": n})


FILTERS = [
    [(0, "<", "0")], [(0, "=", "7")], [(0, "<>", "-3")], [(1, ">=", "0")], [(1, "==", str(17 * (1 << 31)))],
    [(2, "<", "0")], [(2, "==", "0")], [(2, "!=", "nan")], [(2, ">", "-inf")], [(2, "<=", "inf")],
    [(3, "=", "abc")], [(3, "<", "alpha")], [(3, ">", "ab")], [(3, "<>", "")], [(3, ">=", "abc\xe9")],
    [(3, "==", "delta epsilon")], [(4, "<", "1995-03-15")], [(4, "==", "1994-06-10")],
    [(0, ">", "-5"), (2, "<", "30"), (3, "!=", "zz")],
    [(4, ">=", "1994-01-01"), (4, "<", "1995-01-01"), (1, ">=", "0"), (0, "<>", "0")],
]


@pytest.mark.parametrize("k", range(len(FILTERS)))
def test_filter_matches_oracle_in_order(ctx, k):
    rows = mixed(20_011)
    spec = gin.filter_preds(SCHEMA, FILTERS[k])
    got = ctx.filter(rows, spec)
    want = orc.filter(rows, spec)
    assert got.shape == want.shape
    assert np.array_equal(got, want)


@pytest.mark.parametrize("n", [0, 1, 2047, 2048, 2049, 100_003])
def test_filter_sizes_and_16_byte_tuples(ctx, n):
    # 16-byte tuples take the vector copy; ragged tile edges; none / all pass.
    rows = dg.uniform_keys(n, 1000, dg.seed_for(501)) if n else np.zeros((0, 2), np.int64)
    for spec in ([("long", "<", 0, 500)], [("long", "<", 0, -1)], [("long", ">=", 0, 0)],
                 [("long", ">", 8, 1 << 30), ("long", "<", 0, 900)]):
        got = ctx.filter(rows, spec)
        assert np.array_equal(got, orc.filter(rows, spec))


def test_filter_12_byte_tuples(ctx):
    # Widths that are multiples of 4 but not of 16 copy word by word.
    a = (dg.raw_words(dg.seed_for(502), 0, 3 * 50_000) % 1000).astype(np.int32).reshape(-1, 3)
    spec = [("int", ">=", 4, 250), ("int", "!=", 8, 7)]
    assert np.array_equal(ctx.filter(a, spec), orc.filter(a, spec))


@pytest.mark.parametrize("proj", ["3,0", "4,2,1", "0,0,1", "2", "1,4,3,2,0"])
def test_project_matches_oracle(ctx, proj):
    rows = mixed(30_007)
    cols = gin.schema_columns(SCHEMA)
    spec = [(cols[int(i)][1], cols[int(i)][2]) for i in proj.split(",")]
    assert np.array_equal(ctx.project(rows, spec), orc.project(rows, spec))


def test_filter_rejects_bad_predicates(ctx):
    rows = mixed(100)
    for spec in ([("long", "<", 36, 0)],            # runs past the tuple
                 [("int", "<", 2, 0)],              # not 4-byte aligned
                 [("char", "<", 20, "a", 200)]):    # wider than 128 bytes
        with pytest.raises(gpu.PgError):
            ctx.filter(rows, spec)


# ---------------------------------------------------------------- fused probe
def _where_check(ctx, R, S, where, proj=(("P", 8, 8), ("B", 8, 8)), out_cap=None):
    t = ctx.build_table(R, proj)
    try:
        got, n, _ = t.probe(S, where=where, out_cap=out_cap)
        _, n2, s2 = t.probe(S, where=where, flags=gpu.JOIN_COUNT | gpu.JOIN_SUM, sum_col=len(proj) - 1)
    finally:
        t.free()
    Sf = orc.filter(S, where)
    want, wn, _ = orc.hashjoin(R, Sf, proj=proj, hash=orc.hashcfg("modulo", 1 << 12))
    _, wn2, ws2 = orc.hashjoin(R, Sf, proj=proj, materialise=False, sum_col=len(proj) - 1,
                               hash=orc.hashcfg("modulo", 1 << 12))
    assert n == wn and (n2, s2) == (wn2, ws2)
    assert np.array_equal(canon(got), canon(want))
    return n


@pytest.mark.parametrize("where", [[("long", "<", 8, 1 << 30)], [("long", ">=", 0, 5000), ("long", "<", 0, 60_000)],
                                   [("int", "<", 8, 1 << 29)], [("dec", ">", 8, 0.5)]])
def test_probe_where_fused_dense(ctx, where):
    # 16-byte probe tuples on dense tables: the predicates run in the probe
    # kernel (narrow table: the deep pipeline for (P$1, B$1) rows).
    R = dg.build_relation(80_000, dg.seed_for(503))
    S = dg.probe_uniform(900_001, R, dg.seed_for(504))
    S[::41, 0] += 200_000
    if where[0][0] == "dec":
        raw = dg.raw_words(dg.seed_for(505), 1, S.shape[0]) >> np.uint64(11)
        S[:, 1] = (raw.astype(np.float64) / 2.0 ** 53).view(np.int64)
    n = _where_check(ctx, R, S, where)
    assert 0 < n < S.shape[0]
    Rw = R.copy()
    Rw[:, 1] = dg.raw_words(dg.seed_for(503), 1, R.shape[0]).view(np.int64)      # wide dense table
    _where_check(ctx, Rw, S, where)
    _where_check(ctx, R, S, where, proj=(("B", 8, 8), ("P", 0, 8)))              # other word order


def test_probe_where_unfused_cases(ctx):
    # Hashed tables, char predicates, wider tuples and a small output buffer
    # filter the probe side first: same rows.
    R = dg.build_relation(20_000, dg.seed_for(506))
    S = dg.probe_uniform(150_000, R, dg.seed_for(507))
    Rh = R.copy(); Rh[:, 0] *= 7
    Sh = S.copy(); Sh[:, 0] *= 7
    _where_check(ctx, Rh, Sh, [("long", "<", 8, 1 << 30)])
    n_all = _where_check(ctx, R, S, [("long", "<", 8, 1 << 29)])
    _where_check(ctx, R, S, [("long", "<", 8, 1 << 29)], out_cap=n_all)
    # A 40-byte mixed probe side joined on its long column.
    M = mixed(60_000)
    keys = (np.arange(60_000) % 20_000 + 1).astype(np.int64)
    M[:, 4:12] = keys.view(np.uint8).reshape(-1, 8)
    t = ctx.build_table(R, (("P", 0, 4), ("B", 8, 8)))
    where = gin.filter_preds(SCHEMA, [(3, ">=", "b"), (2, "!=", "nan")])
    try:
        got, n, _ = t.probe(M, pkey=(4, 8), proj=(("P", 0, 4), ("B", 8, 8)), where=where)
    finally:
        t.free()
    Mf = orc.filter(M, where)
    want, wn, _ = orc.hashjoin(R, Mf, proj=(("P", 0, 4), ("B", 8, 8)), pkey=(4, 8),
                               hash=orc.hashcfg("modulo", 1 << 12))
    assert n == wn and np.array_equal(canon(got), canon(want))


# ---------------------------------------------------------------- operator layer
def test_gpufilter_and_gpuproject_operators():
    rows = mixed(40_000)
    plans.register("M", rows)
    base = '''
    buffsize = 4096;
    scan = { type = "memscan"; relation = "M"; schema = ("int", "long", "dec", "char(11)", "date(%Y-%m-%d)"); };
    '''
    # Filter over filter (fused into one pass), each thread its own slice.
    plan = base + '''
    treeroot = { name = "f2"; input = { name = "f1"; input = { name = "scan"; }; }; };
    f1 = { type = "gpufilter"; field = 3; op = ">="; value = "alpha"; };
    f2 = { type = "gpufilter"; field = 4; op = "<"; value = "1996-01-01"; };
    '''
    got, per = plans.run(plan, threads=4)
    spec = gin.filter_preds(SCHEMA, [(3, ">=", "alpha"), (4, "<", "1996-01-01")])
    parts = [orc.filter(rows[a:b], spec) for a, b in [(40_000 * t // 4, 40_000 * (t + 1) // 4) for t in range(4)]]
    assert per == [p.shape[0] for p in parts]
    assert np.array_equal(got, np.concatenate(parts))          # thread order, input order
    # Project alone.
    plan = base + '''
    treeroot = { name = "p"; input = { name = "scan"; }; };
    p = { type = "gpuproject"; projection = ("$4", "$0"); };
    '''
    got, _ = plans.run(plan, threads=3)
    assert np.array_equal(got, orc.project(rows, [(32, 8), (0, 4)]))


def test_filter_fused_into_join_probe_and_project_folded_into_join():
    R = dg.build_relation(50_000, dg.seed_for(508))
    S = dg.probe_uniform(400_000, R, dg.seed_for(509))
    S[::29, 0] += 100_000
    plans.register("R", R); plans.register("S", S)
    plan = '''
    buffsize = 8192;
    treeroot = { name = "proj"; input = { name = "join"; build = { name = "r"; }; probe = { name = "flt"; input = { name = "s"; }; }; }; };
    r = { type = "memscan"; relation = "R"; schema = ("long", "long"); };
    s = { type = "memscan"; relation = "S"; schema = ("long", "long"); };
    flt = { type = "gpufilter"; field = 1; op = "<"; value = "1000000000"; };
    join = { type = "gpuhashjoin"; buildjattr = 0; probejattr = 0; projection = ("P$0", "P$1", "B$1");
             threadgroups = ((0, 1, 2, 3)); hash = { fn = "modulo"; buckets = 1024; }; tuplesperbucket = 4; };
    proj = { type = "gpuproject"; projection = ("$1", "$2"); };
    '''
    where = [("long", "<", 8, 1_000_000_000)]
    want, n, _ = orc.hashjoin(R, orc.filter(S, where), proj=(("P", 8, 8), ("B", 8, 8)),
                              hash=orc.hashcfg("modulo", 1 << 12))
    for on in (True, False):
        plans.set_device_exchange(on)
        try:
            plans.transfer_stats(reset=True)
            got, per = plans.run(plan, threads=4)
            st = plans.transfer_stats(reset=True)
        finally:
            plans.set_device_exchange(True)
        assert sum(per) == n
        assert np.array_equal(canon(got), canon(want))
        if on:
            # Fused: the filter's input goes up once and only the projected
            # 16-byte rows come down.
            assert st["h2d"] == R.nbytes + S.nbytes and st["d2h"] == n * 16
