"""Device-resident exchange between adjacent GPU operators in plans.

A GPU operator under a GPU parent keeps its output on the device and the
parent's threads take their shares there (the parent's group launch reads
them in place, or gathers them with device copies when they are not
adjacent). Every plan runs twice, with the exchange on and off (host pages
between operators), and must give the same rows, equal to the oracle's; the
operator layer's transfer counters show what crossed the host link: with the
exchange on, only the leaves' pages go up and only the top operator's output
comes back. Plans follow the reference's multi-operator shapes: partition ->
join (PartitionOp under HashJoinOp) and q1's join -> join -> aggregate
(drivers/sample_queries/q1/query1.conf:115-166).
"""
import numpy as np
import pytest

from oracle import oracle as orc
from pythia_gb300 import datagen as dg
from pythia_gb300 import plans

pytestmark = pytest.mark.gpu
DEC_RTOL = 1e-12


def canon(a):
    return orc.canonical(np.ascontiguousarray(a))


def run_both(plan, threads):
    """(rows, per-thread counts, transfer counters) with the exchange on, then off."""
    out = []
    for on in (True, False):
        plans.set_device_exchange(on)
        try:
            plans.transfer_stats(reset=True)
            rows, per = plans.run(plan, threads=threads)
            out.append((rows, per, plans.transfer_stats(reset=True)))
        finally:
            plans.set_device_exchange(True)
    return out


PART_JOIN = '''
buffsize = 8192;
treeroot = {{ name = "join"; build = {{ name = "pr"; input = {{ name = "r"; }}; }};
                            probe = {{ name = "ps"; input = {{ name = "s"; }}; }}; }};
r = {{ type = "memscan"; relation = "R"; schema = ("long", "long"); }};
s = {{ type = "memscan"; relation = "S"; schema = ("long", "long"); }};
pr = {{ type = "gpupartition"; attr = 0; range = (1, {hi}); buckets = 4; sort = "no"; }};
ps = {{ type = "gpupartition"; attr = 0; range = (1, {hi}); buckets = 4; sort = "no"; }};
join = {{ type = "{jtype}"; buildjattr = 0; probejattr = 0; projection = ("P$1", "B$1");
         threadgroups = {groups}; hash = {{ fn = "modulo"; buckets = 1024; }}; tuplesperbucket = 4; }};
'''


@pytest.mark.parametrize("jtype", ["gpuhashjoin", "gpumpsmjoin"])
def test_partition_join_exchange_on_device(jtype):
    R = dg.build_relation(20_000, dg.seed_for(401))
    S = dg.probe_uniform(90_000, R, dg.seed_for(402))
    plans.register("R", R); plans.register("S", S)
    plan = PART_JOIN.format(hi=20_000, jtype=jtype, groups="((0), (1), (2), (3))")
    (rows_on, per_on, st_on), (rows_off, per_off, st_off) = run_both(plan, 4)
    want, n, _ = orc.hashjoin(R, S, proj=(("P", 8, 8), ("B", 8, 8)), hash=orc.hashcfg("modulo", 1 << 12))
    assert sum(per_on) == sum(per_off) == n == 90_000
    assert per_on == per_off                      # thread t joins partition t either way
    assert np.array_equal(canon(rows_on), canon(want))
    assert np.array_equal(canon(rows_off), canon(want))
    out_bytes = n * 16
    # On: the leaves go up once, the join's rows come down once, and each of
    # the 4 join groups takes both inputs in place.
    assert st_on["h2d"] == R.nbytes + S.nbytes
    assert st_on["d2h"] == out_bytes
    assert st_on["d2d"] == 0 and st_on["in_place"] == 8
    # Off: the partitions' outputs make the round trip as well.
    assert st_off["h2d"] == 2 * (R.nbytes + S.nbytes)
    assert st_off["d2h"] == R.nbytes + S.nbytes + out_bytes
    assert st_off["in_place"] == 0


def test_non_adjacent_shares_are_gathered_on_device():
    # Groups (0, 2) and (1, 3): partitions 0 and 2 are not neighbours in the
    # partition output, so the join gathers them with device copies.
    R = dg.build_relation(16_000, dg.seed_for(403))
    S = dg.probe_uniform(70_000, R, dg.seed_for(404))
    plans.register("R", R); plans.register("S", S)
    plan = PART_JOIN.format(hi=16_000, jtype="gpuhashjoin", groups="((0, 2), (1, 3))")
    (rows_on, per_on, st_on), (rows_off, _, st_off) = run_both(plan, 4)
    want, n, _ = orc.hashjoin(R, S, proj=(("P", 8, 8), ("B", 8, 8)), hash=orc.hashcfg("modulo", 1 << 12))
    assert sum(per_on) == n
    assert np.array_equal(canon(rows_on), canon(want))
    assert np.array_equal(canon(rows_off), canon(want))
    assert st_on["d2d"] == R.nbytes + S.nbytes
    assert st_on["h2d"] == R.nbytes + S.nbytes and st_on["d2h"] == n * 16


def test_many_to_many_join_on_device_grows_its_output():
    # Repeated keys on both sides: the device join's first output guess (|S|
    # rows) is too small and is grown once, as on the host path.
    R = dg.uniform_keys(6000, 400, dg.seed_for(405))
    S = dg.uniform_keys(9000, 400, dg.seed_for(406))
    R[:, 0] += 1; S[:, 0] += 1
    plans.register("R", R); plans.register("S", S)
    plan = PART_JOIN.format(hi=400, jtype="gpuhashjoin", groups="((0, 1, 2, 3))")
    (rows_on, _, st_on), (rows_off, _, _) = run_both(plan, 4)
    want, n, _ = orc.hashjoin(R, S, proj=(("P", 8, 8), ("B", 8, 8)), hash=orc.hashcfg("modulo", 1 << 12))
    assert n > S.shape[0]
    assert np.array_equal(canon(rows_on), canon(want))
    assert np.array_equal(canon(rows_off), canon(want))
    assert st_on["in_place"] == 2


Q1_SHAPE = '''
buffsize = 16384;
treeroot = { name = "sum"; input = { name = "joinO"; build = { name = "scanO"; };
             probe = { name = "joinP"; build = { name = "scanP"; }; probe = { name = "scanL"; }; }; }; };
scanO = { type = "memscan"; relation = "O"; schema = ("long", "long"); };
scanP = { type = "memscan"; relation = "P"; schema = ("long", "long"); };
scanL = { type = "memscan"; relation = "L"; schema = ("long", "long", "dec"); };
joinP = { type = "gpuhashjoin"; buildjattr = 0; probejattr = 1; projection = ("P$0", "P$2", "B$1");
          threadgroups = ((0, 1, 2, 3)); hash = { fn = "modulo"; buckets = 1024; }; tuplesperbucket = 4; };
joinO = { type = "gpuhashjoin"; buildjattr = 0; probejattr = 0; projection = ("B$1", "P$1");
          threadgroups = ((0, 1, 2, 3)); hash = { fn = "modulo"; buckets = 1024; }; tuplesperbucket = 4; };
sum = { type = "gpuaggregate_sum"; field = 0; sumfield = 1; global = true; threads = 4; };
'''


def _q1_inputs():
    nO, nP, nL = 50_000, 20_000, 400_000
    O = dg.build_relation(nO, dg.seed_for(407))
    O[:, 1] = O[:, 0] % 97                                   # the group of an order
    P = dg.build_relation(nP, dg.seed_for(408))
    lo = dg.probe_uniform(nL, O, dg.seed_for(409))
    lp = dg.probe_uniform(nL, P, dg.seed_for(410))
    L = np.zeros((nL, 3), np.int64)
    L[:, 0] = lo[:, 0]
    L[:, 1] = lp[:, 0]
    L[:, 2] = ((dg.raw_words(dg.seed_for(411), 2, nL) >> np.uint64(11)).astype(np.float64) * 1e-9).view(np.int64)
    L[::37, 1] += nP                                         # lines whose part is missing
    return O, P, L


def test_q1_shaped_join_join_aggregate():
    O, P, L = _q1_inputs()
    plans.register("O", O); plans.register("P", P); plans.register("L", L)
    (rows_on, _, st_on), (rows_off, _, st_off) = run_both(Q1_SHAPE, 4)
    jp, _, _ = orc.hashjoin(P, L, proj=(("P", 0, 8), ("P", 16, 8), ("B", 8, 8)), pkey=(8, 8),
                            hash=orc.hashcfg("modulo", 1 << 12))
    jo, _, _ = orc.hashjoin(O, jp.view(np.int64).reshape(-1, 3), proj=(("B", 8, 8), ("P", 8, 8)),
                            hash=orc.hashcfg("modulo", 1 << 12))
    want = canon(orc.groupby_exact(jo.view(np.int64).reshape(-1, 2)))
    for rows in (rows_on, rows_off):
        got = canon(rows)
        assert np.array_equal(got[:, :8], want[:, :8])
        g, e = got[:, 8:].copy().view(np.float64).ravel(), want[:, 8:].copy().view(np.float64).ravel()
        assert np.all(np.abs(g - e) <= DEC_RTOL * np.abs(e))
    # On: the three leaves go up, 97 groups come down; both joins' outputs stay.
    assert st_on["h2d"] == O.nbytes + P.nbytes + L.nbytes
    assert st_on["d2h"] == rows_on.nbytes
    assert st_on["in_place"] == 2
    nP_rows = jp.shape[0]
    nO_rows = jo.shape[0]
    assert st_off["h2d"] == O.nbytes + P.nbytes + L.nbytes + nP_rows * 24 + nO_rows * 16
    assert st_off["d2h"] == nP_rows * 24 + nO_rows * 16 + rows_off.nbytes


def test_thread_local_aggregate_over_device_join():
    # Each thread aggregates its own share of the join's device output; the
    # shares cover the join exactly once.
    R = dg.build_relation(30_000, dg.seed_for(412))
    R[:, 1] = R[:, 0] % 50
    S = dg.probe_uniform(200_000, R, dg.seed_for(413))
    plans.register("R", R); plans.register("S", S)
    plan = '''
    buffsize = 4096;
    treeroot = { name = "cnt"; input = { name = "join"; build = { name = "r"; }; probe = { name = "s"; }; }; };
    r = { type = "memscan"; relation = "R"; schema = ("long", "long"); };
    s = { type = "memscan"; relation = "S"; schema = ("long", "long"); };
    join = { type = "gpuhashjoin"; buildjattr = 0; probejattr = 0; projection = ("B$1", "P$1");
             threadgroups = ((0, 1, 2, 3)); hash = { fn = "modulo"; buckets = 1024; }; tuplesperbucket = 4; };
    cnt = { type = "gpuaggregate_count"; field = 0; };
    '''
    (rows_on, _, st_on), (rows_off, _, _) = run_both(plan, 4)
    for rows in (rows_on, rows_off):
        g = rows.view(np.int64).reshape(-1, 2)
        tot = np.zeros(50, np.int64)
        np.add.at(tot, g[:, 0], g[:, 1])
        assert tot.sum() == 200_000
        assert np.array_equal(tot, np.bincount(S[:, 0] % 50, minlength=50))
    assert st_on["in_place"] == 4 and st_on["d2d"] == 0


def test_pinned_leaves_copy_to_the_device_directly():
    # Relations in registered memory (a loader that reads into pinned memory):
    # their pages go to the device without the staging copy; same rows.
    R = dg.build_relation(20_000, dg.seed_for(414))
    S = dg.probe_uniform(90_000, R, dg.seed_for(415))
    plan = PART_JOIN.format(hi=20_000, jtype="gpuhashjoin", groups="((0), (1), (2), (3))")
    want, n, _ = orc.hashjoin(R, S, proj=(("P", 8, 8), ("B", 8, 8)), hash=orc.hashcfg("modulo", 1 << 12))
    try:
        plans.register("R", R, pin=True); plans.register("S", S, pin=True)
        plans.transfer_stats(reset=True)
        rows, per = plans.run(plan, threads=4)
        st = plans.transfer_stats(reset=True)
    finally:
        plans.register("R", R); plans.register("S", S)      # unpins
    assert sum(per) == n
    assert np.array_equal(canon(rows), canon(want))
    assert st["h2d"] == R.nbytes + S.nbytes == st["direct"]


def test_ordinary_pages_go_in_place_where_the_device_reads_host_memory():
    # Pages of an ordinary (pageable) relation are uploaded by the SMs' loads
    # when the device reads pageable memory (GB300 over NVLink-C2C), and are
    # staged through pinned buffers otherwise; the rows are the same.
    from pythia_gb300 import gpu
    R = dg.build_relation(20_000, dg.seed_for(416))
    S = dg.probe_uniform(90_000, R, dg.seed_for(417))
    plans.register("R", R); plans.register("S", S)
    plan = PART_JOIN.format(hi=20_000, jtype="gpuhashjoin", groups="((0), (1), (2), (3))")
    want, n, _ = orc.hashjoin(R, S, proj=(("P", 8, 8), ("B", 8, 8)), hash=orc.hashcfg("modulo", 1 << 12))
    plans.transfer_stats(reset=True)
    rows, per = plans.run(plan, threads=4)
    st = plans.transfer_stats(reset=True)
    assert sum(per) == n and np.array_equal(canon(rows), canon(want))
    ctx = gpu.Context(0)
    try:
        readable = gpu.lib().pg_host_readable(ctx.h, S.ctypes.data) == 1
    finally:
        ctx.close()
    assert st["h2d"] == R.nbytes + S.nbytes
    assert st["direct"] == (st["h2d"] if readable else 0)


def test_join_over_join_reads_only_the_columns_it_uses():
    # The parent joins on the child's third column and projects its first;
    # the child's second column is dropped on the device (column pruning)
    # and the parent's key is remapped. Same rows with the exchange off.
    nR, nT = 30_000, 5_000
    R = dg.build_relation(nR, dg.seed_for(418))
    R[:, 1] = R[:, 0] % nT + 1
    T = dg.build_relation(nT, dg.seed_for(419))
    S = dg.probe_uniform(120_000, R, dg.seed_for(420))
    plans.register("R", R); plans.register("S", S); plans.register("T", T)
    plan = """
    buffsize = 8192;
    treeroot = { name = "jb"; build = { name = "t"; }; probe = { name = "ja"; build = { name = "r"; }; probe = { name = "s"; }; }; };
    r = { type = "memscan"; relation = "R"; schema = ("long", "long"); };
    s = { type = "memscan"; relation = "S"; schema = ("long", "long"); };
    t = { type = "memscan"; relation = "T"; schema = ("long", "long"); };
    ja = { type = "gpuhashjoin"; buildjattr = 0; probejattr = 0; projection = ("P$0", "P$1", "B$1");
           threadgroups = ((0, 1, 2, 3)); hash = { fn = "modulo"; buckets = 1024; }; tuplesperbucket = 4; };
    jb = { type = "gpuhashjoin"; buildjattr = 0; probejattr = 2; projection = ("P$0", "B$1");
           threadgroups = ((0, 1, 2, 3)); hash = { fn = "modulo"; buckets = 1024; }; tuplesperbucket = 4; };
    """
    ja, _, _ = orc.hashjoin(R, S, proj=(("P", 0, 8), ("P", 8, 8), ("B", 8, 8)), hash=orc.hashcfg("modulo", 1 << 12))
    want, n, _ = orc.hashjoin(T, ja.view(np.int64).reshape(-1, 3), proj=(("P", 0, 8), ("B", 8, 8)), pkey=(16, 8),
                              hash=orc.hashcfg("modulo", 1 << 12))
    assert n == 120_000
    (rows_on, _, st_on), (rows_off, _, st_off) = run_both(plan, 4)
    assert np.array_equal(canon(rows_on), canon(want))
    assert np.array_equal(canon(rows_off), canon(want))
    assert st_on["in_place"] == 1 and st_on["d2h"] == n * 16            # jb takes ja's rows in place
    # Off, the child's rows travel whole: 24 bytes each, down and up again.
    assert st_off["d2h"] == 120_000 * 24 + n * 16
