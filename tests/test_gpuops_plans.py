"""GPU operators inside plans (C++ operator layer, mirror of the engine's
operator interface): the same scenarios the reference's query tests run with
the CPU operator types, with gpu* types substituted and checked against the
oracle. Threads read consecutive slices of each memscan relation; thread
groups, page sizes, partition-to-thread assignment and thread-local versus
global aggregation follow the engine's contracts."""
import numpy as np
import pytest

from oracle import oracle as orc
from pythia_gb300 import datagen as dg
from pythia_gb300 import plans

pytestmark = pytest.mark.gpu
DEC_RTOL = 1e-12


def canon(a):
    return orc.canonical(np.ascontiguousarray(a))


def slices(n, threads):
    return [(n * t // threads, n * (t + 1) // threads) for t in range(threads)]


def join_plan(jtype, groups, projection='("P$1", "B$1")', buffsize=4096, bschema='("long", "long")',
              pschema='("long", "long")', extra=""):
    return f'''
    buffsize = {buffsize};
    treeroot = {{ name = "join"; build = {{ name = "r"; }}; probe = {{ name = "s"; }}; }};
    r = {{ type = "memscan"; relation = "R"; schema = {bschema}; }};
    s = {{ type = "memscan"; relation = "S"; schema = {pschema}; }};
    join = {{ type = "{jtype}"; buildjattr = 0; probejattr = 0; projection = {projection};
             threadgroups = {groups}; hash = {{ fn = "modulo"; buckets = 1024; }}; tuplesperbucket = 4; {extra} }};
    '''


@pytest.mark.parametrize("jtype", ["gpuhashjoin", "gpumpsmjoin"])
def test_join_one_group_pkfk(jtype):
    R = dg.build_relation(30_000, dg.seed_for(71))
    S = dg.probe_uniform(250_000, R, dg.seed_for(72))
    plans.register("R", R); plans.register("S", S)
    rows, per = plans.run(join_plan(jtype, "((0, 1, 2, 3))"), threads=4)
    want, n, _ = orc.hashjoin(R, S, proj=(("P", 8, 8), ("B", 8, 8)), hash=orc.hashcfg("modulo", 1 << 12))
    assert rows.shape == (n, 16) and sum(per) == n
    assert max(per) - min(per) <= 1                      # the group's rows spread evenly
    assert np.array_equal(canon(rows), canon(want))


@pytest.mark.parametrize("jtype", ["gpuhashjoin", "gpumpsmjoin"])
def test_join_two_groups_join_their_own_inputs(jtype):
    # Group (0, 1) joins the rows threads 0 and 1 read, group (2, 3) the rest:
    # keys the two halves share must not meet across groups.
    R = dg.uniform_keys(4000, 500, dg.seed_for(73))
    S = dg.uniform_keys(6000, 500, dg.seed_for(74))
    plans.register("R", R); plans.register("S", S)
    rows, per = plans.run(join_plan(jtype, "((0, 1), (2, 3))", projection='("B$0", "B$1", "P$1")'), threads=4)
    proj = (("B", 0, 8), ("B", 8, 8), ("P", 8, 8))
    halves = []
    for (r0, r1), (s0, s1) in zip([(0, 2000), (2000, 4000)], [(0, 3000), (3000, 6000)]):
        w, _, _ = orc.hashjoin(R[r0:r1], S[s0:s1], proj=proj, hash=orc.hashcfg("modulo", 1 << 10))
        halves.append(w)
    g0 = sum(per[:2])
    assert g0 == halves[0].shape[0] and sum(per[2:]) == halves[1].shape[0]
    assert np.array_equal(canon(rows[:g0]), canon(halves[0]))
    assert np.array_equal(canon(rows[g0:]), canon(halves[1]))


@pytest.mark.parametrize("sort_r,sort_s", [(True, True), (True, False)])
def test_mpsm_plan_presorted_keys(sort_r, sort_s):
    # buildpresorted / probepresorted = "yes" (join.cpp:750-762) on a
    # gpumpsmjoin: sorted relations skip the device's sort or partition; a
    # side declared sorted that is not (sort_s False: S shuffled) still joins
    # right. The run-size, buffer and range keys are accepted and change
    # nothing.
    R = dg.uniform_keys(40_000, 1 << 18, dg.seed_for(75))
    S = dg.uniform_keys(90_000, 1 << 18, dg.seed_for(76))
    if sort_r:
        R = R[np.argsort(R[:, 0], kind="stable")]
    if sort_s:
        S = S[np.argsort(S[:, 0], kind="stable")]
    plans.register("R", R); plans.register("S", S)
    extra = ('buildpresorted = "yes"; probepresorted = "yes"; maxbuildtuplesinM = 1; maxprobetuplesinM = 1; '
             'mostfreqbuildkeyoccurances = 16; buildprepartitioned = { range = [0, 262143]; buckets = 2; };')
    rows, per = plans.run(join_plan("gpumpsmjoin", "((0, 1))", extra=extra), threads=2)
    want, n, _ = orc.mergejoin(R, S)
    assert rows.shape == (n, 16) and sum(per) == n
    assert np.array_equal(canon(rows), canon(want))


def test_hashjoin_reference_unit_scenario():
    # The reference's hash join test: build keys 1..20 with payload k + 0.1
    # (dec), probe keys 1..20 (int-valued long payload), projection
    # (P$0, B$1): every key once, with the matching decimal.
    N = 20
    R = np.zeros(N, dtype=[("k", "<i8"), ("d", "<f8")]); R["k"] = np.arange(1, N + 1); R["d"] = R["k"] + 0.1
    S = np.zeros((N, 2), np.int64); S[:, 0] = np.arange(1, N + 1); S[:, 1] = S[:, 0]
    plans.register("R", R.view(np.uint8).reshape(N, 16)); plans.register("S", S)
    rows, _ = plans.run(join_plan("gpuhashjoin", "((0, 1, 2, 3))", projection='("P$0", "B$1")', buffsize=16,
                                  bschema='("long", "dec")'), threads=4)
    out = rows.view(np.uint8).reshape(-1, 16)
    k = out[:, :8].copy().view(np.int64).ravel()
    d = out[:, 8:].copy().view(np.float64).ravel()
    assert sorted(k.tolist()) == list(range(1, N + 1))
    assert np.all(d == k + 0.1)


def part_plan(extra, buffsize=4096):
    return f'''
    buffsize = {buffsize};
    treeroot = {{ name = "part"; input = {{ name = "scan"; }}; }};
    scan = {{ type = "memscan"; relation = "R"; schema = ("long", "long"); }};
    part = {{ type = "gpupartition"; attr = 0; {extra} maxtuples = 1000000; }};
    '''


def test_partition_exactrange_bit_exact_with_order():
    R = dg.uniform_keys(100_000, 1000, dg.seed_for(75))
    R[:, 0] += 1
    plans.register("R", R)
    rows, per = plans.run(part_plan('range = (1, 1000); buckets = 4; sort = "no";'), threads=4)
    want, offs = orc.partition(R, orc.hashcfg("exactrange", 4, 1, 1000))
    assert per == [int(offs[t + 1] - offs[t]) for t in range(4)]
    assert np.array_equal(rows.view(np.int64).reshape(-1, 2), want)      # order included


def test_partition_radix_and_sorted_partitions():
    R = dg.uniform_keys(80_000, 1 << 20, dg.seed_for(76))
    plans.register("R", R)
    rows, per = plans.run(part_plan('fn = "parammodulo"; buckets = 8; skipbits = 4; sort = "no";'), threads=8)
    want, offs = orc.partition(R, orc.hashcfg("parammodulo", 8, skipbits=4))
    assert np.array_equal(rows.view(np.int64).reshape(-1, 2), want)
    rows, per = plans.run(part_plan('fn = "parammodulo"; buckets = 8; skipbits = 4; sort = "yes"; sortattr = 0;'),
                          threads=8)
    got = rows.view(np.int64).reshape(-1, 2)
    at = 0
    for t in range(8):
        seg, ref = got[at:at + per[t]], want[offs[t]:offs[t + 1]]
        assert np.all(np.diff(seg[:, 0]) >= 0)
        assert np.array_equal(canon(seg), canon(ref))
        at += per[t]


def agg_plan(atype, keys, extra="", schema='("long", "dec")'):
    return f'''
    buffsize = 4096;
    treeroot = {{ name = "agg"; input = {{ name = "scan"; }}; }};
    scan = {{ type = "memscan"; relation = "R"; schema = {schema}; }};
    agg = {{ type = "{atype}"; {keys} {extra} }};
    '''


def test_aggregate_sum_global_dec():
    G = dg.groupby_rows(200_000, 3000, 1e4, dg.seed_for(77))
    plans.register("R", G)
    rows, per = plans.run(agg_plan("gpuaggregate_sum", "field = 0; sumfield = 1;", "global = true; threads = 4;"),
                          threads=4)
    assert max(per) - min(per) <= 1
    got = canon(rows)
    exact = canon(orc.groupby_exact(G))
    assert np.array_equal(got[:, :8], exact[:, :8])
    g, e = got[:, 8:].copy().view(np.float64).ravel(), exact[:, 8:].copy().view(np.float64).ravel()
    assert np.all(np.abs(g - e) <= DEC_RTOL * np.abs(e))


def test_aggregate_more_groups_than_its_first_output_room():
    # 1.2M groups: more than the 1M rows of output room a GPU aggregate starts
    # with; the operator reruns with room for the count pg_groupby reported.
    n, groups = 1_500_000, 1_200_000
    R = dg.uniform_keys(n, groups, dg.seed_for(79))
    R[:, 0] = np.arange(n, dtype=np.int64) * 7919 % groups          # exactly 1.2M keys
    plans.register("R", R)
    rows, _ = plans.run(agg_plan("gpuaggregate_sum", "field = 0; sumfield = 1;", "global = true; threads = 4;",
                                 schema='("long", "long")'), threads=4)
    want = orc.groupby(R, key=(0, 8), val=(8, "long"), agg="sum", hash=orc.hashcfg("modulo", 1 << 20))
    assert rows.shape[0] == want.shape[0] > (1 << 20)
    assert np.array_equal(canon(rows), canon(want))


def test_aggregate_thread_local_each_thread_its_own_groups():
    R = dg.uniform_keys(50_000, 700, dg.seed_for(78))
    plans.register("R", R)
    rows, per = plans.run(agg_plan("gpuaggregate_sum", "field = 0; sumfield = 1;", schema='("long", "long")'),
                          threads=3)
    at = 0
    for t, (a, b) in enumerate(slices(50_000, 3)):
        want = orc.groupby(R[a:b], key=(0, 8), val=(8, "long"), agg="sum")
        assert np.array_equal(canon(rows[at:at + per[t]]), canon(want))
        at += per[t]


def test_aggregate_count_and_sum_global_no_key():
    # The reference's global aggregate tests: values 1..N, no GROUP BY:
    # count N and sum N (N + 1) / 2.
    N = 10_000
    R = np.zeros((N, 2), np.int64); R[:, 0] = np.arange(1, N + 1); R[:, 1] = R[:, 0]
    plans.register("R", R)
    rows, per = plans.run(agg_plan("gpuaggregate_count", "fields = ();", "global = true; threads = 2;",
                                   schema='("long", "long")'), threads=2)
    assert rows.view(np.int64).ravel().tolist() == [N]
    rows, per = plans.run(agg_plan("gpuaggregate_sum", "fields = (); sumfield = 1;", "global = true; threads = 2;",
                                   schema='("long", "long")'), threads=2)
    assert rows.view(np.int64).ravel().tolist() == [N * (N + 1) // 2]


def test_partition_then_join_per_thread():
    # Plans chain GPU operators: both sides partitioned into 4 ranges, thread t
    # joins partition t of R with partition t of S (one group per thread),
    # which together is the whole join.
    R = dg.build_relation(20_000, dg.seed_for(79))
    S = dg.probe_uniform(90_000, R, dg.seed_for(80))
    plans.register("R", R); plans.register("S", S)
    plan = '''
    buffsize = 8192;
    treeroot = { name = "join"; build = { name = "pr"; input = { name = "r"; }; };
                                probe = { name = "ps"; input = { name = "s"; }; }; };
    r = { type = "memscan"; relation = "R"; schema = ("long", "long"); };
    s = { type = "memscan"; relation = "S"; schema = ("long", "long"); };
    pr = { type = "gpupartition"; attr = 0; range = (1, 20000); buckets = 4; sort = "no"; maxtuples = 100000; };
    ps = { type = "gpupartition"; attr = 0; range = (1, 20000); buckets = 4; sort = "no"; maxtuples = 100000; };
    join = { type = "gpuhashjoin"; buildjattr = 0; probejattr = 0; projection = ("P$1", "B$1");
             threadgroups = ((0), (1), (2), (3)); hash = { fn = "modulo"; buckets = 1024; }; tuplesperbucket = 4; };
    '''
    rows, per = plans.run(plan, threads=4)
    want, n, _ = orc.hashjoin(R, S, proj=(("P", 8, 8), ("B", 8, 8)), hash=orc.hashcfg("modulo", 1 << 12))
    assert sum(per) == n == 90_000
    assert np.array_equal(canon(rows), canon(want))
