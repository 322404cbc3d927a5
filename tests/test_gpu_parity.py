"""GPU parity: every operator through the C ABI against the oracle.

Integer work (hash buckets, partitions, join rows, counts, integer sums, sort
keys) must match bit for bit; unordered outputs (joins, group-by) compare as
sorted multisets. Double (dec) sums are exact 192-bit fixed-point sums rounded
once: on these inputs they equal the correctly rounded exact sum bit for bit,
which is stricter than the contract's relative error of 1e-12, and they do not
depend on row order or launch shape.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from pythia_gb300 import datagen as dg
from pythia_gb300 import gpu
from tests.golden import inputs as gin

pytestmark = pytest.mark.gpu
DEC_RTOL = 1e-12


def canon(a):
    return orc.canonical(np.ascontiguousarray(a))


# ---------------------------------------------------------------- hashing
HASHES = [("bytes", {}), ("modulo", {}), ("range", {"min": -1000, "max": 1000}),
          ("exactrange", {"min": -1000, "max": 1000}), ("parammodulo", {"skipbits": 3, "offset": 7}),
          ("knuth", {"skipbits": 2, "offset": 5}), ("tpchorderkey", {}), ("willis", {}),
          ("alwayszero", {}), ("tpchq1magic", {})]


@pytest.mark.parametrize("fn,extra", HASHES)
@pytest.mark.parametrize("buckets", [1, 7, 100, 4096])
def test_hash_functions(ctx, fn, extra, buckets):
    rows = gin.make({"gen": "formula", "name": "signed_keys", "n": 5000})
    cfg_g = gpu.hashcfg(fn, buckets, **extra)
    cfg_o = orc.hashcfg(fn, buckets, **extra)
    assert ctx.nbuckets(cfg_g) == orc.hashfn(cfg_o).nbuckets
    for off, size in ((0, 8), (8, 8)):
        got = ctx.hash_tuples(rows, cfg_g, off, size)
        want = orc.hash_column(cfg_o, rows, off, size)
        assert np.array_equal(got, want), fn


def test_hash_int32_keys(ctx):
    rows = gin.make({"gen": "formula", "name": "int_pairs", "n": 4096})
    for fn in ("modulo", "bytes", "knuth", "willis", "parammodulo"):
        got = ctx.hash_tuples(rows, gpu.hashcfg(fn, 256), 4, 4)
        want = orc.hash_column(orc.hashcfg(fn, 256), rows, 4, 4)
        assert np.array_equal(got, want), fn


# ---------------------------------------------------------------- partition
def _part_check(ctx, rows, cfg_g, cfg_o, key=(0, 8)):
    got, goffs = ctx.partition(rows, cfg_g, *key)
    want, woffs = orc.partition(rows, cfg_o, key)
    assert np.array_equal(goffs, woffs)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), "partition output (stable order) differs"


@pytest.mark.parametrize("T", [1, 3, 7, 15, 127])
def test_partition_exactrange(ctx, T):
    rows = dg.uniform_keys(100_000, 50_000, dg.seed_for(20 + T))
    _part_check(ctx, rows, gpu.hashcfg("exactrange", T, 0, 49_999), orc.hashcfg("exactrange", T, 0, 49_999))


@pytest.mark.parametrize("bits", [4, 6, 8, 10, 12])
def test_partition_radix(ctx, bits):
    rows = dg.uniform_keys(300_001, 1 << 40, dg.seed_for(30 + bits))
    cfg = dict(buckets=1 << bits, skipbits=3)
    _part_check(ctx, rows, gpu.hashcfg("parammodulo", **cfg), orc.hashcfg("parammodulo", **cfg))


def test_partition_zipf_skew(ctx):
    rows = dg.zipf_keys(200_000, 10_000, 1.0, dg.seed_for(40))
    _part_check(ctx, rows, gpu.hashcfg("exactrange", 5, 0, 9999), orc.hashcfg("exactrange", 5, 0, 9999))


def test_partition_widths(ctx):
    # 20-byte tuples (int, long, long) keyed on the long at offset 4, and
    # 8-byte (int, int) tuples keyed on an int.
    base = dg.uniform_keys(50_003, 1000, dg.seed_for(41))
    t20 = np.zeros((base.shape[0], 5), dtype=np.int32)
    t20[:, 0] = np.arange(base.shape[0])
    t20[:, 1:5] = base.view(np.int32)
    _part_check(ctx, t20, gpu.hashcfg("exactrange", 9, 0, 999), orc.hashcfg("exactrange", 9, 0, 999), key=(4, 8))
    t8 = gin.make({"gen": "formula", "name": "int_pairs", "n": 70_000})
    _part_check(ctx, t8, gpu.hashcfg("modulo", 64), orc.hashcfg("modulo", 64), key=(0, 4))


def test_partition_edge_sizes(ctx):
    for n in (0, 1, 2047, 2048, 2049, 4096):
        rows = dg.uniform_keys(n, 100, dg.seed_for(42))
        _part_check(ctx, rows, gpu.hashcfg("modulo", 16), orc.hashcfg("modulo", 16))


def test_partition_out_of_range_is_an_error(ctx):
    rows = dg.uniform_keys(1000, 100, dg.seed_for(43))
    with pytest.raises(gpu.PgError):
        ctx.partition(rows, gpu.hashcfg("exactrange", 4, 0, 49))   # keys up to 99 exceed the range


# ---------------------------------------------------------------- hash join
def _join_check(ctx, R, S, proj=(("P", 8, 8), ("B", 8, 8)), bkey=(0, 8), pkey=(0, 8), buckets=1024):
    got, n, _ = ctx.hashjoin(R, S, proj=proj, bkey=bkey, pkey=pkey)
    want, wn, _ = orc.hashjoin(R, S, proj=proj, bkey=bkey, pkey=pkey, hash=orc.hashcfg("modulo", buckets))
    assert n == wn
    assert np.array_equal(canon(got), canon(want))
    sc = len(proj) - 1
    _, n2, s2 = ctx.hashjoin(R, S, proj=proj, bkey=bkey, pkey=pkey, flags=gpu.JOIN_COUNT | gpu.JOIN_SUM, sum_col=sc)
    _, wn2, ws2 = orc.hashjoin(R, S, proj=proj, bkey=bkey, pkey=pkey, materialise=False, sum_col=sc,
                               hash=orc.hashcfg("modulo", buckets))
    assert (n2, s2) == (wn2, ws2)
    return n


def test_join_pkfk_uniform(ctx):
    R = dg.build_relation(50_000, dg.seed_for(1))
    S = dg.probe_uniform(400_000, R, dg.seed_for(2))
    assert _join_check(ctx, R, S) == 400_000


def test_join_pkfk_zipf(ctx):
    R = dg.build_relation(30_000, dg.seed_for(11))
    S = dg.probe_zipf(300_000, 1.0, R, dg.seed_for(12))
    _join_check(ctx, R, S)


def test_join_sparse_unique_keys(ctx):
    # Unique keys spread over a wide domain take the hashed table (dense
    # tables need the keys within twice |R| consecutive values).
    R = dg.build_relation(60_000, dg.seed_for(17))
    R[:, 0] = R[:, 0] * 7919 - (1 << 40)
    S = dg.probe_uniform(500_000, R, dg.seed_for(18))
    S[::1000, 0] += 3                      # some misses
    R[5, 0] = -1                           # a unique key equal to the empty marker
    S[::777, 0] = -1
    _join_check(ctx, R, S)
    _join_check(ctx, R, S, proj=(("B", 8, 8), ("P", 0, 8)))
    # The probe side partitioned on the keys' hash first (large hashed tables
    # take this path; forced here): the same rows, in another order.
    try:
        ctx.tune(hash_partition=2)
        _join_check(ctx, R, S)
        _join_check(ctx, R, S, proj=(("B", 8, 8), ("P", 0, 8)))
        _, n, sm = ctx.hashjoin(R, S, flags=gpu.JOIN_COUNT | gpu.JOIN_SUM, sum_col=1)
        _, wn, ws = orc.hashjoin(R, S, sum_col=1, materialise=False, hash=orc.hashcfg("modulo", 1 << 12))
        assert (n, sm) == (wn, ws)
    finally:
        ctx.tune(hash_partition=0)


def test_join_dense_keys_wide_values(ctx):
    # Dense keys whose build values span more than 2^32 values take the wide
    # dense layout (8-byte values + presence bits) instead of 4-byte entries.
    R = dg.build_relation(40_000, dg.seed_for(19))
    R[:, 1] = dg.raw_words(dg.seed_for(19), 1, 40_000).view(np.int64)
    S = dg.probe_uniform(300_000, R, dg.seed_for(20))
    S[::5, 0] += 100_000                      # misses beyond the key range
    _join_check(ctx, R, S)
    R[::3, 0] += 20_000                       # holes inside the key range
    _join_check(ctx, R, S)


@pytest.mark.parametrize("knobs", [dict(probe_variant=1), dict(probe_variant=1, probe_items=8),
                                   dict(probe_variant=1, probe_passes=2, probe_items=8), dict(probe_cache=1),
                                   dict(probe_cache=14), dict(probe_passes=2), dict(probe_variant=4),
                                   dict(probe_variant=4, probe_passes=2, probe_ctas_per_sm=5),
                                   dict(probe_variant=2), dict(probe_variant=3), dict(probe_variant=5),
                                   dict(probe_cache=64), dict(probe_cache=192), dict(probe_cache=48 + 4),
                                   dict(probe_cache=256)])
def test_join_probe_launch_shapes(ctx, knobs):
    # Probe kernel variants, lookups in flight, L2 policies, passes and grid
    # shapes change speed, never rows: narrow and wide dense tables, with
    # misses (compaction) and a ragged tail (n not a multiple of 256).
    R = dg.build_relation(70_001, dg.seed_for(23))
    S = dg.probe_uniform(555_555, R, dg.seed_for(24))
    S[::97, 0] += 200_000
    Rw = R.copy()
    Rw[:, 1] = dg.raw_words(dg.seed_for(23), 1, 70_001).view(np.int64)
    try:
        ctx.tune(**knobs)
        _join_check(ctx, R, S)
        _join_check(ctx, Rw, S)
        _join_check(ctx, R, S[:1000])
    finally:
        ctx.tune(probe_items=0, probe_cache=0, probe_passes=0, probe_variant=0, probe_ctas_per_sm=0)


def test_join_dense_keys_with_repeated_rows(ctx):
    # A dense key domain whose build side repeats whole rows (same key and
    # payload) must still join every copy: the dense build detects repeats by
    # counting present entries and falls back to the hashed table.
    R = dg.build_relation(20_000, dg.seed_for(25))
    R = np.concatenate([R, R[:3], R[100:101]])
    S = dg.probe_uniform(200_000, R[:20_000], dg.seed_for(26))
    _join_check(ctx, R, S)


def _spec_cases():
    """Build sides for the device-only dense build: ones it keeps and ones
    its checks refute (rebuilt exactly at the table's first use)."""
    R = dg.build_relation(100_000, dg.seed_for(41))
    cases = {"dense": R}
    d = np.concatenate([R, R[:2]])                       # a repeated row: fewer entries than tuples
    cases["repeated_row"] = d
    o = R.copy(); o[12_345, 0] = 5_000_000_000           # one key far outside the sampled window
    cases["key_outlier"] = o
    v = R.copy(); v[:, 1] %= 1000; v[777, 1] = 1 << 40   # one value outside the 32-bit entry range
    cases["value_outlier"] = v
    w = R.copy(); w[:, 1] = dg.raw_words(dg.seed_for(41), 1, R.shape[0]).view(np.int64)   # 64-bit values
    cases["wide_values"] = w
    n = R.copy(); n[:, 1] = -n[:, 1] - 1; n[:, 0] -= 200_000   # negative keys and values
    cases["negative"] = n
    h = R.copy(); h[:, 1] = 7_000_000_000 + (h[:, 1] % 100_000)   # values far from 0 (base not 0)
    cases["high_values"] = h
    z = R.copy(); z[:, 1] %= 1000                        # values from 0: the sample's base is the smallest value
    cases["zero_based_values"] = z
    return cases


@pytest.mark.parametrize("spec", [1, 2])
@pytest.mark.parametrize("case", sorted(_spec_cases()))
def test_join_dense_build_on_device(ctx, spec, case):
    # The dense build that takes its key window and value base from a sample
    # (build_spec=1 forces it at every size, 2 is the host-checked build) must
    # give the same rows, counts and sums whether the sample's layout holds or
    # the table is rebuilt at its first use.
    R = _spec_cases()[case]
    S = dg.probe_uniform(300_000, R[:100_000], dg.seed_for(42))
    S[::101, 0] += 3_000_000                              # misses outside every window
    # Misses past the sampled window but inside the build's allocation.
    S[::97, 0] = R[:100_000, 0].max() + 50_000 + (S[::97, 1] % 60_000)
    try:
        ctx.tune(build_spec=spec)
        _join_check(ctx, R, S)
        _join_check(ctx, R, S, proj=(("B", 8, 8), ("P", 8, 8)))      # a projection the fast kernels do not take
        small = R[:5000].copy()
        _join_check(ctx, small, S[:20_000])
    finally:
        ctx.tune(build_spec=0)


@pytest.mark.parametrize("case", ["dense", "high_values", "negative", "zero_based_values"])
def test_dense_build_on_device_settles_to_the_exact_table(ctx, case):
    # A table built on the device and then used by a path that needs its
    # exact layout (an image here) is the table the host-checked build makes,
    # byte for byte; so is the one-pass join + group-by on it.
    R = _spec_cases()[case]
    images = []
    for spec in (1, 2):
        ctx.tune(build_spec=spec)
        try:
            t = ctx.build_table(R)
            try:
                images.append(t.serialize())
            finally:
                t.free()
        finally:
            ctx.tune(build_spec=0)
    assert np.array_equal(images[0], images[1])
    G = R.copy()
    G[:, 1] = (G[:, 1] % 997) + 5000                      # group column with its smallest value far from 0
    S = dg.probe_uniform(200_000, G, dg.seed_for(43))
    S[:, 1] = (S[:, 1] % 1000)
    outs = []
    for spec in (1, 2):
        ctx.tune(build_spec=spec)
        try:
            outs.append(canon(ctx.hashjoin_groupby(G, S, group=(8, 8), val=(8, "long"))))
        finally:
            ctx.tune(build_spec=0)
    assert np.array_equal(outs[0], outs[1])


def test_join_many_to_many(ctx):
    R = dg.uniform_keys(5000, 700, dg.seed_for(5))
    S = dg.uniform_keys(9000, 900, dg.seed_for(6))
    _join_check(ctx, R, S)
    try:
        ctx.tune(hash_partition=2, dense=2)          # hashed table, probe side partitioned first
        _join_check(ctx, R, S)
    finally:
        ctx.tune(hash_partition=0, dense=0)


def test_join_projection_orders(ctx):
    R = dg.build_relation(3000, dg.seed_for(7))
    S = dg.probe_uniform(9000, R, dg.seed_for(8))
    _join_check(ctx, R, S, proj=(("B", 0, 8), ("P", 8, 8), ("B", 8, 8)))   # 24-byte rows
    _join_check(ctx, R, S, proj=(("B", 8, 8), ("P", 8, 8)))
    _join_check(ctx, R, S, proj=(("P", 0, 8), ("P", 8, 8), ("B", 8, 4), ("B", 12, 4)))
    _join_check(ctx, R, S, proj=(("B", 0, 8), ("B", 8, 8), ("P", 8, 8)))   # 16 B of build columns: row-index path


def test_join_edge_cases(ctx):
    R = dg.build_relation(1000, dg.seed_for(9))
    empty = np.zeros((0, 2), dtype=np.int64)
    assert _join_check(ctx, R, empty) == 0
    assert _join_check(ctx, empty, R) == 0
    big = gin.make({"gen": "formula", "name": "big_keys", "n": 5000})
    assert _join_check(ctx, R, big) == 0
    one = R[:1].copy()
    assert _join_check(ctx, one, one) == 1


def test_join_empty_marker_key(ctx):
    # -1 is the tables' empty marker; a real key -1 must still join.
    R = dg.build_relation(2000, dg.seed_for(13))
    R[17, 0] = -1
    S = dg.probe_uniform(10_000, R, dg.seed_for(14))
    S[::97, 0] = -1
    _join_check(ctx, R, S)
    R2 = R.copy()
    R2[18, 0] = -1                           # two build tuples with key -1
    _join_check(ctx, R2, S)


def test_join_negative_and_int32_keys(ctx):
    R = gin.make({"gen": "formula", "name": "signed_keys", "n": 3000})
    S = gin.make({"gen": "formula", "name": "signed_keys", "n": 3000})
    _join_check(ctx, R, S)
    I = gin.make({"gen": "formula", "name": "int_pairs", "n": 4000})
    I[:, 0] %= 500
    _join_check(ctx, I, I, proj=(("P", 4, 4), ("B", 4, 4)), bkey=(0, 4), pkey=(0, 4))


def test_join_wide_tuples(ctx):
    base = dg.build_relation(4000, dg.seed_for(15))
    R = np.zeros((4000, 5), dtype=np.int32)
    R[:, 1:] = base.view(np.int32)
    sb = dg.probe_uniform(12000, base, dg.seed_for(16))
    S = np.zeros((12000, 5), dtype=np.int32)
    S[:, 0] = np.arange(12000)
    S[:, 1:] = sb.view(np.int32)
    _join_check(ctx, R, S, proj=(("P", 0, 4), ("P", 12, 8), ("B", 12, 8)), bkey=(4, 8), pkey=(4, 8))


def _lines(n, R, seed, miss_every=0):
    """(order, part, price) 24-byte probe tuples whose part keys are drawn from R."""
    fk = dg.probe_uniform(n, R, dg.seed_for(seed))
    L = np.zeros((n, 3), np.int64)
    L[:, 0] = np.arange(n) * 3 + 1
    L[:, 1] = fk[:, 0]
    L[:, 2] = ((dg.raw_words(dg.seed_for(seed + 1), 2, n) >> np.uint64(11)).astype(np.float64) * 1e-9).view(np.int64)
    if miss_every:
        L[::miss_every, 1] += 1 << 40
    return L


@pytest.mark.parametrize("wide", [0, 1, 2, 3])
def test_join_other_widths(ctx, wide):
    # Probe tuples and output rows other than 16 bytes: staged through shared
    # memory (2: 4 lookups per thread, 3: 2; 0: rows of dense tables staged,
    # hashed tables, counts and sums per thread) or loaded per thread (1);
    # same rows, counts and sums. Dense narrow, dense wide and hashed
    # tables; ragged final tiles whose bytes are not a multiple of 16.
    R = dg.build_relation(60_000, dg.seed_for(601))
    Rw = R.copy(); Rw[:, 1] = dg.raw_words(dg.seed_for(602), 1, 60_000).view(np.int64)
    Rh = R.copy(); Rh[:, 0] = Rh[:, 0] * 7919 - (1 << 40)
    try:
        ctx.tune(probe_wide=wide)
        L = _lines(300_001, R, 603, miss_every=37)
        for table in (R, Rw):
            _join_check(ctx, table, L, proj=(("P", 0, 8), ("P", 16, 8), ("B", 8, 8)), pkey=(8, 8))
            _join_check(ctx, table, L, proj=(("P", 16, 8), ("B", 8, 8)), pkey=(8, 8))
            _join_check(ctx, table, L, proj=(("B", 8, 4), ("P", 4, 8), ("P", 20, 4), ("B", 12, 4)), pkey=(8, 8))
        Lh = L.copy(); Lh[:, 1] = Lh[:, 1] * 7919 - (1 << 40)
        Lh[::101, 1] = -1; Rh[7, 0] = -1                      # the empty marker as a real key
        _join_check(ctx, Rh, Lh, proj=(("P", 0, 8), ("P", 16, 8), ("B", 8, 8)), pkey=(8, 8))
        # 12-byte tuples with an int key at byte 4; odd counts leave 4 or 8
        # bytes past the last multiple of 16.
        I = np.zeros((20_001, 3), np.int32)
        I[:, 0] = np.arange(20_001); I[:, 1] = (np.arange(20_001) * 7) % 5000; I[:, 2] = -np.arange(20_001)
        Ri = np.zeros((5000, 2), np.int32); Ri[:, 0] = np.arange(5000); Ri[:, 1] = np.arange(5000) * 3 - 7000
        for n in (20_001, 20_002, 3, 1):
            _join_check(ctx, Ri, I[:n], proj=(("P", 8, 4), ("B", 4, 4), ("P", 0, 4)), bkey=(0, 4), pkey=(4, 4))
        # 16-byte tuples keyed at byte 4 and 12-byte rows; 64-byte tuples (the
        # widest staged) and 68-byte ones (per-thread loads).
        S16 = dg.probe_uniform(100_003, R, dg.seed_for(604)).view(np.int32)
        S16 = np.ascontiguousarray(np.roll(S16, 1, axis=1))
        _join_check(ctx, R, S16, proj=(("P", 0, 4), ("B", 8, 8)), pkey=(4, 8))
        for words in (16, 17):
            Wd = np.zeros((70_000, words), np.int32)
            Wd[:, :] = np.arange(words)[None, :] + np.arange(70_000)[:, None]
            Wd[:, 10:12] = dg.probe_uniform(70_000, R, dg.seed_for(605))[:, :1].view(np.int32)
            _join_check(ctx, R, Wd, proj=(("P", 60, 4), ("P", 0, 8), ("B", 8, 8), ("P", 36, 4)), pkey=(40, 8))
        # A probe side several grid waves long; an exact and a short output.
        Lbig = _lines(2_000_000, R, 606, miss_every=13)
        n = _join_check(ctx, R, Lbig, proj=(("P", 0, 8), ("P", 16, 8), ("B", 8, 8)), pkey=(8, 8))
        t = ctx.build_table(R, (("P", 0, 8), ("P", 16, 8), ("B", 8, 8)))
        try:
            got, n2, _ = t.probe(Lbig, pkey=(8, 8), out_cap=n)
            assert n2 == n and got.shape[0] == n
            with pytest.raises(gpu.PgError):
                t.probe(Lbig, pkey=(8, 8), out_cap=n - 1)
        finally:
            t.free()
    finally:
        ctx.tune(probe_wide=0)


def _probe_spans(ctx, R, parts, proj, pkey, bkey=(0, 8), flags=gpu.JOIN_MATERIALIZE, sum_col=-1):
    # The probe side as separate device arrays, probed as one relation.
    import ctypes
    L = gpu.lib()
    t = ctx.build_table(R, proj, bkey)
    try:
        bufs = [ctx.upload(np.ascontiguousarray(p)) for p in parts]
        rels = (gpu.Rel * len(parts))(*[ctx.rel(b, p.shape[0], gpu.row_width(p), *pkey) for b, p in zip(bufs, parts)])
        c, nc = gpu.cols(proj)
        ow = sum(b for _, _, b in proj)
        total = sum(p.shape[0] for p in parts)
        o = ctx.alloc(max(total, 1) * ow)
        res = gpu.JoinResult()
        ctx._check(L.pg_hashjoin_probe_spans(ctx.h, ctx.stream, t.h, rels, len(parts), c, nc,
                                             o.ptr if flags & gpu.JOIN_MATERIALIZE else None, total, flags, sum_col,
                                             ctypes.byref(res)))
        rows = ctx.download(o, res.n_out * ow).reshape(-1, ow) if flags & gpu.JOIN_MATERIALIZE else None
        return rows, res.n_out, res.sum
    finally:
        t.free()


def test_join_probe_spans_as_one_relation(ctx):
    # 24-byte lines split into uneven arrays (one empty) against dense narrow,
    # dense wide and hashed tables; 16-byte tuples too: the rows, count and
    # sum of one probe over the concatenation.
    R = dg.build_relation(50_000, dg.seed_for(620))
    Rw = R.copy(); Rw[:, 1] = dg.raw_words(dg.seed_for(621), 1, 50_000).view(np.int64)
    Rh = R.copy(); Rh[:, 0] = Rh[:, 0] * 7919 - (1 << 40)
    L = _lines(210_001, R, 622, miss_every=31)
    Lh = L.copy(); Lh[:, 1] = Lh[:, 1] * 7919 - (1 << 40)
    cuts = [0, 70_000, 70_000, 150_001, 210_001]
    proj = (("P", 0, 8), ("P", 16, 8), ("B", 8, 8))
    for table, lines in ((R, L), (Rw, L), (Rh, Lh)):
        parts = [lines[a:b] for a, b in zip(cuts, cuts[1:])]
        got, n, _ = _probe_spans(ctx, table, parts, proj, (8, 8))
        want, wn, _ = orc.hashjoin(table, lines, proj=proj, pkey=(8, 8), hash=orc.hashcfg("modulo", 1024))
        assert n == wn and np.array_equal(canon(got), canon(want))
        _, n2, s2 = _probe_spans(ctx, table, parts, proj, (8, 8), flags=gpu.JOIN_COUNT | gpu.JOIN_SUM, sum_col=2)
        _, wn2, ws2 = orc.hashjoin(table, lines, proj=proj, pkey=(8, 8), materialise=False, sum_col=2,
                                   hash=orc.hashcfg("modulo", 1024))
        assert (n2, s2) == (wn2, ws2)
    S = dg.probe_uniform(100_000, R, dg.seed_for(623))
    got, n, _ = _probe_spans(ctx, R, [S[:33_333], S[33_333:]], (("P", 8, 8), ("B", 8, 8)), (0, 8))
    want, wn, _ = orc.hashjoin(R, S, hash=orc.hashcfg("modulo", 1024))
    assert n == wn and np.array_equal(canon(got), canon(want))


def test_join_probe_spans_refuses_repeated_build_keys(ctx):
    R = dg.uniform_keys(5000, 700, dg.seed_for(624))
    S = dg.uniform_keys(9000, 900, dg.seed_for(625))
    with pytest.raises(gpu.PgError) as e:
        _probe_spans(ctx, R, [S[:4000], S[4000:]], (("P", 8, 8), ("B", 8, 8)), (0, 8))
    assert e.value.code == gpu.PG_ERR_UNSUPPORTED


def _golden_joins():
    import json
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "golden.json")
    with open(path) as f:
        return [c for c in json.load(f)["cases"] if c["op"] == "hashjoin"]


@pytest.mark.parametrize("case", _golden_joins(), ids=lambda c: c["name"])
def test_join_matches_reference_engine_digest(ctx, case):
    # The GPU join's rows against the digest the reference engine's own
    # HashJoinOp recorded for the same inputs (tests/golden/make_golden.py):
    # row count, count and canonical SHA-256 of the sorted rows.
    import hashlib
    p, ref = case["params"], case["ref"]
    R, S = gin.make(case["inputs"]["R"]), gin.make(case["inputs"]["S"])
    width = lambda schema: [4 if c == "int" else 8 for c in schema.split(",")]
    bw, pw = width(p["bschema"]), width(p["pschema"])
    proj = []
    for col in p["proj"].split(","):
        side, i = col.split("$")
        w = bw if side == "B" else pw
        proj.append((side, sum(w[:int(i)]), w[int(i)]))
    ba, pa = p.get("buildjattr", 0), p.get("probejattr", 0)
    got, n, _ = ctx.hashjoin(R, S, proj=tuple(proj), bkey=(sum(bw[:ba]), bw[ba]), pkey=(sum(pw[:pa]), pw[pa]))
    assert n == ref["n_out"] == ref["count"]
    if n:
        digest = hashlib.sha256(np.ascontiguousarray(canon(got)).view(np.uint8).tobytes()).hexdigest()
        assert digest == ref["canonical_sha256"]


def _golden_cases(ops):
    import json
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "golden.json")
    with open(path) as f:
        return [c for c in json.load(f)["cases"] if c["op"] in ops]


@pytest.mark.parametrize("case", _golden_cases(("partition", "sort", "filter", "project")), ids=lambda c: c["name"])
def test_ordered_ops_match_reference_engine_digest(ctx, case):
    # Partition (stable order within a partition), sort, Filter and Project
    # on the GPU against the SHA-256 digests of the reference engine's own
    # operators on the same inputs.
    import hashlib
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()
    p, ref, op = case["params"], case["ref"], case["op"]
    a = gin.make(case["inputs"]["in"])
    if op == "partition":
        out, offs = ctx.partition(a, gpu.hashcfg("exactrange", p["buckets"], p["min"], p["max"]))
        for b, part in enumerate(ref["partitions"]):
            rows = out[offs[b]:offs[b + 1]]
            assert rows.shape[0] == part["n"] and sha(rows) == part["sha256"], f"partition {b}"
    elif op == "sort":
        out = np.ascontiguousarray(ctx.sort(a)).view(np.uint8).reshape(a.shape[0], -1)
        assert sha(out[:, :8]) == ref["keys_sha256"]
        assert sha(canon(out)) == ref["canonical_sha256"]
    else:
        cols = gin.schema_columns(p["schema"])
        w = sum(cw for _, _, cw in cols)
        rows = np.ascontiguousarray(a).view(np.uint8).reshape(a.shape[0], w)
        if op == "filter":
            out = ctx.filter(rows, gin.filter_preds(p["schema"], p["filters"]))
            assert out.shape[0] == ref["n"] and sha(out) == ref["sha256"]
        else:
            out = ctx.project(rows, [(cols[int(i)][1], cols[int(i)][2]) for i in p["projection"].split(",")])
            assert out.size == ref["bytes"] and sha(out) == ref["sha256"]


def test_join_reference_unit_test(ctx):
    # unit_tests/queryhashjoin.cpp: build (i, i), probe (i, i+0.1), i = 1..20.
    R = gin.make({"gen": "formula", "name": "i_i", "n": 20})
    S = gin.make({"gen": "formula", "name": "i_i_plus_0.1", "n": 20})
    got, n, _ = ctx.hashjoin(R, S, proj=(("B", 8, 8), ("P", 8, 8)))
    assert n == 20
    rows = got.view(np.int64).reshape(-1, 2)
    assert sorted(rows[:, 0].tolist()) == list(range(1, 21))
    assert np.allclose(rows[:, 1].view(np.float64), rows[:, 0] + 0.1)


# ---------------------------------------------------------------- group-by
def _gb_int_check(ctx, rows, agg, vtype, key=(0, 8), hint=0, has_key=True):
    got = ctx.groupby(rows, key=key, val=(8 if vtype != "int" else 4, vtype), agg=agg,
                      groups_hint=hint, has_key=has_key)
    want = orc.groupby(rows, key=key, val=(8 if vtype != "int" else 4, vtype), agg=agg,
                       hash=orc.hashcfg("modulo", 1024), has_key=has_key)
    assert np.array_equal(canon(got), canon(want))


@pytest.mark.parametrize("groups", [1, 10, 1000, 20_000, 200_000])
def test_groupby_long_sum_and_count(gbctx, groups):
    ctx = gbctx
    rows = dg.uniform_keys(500_000, groups, dg.seed_for(50))
    rows[:, 1] -= 1 << 30    # negative values too
    for agg in ("sum", "count"):
        _gb_int_check(ctx, rows, agg, "long")
        _gb_int_check(ctx, rows, agg, "long", hint=groups)


def test_groupby_int_sum_wraps(gbctx):
    ctx = gbctx
    rows = gin.make({"gen": "formula", "name": "int_big", "n": 100_000})
    got = ctx.groupby(rows, key=(0, 4), val=(4, "int"), agg="sum")
    want = orc.groupby(rows, key=(0, 4), val=(4, "int"), agg="sum")
    assert np.array_equal(canon(got), canon(want))


def test_groupby_no_group_by(ctx):
    rows = dg.uniform_keys(123_457, 1000, dg.seed_for(51))
    _gb_int_check(ctx, rows, "count", "long", has_key=False)
    _gb_int_check(ctx, rows, "sum", "long", has_key=False)
    assert ctx.groupby(rows[:0], agg="count", has_key=False).shape[0] == 0


def test_groupby_empty_marker_key(gbctx):
    ctx = gbctx
    rows = dg.uniform_keys(20_000, 300, dg.seed_for(52))
    rows[::7, 0] = -1
    _gb_int_check(ctx, rows, "sum", "long")
    _gb_int_check(ctx, rows, "count", "long", hint=10_000)


# Every group-by path: 0 chooses (dense direct-indexed table for compact key
# ranges, summed per CTA in shared memory first for windows up to 4096 keys),
# 3 hashed global table, 4 partitioned, 1 and 2 the same with warp combining of
# equal keys, 7 dense with global atomics only.
GB_PATHS = [0, 1, 2, 3, 4, 7]


@pytest.fixture(params=GB_PATHS)
def gbctx(ctx, request):
    ctx.tune(groupby_path=request.param)
    yield ctx
    ctx.tune(groupby_path=0)


def _gb_dec_check(ctx, rows, hint=0, has_key=True):
    # Bit for bit against the exactly rounded sum of each group (Shewchuk's
    # summation in the oracle); within the contract's 1e-12 a fortiori.
    got = ctx.groupby(rows, val=(8, "dec"), agg="sum", groups_hint=hint, has_key=has_key)
    exact = orc.groupby_exact(rows, has_key=has_key)
    if not has_key:
        assert np.array_equal(got.view(np.int64), exact.view(np.int64))
        return got
    g = got.view(np.int64).reshape(-1, 2)
    e = exact.view(np.int64).reshape(-1, 2)
    g = g[np.argsort(g[:, 0], kind="stable")]
    assert np.array_equal(g[:, 0], e[:, 0])
    gv, ev = g[:, 1].view(np.float64), e[:, 1].view(np.float64)
    rel = np.abs(gv - ev) / np.maximum(np.abs(ev), 1e-300)
    assert rel.max() <= DEC_RTOL, rel.max()
    assert np.array_equal(g[:, 1], e[:, 1]), np.flatnonzero(g[:, 1] != e[:, 1])[:5]
    return got


@pytest.mark.parametrize("groups", [1, 300, 100_000])
def test_groupby_dec_exact(gbctx, groups):
    ctx = gbctx
    rows = dg.groupby_rows(1_000_000, groups, 1e4, dg.seed_for(53))
    _gb_dec_check(ctx, rows)
    _gb_dec_check(ctx, rows, hint=groups)


@pytest.mark.parametrize("path", [0, 7])
def test_groupby_few_groups_large_input(ctx, path):
    # 5M rows in 1000 groups take the key window from a sample; path 0 sums
    # each CTA's rows in shared memory before one flush per group, path 7
    # adds every row into the global table. Integer results are exact, dec
    # sums within the contract; one key holding a third of the rows too.
    rows = dg.groupby_rows(5_000_000, 1000, 1e4, dg.seed_for(56))
    rows[::3, 0] = 17
    try:
        ctx.tune(groupby_path=path)
        _gb_dec_check(ctx, rows)
        ints = rows.copy()
        ints[:, 1] = (ints[:, 1] & 0xFFFFF) - 0x80000
        for agg in ("sum", "count"):
            _gb_int_check(ctx, ints, agg, "long")
        i32 = np.ascontiguousarray(ints.view(np.int32)[:, [0, 2]])
        got = ctx.groupby(i32, key=(0, 4), val=(4, "int"), agg="sum")
        assert np.array_equal(canon(got), canon(orc.groupby(i32, key=(0, 4), val=(4, "int"), agg="sum")))
    finally:
        ctx.tune(groupby_path=0)


def test_groupby_dec_ill_conditioned(gbctx):
    ctx = gbctx
    # Large values that cancel plus many small ones: naive summation loses the
    # small ones entirely; the exact fixed-point sum keeps them.
    n = 200_000
    rows = np.zeros((n, 2), dtype=np.int64)
    rows[:, 0] = np.arange(n) % 10
    v = np.full(n, 1e-3)
    v[0:20:2] = 1e16
    v[1:20:2] = -1e16
    rows[:, 1] = v.view(np.int64)
    _gb_dec_check(ctx, rows)


def test_groupby_dec_independent_of_row_order(gbctx):
    # The same rows in another order (and again) give the same bits: integer
    # adds do not depend on which thread arrives first.
    ctx = gbctx
    rows = dg.groupby_rows(300_000, 2000, 1e4, dg.seed_for(57))
    rows[::5, 1] = (-rows[::5, 1].view(np.float64) * 1e-7).view(np.int64)       # mixed signs and scales
    first = canon(_gb_dec_check(ctx, rows))
    perm = np.random.default_rng(58).permutation(rows.shape[0])
    assert np.array_equal(canon(ctx.groupby(rows[perm], val=(8, "dec"), agg="sum")), first)
    assert np.array_equal(canon(ctx.groupby(rows, val=(8, "dec"), agg="sum")), first)
    assert np.array_equal(canon(ctx.groupby(rows[::-1], val=(8, "dec"), agg="sum", groups_hint=2000)), first)
    try:
        ctx.tune(groupby_ilp=8)                     # eight rows in flight per thread: same bits
        assert np.array_equal(canon(ctx.groupby(rows[perm], val=(8, "dec"), agg="sum")), first)
    finally:
        ctx.tune(groupby_ilp=0)


def test_groupby_dec_infinities_and_nans(gbctx):
    # Groups that meet infinities or NaNs get IEEE's result (+inf, -inf, or NaN
    # for NaN or both infinities); every other group its exact sum.
    ctx = gbctx
    rows = dg.groupby_rows(100_000, 400, 1e4, dg.seed_for(59))
    keys = rows[:, 0]
    vals = rows[:, 1].view(np.float64)
    ks = np.unique(keys)[[3, 5, 8, 13, 21]]
    specials = {ks[0]: ([np.inf], np.inf), ks[1]: ([-np.inf, np.inf], np.nan), ks[2]: ([-np.inf, -np.inf], -np.inf),
                ks[3]: ([np.nan], np.nan), ks[4]: ([np.inf, np.nan], np.nan)}
    for k, (vs, _) in specials.items():
        vals[np.flatnonzero(keys == k)[: len(vs)]] = vs
    got = canon(ctx.groupby(rows, val=(8, "dec"), agg="sum")).view(np.int64).reshape(-1, 2)
    plain = ~np.isin(keys, ks)
    exact = canon(orc.groupby_exact(rows[plain])).view(np.int64).reshape(-1, 2)
    sp = np.isin(got[:, 0], ks)
    assert sp.sum() == len(ks)
    assert np.array_equal(got[~sp], exact)
    for k, v in zip(got[sp, 0], got[sp, 1].view(np.float64)):
        want = specials[k][1]
        assert (np.isnan(v) and np.isnan(want)) or v == want, (k, v, want)
    # One group (no GROUP BY): an infinity anywhere makes the sum infinite.
    one = rows.copy()
    v1 = one[:, 1].view(np.float64)
    v1[~np.isfinite(v1)] = 1.0
    v1[777] = -np.inf
    assert np.isneginf(ctx.groupby(one, val=(8, "dec"), agg="sum", has_key=False).view(np.float64)[0, 0])


def test_groupby_dec_value_above_the_sampled_unit(ctx):
    # 4M+ rows take the sum's unit from every 1024th row with a 4x margin; a
    # value far above them (at a row the sample skips) makes the operator redo
    # the sum on the exact unit. Values 2^100 apart still sum exactly.
    n = (1 << 22) + 4097
    rows = dg.uniform_keys(n, 5000, dg.seed_for(82))
    rows[:, 1] = (rows[:, 1] % 1000).astype(np.float64).view(np.int64)
    r = rows.copy()
    r[1025, 1] = np.float64(3.0e33).view(np.int64)
    r[4097, 1] = np.float64(-2.5e-3).view(np.int64)
    for path in (0, 3):
        try:
            ctx.tune(groupby_path=path)
            _gb_dec_check(ctx, r, hint=5000)
        finally:
            ctx.tune(groupby_path=0)


def test_groupby_dec_zipf(gbctx):
    ctx = gbctx
    rows = gin.make({"gen": "groupby_zipf", "n": 300_000, "groups": 20_000, "rel": 54})
    _gb_dec_check(ctx, rows)
    _gb_dec_check(ctx, rows, hint=20_000)     # partitioned path with skewed partitions


def test_groupby_partition_overflow(gbctx):
    ctx = gbctx
    # A hint far below the real group count: partitions overflow their shared
    # tables into the global one, and the global table itself regrows.
    rows = dg.uniform_keys(400_000, 90_000, dg.seed_for(55))
    got = ctx.groupby(rows, val=(8, "long"), agg="sum", groups_hint=5000)
    want = orc.groupby(rows, val=(8, "long"), agg="sum", hash=orc.hashcfg("modulo", 1024))
    assert np.array_equal(canon(got), canon(want))


def _fused_rows(n_build, groups, n_probe, seed):
    R = dg.build_relation(n_build, dg.seed_for(seed))
    R[:, 1] = dg.raw_words(dg.seed_for(seed), 3, n_build) % np.uint64(groups)
    S = dg.probe_uniform(n_probe, R, dg.seed_for(seed + 1))
    S[:, 1] = (dg.raw_words(dg.seed_for(seed + 1), 4, n_probe) >> np.uint64(11)).astype(np.float64).view(np.int64)
    return R, S


@pytest.mark.parametrize("n_build,groups", [(1000, 7), (60_000, 600), (200_000, 50_000)])
def test_hashjoin_groupby_fused(ctx, n_build, groups):
    # Join then aggregate in one pass == materialised join, then exact group-by.
    R, S = _fused_rows(n_build, groups, 8 * n_build, 90 + groups % 7)
    S[::53, 0] += 10 * n_build                     # probe misses
    joined, n, _ = orc.hashjoin(R, S, proj=(("B", 8, 8), ("P", 8, 8)), hash=orc.hashcfg("modulo", 1 << 12))
    exact = canon(orc.groupby_exact(joined.view(np.int64).reshape(-1, 2)))
    got = canon(ctx.hashjoin_groupby(R, S, val=(8, "dec")))
    assert np.array_equal(got, exact)              # keys, and sums bit for bit
    # Count and long sum on the same plan.
    Sl = S.copy(); Sl[:, 1] = dg.raw_words(dg.seed_for(7), 5, S.shape[0]).view(np.int64) >> 20
    jl, _, _ = orc.hashjoin(R, Sl, proj=(("B", 8, 8), ("P", 8, 8)), hash=orc.hashcfg("modulo", 1 << 12))
    for agg in ("sum", "count"):
        want = orc.groupby(jl.view(np.int64).reshape(-1, 2), val=(8, "long"), agg=agg)
        assert np.array_equal(canon(ctx.hashjoin_groupby(R, Sl, val=(8, "long"), agg=agg)), canon(want))


def test_hashjoin_groupby_dec_unit_and_specials(ctx):
    # The fused plan's dec unit comes from a sample of 4M+ probe tuples; a value
    # above it makes the plan redo the sum exactly. Infinities or NaNs in the
    # summed column return PG_ERR_UNSUPPORTED (the caller probes, then groups).
    R, S = _fused_rows(100_000, 700, (1 << 22) + 300, 93)
    S[1025, 1] = np.float64(7.0e40).view(np.int64)
    got = canon(ctx.hashjoin_groupby(R, S, val=(8, "dec")))
    joined, _, _ = orc.hashjoin(R, S, proj=(("B", 8, 8), ("P", 8, 8)), hash=orc.hashcfg("modulo", 1 << 12))
    assert np.array_equal(got, canon(orc.groupby_exact(joined.view(np.int64).reshape(-1, 2))))
    S[77, 1] = np.float64(np.nan).view(np.int64)
    with pytest.raises(gpu.PgError) as e:
        ctx.hashjoin_groupby(R, S, val=(8, "dec"))
    assert e.value.code == gpu.PG_ERR_UNSUPPORTED


def test_hashjoin_groupby_unsupported_layouts(ctx):
    # A hashed (sparse-key) table cannot take the one-pass plan: the caller is
    # told so and falls back to probe + group-by.
    R, S = _fused_rows(5000, 50, 20_000, 97)
    R[:, 0] *= 7919
    S[:, 0] *= 7919
    with pytest.raises(gpu.PgError) as e:
        ctx.hashjoin_groupby(R, S)
    assert e.value.code == gpu.PG_ERR_UNSUPPORTED


def test_groupby_key_window_from_sample(ctx):
    # Inputs of 4M+ rows take the dense window from a sample of every 1024th
    # row. Keys outside it (rows the sample skipped) send the operator to the
    # exact window; keys the sample caught only widen it. Same groups either way.
    n = (1 << 22) + 4097
    rows = dg.uniform_keys(n, 5000, dg.seed_for(81))
    rows[:, 1] = (rows[:, 1] % 1000).astype(np.float64).view(np.int64)
    for outlier_at, key in ((1025, 7000), (2048, 9999), (n - 1, -3000)):
        r = rows.copy()
        r[outlier_at, 0] = key
        got = ctx.groupby(r, val=(8, "dec"), agg="sum", groups_hint=5000)
        want = orc.groupby_exact(r)
        g, w = canon(got), canon(want)
        assert np.array_equal(g[:, :8], w[:, :8])
        gv, wv = g[:, 8:].copy().view(np.float64).ravel(), w[:, 8:].copy().view(np.float64).ravel()
        assert np.all(np.abs(gv - wv) <= DEC_RTOL * np.abs(wv))
    got = ctx.groupby(rows, val=(8, "long"), agg="count", groups_hint=5000)
    assert np.array_equal(canon(got), canon(orc.groupby(rows, val=(8, "long"), agg="count",
                                                        hash=orc.hashcfg("modulo", 1024))))


def test_groupby_reference_unit_test(gbctx):
    ctx = gbctx
    # unit_tests/queryaggsum.cpp: group i holds 1..i; sum must be i(i+1)/2.
    rows = gin.make({"gen": "formula", "name": "agg_1_to_i", "n": 20})
    got = ctx.groupby(rows, val=(8, "dec"), agg="sum").view(np.int64).reshape(-1, 2)
    d = {int(k): float(v) for k, v in zip(got[:, 0], got[:, 1].view(np.float64))}
    assert d == {i: i * (i + 1) / 2 for i in range(1, 21)}


# ---------------------------------------------------------------- sort
def _sort_check(ctx, rows, key=(0, 8)):
    got = ctx.sort(rows, key)
    want = orc.sort(rows, key)
    if rows.shape[0] == 0:
        assert got.shape == rows.shape
        return
    kb = key[1]
    gk = got.view(np.uint8).reshape(got.shape[0], -1)[:, key[0]:key[0] + kb].copy().view(np.int64 if kb == 8 else np.int32)
    wk = want.view(np.uint8).reshape(want.shape[0], -1)[:, key[0]:key[0] + kb].copy().view(np.int64 if kb == 8 else np.int32)
    assert np.array_equal(gk, wk)
    assert np.array_equal(canon(got), canon(want))


@pytest.mark.parametrize("n", [0, 1, 100, 4095, 4096, 4097, 8192, 100_000, 1_000_003])
@pytest.mark.parametrize("path", [0, 1, 2])
def test_sort_sizes(ctx, n, path):
    # Keys over 2^40: path 0 sorts by 8-bit LSD radix passes above 2^18 tuples and
    # by bitonic tiles and merges below, 1 always radix, 2 always bitonic.
    try:
        ctx.tune(sort_path=path)
        _sort_check(ctx, dg.uniform_keys(n, 1 << 40, dg.seed_for(60)))
    finally:
        ctx.tune(sort_path=0)


def test_sort_duplicates_and_negatives(ctx):
    _sort_check(ctx, dg.uniform_keys(300_000, 50, dg.seed_for(61)))
    _sort_check(ctx, gin.make({"gen": "formula", "name": "signed_keys", "n": 50_000}))
    a = dg.uniform_keys(10_000, 10, dg.seed_for(62))
    a[:, 0] = np.iinfo(np.int64).max - a[:, 0]
    a[::3, 0] = np.iinfo(np.int64).min
    _sort_check(ctx, a)                              # span 2^64 - 1: bitonic
    b = dg.uniform_keys(400_000, 1 << 62, dg.seed_for(65))
    b[::2, 0] -= 1 << 61                             # span just under 2^63, negatives: eight radix passes
    _sort_check(ctx, b)


def test_sort_layouts(ctx):
    a = dg.uniform_keys(70_000, 1 << 30, dg.seed_for(63))
    _sort_check(ctx, a, key=(8, 8))                  # key in the second column
    t8 = gin.make({"gen": "formula", "name": "int_pairs", "n": 50_000})
    _sort_check(ctx, t8, key=(4, 4))                 # int key
    t20 = np.zeros((30_000, 5), dtype=np.int32)
    t20[:, 0] = np.arange(30_000)
    t20[:, 1:] = dg.uniform_keys(30_000, 999, dg.seed_for(64)).view(np.int32)
    _sort_check(ctx, t20, key=(4, 8))


# ---------------------------------------------------------------- MPSM
def _mpsm_check(ctx, R, S, proj=(("P", 8, 8), ("B", 8, 8)), bkey=(0, 8), pkey=(0, 8)):
    got, n, _ = ctx.mpsm(R, S, proj=proj, bkey=bkey, pkey=pkey)
    want, wn, _ = orc.mergejoin(R, S, proj=proj, bkey=bkey, pkey=pkey)
    assert n == wn
    assert np.array_equal(canon(got), canon(want))
    for sc in range(len(proj)):
        _, n2, s2 = ctx.mpsm(R, S, proj=proj, bkey=bkey, pkey=pkey, flags=gpu.JOIN_COUNT | gpu.JOIN_SUM, sum_col=sc)
        _, wn2, ws2 = orc.mergejoin(R, S, proj=proj, bkey=bkey, pkey=pkey, materialise=False, sum_col=sc)
        assert (n2, s2) == (wn2, ws2)
    return n


def test_mpsm_reference_unit_tests(ctx):
    f = lambda name, n: gin.make({"gen": "formula", "name": name, "n": n})  # noqa: E731
    assert _mpsm_check(ctx, f("i_i", 2000), f("i_i", 2000)) == 2000
    assert _mpsm_check(ctx, f("i_i", 2000), f("fk_i_and_3", 2000)) == 5000
    assert _mpsm_check(ctx, f("ones", 200), f("ones", 200)) == 40_000


@pytest.mark.parametrize("span_bits", [13, 17, 21, 24])
def test_mpsm_count_sum_bucketed_key_spans(ctx, span_bits):
    # Count/sum joins with key spans of 2^13..2^24 take the bucketed merge (one
    # radix pass of up to 8 bucket bits, or two halves); both summed sides,
    # a hot key and negative keys included.
    n = 300_000
    R = dg.uniform_keys(n, 1 << span_bits, dg.seed_for(72 + span_bits))
    S = dg.uniform_keys(n, 1 << span_bits, dg.seed_for(73 + span_bits))
    R[::50, 0] = 77                                   # a hot key on both sides
    S[::40, 0] = 77
    R[:, 0] -= 1 << (span_bits - 1)
    S[:, 0] -= 1 << (span_bits - 1)
    proj = (("P", 8, 8), ("B", 8, 8))
    for sc in (0, 1):
        _, n2, s2 = ctx.mpsm(R, S, proj=proj, flags=gpu.JOIN_COUNT | gpu.JOIN_SUM, sum_col=sc)
        _, wn2, ws2 = orc.mergejoin(R, S, proj=proj, materialise=False, sum_col=sc)
        assert (n2, s2) == (wn2, ws2)
    I = gin.make({"gen": "formula", "name": "int_pairs", "n": 60_000})
    I[:, 0] %= 1 << 15
    _, n3, s3 = ctx.mpsm(I, I, proj=(("P", 4, 4), ("B", 4, 4)), bkey=(0, 4), pkey=(0, 4),
                         flags=gpu.JOIN_COUNT | gpu.JOIN_SUM, sum_col=1)
    _, wn3, ws3 = orc.mergejoin(I, I, proj=(("P", 4, 4), ("B", 4, 4)), bkey=(0, 4), pkey=(0, 4),
                                materialise=False, sum_col=1)
    assert (n3, s3) == (wn3, ws3)


@pytest.mark.parametrize("span_bits", [13, 16, 20, 24])
def test_mpsm_materialised_bucketed_key_spans(ctx, span_bits):
    # Materialised joins of 16-byte tuples with key spans of 2^13..2^24 take
    # the bucketed form (each bucket pair joined in shared memory): rows must
    # be the oracle's multiset for every 16-byte projection, including the
    # build key (taken from the probe's equal key) and the probe key, with a
    # hot key and negative keys.
    n = 300_000
    R = dg.uniform_keys(n, 1 << span_bits, dg.seed_for(90 + span_bits))
    S = dg.uniform_keys(n, 1 << span_bits, dg.seed_for(91 + span_bits))
    R[::97, 0] = 4242                                 # a hot key on both sides
    S[::89, 0] = 4242
    R[:, 0] -= 1 << (span_bits - 1)
    S[:, 0] -= 1 << (span_bits - 1)
    for proj in ((("P", 8, 8), ("B", 8, 8)), (("B", 0, 8), ("P", 8, 8)), (("B", 8, 8), ("P", 0, 8)),
                 (("P", 8, 4), ("B", 12, 4), ("B", 0, 8)), (("B", 8, 8), ("B", 0, 4), ("P", 12, 4))):
        _mpsm_check(ctx, R, S, proj=proj)


def test_mpsm_materialised_bucket_too_large_for_shared_memory(ctx):
    # One key bucket holding more build tuples than shared memory takes
    # (30,000 > 24,576): the join falls back to sorting, with the same rows.
    R = dg.uniform_keys(100_000, 1 << 20, dg.seed_for(96))
    R[:30_000, 0] = (R[:30_000, 0] % 4096) + (1 << 19)     # all in one 4096-key bucket
    S = dg.uniform_keys(100_000, 1 << 20, dg.seed_for(97))
    S[::3, 0] = (S[::3, 0] % 4096) + (1 << 19)
    _mpsm_check(ctx, R, S)


@pytest.mark.parametrize("span", [1 << 20, 1 << 40])
def test_mpsm_presorted_sides(ctx, span):
    # buildpresorted / probepresorted: a side the device confirms sorted skips
    # its partition (key spans up to 2^24) or its sort (wider spans); a side
    # flagged sorted that is not must still join correctly.
    R = dg.uniform_keys(200_000, span, dg.seed_for(98))
    S = dg.uniform_keys(300_000, span, dg.seed_for(99))
    m = R[::7].shape[0]
    S[: 7 * m : 7, 0] = R[::7, 0]                     # some matches at the wide span
    Rs = R[np.argsort(R[:, 0], kind="stable")]
    Ss = S[np.argsort(S[:, 0], kind="stable")]
    want, wn, _ = orc.mergejoin(R, S)
    both = gpu.JOIN_MATERIALIZE | gpu.JOIN_BUILD_SORTED | gpu.JOIN_PROBE_SORTED
    for r, s_, fl in ((Rs, Ss, both), (Rs, S, both), (R, Ss, both), (Rs, Ss, gpu.JOIN_MATERIALIZE)):
        got, n, _ = ctx.mpsm(r, s_, flags=fl)
        assert n == wn
        assert np.array_equal(canon(got), canon(want))
        _, n2, s2 = ctx.mpsm(r, s_, flags=(fl & ~gpu.JOIN_MATERIALIZE) | gpu.JOIN_COUNT | gpu.JOIN_SUM, sum_col=1)
        assert (n2, s2) == orc.mergejoin(R, S, materialise=False, sum_col=1)[1:]


def test_mpsm_duplicates(ctx):
    R = dg.uniform_keys(50_000, 12_500, dg.seed_for(70))
    S = dg.uniform_keys(50_000, 12_500, dg.seed_for(71))
    _mpsm_check(ctx, R, S)


def test_mpsm_skew_and_edges(ctx):
    R = dg.zipf_keys(20_000, 2000, 1.0, dg.seed_for(72))
    S = dg.zipf_keys(20_000, 2000, 1.0, dg.seed_for(73))
    _mpsm_check(ctx, R, S)
    empty = np.zeros((0, 2), dtype=np.int64)
    assert _mpsm_check(ctx, R, empty) == 0
    neg = gin.make({"gen": "formula", "name": "signed_keys", "n": 6000})
    _mpsm_check(ctx, neg, neg, proj=(("B", 0, 8), ("P", 8, 8), ("B", 8, 8)))


def test_mpsm_matches_hashjoin(ctx):
    R = dg.uniform_keys(40_000, 10_000, dg.seed_for(74))
    S = dg.uniform_keys(40_000, 10_000, dg.seed_for(75))
    a, n1, _ = ctx.mpsm(R, S)
    b, n2, _ = ctx.hashjoin(R, S)
    assert n1 == n2 and np.array_equal(canon(a), canon(b))


# ---------------------------------------------------------------- batches
def test_batch_join_count_matches_oracle(ctx):
    from pythia_gb300 import autotune
    rng = np.random.default_rng(3)
    sizes = np.concatenate([rng.integers(1, 3000, 40), [1, 4096, 20_000]])
    rels, items, want = [], [], []
    for i, r in enumerate(sizes):
        R = dg.build_relation(int(r), dg.seed_for(300 + i))
        if i % 3 == 0:
            R[:, 0] = R[:, 0] * 1_000_003            # sparse keys
        S = dg.probe_uniform(int(8 * r), R, dg.seed_for(600 + i))
        S[::11, 0] += 5_000_000                       # some misses
        if i % 5 == 0:
            R[: max(1, int(r) // 4), 0] = R[0, 0]     # duplicate build keys
        dR, dS = ctx.upload(R), ctx.upload(S)
        rels += [dR, dS]
        items.append((dR.ptr, R.shape[0], dS.ptr, S.shape[0]))
        _, n, _ = orc.hashjoin(R, S, materialise=False, hash=orc.hashcfg("modulo", 1024))
        want.append(n)
    items.append((rels[0].ptr, 0, rels[1].ptr, 0))    # an empty instance
    want.append(0)
    for shape in (autotune.BATCH_SHAPES[0], autotune.BATCH_SHAPES[3],
                  dict(autotune.BATCH_SHAPES[8], use_graph=0)):
        b = autotune.prepare(ctx, items, shape)
        try:
            for _ in range(2):                         # replays give the same counts
                counts = np.zeros(len(items), dtype=np.uint64)
                autotune.run(ctx, b, counts)
                assert counts.tolist() == want
        finally:
            autotune.free(ctx, b)
    # The library autotuner times every candidate and picks one of them; the
    # pick gives the same counts.
    shapes = autotune.BATCH_SHAPES[:4]
    best, table = autotune.tune_batch(ctx, {"mixed": items}, shapes=shapes, repeats=2)
    assert best["mixed"] in shapes and len(table["mixed"]) == 4
    assert all(r["ms"] > 0 for r in table["mixed"])
    assert table["mixed"][0]["ms"] == min(r["ms"] for r in table["mixed"])
    b = autotune.prepare(ctx, items, best["mixed"])
    try:
        counts = np.zeros(len(items), dtype=np.uint64)
        autotune.run(ctx, b, counts)
        assert counts.tolist() == want
    finally:
        autotune.free(ctx, b)


def test_batch_rejects_empty_marker_build_key(ctx):
    # Batched tables use -1 as their empty-slot marker; a build key equal to it
    # fails the batch at prepare instead of producing a wrong count.
    from pythia_gb300 import autotune
    R = dg.build_relation(3000, dg.seed_for(320))
    R[7, 0] = -1
    S = dg.probe_uniform(24_000, R, dg.seed_for(321))
    dR, dS = ctx.upload(R), ctx.upload(S)
    with pytest.raises(gpu.PgError) as e:
        autotune.prepare(ctx, [(dR.ptr, R.shape[0], dS.ptr, S.shape[0])], autotune.BATCH_SHAPES[0])
    assert e.value.code == gpu.PG_ERR_UNSUPPORTED
    assert gpu.lib().pg_device_status(ctx.h) == 0      # the failing check cleared the status word


def test_generate_fk_matches_host_replica(ctx):
    import bench
    R = dg.build_relation(5000, dg.seed_for(700))
    dR = ctx.upload(R)
    dS = ctx.alloc(16 * 40_000)
    ctx._check(gpu.lib().pg_generate_fk(ctx.h, ctx.stream, dR.ptr, 5000, 12345, dS.ptr, 40_000))
    got = ctx.download(dS, 16 * 40_000).view(np.int64).reshape(-1, 2)
    assert np.array_equal(got, bench.fk_host(R, 12345, 40_000))


# ---------------------------------------------------------------- host ingest
def test_h2d_by_sm_loads_any_alignment(ctx):
    # pg_h2d_sm: bytes arrive exactly for every source and destination
    # alignment (byte head, 16/8/4/1-byte units, byte tail) from registered
    # memory, and from ordinary memory where the device reads it in place.
    L = gpu.lib()
    src = dg.raw_words(dg.seed_for(710), 0, (3 << 20) // 8).view(np.uint8)
    reg = src.copy()
    ctx._check(L.pg_host_register(ctx.h, reg.ctypes.data, reg.nbytes))
    try:
        assert L.pg_host_readable(ctx.h, reg.ctypes.data) == 1
        sources = [reg] + ([src] if L.pg_host_readable(ctx.h, src.ctypes.data) else [])
        dst = ctx.alloc(3 << 20)
        for host in sources:
            for so in (0, 1, 3, 4, 8, 12, 16):
                for do in (0, 1, 5, 8, 15):
                    for n in (0, 1, 15, 16, 17, 1000, (1 << 20) + 7):
                        ctx._check(L.pg_memset(ctx.h, ctx.stream, dst.ptr, 0xA5, do + n + 16))
                        ctx._check(L.pg_h2d_sm(ctx.h, ctx.stream, dst.ptr + do, host.ctypes.data + so, n))
                        got = ctx.download(dst, do + n + 16, np.uint8)
                        assert np.array_equal(got[do:do + n], host[so:so + n]), (so, do, n)
                        assert (got[:do] == 0xA5).all() and (got[do + n:] == 0xA5).all(), (so, do, n)
    finally:
        ctx._check(L.pg_host_unregister(ctx.h, reg.ctypes.data))


# ---------------------------------------------------------------- bounded waits
PG_ERR_TIMEOUT = 4


@pytest.mark.parametrize("op", ["sort", "partition", "staged_probe"])
def test_bounded_wait_gives_up_and_the_next_call_succeeds(ctx, op):
    # Kernels that stage input through bulk copies wait on an mbarrier for
    # each copy. With the context's wait limit at one non-blocking poll the
    # first wait gives up before its copy lands: the call must fail with
    # PG_ERR_TIMEOUT (the kernel still waits for the copy before its block
    # ends), and the next call with the built-in limit must be right.
    rows = dg.uniform_keys(1 << 20, 1 << 40, dg.seed_for(70))   # key span over 2^32: bitonic tiles
    R = dg.build_relation(70_000, dg.seed_for(71))
    S = dg.probe_uniform(500_000, R, dg.seed_for(72))

    def run():
        if op == "sort":
            return ctx.sort(rows)
        if op == "partition":
            return ctx.partition(rows, gpu.hashcfg("parammodulo", 256), 0, 8)[0]
        return ctx.hashjoin(R, S)[0]

    ctx.tune(spin_limit=1, probe_variant=1 if op == "staged_probe" else 0)
    try:
        with pytest.raises(gpu.PgError) as err:
            run()
        assert err.value.code == PG_ERR_TIMEOUT
    finally:
        ctx.tune(spin_limit=0)
    try:
        got = run()
    finally:
        ctx.tune(probe_variant=0)
    if op == "sort":
        _sort_check(ctx, rows)
    elif op == "partition":
        want, _ = orc.partition(rows, orc.hashcfg("parammodulo", 256))
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    else:
        want, _, _ = orc.hashjoin(R, S, hash=orc.hashcfg("modulo", 1 << 16))
        assert np.array_equal(canon(got), canon(want))
