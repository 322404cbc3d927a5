"""Join-table images (pg_hashtable_serialize / _deserialize / _save / _load).

The reference's HashTable::serialize / deserialize (util/hashtable.cpp:99-201)
is tested by unit_tests/testhashtable.cpp:87-181: a table of n < 10000 int
tuples is written to a segment file, a fresh table is loaded from it, and every
value must appear exactly once. The same scenario runs here, and every table
layout (narrow dense, wide dense, hashed, hashed with repeated keys and with
the empty-marker key, 4-byte keys, empty) must probe identically after a round
trip and match the oracle join. The narrow dense image is also rebuilt byte for
byte in numpy from the relation, which pins the format.
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from pythia_gb300 import datagen as dg
from pythia_gb300 import gpu
from tests.golden import inputs as gin

pytestmark = pytest.mark.gpu
PROJ = (("P", 8, 8), ("B", 8, 8))
HEADER = 512
LAYOUT_OFF = 16        # u32 layout: 0 hashed, 1 dense, 2 narrow dense


def canon(a):
    return orc.canonical(np.ascontiguousarray(a))


def wsum(b, base_word=0):
    """sum_i w_i * (2 i + 1) mod 2^64 over zero-padded 8-byte words."""
    b = np.frombuffer(bytes(b) + b"\0" * (-len(b) % 8), dtype="<u8")
    i = np.arange(base_word, base_word + b.size, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return int(np.sum(b * (i * np.uint64(2) + np.uint64(1)), dtype=np.uint64))


def layout(img):
    return int(np.frombuffer(img[LAYOUT_OFF:LAYOUT_OFF + 4], dtype="<u4")[0])


def _round_trip(ctx, R, S, proj=PROJ, bkey=(0, 8), pkey=(0, 8)):
    t = ctx.build_table(R, proj, bkey)
    try:
        img = t.serialize()
        assert img.size == t.image_size() and img.size % 256 == 0
        before = t.probe(S, pkey=pkey)
    finally:
        t.free()
    t2 = ctx.load_table(img, proj)
    try:
        after = t2.probe(S, pkey=pkey)
        sc = len(proj) - 1
        _, n2, s2 = t2.probe(S, pkey=pkey, flags=gpu.JOIN_COUNT | gpu.JOIN_SUM, sum_col=sc)
    finally:
        t2.free()
    want, wn, _ = orc.hashjoin(R, S, proj=proj, bkey=bkey, pkey=pkey, hash=orc.hashcfg("modulo", 1024))
    _, wn2, ws2 = orc.hashjoin(R, S, proj=proj, bkey=bkey, pkey=pkey, materialise=False, sum_col=sc,
                               hash=orc.hashcfg("modulo", 1024))
    assert before[1] == after[1] == wn
    assert np.array_equal(canon(before[0]), canon(after[0]))
    assert np.array_equal(canon(after[0]), canon(want))
    assert (n2, s2) == (wn2, ws2)
    return img


def test_narrow_dense_round_trip(ctx):
    R = dg.build_relation(50_000, dg.seed_for(301))
    S = dg.probe_uniform(300_000, R, dg.seed_for(302))
    S[::91, 0] += 100_000
    assert layout(_round_trip(ctx, R, S)) == 2


def test_wide_dense_round_trip(ctx):
    R = dg.build_relation(40_000, dg.seed_for(303))
    R[:, 1] = dg.raw_words(dg.seed_for(303), 1, 40_000).view(np.int64)
    R[:, 0] = R[:, 0] * 5 // 4                        # holes inside the key range
    S = dg.probe_uniform(200_000, R, dg.seed_for(304))
    assert layout(_round_trip(ctx, R, S)) == 1


def test_hashed_round_trip_with_empty_marker_keys(ctx):
    R = dg.build_relation(60_000, dg.seed_for(305))
    R[:, 0] = R[:, 0] * 7919 - (1 << 40)
    R[5, 0] = -1
    R[6, 0] = -1                                      # two side-list entries
    S = dg.probe_uniform(400_000, R, dg.seed_for(306))
    S[::777, 0] = -1
    S[::1000, 0] += 3
    assert layout(_round_trip(ctx, R, S)) == 0
    assert layout(_round_trip(ctx, R, S, proj=(("B", 8, 8), ("P", 0, 8)))) == 0


def test_hashed_round_trip_repeated_keys(ctx):
    R = dg.uniform_keys(5000, 700, dg.seed_for(307))
    S = dg.uniform_keys(9000, 900, dg.seed_for(308))
    assert layout(_round_trip(ctx, R, S)) == 0


def test_round_trip_int32_keys_and_4_byte_columns(ctx):
    I = gin.make({"gen": "formula", "name": "int_pairs", "n": 4000})
    I[:, 0] %= 500
    _round_trip(ctx, I, I, proj=(("P", 4, 4), ("B", 4, 4)), bkey=(0, 4), pkey=(0, 4))
    R = dg.build_relation(3000, dg.seed_for(309))
    S = dg.probe_uniform(9000, R, dg.seed_for(310))
    _round_trip(ctx, R, S, proj=(("P", 0, 8), ("P", 8, 8), ("B", 8, 4), ("B", 12, 4)))


def test_round_trip_empty_build(ctx):
    R = np.zeros((0, 2), dtype=np.int64)
    S = dg.build_relation(1000, dg.seed_for(311))
    _round_trip(ctx, R, S)


def test_reference_serialize_deserialize_scenario(ctx):
    # testhashtable.cpp:87-181: keys and values 0..n-1 (n < 10000), written,
    # loaded into a fresh table, every value found exactly once; the same on a
    # sparse key domain (hashed layout).
    rng = np.random.default_rng(20240613)
    for spread in (1, 7919):
        n = int(rng.integers(1, 10_000))
        R = np.stack([np.arange(n) * spread, np.arange(n)], axis=1).astype(np.int64)
        t = ctx.build_table(R, (("B", 8, 8),))
        img = t.serialize()
        t.free()
        t2 = ctx.load_table(img, (("B", 8, 8),))
        rows, cnt, _ = t2.probe(R)
        t2.free()
        assert cnt == n
        assert np.array_equal(np.bincount(rows.view(np.int64).ravel(), minlength=n), np.ones(n, dtype=np.int64))


def test_narrow_dense_image_bytes(ctx):
    # The image of a narrow dense table, rebuilt from the relation in numpy.
    n = 30_001
    R = dg.build_relation(n, dg.seed_for(312), key_base=-12_345)
    R[:, 0] = -12_345 + (R[:, 0] + 12_345) * 5 // 4   # holes: range 1.25 |R|, below 2 |R|
    R = R[np.argsort(R[:, 0] % 7, kind="stable")]     # any row order
    t = ctx.build_table(R, PROJ)
    img = t.serialize()
    t.free()
    keys, vals = R[:, 0], R[:, 1].view(np.uint64)
    kmin, kmax = int(keys.min()), int(keys.max())
    drange = kmax - kmin + 1
    vmin, vmax = int(vals.min()), int(vals.max())
    entries = np.full(drange, 0xFFFFFFFF, dtype="<u4")
    entries[keys - kmin] = (vals - np.uint64(vmin)).astype(np.uint32)
    sec = entries.tobytes()
    size = HEADER + (len(sec) + 255) // 256 * 256
    h = np.zeros(HEADER, dtype=np.uint8)

    def put(off, dt, v):
        a = np.asarray(v, dtype=dt)
        h[off:off + a.nbytes] = np.frombuffer(a.tobytes(), dtype=np.uint8)
    h[0:8] = np.frombuffer(b"PGJTABLE", dtype=np.uint8)
    put(8, "<u4", [1, HEADER, 2, 1])                   # version, header bytes, layout, unique
    put(24, "<u8", n)
    put(32, "<u4", [16, 8, 0, 0])                      # tuple width, key bytes, log2cap, side entries
    put(48, "<i8", kmin)
    put(56, "<u8", [drange, vmin, vmax])
    put(80, "<u4", [2, 0])                             # projected columns
    put(88, "<u4", [1, 8, 8, 0, 8, 8])                 # P$1, B$1 (side, offset, bytes)
    put(280 + 4 * 8, "<u8", HEADER)                    # section offsets: narrow dense entries
    put(320 + 4 * 8, "<u8", len(sec))                  # section sizes
    put(360, "<u8", [size, wsum(sec, HEADER // 8)])    # image size, payload checksum
    put(504, "<u8", wsum(h[:504].tobytes()))
    want = np.zeros(size, dtype=np.uint8)
    want[:HEADER] = h
    want[HEADER:HEADER + len(sec)] = np.frombuffer(sec, dtype=np.uint8)
    assert img.size == size
    assert np.array_equal(img, want)


def test_damaged_images_are_refused(ctx):
    R = dg.build_relation(20_000, dg.seed_for(313))
    S = dg.probe_uniform(50_000, R, dg.seed_for(314))
    t = ctx.build_table(R, PROJ)
    img = t.serialize()
    t.free()
    cases = {}
    bad = img.copy(); bad[HEADER + 1000] ^= 0x10; cases["payload"] = bad
    bad = img.copy(); bad[24] ^= 1; cases["header field"] = bad
    bad = img.copy(); bad[0] = ord("X"); cases["magic"] = bad
    cases["truncated"] = img[:-256]
    cases["short"] = img[:100]
    for what, b in cases.items():
        with pytest.raises(gpu.PgError) as e:
            ctx.load_table(b, PROJ)
        assert e.value.code == gpu.PG_ERR_ARG, what
    # The context is still usable, and the intact image still loads.
    t2 = ctx.load_table(img, PROJ)
    _, n, _ = t2.probe(S, flags=gpu.JOIN_COUNT)
    t2.free()
    assert n == 50_000


def test_row_index_tables_have_no_image(ctx):
    R = dg.build_relation(3000, dg.seed_for(315))
    t = ctx.build_table(R, (("B", 0, 8), ("B", 8, 8), ("P", 8, 8)))   # 16 B of build columns
    try:
        with pytest.raises(gpu.PgError) as e:
            t.serialize()
        assert e.value.code == gpu.PG_ERR_UNSUPPORTED
    finally:
        t.free()


def test_file_round_trip_and_exclusive_create(ctx, tmp_path):
    R = dg.build_relation(25_000, dg.seed_for(316))
    R[:, 0] *= 3                                       # hashed layout
    S = dg.probe_uniform(100_000, R, dg.seed_for(317))
    p = os.path.join(tmp_path, "table.img")
    t = ctx.build_table(R, PROJ)
    want = t.probe(S)
    t.save(p)
    with pytest.raises(gpu.PgError):
        t.save(p)                                      # the file exists
    assert os.path.getsize(p) == t.image_size()
    t.free()
    t2 = ctx.load_table(p, PROJ)
    got = t2.probe(S)
    t2.free()
    assert got[1] == want[1] and np.array_equal(canon(got[0]), canon(want[0]))
    with pytest.raises(gpu.PgError):
        ctx.load_table(os.path.join(tmp_path, "missing.img"), PROJ)


def test_loaded_table_on_another_context_and_fused_groupby(ctx):
    # A served table restored into a second context feeds the one-pass
    # join + group-by like the original.
    R = dg.build_relation(60_000, dg.seed_for(318))
    R[:, 1] = dg.raw_words(dg.seed_for(318), 3, 60_000) % np.uint64(600)
    S = dg.probe_uniform(480_000, R, dg.seed_for(319))
    S[:, 1] = dg.raw_words(dg.seed_for(319), 5, S.shape[0]).view(np.int64) >> 20
    gproj = (("B", 8, 8), ("P", 8, 8))
    t = ctx.build_table(R, gproj)
    img = t.serialize()
    want = canon(t.groupby(S, val=(8, "long"), agg="sum", cap=R.shape[0]))
    t.free()
    c2 = gpu.Context(0)
    try:
        t2 = c2.load_table(img, gproj)
        got = canon(t2.groupby(S, val=(8, "long"), agg="sum", cap=R.shape[0]))
        t2.free()
    finally:
        c2.close()
    jl, _, _ = orc.hashjoin(R, S, proj=gproj, hash=orc.hashcfg("modulo", 1 << 12))
    assert np.array_equal(got, want)
    assert np.array_equal(got, canon(orc.groupby(jl.view(np.int64).reshape(-1, 2), val=(8, "long"), agg="sum")))
