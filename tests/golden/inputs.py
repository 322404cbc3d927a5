"""Rebuilds the inputs that tests/golden/golden.json names.

A spec is either a call of the seeded generator (pythia_gb300.datagen, seed =
SEED_BASE + rel) or one of the closed-form relations the reference's own unit
tests use (unit_tests/common.h:55-63 writes i|i; queryhashjoin.cpp:102-111
writes i|i+0.1; queryaggsum.cpp:100-110 writes group i with values 1..i;
querympsmpkfkjoin.cpp gives key i multiplicity (i&3)+1;
querympsmcartesianprod.cpp uses all-ones keys).
"""
import numpy as np

from pythia_gb300 import datagen as dg


def _formula(name, n):
    if name == "empty":
        return np.zeros((0, 2), dtype=np.int64)
    if name == "i_i":
        i = np.arange(1, n + 1, dtype=np.int64)
        return np.stack([i, i], axis=1)
    if name == "i_i_plus_0.1":
        i = np.arange(1, n + 1, dtype=np.int64)
        out = np.empty((n, 2), dtype=np.int64)
        out[:, 0] = i
        out[:, 1] = (i.astype(np.float64) + 0.1).view(np.int64)
        return out
    if name == "agg_1_to_i":
        keys, vals = [], []
        for i in range(1, n + 1):
            for k in range(1, i + 1):
                keys.append(i)
                vals.append(float(k))
        out = np.empty((len(keys), 2), dtype=np.int64)
        out[:, 0] = keys
        out[:, 1] = np.array(vals, dtype=np.float64).view(np.int64)
        return out
    if name == "fk_i_and_3":
        keys = [i for i in range(1, n + 1) for _ in range((i & 3) + 1)]
        k = np.array(keys, dtype=np.int64)
        return np.stack([k, np.arange(k.shape[0], dtype=np.int64) * 7 + 1], axis=1)
    if name == "ones":
        return np.stack([np.ones(n, dtype=np.int64), np.arange(n, dtype=np.int64)], axis=1)
    if name == "signed_keys":
        w = dg.raw_words(dg.seed_for(40), 0, 2 * n).view(np.int64).reshape(n, 2)
        out = w.copy()
        out[:, 0] = (w[:, 0] % 2001) - 1000
        out[:, 1] = w[:, 1] & 0x7FFFFFFF
        return out
    if name == "big_keys":
        i = np.arange(n, dtype=np.int64)
        return np.stack([i + (1 << 40), i], axis=1)
    if name == "int_pairs":
        w = dg.raw_words(dg.seed_for(41), 0, n).astype(np.uint64)
        return w.view(np.int32).reshape(n, 2).copy()
    if name == "int_big":
        w = dg.raw_words(dg.seed_for(42), 0, n).astype(np.uint64)
        out = w.view(np.int32).reshape(n, 2).copy()
        out[:, 0] = np.abs(out[:, 0] % 37)
        return out
    if name == "mixed_cols":
        return mixed_cols(n)
    raise KeyError(name)


MIXED_SCHEMA = "int;long;dec;char(11);date(%Y-%m-%d)"
MIXED_OFF = {"int": 0, "long": 4, "dec": 12, "char": 20, "date": 32}
MIXED_WIDTH = 40
WORDS = [b"", b"a", b"ab", b"abc", b"abd", b"b", b"alpha", b"alphabet", b"beta", b"gamma",
         b"delta epsil", b"zz", b"Zeta", b"abc\xe9"]


def date_bits(year, month, day):
    """The engine's packed date (schema.h:66-104): years since 1900 << 46,
    month - 1 << 42, day << 37."""
    return ((year - 1900) << 46) | ((month - 1) << 42) | (day << 37)


def mixed_cols(n):
    """Rows (int, long, dec, char(11), date) = 40 bytes: small-domain ints
    and longs (many equal to the filter constants), decs with NaN, signed
    zeros and infinities, strings sharing prefixes, dates over seven years."""
    w = dg.raw_words(dg.seed_for(43), 0, 5 * n).astype(np.uint64).reshape(5, n) if n else np.zeros((5, 0), np.uint64)
    out = np.zeros((n, MIXED_WIDTH), dtype=np.uint8)
    ints = (w[0] % 41).astype(np.int64) - 20
    longs = (w[1] % 2001).astype(np.int64) * (1 << 31) - 1000 * (1 << 31)
    decs = (w[2] % 1000).astype(np.float64) / 8.0 - 60.0
    sel = w[2] >> np.uint64(40)
    decs[(sel % 53) == 0] = np.nan
    decs[(sel % 59) == 1] = -0.0
    decs[(sel % 61) == 2] = 0.0
    decs[(sel % 67) == 3] = np.inf
    decs[(sel % 71) == 4] = -np.inf
    out[:, 0:4] = ints.astype(np.int32).view(np.uint8).reshape(n, 4)
    out[:, 4:12] = longs.view(np.uint8).reshape(n, 8)
    out[:, 12:20] = decs.view(np.uint8).reshape(n, 8)
    for i in range(n):
        s = WORDS[int(w[3][i] % len(WORDS))]
        out[i, 20:20 + len(s)] = np.frombuffer(s, dtype=np.uint8)
    years = 1992 + (w[4] % 7).astype(np.int64)
    months = 1 + ((w[4] >> np.uint64(8)) % 12).astype(np.int64)
    days = 1 + ((w[4] >> np.uint64(16)) % 28).astype(np.int64)
    out[:, 32:40] = date_bits(years, months, days).astype(np.int64).view(np.uint8).reshape(n, 8)
    return out


def schema_columns(schema):
    """[(type, offset, width)] of a ';'-separated schema list (Schema::create,
    schema.cpp:221-259: char(N) holds N + 1 bytes)."""
    out, off = [], 0
    for c in schema.split(";"):
        if c == "int":
            t, w = "int", 4
        elif c.startswith("char("):
            t, w = "char", int(c[5:-1]) + 1
        elif c.startswith("date"):
            t, w = "date", 8
        else:
            t, w = ("dec" if c == "dec" else "long"), 8
        out.append((t, off, w))
        off += w
    return out


def filter_value(t, text):
    """Filter's constant parsed as Schema::parseTuple does (schema.cpp:129-168):
    atoi / atoll / atof, strncpy of the text, strptime + packed date."""
    import time
    if t == "int":
        return int(text)
    if t == "long":
        return int(text)
    if t == "dec":
        return float(text)
    if t == "date":
        tm = time.strptime(text, "%Y-%m-%d")
        return date_bits(tm.tm_year, tm.tm_mon, tm.tm_mday)
    return text.encode()


def filter_preds(schema, filters):
    """Oracle / GPU predicate specs [(type, op, offset, value, width)] of
    [(field index, op, text)] filters (Filter's field / op / value keys)."""
    cols = schema_columns(schema)
    out = []
    for field, op, text in filters:
        t, off, w = cols[field]
        out.append(("long" if t == "date" else t, op, off, filter_value(t, text), w))
    return out


def _lines(spec):
    """(order, part, price) 24-byte lines: orders 3i + 1, parts drawn from the
    build relation, prices as float64 bits; every miss_every-th part lies past
    the build's keys."""
    n = spec["n"]
    fk = dg.probe_uniform(n, make(spec["build"]), dg.seed_for(spec["rel"]))
    L = np.zeros((n, 3), np.int64)
    L[:, 0] = np.arange(n, dtype=np.int64) * 3 + 1
    L[:, 1] = fk[:, 0]
    raw = dg.raw_words(dg.seed_for(spec["rel"] + 1), 2, n) >> np.uint64(11)
    L[:, 2] = (raw.astype(np.float64) * 1e-9).view(np.int64)
    if spec.get("miss_every"):
        L[::spec["miss_every"], 1] += 1 << 40
    return L


def make(spec):
    g = spec["gen"]
    if g == "formula":
        return _formula(spec["name"], spec["n"])
    if g == "lines":
        return _lines(spec)
    seed = dg.seed_for(spec["rel"])
    if g == "build":
        return dg.build_relation(spec["n"], seed)
    if g == "probe_uniform":
        return dg.probe_uniform(spec["n"], make(spec["build"]), seed)
    if g == "probe_zipf":
        return dg.probe_zipf(spec["n"], spec["s"], make(spec["build"]), seed)
    if g == "uniform_keys":
        return dg.uniform_keys(spec["n"], spec["range"], seed)
    if g == "zipf_keys":
        return dg.zipf_keys(spec["n"], spec["range"], spec["s"], seed)
    if g == "groupby":
        return dg.groupby_rows(spec["n"], spec["groups"], spec["vmax"], seed)
    if g == "groupby_zipf":
        rows = dg.zipf_keys(spec["n"], spec["groups"], 1.0, seed)
        vals = dg.groupby_rows(spec["n"], 1, 1e4, seed)[:, 1]
        rows[:, 1] = vals
        return rows
    raise KeyError(g)
