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
    raise KeyError(name)


def make(spec):
    g = spec["gen"]
    if g == "formula":
        return _formula(spec["name"], spec["n"])
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
