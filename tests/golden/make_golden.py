"""Regenerates tests/golden/golden.json from the REFERENCE engine.

Runs the reference Pythia operators (compiled from the reference source tree
by oracle/Makefile.ref into oracle/_ref/ref_driver) on seeded synthetic
inputs and records compact digests of their outputs. The digests pin both the
C oracle (tests/test_oracle_golden.py) and, through it, the GPU operators.

Inputs are not stored: each case names the generator call that makes it
(pythia_gb300.datagen) and the SHA-256 of the bytes, so a test can rebuild
the input on any machine and first check that the generator agrees.

Run where the reference source tree exists (REF names it):
    make -f oracle/Makefile.ref REF=<reference source tree> -j8
    python tests/golden/make_golden.py [--keep-existing]
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from pythia_gb300 import datagen as dg  # noqa: E402
from tests.golden import inputs as gin  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def canonical(rows):
    if rows.shape[0] == 0:
        return np.zeros((0, 0), dtype=np.uint8)
    u8 = np.ascontiguousarray(rows).view(np.uint8).reshape(rows.shape[0], -1)
    return np.sort(u8.view(f"V{u8.shape[1]}").ravel()).view(np.uint8).reshape(-1, u8.shape[1])


def run(tmp, mode, files, **kw):
    args = [DRIVER, mode]
    for k, a in files.items():
        p = os.path.join(tmp, k + ".bin")
        np.ascontiguousarray(a).tofile(p)
        args.append(f"{k}={p}")
    out = os.path.join(tmp, "out.bin")
    args.append(f"out={out}")
    args += [f"{k}={v}" for k, v in kw.items()]
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"{args}: {r.stderr}")
    return np.fromfile(out, dtype=np.uint8)


def join_digest(raw, ow):
    rows = raw.reshape(-1, ow)
    return {"n_out": int(rows.shape[0]), "canonical_sha256": sha(canonical(rows))}


def main():
    cases = []
    with tempfile.TemporaryDirectory() as tmp:
        # ---- hash functions (hash.h:51-479 via TupleHasher::create) ----
        A = gin.make({"gen": "uniform_keys", "n": 20000, "range": 5000, "rel": 3})
        neg = gin.make({"gen": "formula", "name": "signed_keys", "n": 4096})
        for fn, extra in [("bytes", {}), ("modulo", {}), ("range", {"min": 0, "max": 4999}),
                          ("exactrange", {"min": 0, "max": 4999}),
                          ("parammodulo", {"skipbits": 3, "offset": 7}),
                          ("knuth", {"skipbits": 2, "offset": 5}),
                          ("tpchorderkey", {}), ("willis", {})]:
            for buckets in (100, 1024):
                for src, spec in (("A", {"gen": "uniform_keys", "n": 20000, "range": 5000, "rel": 3}),
                                  ("neg", {"gen": "formula", "name": "signed_keys", "n": 4096})):
                    data = A if src == "A" else neg
                    if fn in ("range", "exactrange") and src == "neg":
                        continue
                    h = run(tmp, "hash", {"in": data}, fn=fn, buckets=buckets, **extra).view(np.uint32)
                    cases.append({"name": f"hash_{fn}_{buckets}_{src}", "op": "hash",
                                  "inputs": {"in": spec}, "input_sha256": {"in": sha(data)},
                                  "params": {"fn": fn, "buckets": buckets, **extra},
                                  "ref": {"buckets": int(h[-1]), "sha256": sha(h[:-1])}})
        # int32 key column (numericalize sign-extends CtInt): schema int,int.
        I = gin.make({"gen": "formula", "name": "int_pairs", "n": 4096})
        for fn in ("modulo", "bytes", "knuth", "willis"):
            h = run(tmp, "hash", {"in": I}, schema="int,int", fn=fn, buckets=256).view(np.uint32)
            cases.append({"name": f"hash_{fn}_int32", "op": "hash",
                          "inputs": {"in": {"gen": "formula", "name": "int_pairs", "n": 4096}},
                          "input_sha256": {"in": sha(I)},
                          "params": {"fn": fn, "buckets": 256, "schema": "int,int"},
                          "ref": {"buckets": int(h[-1]), "sha256": sha(h[:-1])}})

        # ---- hash join (join.cpp:273-675) ----
        def hj(name, rspec, sspec, threads=4, buckets=1024, fn="modulo", tpb=4,
               proj="P$1,B$1", bschema="long,long", pschema="long,long", ow=16, agg=None, keys=None):
            R, S = gin.make(rspec), gin.make(sspec)
            kw = dict(threads=threads, buckets=buckets, fn=fn, tuplesperbucket=tpb, proj=proj,
                      bschema=bschema, pschema=pschema, buffsize=4096)
            if keys:
                kw.update(buildjattr=keys[0], probejattr=keys[1])
            raw = run(tmp, "hashjoin", {"build": R, "probe": S}, **kw)
            ref = join_digest(raw, ow)
            for a in ("count", "sum"):
                v = run(tmp, "hashjoin", {"build": R, "probe": S}, agg=a, sumfield=1, **kw)
                ref[a] = int(v.view(np.int64)[0]) if v.size else 0
            cases.append({"name": name, "op": "hashjoin", "inputs": {"R": rspec, "S": sspec},
                          "input_sha256": {"R": sha(R), "S": sha(S)},
                          "params": dict({"threads": threads, "buckets": buckets, "fn": fn,
                                          "tuplesperbucket": tpb, "proj": proj, "bschema": bschema,
                                          "pschema": pschema},
                                         **({"buildjattr": keys[0], "probejattr": keys[1]} if keys else {})),
                          "ref": ref})

        hj("hashjoin_reference_test_20", {"gen": "formula", "name": "i_i", "n": 20},
           {"gen": "formula", "name": "i_i_plus_0.1", "n": 20}, buckets=16, tpb=2,
           proj="B$1,P$1", pschema="long,dec")
        hj("hashjoin_pkfk_4k_32k", {"gen": "build", "n": 4096, "rel": 1},
           {"gen": "probe_uniform", "n": 32768, "build": {"gen": "build", "n": 4096, "rel": 1}, "rel": 2})
        hj("hashjoin_pkfk_zipf", {"gen": "build", "n": 8192, "rel": 11},
           {"gen": "probe_zipf", "n": 65536, "s": 1.0, "build": {"gen": "build", "n": 8192, "rel": 11}, "rel": 12})
        hj("hashjoin_many_to_many", {"gen": "uniform_keys", "n": 2048, "range": 512, "rel": 5},
           {"gen": "uniform_keys", "n": 4096, "range": 600, "rel": 6}, buckets=256)
        hj("hashjoin_knuth_proj3", {"gen": "build", "n": 3000, "rel": 7},
           {"gen": "probe_uniform", "n": 9000, "build": {"gen": "build", "n": 3000, "rel": 7}, "rel": 8},
           fn="knuth", proj="B$0,P$1,B$1", ow=24, buckets=2048)
        hj("hashjoin_empty_probe", {"gen": "build", "n": 100, "rel": 9},
           {"gen": "formula", "name": "empty", "n": 0})
        hj("hashjoin_no_matches", {"gen": "build", "n": 1000, "rel": 9},
           {"gen": "formula", "name": "big_keys", "n": 5000})
        # The q1 plan's part join: 24-byte lines (order, part, price) keyed on
        # their second column, into 24- and 16-byte rows.
        lines = {"gen": "lines", "n": 40000, "build": {"gen": "build", "n": 6000, "rel": 21}, "rel": 22,
                 "miss_every": 37}
        hj("hashjoin_q1_lines_24B", {"gen": "build", "n": 6000, "rel": 21}, lines,
           proj="P$0,P$2,B$1", pschema="long,long,dec", ow=24, keys=(0, 1))
        hj("hashjoin_q1_lines_16B", {"gen": "build", "n": 6000, "rel": 21}, lines,
           proj="P$2,B$1", pschema="long,long,dec", ow=16, keys=(0, 1))

        # ---- partition (partition.cpp:45-404), stable order per partition ----
        for T, spec in [(1, {"gen": "uniform_keys", "n": 20000, "range": 5000, "rel": 3}),
                        (3, {"gen": "uniform_keys", "n": 20000, "range": 5000, "rel": 3}),
                        (7, {"gen": "uniform_keys", "n": 20000, "range": 5000, "rel": 3}),
                        (15, {"gen": "uniform_keys", "n": 131072, "range": 131072, "rel": 13}),
                        (5, {"gen": "zipf_keys", "n": 50000, "range": 10000, "s": 1.0, "rel": 14})]:
            data = gin.make(spec)
            lo, hi = 0, int(spec["range"]) - 1
            raw = run(tmp, "partition", {"in": data}, threads=T, min=lo, max=hi, buffsize=4096)
            raw = raw.reshape(-1, 20)
            tid = raw[:, :4].copy().view(np.int32).ravel()
            rows = raw[:, 4:].copy()
            parts = [{"n": int((tid == p).sum()), "sha256": sha(rows[tid == p])} for p in range(T)]
            cases.append({"name": f"partition_exactrange_T{T}_{spec['gen']}", "op": "partition",
                          "inputs": {"in": spec}, "input_sha256": {"in": sha(data)},
                          "params": {"buckets": T, "min": lo, "max": hi}, "ref": {"partitions": parts}})

        # ---- aggregates (genericaggregate.cpp, aggregatesum.cpp, aggregatecount.cpp) ----
        def agg(name, spec, mode, schema, aggmode="twostage", threads=4, buckets=1024, ow=16):
            data = gin.make(spec)
            raw = run(tmp, mode, {"in": data}, schema=schema, threads=threads, buckets=buckets,
                      aggmode=aggmode, buffsize=4096)
            rows = raw.reshape(-1, ow)
            ref = {"ngroups": int(rows.shape[0])}
            if schema.endswith("dec") and mode == "aggsum":
                srt = rows[np.argsort(rows[:, :8].copy().view(np.int64).ravel(), kind="stable")]
                ref["keys_sha256"] = sha(srt[:, :8])
                ref["sums"] = [float(v) for v in srt[:, 8:].copy().view(np.float64).ravel()][:4096]
            else:
                ref["canonical_sha256"] = sha(canonical(rows))
            cases.append({"name": name, "op": mode, "inputs": {"in": spec},
                          "input_sha256": {"in": sha(data)},
                          "params": {"schema": schema, "aggmode": aggmode, "threads": threads,
                                     "buckets": buckets}, "ref": ref})

        agg("aggsum_reference_test_1_to_i", {"gen": "formula", "name": "agg_1_to_i", "n": 20},
            "aggsum", "long,dec", buckets=4)
        agg("aggsum_global_reference_test", {"gen": "formula", "name": "agg_1_to_i", "n": 20},
            "aggsum", "long,dec", aggmode="global", buckets=4096, threads=8)
        agg("aggsum_long_5k_groups", {"gen": "uniform_keys", "n": 20000, "range": 5000, "rel": 3},
            "aggsum", "long,long")
        agg("aggcount_long_5k_groups", {"gen": "uniform_keys", "n": 20000, "range": 5000, "rel": 3},
            "aggcount", "long,long")
        agg("aggsum_dec_300_groups", {"gen": "groupby", "n": 20000, "groups": 300, "vmax": 1e4, "rel": 4},
            "aggsum", "long,dec")
        agg("aggsum_dec_zipf_keys", {"gen": "groupby_zipf", "n": 30000, "groups": 2000, "rel": 15},
            "aggsum", "long,dec")
        agg("aggsum_int_wrap", {"gen": "formula", "name": "int_big", "n": 8192},
            "aggsum", "int,int", ow=8, buckets=64)
        agg("aggcount_global_one_group", {"gen": "uniform_keys", "n": 5000, "range": 1, "rel": 16},
            "aggcount", "long,long", aggmode="global", threads=3)

        # ---- sort-merge / MPSM join (join.cpp:945-1371) and page sort ----
        def mj(name, rspec, sspec, threads=4):
            R, S = gin.make(rspec), gin.make(sspec)
            mf = int(np.bincount(R[:, 0] - R[:, 0].min()).max()) if R.shape[0] else 1
            raw = run(tmp, "oldmpsm", {"build": R, "probe": S}, threads=threads,
                      maxbuildtuples=2 * R.shape[0] + 64, maxprobetuples=2 * S.shape[0] + 64,
                      mostfreq=mf, buffsize=4096)
            ref = join_digest(raw, 16)
            rows = raw.reshape(-1, 16)
            ref["sum_build_plus_probe"] = int(
                (rows[:, :8].copy().view(np.int64).astype(np.uint64).sum(dtype=np.uint64)
                 + rows[:, 8:].copy().view(np.int64).astype(np.uint64).sum(dtype=np.uint64))
                .astype(np.int64)) if rows.shape[0] else 0
            cases.append({"name": name, "op": "mpsm", "inputs": {"R": rspec, "S": sspec},
                          "input_sha256": {"R": sha(R), "S": sha(S)},
                          "params": {"threads": threads, "proj": "P$1,B$1"}, "ref": ref})

        mj("mpsm_pk_pk_2000", {"gen": "formula", "name": "i_i", "n": 2000},
           {"gen": "formula", "name": "i_i", "n": 2000})
        mj("mpsm_pk_fk_multiplicity", {"gen": "formula", "name": "i_i", "n": 2000},
           {"gen": "formula", "name": "fk_i_and_3", "n": 2000})
        mj("mpsm_cartesian_200", {"gen": "formula", "name": "ones", "n": 200},
           {"gen": "formula", "name": "ones", "n": 200})
        mj("mpsm_dups_4k", {"gen": "uniform_keys", "n": 4096, "range": 1024, "rel": 5},
           {"gen": "uniform_keys", "n": 4096, "range": 1024, "rel": 6})
        mj("mpsm_negative_keys", {"gen": "formula", "name": "signed_keys", "n": 4096},
           {"gen": "formula", "name": "signed_keys", "n": 4096}, threads=3)

        for spec in ({"gen": "uniform_keys", "n": 20000, "range": 5000, "rel": 3},
                     {"gen": "formula", "name": "signed_keys", "n": 4096},
                     {"gen": "uniform_keys", "n": 4096, "range": 1 << 40, "rel": 17}):
            data = gin.make(spec)
            raw = run(tmp, "sort", {"in": data}).reshape(-1, 16)
            cases.append({"name": f"sort_{spec.get('name', spec['gen'])}_{spec['n']}", "op": "sort",
                          "inputs": {"in": spec}, "input_sha256": {"in": sha(data)},
                          "params": {"keyoff": 0},
                          "ref": {"keys_sha256": sha(raw[:, :8]),
                                  "canonical_sha256": sha(canonical(raw))}})

        # ---- Filter (filter.cpp:37-85) and Project (project.cpp:37-104) ----
        # One scanning thread: the output keeps the input order exactly.
        MIX = {"gen": "formula", "name": "mixed_cols", "n": 5000}
        mixed = gin.make(MIX)
        FIELD = {"int": 0, "long": 1, "dec": 2, "char": 3, "date": 4}
        filters = [
            [("int", "<", "0")], [("int", "=", "7")], [("int", "!=", "-3")], [("int", ">=", "15")],
            [("long", "<=", str(-300 * (1 << 31)))], [("long", ">", "0")], [("long", "==", str(17 * (1 << 31)))],
            [("dec", "<", "0")], [("dec", "==", "0")], [("dec", "!=", "nan")], [("dec", ">", "-inf")],
            [("dec", "<>", "1.5")], [("dec", ">=", "inf")], [("dec", "<=", "-12.375")],
            [("char", "=", "abc")], [("char", "<", "alpha")], [("char", ">", "ab")], [("char", "<>", "")],
            [("char", ">=", "b")], [("char", "==", "delta epsilon")], [("char", "<", "abc\xe9")],
            [("date", "<", "1995-03-15")], [("date", ">=", "1993-01-01")], [("date", "==", "1994-06-10")],
            [("int", ">", "-5"), ("dec", "<", "30"), ("char", "!=", "zz")],
            [("date", ">=", "1994-01-01"), ("date", "<", "1995-01-01"), ("long", ">=", "0"), ("int", "<>", "0")],
        ]
        for k, flt in enumerate(filters):
            kw = {}
            for j, (col, op, val) in enumerate(flt):
                sfx = str(j + 1) if j else ""
                kw["field" + sfx] = FIELD[col]
                kw["op" + sfx] = op
                kw["value" + sfx] = val
            raw = run(tmp, "filter", {"in": mixed}, schema=gin.MIXED_SCHEMA, buffsize=4096, **kw)
            rows = raw.reshape(-1, gin.MIXED_WIDTH)
            cases.append({"name": f"filter_{k}_{'_'.join(c for c, _, _ in flt)}", "op": "filter",
                          "inputs": {"in": MIX}, "input_sha256": {"in": sha(mixed)},
                          "params": {"schema": gin.MIXED_SCHEMA,
                                     "filters": [[FIELD[c], o, v] for c, o, v in flt]},
                          "ref": {"n": int(rows.shape[0]), "sha256": sha(rows)}})
        # The reference's own test: 20 rows (i, i), field 0 < 10 (unit_tests/querymap.cpp:41-190).
        ii = {"gen": "formula", "name": "i_i", "n": 20}
        raw = run(tmp, "filter", {"in": gin.make(ii)}, schema="long;long", field=0, op="<", value="10", buffsize=64)
        cases.append({"name": "filter_reference_querymap", "op": "filter", "inputs": {"in": ii},
                      "input_sha256": {"in": sha(gin.make(ii))},
                      "params": {"schema": "long;long", "filters": [[0, "<", "10"]]},
                      "ref": {"n": int(raw.size // 16), "sha256": sha(raw.reshape(-1, 16))}})
        for proj in ("3,0", "4,2,1", "0,0,1", "2"):
            raw = run(tmp, "project", {"in": mixed}, schema=gin.MIXED_SCHEMA, projection=proj, buffsize=4096)
            cases.append({"name": f"project_{proj.replace(',', '_')}", "op": "project", "inputs": {"in": MIX},
                          "input_sha256": {"in": sha(mixed)}, "params": {"schema": gin.MIXED_SCHEMA, "projection": proj},
                          "ref": {"bytes": int(raw.size), "sha256": sha(raw)}})
        # unit_tests/queryproject.cpp: ("$1") of 20 rows (i, i).
        raw = run(tmp, "project", {"in": gin.make(ii)}, schema="long;long", projection="1", buffsize=64)
        cases.append({"name": "project_reference_queryproject", "op": "project", "inputs": {"in": ii},
                      "input_sha256": {"in": sha(gin.make(ii))}, "params": {"schema": "long;long", "projection": "1"},
                      "ref": {"bytes": int(raw.size), "sha256": sha(raw)}})

    path = os.path.join(ROOT, "tests", "golden", "golden.json")
    if "--keep-existing" in sys.argv and os.path.exists(path):
        # Cases already in the file keep their recorded digests (some dec
        # sums of threaded reference runs differ in the last bits between
        # runs); only new case names take the fresh ones.
        with open(path) as f:
            old = {c["name"]: c for c in json.load(f)["cases"]}
        cases = [old.get(c["name"], c) for c in cases]
    with open(path, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "reference": "sblanas/pythia operators via oracle/_ref/ref_driver",
                   "cases": cases}, f, indent=1)
    print(f"wrote {len(cases)} cases to {path}")


if __name__ == "__main__":
    main()
