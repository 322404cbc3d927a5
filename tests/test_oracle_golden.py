"""The oracle against the reference engine's own outputs (tests/golden).

Each case rebuilds its input from the named generator call, checks the bytes
against the recorded SHA-256 (so generator drift is caught first), runs the
C restatement and compares its output digest with the reference's.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc
from tests.golden import inputs as gin

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
CASES = GOLDEN["cases"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def widths(schema):
    return [4 if c == "int" else 8 for c in schema.split(",")]


def proj_types(spec):
    return [(p.split("$")[0], int(p.split("$")[1])) for p in spec.split(",")]


def parse_proj(spec, bschema, pschema):
    out = []
    for p in spec.split(","):
        side, idx = p.split("$")
        ws = widths(bschema if side == "B" else pschema)
        out.append((side, sum(ws[: int(idx)]), ws[int(idx)]))
    return out


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_golden(case):
    inputs = {k: gin.make(spec) for k, spec in case["inputs"].items()}
    for k, a in inputs.items():
        assert sha(a) == case["input_sha256"][k], f"generator drift for input {k}"
    p, ref, op = case["params"], case["ref"], case["op"]
    if op == "hash":
        w = widths(p.get("schema", "long,long"))
        cfg = orc.hashcfg(p["fn"], p["buckets"], p.get("min", 0), p.get("max", 0),
                          p.get("skipbits", 0), p.get("offset", 0))
        h = orc.hash_column(cfg, inputs["in"], 0, w[0], sum(w))
        assert orc.hashfn(cfg).nbuckets == ref["buckets"]
        assert sha(h) == ref["sha256"]
    elif op in ("hashjoin", "mpsm"):
        R, S = inputs["R"], inputs["S"]
        proj = parse_proj(p["proj"], p.get("bschema", "long,long"), p.get("pschema", "long,long"))
        if op == "hashjoin":
            cfg = orc.hashcfg(p["fn"], p["buckets"])
            bw, pw = widths(p.get("bschema", "long,long")), widths(p.get("pschema", "long,long"))
            ba, pa = p.get("buildjattr", 0), p.get("probejattr", 0)
            out, n, s = orc.hashjoin(R, S, proj=proj, hash=cfg, tuplesperbucket=p["tuplesperbucket"],
                                     threads=p["threads"], sum_col=1, bkey=(sum(bw[:ba]), bw[ba]),
                                     pkey=(sum(pw[:pa]), pw[pa]))
            assert n == ref["n_out"] == ref["count"]
            side, idx = proj_types(p["proj"])[1]
            if (p["bschema"] if side == "B" else p["pschema"]).split(",")[idx] == "dec":
                # aggregate_sum over a dec column sums doubles.
                col = out[:, 8:16].copy().view(np.float64).ravel()
                want = np.array([ref["sum"]], dtype=np.int64).view(np.float64)[0]
                assert abs(orc.fsum(col) - want) <= 1e-12 * abs(want)
            else:
                assert s == ref["sum"]
        else:
            out, n, _ = orc.mergejoin(R, S, proj=proj, threads=p["threads"])
            assert n == ref["n_out"]
            rows = out.view(np.int64).reshape(-1, 2) if n else np.zeros((0, 2), np.int64)
            tot = int((rows[:, 0].astype(np.uint64).sum(dtype=np.uint64) +
                       rows[:, 1].astype(np.uint64).sum(dtype=np.uint64)).astype(np.int64)) if n else 0
            assert tot == ref["sum_build_plus_probe"]
        if n:
            assert sha(orc.canonical(out)) == ref["canonical_sha256"]
    elif op == "partition":
        a = inputs["in"]
        out, offs = orc.partition(a, orc.hashcfg("exactrange", p["buckets"], p["min"], p["max"]),
                                  threads=3)
        for b, part in enumerate(ref["partitions"]):
            rows = out[offs[b]:offs[b + 1]]
            assert rows.shape[0] == part["n"]
            assert sha(rows) == part["sha256"], f"partition {b}"
    elif op in ("aggsum", "aggcount"):
        a = inputs["in"]
        w = widths(p["schema"])
        vt = {"int": "int", "long": "long", "dec": "dec"}[p["schema"].split(",")[1]]
        agg = "sum" if op == "aggsum" else "count"
        got = orc.groupby(a, key=(0, w[0]), val=(w[0], vt), agg=agg, threads=p["threads"],
                          hash=orc.hashcfg("modulo", p["buckets"]))
        assert got.shape[0] == ref["ngroups"]
        if "sums" in ref:
            g = got.view(np.int64).reshape(-1, 2)
            g = g[np.argsort(g[:, 0], kind="stable")]
            assert sha(g[:, 0]) == ref["keys_sha256"]
            exact = orc.groupby_exact(a).view(np.int64).reshape(-1, 2)[:, 1].view(np.float64)
            refs = np.array(ref["sums"])
            # Both naive sums are within 1e-12 of the exactly rounded sum.
            for v in (refs, g[:, 1].view(np.float64)[: len(refs)]):
                rel = np.abs(v - exact[: len(refs)]) / np.maximum(np.abs(exact[: len(refs)]), 1e-300)
                assert rel.max() <= 1e-12
        else:
            assert sha(orc.canonical(got)) == ref["canonical_sha256"]
    elif op == "sort":
        a = inputs["in"]
        out = orc.sort(a)
        assert sha(out[:, :1].copy()) == ref["keys_sha256"]
        assert sha(orc.canonical(out)) == ref["canonical_sha256"]
    elif op == "filter":
        a = inputs["in"]
        w = sum(cw for _, _, cw in gin.schema_columns(p["schema"]))
        rows = np.ascontiguousarray(a).view(np.uint8).reshape(a.shape[0], w)
        out = orc.filter(rows, gin.filter_preds(p["schema"], p["filters"]))
        assert out.shape[0] == ref["n"]
        assert sha(out) == ref["sha256"]
    elif op == "project":
        a = inputs["in"]
        cols = gin.schema_columns(p["schema"])
        w = sum(cw for _, _, cw in cols)
        rows = np.ascontiguousarray(a).view(np.uint8).reshape(a.shape[0], w)
        out = orc.project(rows, [(cols[int(i)][1], cols[int(i)][2]) for i in p["projection"].split(",")])
        assert out.size == ref["bytes"]
        assert sha(out) == ref["sha256"]
    else:
        pytest.fail(f"unknown op {op}")
