"""TEST INFRASTRUCTURE — the oracle (ctypes over oracle/liboracle.so).

Python face of the C restatement of the reference operators
(oracle/pythia_oracle.c). Only tests/, __graft_entry__.smoke() and bench.py's
CPU baseline / reference arm import this module.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

FN = {"bytes": 0, "modulo": 1, "range": 2, "exactrange": 3, "parammodulo": 4,
      "knuth": 5, "tpchorderkey": 6, "willis": 7, "alwayszero": 8, "tpchq1magic": 9}
VAL = {"int": 0, "long": 1, "dec": 2}
AGG = {"sum": 0, "count": 1}


class HashCfg(ctypes.Structure):
    _fields_ = [("fn", ctypes.c_int32), ("buckets", ctypes.c_uint32),
                ("min", ctypes.c_int64), ("max", ctypes.c_int64),
                ("skipbits", ctypes.c_uint32), ("offset", ctypes.c_uint32)]


class HashFn(ctypes.Structure):
    _fields_ = [("fn", ctypes.c_int32), ("k", ctypes.c_int64), ("min", ctypes.c_int64),
                ("max", ctypes.c_int64), ("bucketrange", ctypes.c_int64),
                ("skipbits", ctypes.c_uint32), ("nbuckets", ctypes.c_uint32)]


class Col(ctypes.Structure):
    _fields_ = [("side", ctypes.c_uint32), ("off", ctypes.c_uint32), ("bytes", ctypes.c_uint32)]


class JoinResult(ctypes.Structure):
    _fields_ = [("n_out", ctypes.c_uint64), ("sum", ctypes.c_int64)]


class Digest(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint64), ("w0", ctypes.c_uint64), ("w1", ctypes.c_uint64), ("h", ctypes.c_uint64)]

    def as_dict(self):
        return {"rows": int(self.n), "sum_word0": int(self.w0), "sum_word1": int(self.w1), "sum_row_hash": int(self.h)}


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(path)
        vp, u64, u32, ci = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int
        P = ctypes.POINTER
        L.or_getlogarithm.argtypes = [u32]; L.or_getlogarithm.restype = u32
        L.or_hashfn_make.argtypes = [P(HashCfg), P(HashFn)]; L.or_hashfn_make.restype = ci
        L.or_hash_value.argtypes = [P(HashFn), vp, u32]; L.or_hash_value.restype = u32
        L.or_hash_column.argtypes = [P(HashFn), vp, u64, u32, u32, u32, vp]
        L.or_hash_column.restype = None
        L.or_exactrange_minimumforbucket.argtypes = [P(HashFn), u32]
        L.or_exactrange_minimumforbucket.restype = ctypes.c_int64
        L.or_parammodulo_generate.argtypes = [P(HashFn), u32, P(HashFn)]
        L.or_parammodulo_generate.restype = ci
        L.or_hashjoin.argtypes = [vp, u64, u32, u32, u32, vp, u64, u32, u32, u32,
                                  P(HashCfg), u32, P(Col), ci, vp, u64, ci, ci, P(JoinResult)]
        L.or_hashjoin.restype = ci
        L.or_partition.argtypes = [vp, u64, u32, u32, u32, P(HashCfg), vp, vp, ci]
        L.or_partition.restype = ci
        L.or_groupby.argtypes = [vp, u64, u32, ci, u32, u32, u32, ci, ci, P(HashCfg),
                                 vp, u64, P(u64), ci]
        L.or_groupby.restype = ci
        L.or_groupby_exact.argtypes = [vp, u64, u32, ci, u32, u32, u32, vp, u64, P(u64)]
        L.or_groupby_exact.restype = ci
        L.or_fsum.argtypes = [vp, u64, u64]; L.or_fsum.restype = ctypes.c_double
        L.or_sort.argtypes = [vp, u64, u32, u32, u32, vp]; L.or_sort.restype = ci
        L.or_mergejoin.argtypes = [vp, u64, u32, u32, u32, vp, u64, u32, u32, u32,
                                   P(Col), ci, vp, u64, ci, ci, P(JoinResult)]
        L.or_mergejoin.restype = ci
        L.or_hashjoin_paged.argtypes = [vp, u64, u32, u32, u32, vp, u64, u32, u32, u32,
                                        P(HashCfg), u32, P(Col), ci, u32, ci, ci, P(JoinResult)]
        L.or_hashjoin_paged.restype = ci
        L.or_rows_digest.argtypes = [vp, u64, u32, ci, P(Digest)]; L.or_rows_digest.restype = None
        L.or_hashjoin_digest.argtypes = [vp, u64, u32, u32, u32, vp, u64, u32, u32, u32,
                                         P(HashCfg), u32, P(Col), ci, ci, P(Digest)]
        L.or_hashjoin_digest.restype = ci
        L.or_mergejoin_digest.argtypes = [vp, u64, u32, u32, u32, vp, u64, u32, u32, u32,
                                          P(Col), ci, ci, P(Digest)]
        L.or_mergejoin_digest.restype = ci
        L.or_filter.argtypes = [vp, u64, u32, P(Pred), ci, vp]; L.or_filter.restype = u64
        L.or_project.argtypes = [vp, u64, u32, P(Col), ci, vp]; L.or_project.restype = None
        _LIB = L
    return _LIB


class Pred(ctypes.Structure):
    _fields_ = [("type", ctypes.c_uint32), ("op", ctypes.c_uint32), ("off", ctypes.c_uint32),
                ("bytes", ctypes.c_uint32), ("value", ctypes.c_uint8 * 128)]


PRED_TYPE = {"int": 1, "long": 2, "date": 2, "dec": 3, "char": 4}
PRED_OP = {"=": 0, "==": 0, "<>": 1, "!=": 1, "<": 2, "<=": 3, ">": 4, ">=": 5}


def preds(spec):
    """spec: [(type, op, byte offset, value[, char width])] -> (Pred array, n)."""
    arr = (Pred * max(1, len(spec)))()
    for i, sp in enumerate(spec):
        t, op, off, v = sp[:4]
        p = arr[i]
        p.type, p.op, p.off = PRED_TYPE[t], PRED_OP[op], off
        if t == "int":
            b = np.int32(v).tobytes()
        elif t in ("long", "date"):
            b = np.int64(v).tobytes()
        elif t == "dec":
            b = np.float64(v).tobytes()
        else:
            width = sp[4]
            raw = v if isinstance(v, bytes) else str(v).encode()
            b = (raw[:width] + b"\0" * width)[:width]       # strncpy into the column
        p.bytes = len(b)
        ctypes.memmove(p.value, b, min(len(b), 128))
    return arr, len(spec)


def filter(rows, spec):
    """Filter (filter.cpp:76-85) with the conjunction of `spec` predicates."""
    a, p, n, w = _rows(rows)
    pr, npr = preds(spec)
    out = np.empty_like(a)
    m = lib().or_filter(p, n, w, pr, npr, out.ctypes.data)
    return out[:m]


def project(rows, spec):
    """Project (project.cpp:93-104): spec = [(byte offset, bytes)]."""
    a, p, n, w = _rows(rows)
    c = (Col * len(spec))(*[Col(0, o, b) for o, b in spec])
    ow = sum(b for _, b in spec)
    out = np.empty(n * ow, dtype=np.uint8)
    lib().or_project(p, n, w, c, len(spec), out.ctypes.data)
    return out.reshape(n, ow)


def hashcfg(fn, buckets=1, min=0, max=0, skipbits=0, offset=0):
    return HashCfg(FN[fn] if isinstance(fn, str) else fn, buckets, min, max, skipbits, offset)


def hashfn(cfg):
    f = HashFn()
    if lib().or_hashfn_make(ctypes.byref(cfg), ctypes.byref(f)):
        raise ValueError("invalid hash configuration")
    return f


def _rows(a):
    a = np.ascontiguousarray(a)
    w = int(a.itemsize * int(np.prod(a.shape[1:]))) if a.ndim > 1 else int(a.itemsize)
    return a, a.ctypes.data, a.shape[0], w


def hash_column(cfg, rows, off=0, size=8, width=None):
    a, p, n, w = _rows(rows)
    w = width or w
    out = np.empty(n, dtype=np.uint32)
    f = hashfn(cfg)
    lib().or_hash_column(ctypes.byref(f), p, n, w, off, size, out.ctypes.data)
    return out


def cols(spec):
    """spec: list of (side, off, bytes), side 'B' or 'P' (or 0/1)."""
    arr = (Col * max(1, len(spec)))()
    for i, (s, o, b) in enumerate(spec):
        arr[i] = Col(0 if s in ("B", 0) else 1, o, b)
    return arr, len(spec)


def hashjoin(R, S, proj=(("P", 8, 8), ("B", 8, 8)), hash=None, tuplesperbucket=4,
             bkey=(0, 8), pkey=(0, 8), materialise=True, sum_col=-1, threads=1, out_cap=None):
    Ra, Rp, nR, wR = _rows(R)
    Sa, Sp, nS, wS = _rows(S)
    hash = hash or hashcfg("modulo", 1 << 10)
    c, nc = cols(proj)
    ow = sum(b for _, _, b in proj)
    res = JoinResult()
    if materialise:
        # First pass counts, second writes: the oracle does not guess sizes.
        if out_cap is None:
            rc = lib().or_hashjoin(Rp, nR, wR, bkey[0], bkey[1], Sp, nS, wS, pkey[0], pkey[1],
                                   ctypes.byref(hash), tuplesperbucket, c, nc, None, 0, sum_col,
                                   threads, ctypes.byref(res))
            if rc:
                raise ValueError("or_hashjoin failed")
            out_cap = res.n_out
        out = np.zeros(out_cap * ow, dtype=np.uint8)
        rc = lib().or_hashjoin(Rp, nR, wR, bkey[0], bkey[1], Sp, nS, wS, pkey[0], pkey[1],
                               ctypes.byref(hash), tuplesperbucket, c, nc, out.ctypes.data,
                               out_cap, sum_col, threads, ctypes.byref(res))
        if rc:
            raise ValueError("or_hashjoin failed")
        return out[: min(out_cap, res.n_out) * ow].reshape(-1, ow), res.n_out, res.sum
    rc = lib().or_hashjoin(Rp, nR, wR, bkey[0], bkey[1], Sp, nS, wS, pkey[0], pkey[1],
                           ctypes.byref(hash), tuplesperbucket, c, nc, None, 0, sum_col,
                           threads, ctypes.byref(res))
    if rc:
        raise ValueError("or_hashjoin failed")
    return None, res.n_out, res.sum


def hashjoin_paged(R, S, proj=(("P", 8, 8), ("B", 8, 8)), hash=None, tuplesperbucket=4,
                   bkey=(0, 8), pkey=(0, 8), page_bytes=1 << 20, sum_col=-1, threads=1):
    """The hash join with each thread writing its rows into one reused output
    page of page_bytes (HashJoinOp::getNext's output page), returning
    (rows, wrapping sum of column sum_col)."""
    Ra, Rp, nR, wR = _rows(R)
    Sa, Sp, nS, wS = _rows(S)
    hash = hash or hashcfg("modulo", 1 << 10)
    c, nc = cols(proj)
    res = JoinResult()
    if lib().or_hashjoin_paged(Rp, nR, wR, bkey[0], bkey[1], Sp, nS, wS, pkey[0], pkey[1],
                               ctypes.byref(hash), tuplesperbucket, c, nc, page_bytes, sum_col, threads,
                               ctypes.byref(res)):
        raise ValueError("or_hashjoin_paged failed")
    return res.n_out, res.sum


def rows_digest(rows, threads=1):
    """Order-independent digest of a row array (any row width): row count,
    sums of the first and second 8-byte words, sum of a whole-row hash, all
    mod 2^64 (or_rows_digest)."""
    a, p, n, w = _rows(rows)
    d = Digest()
    lib().or_rows_digest(p, n, w, threads, ctypes.byref(d))
    return d.as_dict()


def hashjoin_digest(R, S, proj=(("P", 8, 8), ("B", 8, 8)), hash=None, tuplesperbucket=4,
                    bkey=(0, 8), pkey=(0, 8), threads=1):
    """rows_digest of the oracle hash join's output, without materialising it."""
    Ra, Rp, nR, wR = _rows(R)
    Sa, Sp, nS, wS = _rows(S)
    hash = hash or hashcfg("modulo", 1 << 10)
    c, nc = cols(proj)
    d = Digest()
    if lib().or_hashjoin_digest(Rp, nR, wR, bkey[0], bkey[1], Sp, nS, wS, pkey[0], pkey[1],
                                ctypes.byref(hash), tuplesperbucket, c, nc, threads, ctypes.byref(d)):
        raise ValueError("or_hashjoin_digest failed")
    return d.as_dict()


def mergejoin_digest(R, S, proj=(("P", 8, 8), ("B", 8, 8)), bkey=(0, 8), pkey=(0, 8), threads=1):
    """rows_digest of the oracle sort-merge join's output, without materialising it."""
    Ra, Rp, nR, wR = _rows(R)
    Sa, Sp, nS, wS = _rows(S)
    c, nc = cols(proj)
    d = Digest()
    if lib().or_mergejoin_digest(Rp, nR, wR, bkey[0], bkey[1], Sp, nS, wS, pkey[0], pkey[1],
                                 c, nc, threads, ctypes.byref(d)):
        raise ValueError("or_mergejoin_digest failed")
    return d.as_dict()


def mergejoin(R, S, proj=(("P", 8, 8), ("B", 8, 8)), bkey=(0, 8), pkey=(0, 8),
              materialise=True, sum_col=-1, threads=1):
    Ra, Rp, nR, wR = _rows(R)
    Sa, Sp, nS, wS = _rows(S)
    c, nc = cols(proj)
    ow = sum(b for _, _, b in proj)
    res = JoinResult()
    rc = lib().or_mergejoin(Rp, nR, wR, bkey[0], bkey[1], Sp, nS, wS, pkey[0], pkey[1],
                            c, nc, None, 0, sum_col, threads, ctypes.byref(res))
    if rc:
        raise ValueError("or_mergejoin failed")
    if not materialise:
        return None, res.n_out, res.sum
    out = np.zeros(res.n_out * ow, dtype=np.uint8)
    rc = lib().or_mergejoin(Rp, nR, wR, bkey[0], bkey[1], Sp, nS, wS, pkey[0], pkey[1],
                            c, nc, out.ctypes.data, res.n_out, sum_col, threads,
                            ctypes.byref(res))
    return out.reshape(-1, ow) if ow else out, res.n_out, res.sum


def partition(rows, hash, key=(0, 8), threads=1):
    a, p, n, w = _rows(rows)
    f = hashfn(hash)
    out = np.empty_like(a)
    offsets = np.zeros(f.nbuckets + 1, dtype=np.uint64)
    rc = lib().or_partition(p, n, w, key[0], key[1], ctypes.byref(hash), out.ctypes.data,
                            offsets.ctypes.data, threads)
    if rc == -2:
        raise ValueError("a tuple hashed outside [0, buckets)")
    if rc:
        raise ValueError("or_partition failed")
    return out, offsets


def groupby(rows, key=(0, 8), val=(8, "long"), agg="sum", hash=None, threads=1, has_key=True):
    a, p, n, w = _rows(rows)
    hash = hash or hashcfg("modulo", 1 << 10)
    vtype = VAL[val[1]]
    aw = 4 if (agg == "sum" and vtype == 0) else 8
    tw = (key[1] if has_key else 0) + aw
    cap = max(n, 1)
    out = np.zeros(cap * tw, dtype=np.uint8)
    ng = ctypes.c_uint64()
    rc = lib().or_groupby(p, n, w, int(has_key), key[0], key[1], val[0], vtype, AGG[agg],
                          ctypes.byref(hash), out.ctypes.data, cap, ctypes.byref(ng), threads)
    if rc:
        raise ValueError("or_groupby failed")
    return out[: ng.value * tw].reshape(-1, tw)


def groupby_exact(rows, key=(0, 8), voff=8, has_key=True):
    a, p, n, w = _rows(rows)
    tw = (key[1] if has_key else 0) + 8
    cap = max(n, 1)
    out = np.zeros(cap * tw, dtype=np.uint8)
    ng = ctypes.c_uint64()
    rc = lib().or_groupby_exact(p, n, w, int(has_key), key[0], key[1], voff, out.ctypes.data,
                                cap, ctypes.byref(ng))
    if rc:
        raise ValueError("or_groupby_exact failed")
    return out[: ng.value * tw].reshape(-1, tw)


def fsum(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib().or_fsum(x.ctypes.data, x.shape[0], 1)


def sort(rows, key=(0, 8)):
    a, p, n, w = _rows(rows)
    out = np.empty_like(a)
    lib().or_sort(p, n, w, key[0], key[1], out.ctypes.data)
    return out


def canonical(rows):
    """Rows as a byte-lexicographically sorted (n, w) uint8 array: the form in
    which unordered operator outputs (joins, group-by) are compared."""
    a = np.ascontiguousarray(rows)
    if a.size == 0:
        return a.reshape(0, a.shape[-1] if a.ndim > 1 else 0).view(np.uint8)
    u8 = a.view(np.uint8).reshape(a.shape[0], -1)
    v = u8.view(f"V{u8.shape[1]}").ravel()
    return np.sort(v).view(np.uint8).reshape(-1, u8.shape[1])
