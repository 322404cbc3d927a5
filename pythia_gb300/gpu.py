"""ctypes binding of the C ABI in include/pythia_gpu.h (libpythia_gpu.so).

This is the same binding a Python caller of the Pythia GPU operators would
write; tests and the benchmark drive every kernel through it. There is no CPU
fallback: a missing library or device raises.
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
_LIB = None

PG_OK, PG_ERR_ARG, PG_ERR_OOM, PG_ERR_CUDA, PG_ERR_TIMEOUT = 0, 1, 2, 3, 4
PG_ERR_TABLE_FULL, PG_ERR_OUTPUT_FULL, PG_ERR_UNSUPPORTED = 5, 6, 7
JOIN_MATERIALIZE, JOIN_COUNT, JOIN_SUM = 1, 2, 4
JOIN_BUILD_SORTED, JOIN_PROBE_SORTED = 8, 16       # pg_mpsm_join: that side is sorted on its key
FN = {"bytes": 0, "modulo": 1, "range": 2, "exactrange": 3, "parammodulo": 4,
      "knuth": 5, "tpchorderkey": 6, "willis": 7, "alwayszero": 8, "tpchq1magic": 9}
VAL = {"int": 0, "long": 1, "dec": 2}
AGG = {"sum": 0, "count": 1}


class PgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"pythia_gpu error {code}: {msg}")
        self.code = code


class Rel(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("n", ctypes.c_uint64), ("width", ctypes.c_uint32),
                ("key_off", ctypes.c_uint32), ("key_bytes", ctypes.c_uint32)]


class HashCfg(ctypes.Structure):
    _fields_ = [("fn", ctypes.c_int32), ("buckets", ctypes.c_uint32), ("min", ctypes.c_int64),
                ("max", ctypes.c_int64), ("skipbits", ctypes.c_uint32), ("offset", ctypes.c_uint32)]


class Col(ctypes.Structure):
    _fields_ = [("side", ctypes.c_uint32), ("off", ctypes.c_uint32), ("bytes", ctypes.c_uint32)]


class JoinResult(ctypes.Structure):
    _fields_ = [("n_out", ctypes.c_uint64), ("sum", ctypes.c_int64)]


class BatchItem(ctypes.Structure):
    _fields_ = [("R", ctypes.c_void_p), ("nR", ctypes.c_uint64), ("S", ctypes.c_void_p),
                ("nS", ctypes.c_uint64)]


class BatchShape(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int32), ("items", ctypes.c_int32), ("tile", ctypes.c_uint32),
                ("ctas_per_sm", ctypes.c_int32), ("load_inverse", ctypes.c_int32),
                ("use_graph", ctypes.c_int32)]


SYMBOLS = ["pg_init", "pg_shutdown", "pg_last_error", "pg_device_status", "pg_stream_create",
           "pg_stream_destroy", "pg_sync", "pg_buffer_alloc", "pg_buffer_free", "pg_host_alloc",
           "pg_host_free", "pg_h2d", "pg_d2h", "pg_d2d", "pg_memset", "pg_kernel_launches",
           "pg_hash_buckets", "pg_hash_tuples", "pg_partition", "pg_partition_sort",
           "pg_hashjoin_build", "pg_hashjoin_probe", "pg_hashtable_free", "pg_hashjoin_host",
           "pg_groupby", "pg_sort_pages", "pg_mpsm_join", "pg_hashjoin_agg_noalloc",
           "pg_tune_set", "pg_tune_get", "pg_batch_prepare", "pg_batch_run", "pg_batch_free",
           "pg_generate_fk", "pg_buffer_alloc_async", "pg_buffer_free_async", "pg_generate_zipf_fk",
           "pg_hashjoin_groupby", "pg_stream_create_urgent", "pg_autotune_batch",
           "pg_hashtable_image_size", "pg_hashtable_serialize", "pg_hashtable_deserialize",
           "pg_hashtable_save", "pg_hashtable_load", "pg_filter", "pg_project", "pg_hashjoin_probe_where",
           "pg_host_register", "pg_host_unregister", "pg_host_is_pinned", "pg_host_readable", "pg_h2d_sm",
           "pg_hashjoin_probe_spans"]
TUNE = {"probe_ctas_per_sm": 0, "probe_variant": 1, "dense": 2, "partition_tile": 3,
        "groupby_smem_groups": 4, "radix_bits": 5, "probe_items": 6, "probe_cache": 7, "probe_passes": 8, "groupby_path": 9,
        "probe_wide": 10, "build_spec": 11, "spin_limit": 12,
        "l2_fetch": 13, "sort_path": 14, "groupby_ilp": 15,
        "hash_partition": 16}


def lib_path():
    return os.path.join(_PKG, "libpythia_gpu.so")


def lib():
    global _LIB
    if _LIB is None:
        p = lib_path()
        if not os.path.exists(p):
            raise RuntimeError(f"{p} is missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(p)
        vp, u64, u32, ci, P = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, ctypes.POINTER
        sig = {
            "pg_init": ([ci, u64, P(vp)], ci),
            "pg_shutdown": ([vp], ci),
            "pg_last_error": ([vp], ctypes.c_char_p),
            "pg_device_status": ([vp], ci),
            "pg_stream_create": ([vp, P(vp)], ci),
            "pg_stream_destroy": ([vp, vp], ci),
            "pg_sync": ([vp, vp], ci),
            "pg_buffer_alloc": ([vp, u64, P(vp)], ci),
            "pg_buffer_free": ([vp, vp], ci),
            "pg_host_alloc": ([vp, u64, P(vp)], ci),
            "pg_host_free": ([vp, vp], ci),
            "pg_host_register": ([vp, vp, u64], ci),
            "pg_host_unregister": ([vp, vp], ci),
            "pg_host_is_pinned": ([vp, vp], ci),
            "pg_host_readable": ([vp, vp], ci),
            "pg_h2d_sm": ([vp, vp, vp, vp, u64], ci),
            "pg_h2d": ([vp, vp, vp, vp, u64], ci),
            "pg_d2h": ([vp, vp, vp, vp, u64], ci),
            "pg_d2d": ([vp, vp, vp, vp, u64], ci),
            "pg_memset": ([vp, vp, vp, ci, u64], ci),
            "pg_kernel_launches": ([], u64),
            "pg_hash_buckets": ([vp, P(HashCfg), P(u32)], ci),
            "pg_hash_tuples": ([vp, vp, P(Rel), P(HashCfg), vp], ci),
            "pg_partition": ([vp, vp, P(Rel), P(HashCfg), vp, vp], ci),
            "pg_partition_sort": ([vp, vp, P(Rel), vp, u32, vp], ci),
            "pg_hashjoin_build": ([vp, vp, P(Rel), P(Col), ci, P(vp)], ci),
            "pg_hashjoin_probe": ([vp, vp, vp, P(Rel), P(Col), ci, vp, u64, ci, ci, P(JoinResult)], ci),
            "pg_hashjoin_probe_spans": ([vp, vp, vp, P(Rel), ci, P(Col), ci, vp, u64, ci, ci, P(JoinResult)], ci),
            "pg_hashtable_free": ([vp, vp], ci),
            "pg_hashjoin_host": ([vp, P(Rel), P(Rel), P(Col), ci, vp, u64, ci, ci, P(JoinResult)], ci),
            "pg_groupby": ([vp, vp, P(Rel), u32, ci, ci, u64, vp, u64, P(u64)], ci),
            "pg_sort_pages": ([vp, vp, P(Rel), vp], ci),
            "pg_mpsm_join": ([vp, vp, P(Rel), P(Rel), P(Col), ci, vp, u64, ci, ci, P(JoinResult)], ci),
            "pg_hashjoin_agg_noalloc": ([vp, vp, P(Rel), P(Rel), P(Col), ci, ci, P(JoinResult)], ci),
            "pg_tune_set": ([vp, ci, ctypes.c_int64], ci),
            "pg_tune_get": ([vp, ci], ctypes.c_int64),
            "pg_batch_prepare": ([vp, vp, P(BatchItem), u32, P(BatchShape), P(vp)], ci),
            "pg_batch_run": ([vp, vp, vp], ci),
            "pg_batch_free": ([vp, vp], ci),
            "pg_generate_fk": ([vp, vp, vp, u64, u64, vp, u64], ci),
            "pg_generate_zipf_fk": ([vp, vp, vp, u64, ctypes.c_double, u64, vp, u64, ctypes.c_double], ci),
            "pg_buffer_alloc_async": ([vp, vp, u64, P(vp)], ci),
            "pg_buffer_free_async": ([vp, vp, vp], ci),
            "pg_hashjoin_groupby": ([vp, vp, vp, P(Rel), u32, ci, ci, vp, u64, P(u64)], ci),
            "pg_stream_create_urgent": ([vp, P(vp)], ci),
            "pg_autotune_batch": ([vp, vp, P(BatchItem), u32, P(BatchShape), u32, ci, P(u32), P(ctypes.c_double)], ci),
            "pg_hashtable_image_size": ([vp, vp, P(u64)], ci),
            "pg_hashtable_serialize": ([vp, vp, vp, vp, u64, P(u64)], ci),
            "pg_hashtable_deserialize": ([vp, vp, vp, u64, P(vp)], ci),
            "pg_hashtable_save": ([vp, vp, vp, ctypes.c_char_p], ci),
            "pg_hashtable_load": ([vp, vp, ctypes.c_char_p, P(vp)], ci),
            "pg_filter": ([vp, vp, P(Rel), P(Pred), ci, vp, P(u64)], ci),
            "pg_project": ([vp, vp, P(Rel), P(Col), ci, vp], ci),
            "pg_hashjoin_probe_where": ([vp, vp, vp, P(Rel), P(Pred), ci, P(Col), ci, vp, u64, ci, ci,
                                         P(JoinResult)], ci),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes, f.restype = args, res
        _LIB = L
    return _LIB


class Pred(ctypes.Structure):
    _fields_ = [("type", ctypes.c_uint32), ("op", ctypes.c_uint32), ("off", ctypes.c_uint32),
                ("bytes", ctypes.c_uint32), ("value", ctypes.c_uint8 * 128)]


PRED_TYPE = {"int": 1, "long": 2, "date": 2, "dec": 3, "char": 4}
PRED_OP = {"=": 0, "==": 0, "<>": 1, "!=": 1, "<": 2, "<=": 3, ">": 4, ">=": 5}


def preds(spec):
    """spec: [(type, op, byte offset, value[, char width])], type int / long /
    date (a long) / dec / char; value a number, or bytes / str for char
    (copied as strncpy copies into the column) -> (pg_pred array, n)."""
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
            b = (raw[:width] + b"\0" * width)[:width]
        p.bytes = len(b)
        ctypes.memmove(p.value, b, min(len(b), 128))
    return arr, len(spec)


def hashcfg(fn, buckets=1, min=0, max=0, skipbits=0, offset=0):
    return HashCfg(FN[fn] if isinstance(fn, str) else fn, buckets, min, max, skipbits, offset)


def cols(spec):
    """spec: [(side, byte offset, bytes)], side "B"/"P" (build/probe)."""
    arr = (Col * max(1, len(spec)))()
    for i, (s, o, b) in enumerate(spec):
        arr[i] = Col(0 if s in ("B", 0) else 1, o, b)
    return arr, len(spec)


class DeviceBuffer:
    def __init__(self, ctx, nbytes):
        self.ctx, self.nbytes = ctx, int(nbytes)
        p = ctypes.c_void_p()
        ctx._check(lib().pg_buffer_alloc(ctx.h, max(16, self.nbytes), ctypes.byref(p)))
        self.ptr = p.value

    def free(self):
        if self.ptr:
            lib().pg_buffer_free(self.ctx.h, self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """One pg_ctx on one device, with one stream."""

    def __init__(self, device=0, reserve=0):
        h = ctypes.c_void_p()
        rc = lib().pg_init(device, reserve, ctypes.byref(h))
        if rc:
            raise PgError(rc, lib().pg_last_error(None).decode())
        self.h = h.value
        s = ctypes.c_void_p()
        self._check(lib().pg_stream_create(self.h, ctypes.byref(s)))
        self.stream = s.value

    def _check(self, rc):
        if rc:
            raise PgError(rc, (lib().pg_last_error(self.h) or b"").decode())
        return rc

    def close(self):
        if self.h:
            lib().pg_stream_destroy(self.h, self.stream)
            lib().pg_shutdown(self.h)
            self.h = None

    # ---- memory ----
    def alloc(self, nbytes):
        return DeviceBuffer(self, nbytes)

    def upload(self, a):
        a = np.ascontiguousarray(a)
        b = DeviceBuffer(self, a.nbytes)
        self._check(lib().pg_h2d(self.h, self.stream, b.ptr, a.ctypes.data, a.nbytes))
        self.sync()
        return b

    def download(self, buf, nbytes, dtype=np.uint8):
        out = np.empty(nbytes, dtype=np.uint8)
        if nbytes:
            self._check(lib().pg_d2h(self.h, self.stream, out.ctypes.data, buf.ptr, nbytes))
            self.sync()
        return out.view(dtype)

    def sync(self):
        self._check(lib().pg_sync(self.h, self.stream))

    def tune(self, **knobs):
        """Sets launch-shape knobs (see PG_TUNE_* in include/pythia_gpu.h)."""
        for k, v in knobs.items():
            self._check(lib().pg_tune_set(self.h, TUNE[k], int(v)))

    @staticmethod
    def rel(buf, n, width, key_off=0, key_bytes=8):
        return Rel(buf.ptr if buf is not None else None, n, width, key_off, key_bytes)

    # ---- operators on numpy inputs (upload, run, download) ----
    def hash_tuples(self, rows, cfg, key_off=0, key_bytes=8):
        a = np.ascontiguousarray(rows)
        n, w = a.shape[0], row_width(a)
        d = self.upload(a)
        o = self.alloc(4 * max(n, 1))
        r = self.rel(d, n, w, key_off, key_bytes)
        self._check(lib().pg_hash_tuples(self.h, self.stream, ctypes.byref(r), ctypes.byref(cfg), o.ptr))
        return self.download(o, 4 * n, np.uint32)

    def nbuckets(self, cfg):
        nb = ctypes.c_uint32()
        self._check(lib().pg_hash_buckets(self.h, ctypes.byref(cfg), ctypes.byref(nb)))
        return nb.value

    def partition(self, rows, cfg, key_off=0, key_bytes=8):
        a = np.ascontiguousarray(rows)
        n, w = a.shape[0], row_width(a)
        nb = self.nbuckets(cfg)
        d = self.upload(a)
        o = self.alloc(a.nbytes)
        offs = self.alloc(8 * (nb + 1))
        r = self.rel(d, n, w, key_off, key_bytes)
        self._check(lib().pg_partition(self.h, self.stream, ctypes.byref(r), ctypes.byref(cfg),
                                       o.ptr, offs.ptr))
        out = self.download(o, a.nbytes).view(a.dtype).reshape(a.shape)
        return out, self.download(offs, 8 * (nb + 1), np.uint64)

    def build_table(self, R, proj=(("P", 8, 8), ("B", 8, 8)), bkey=(0, 8)):
        """Builds the join table of R (pg_hashjoin_build) for the projection
        `proj`; the table stays on the device until JoinTable.free()."""
        Ra = np.ascontiguousarray(R)
        dR = self.upload(Ra)
        rR = self.rel(dR, Ra.shape[0], row_width(Ra), *bkey)
        c, nc = cols(proj)
        ht = ctypes.c_void_p()
        self._check(lib().pg_hashjoin_build(self.h, self.stream, ctypes.byref(rR), c, nc, ctypes.byref(ht)))
        return JoinTable(self, ht.value, proj, dR)

    def load_table(self, image, proj=None):
        """A join table from an image: bytes-like / uint8 array (pg_hashtable_
        deserialize) or a file path (pg_hashtable_load)."""
        ht = ctypes.c_void_p()
        if isinstance(image, (str, os.PathLike)):
            self._check(lib().pg_hashtable_load(self.h, self.stream, os.fsencode(image), ctypes.byref(ht)))
        else:
            a = np.frombuffer(image, dtype=np.uint8) if not isinstance(image, np.ndarray) else image
            a = np.ascontiguousarray(a)
            self._check(lib().pg_hashtable_deserialize(self.h, self.stream, a.ctypes.data, a.nbytes,
                                                       ctypes.byref(ht)))
        return JoinTable(self, ht.value, proj, None)

    def hashjoin(self, R, S, proj=(("P", 8, 8), ("B", 8, 8)), bkey=(0, 8), pkey=(0, 8),
                 flags=JOIN_MATERIALIZE, sum_col=-1, out_cap=None):
        t = self.build_table(R, proj, bkey)
        try:
            return t.probe(S, pkey=pkey, flags=flags, sum_col=sum_col, out_cap=out_cap)
        finally:
            t.free()

    def hashjoin_groupby(self, R, S, group=(8, 8), val=(8, "dec"), agg="sum", bkey=(0, 8), pkey=(0, 8)):
        """Join R and S on their keys and aggregate the probe column `val`
        grouped by the build column `group` in one pass (pg_hashjoin_groupby).
        Returns (group, agg) rows."""
        t = self.build_table(R, (("B", group[0], group[1]), ("P", val[0], 4 if val[1] == "int" else 8)), bkey)
        try:
            return t.groupby(S, val=val, agg=agg, pkey=pkey, cap=max(np.asarray(R).shape[0], 1))
        finally:
            t.free()

    def groupby(self, rows, key=(0, 8), val=(8, "long"), agg="sum", groups_hint=0, has_key=True):
        a = np.ascontiguousarray(rows)
        n, w = a.shape[0], row_width(a)
        d = self.upload(a)
        vtype = VAL[val[1]]
        aw = 4 if (agg == "sum" and vtype == 0) else 8
        kb = key[1] if has_key else 0
        ow = kb + aw
        cap = max(n, 1)
        o = self.alloc(cap * ow)
        ng = ctypes.c_uint64()
        r = self.rel(d, n, w, key[0] if has_key else 0, kb)
        self._check(lib().pg_groupby(self.h, self.stream, ctypes.byref(r), val[0], vtype, AGG[agg],
                                     groups_hint, o.ptr, cap, ctypes.byref(ng)))
        return self.download(o, ng.value * ow).reshape(-1, ow)

    def filter(self, rows, spec):
        """pg_filter: the rows satisfying every predicate of `spec`, in order."""
        a = np.ascontiguousarray(rows)
        n, w = a.shape[0], row_width(a)
        d = self.upload(a)
        o = self.alloc(max(a.nbytes, 16))
        r = self.rel(d, n, w, 0, 0)
        pr, npr = preds(spec)
        m = ctypes.c_uint64()
        self._check(lib().pg_filter(self.h, self.stream, ctypes.byref(r), pr, npr, o.ptr, ctypes.byref(m)))
        return self.download(o, m.value * w).view(a.dtype).reshape((-1,) + a.shape[1:])

    def project(self, rows, spec):
        """pg_project: spec = [(byte offset, bytes)] -> (n, sum of bytes) uint8 rows."""
        a = np.ascontiguousarray(rows)
        n, w = a.shape[0], row_width(a)
        ow = sum(b for _, b in spec)
        d = self.upload(a)
        o = self.alloc(max(n * ow, 16))
        r = self.rel(d, n, w, 0, 0)
        c = (Col * len(spec))(*[Col(0, off, b) for off, b in spec])
        self._check(lib().pg_project(self.h, self.stream, ctypes.byref(r), c, len(spec), o.ptr))
        return self.download(o, n * ow).reshape(n, ow)

    def sort(self, rows, key=(0, 8)):
        a = np.ascontiguousarray(rows)
        n, w = a.shape[0], row_width(a)
        d = self.upload(a)
        o = self.alloc(a.nbytes)
        r = self.rel(d, n, w, *key)
        self._check(lib().pg_sort_pages(self.h, self.stream, ctypes.byref(r), o.ptr))
        return self.download(o, a.nbytes).view(a.dtype).reshape(a.shape)

    def mpsm(self, R, S, proj=(("P", 8, 8), ("B", 8, 8)), bkey=(0, 8), pkey=(0, 8),
             flags=JOIN_MATERIALIZE, sum_col=-1):
        Ra, Sa = np.ascontiguousarray(R), np.ascontiguousarray(S)
        dR, dS = self.upload(Ra), self.upload(Sa)
        rR = self.rel(dR, Ra.shape[0], row_width(Ra), *bkey)
        rS = self.rel(dS, Sa.shape[0], row_width(Sa), *pkey)
        c, nc = cols(proj)
        ow = sum(b for _, _, b in proj)
        res = JoinResult()
        rc = lib().pg_mpsm_join(self.h, self.stream, ctypes.byref(rR), ctypes.byref(rS), c, nc, None, 0,
                                flags & ~JOIN_MATERIALIZE, sum_col, ctypes.byref(res))
        self._check(rc)
        if not flags & JOIN_MATERIALIZE:
            return None, res.n_out, res.sum
        o = self.alloc(max(res.n_out, 1) * ow)
        self._check(lib().pg_mpsm_join(self.h, self.stream, ctypes.byref(rR), ctypes.byref(rS), c, nc,
                                       o.ptr, res.n_out, flags, sum_col, ctypes.byref(res)))
        return self.download(o, res.n_out * ow).reshape(-1, ow), res.n_out, res.sum


class JoinTable:
    """A join table resident on the device (pg_hashtable): built from a
    relation, or loaded from an image, and probed any number of times."""

    def __init__(self, ctx, handle, proj, build_buf):
        self.ctx, self.h, self.proj, self._build_buf = ctx, handle, proj, build_buf

    def free(self):
        if self.h:
            lib().pg_hashtable_free(self.ctx.h, self.h)
            self.h = None
        self._build_buf = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def probe(self, S, proj=None, pkey=(0, 8), flags=JOIN_MATERIALIZE, sum_col=-1, out_cap=None, where=None):
        """pg_hashjoin_probe with S (pg_hashjoin_probe_where when `where`, a
        predicate spec as for preds(), is given); returns (rows or None, n_out, sum)."""
        ctx, L = self.ctx, lib()
        if where:
            pr, npr = preds(where)

            def call(*a):
                return L.pg_hashjoin_probe_where(a[0], a[1], a[2], a[3], pr, npr, *a[4:])
        else:
            call = L.pg_hashjoin_probe
        proj = proj if proj is not None else self.proj
        Sa = np.ascontiguousarray(S)
        dS = ctx.upload(Sa)
        rS = ctx.rel(dS, Sa.shape[0], row_width(Sa), *pkey)
        c, nc = cols(proj)
        ow = sum(b for _, _, b in proj)
        res = JoinResult()
        if not flags & JOIN_MATERIALIZE:
            ctx._check(call(ctx.h, ctx.stream, self.h, ctypes.byref(rS), c, nc,
                            None, 0, flags, sum_col, ctypes.byref(res)))
            return None, res.n_out, res.sum
        cap = Sa.shape[0] if out_cap is None else out_cap
        o = ctx.alloc(max(cap, 1) * ow)
        rc = call(ctx.h, ctx.stream, self.h, ctypes.byref(rS), c, nc,
                  o.ptr, cap, flags, sum_col, ctypes.byref(res))
        if rc == PG_ERR_OUTPUT_FULL and out_cap is None:
            cap = res.n_out
            o = ctx.alloc(max(cap, 1) * ow)
            rc = call(ctx.h, ctx.stream, self.h, ctypes.byref(rS), c, nc,
                      o.ptr, cap, flags, sum_col, ctypes.byref(res))
        ctx._check(rc)
        out = ctx.download(o, res.n_out * ow).reshape(-1, ow) if ow else None
        return out, res.n_out, res.sum

    def groupby(self, S, val=(8, "dec"), agg="sum", pkey=(0, 8), cap=None):
        """pg_hashjoin_groupby with S: (group, agg) rows."""
        ctx, L = self.ctx, lib()
        Sa = np.ascontiguousarray(S)
        dS = ctx.upload(Sa)
        rS = ctx.rel(dS, Sa.shape[0], row_width(Sa), *pkey)
        vtype = VAL[val[1]]
        gbytes = sum(b for s, _, b in self.proj if s in ("B", 0)) if self.proj else 8
        ow = gbytes + (4 if (agg == "sum" and vtype == 0) else 8)
        cap = max(int(cap or 1), 1)
        o = ctx.alloc(cap * ow)
        ng = ctypes.c_uint64()
        ctx._check(L.pg_hashjoin_groupby(ctx.h, ctx.stream, self.h, ctypes.byref(rS), val[0], vtype,
                                         AGG[agg], o.ptr, cap, ctypes.byref(ng)))
        return ctx.download(o, ng.value * ow).reshape(-1, ow)

    def image_size(self):
        n = ctypes.c_uint64()
        self.ctx._check(lib().pg_hashtable_image_size(self.ctx.h, self.h, ctypes.byref(n)))
        return n.value

    def serialize(self):
        """The table's image (pg_hashtable_serialize) as a uint8 array."""
        n = self.image_size()
        out = np.empty(n, dtype=np.uint8)
        m = ctypes.c_uint64()
        self.ctx._check(lib().pg_hashtable_serialize(self.ctx.h, self.ctx.stream, self.h, out.ctypes.data, n,
                                                     ctypes.byref(m)))
        return out[:m.value]

    def save(self, path):
        self.ctx._check(lib().pg_hashtable_save(self.ctx.h, self.ctx.stream, self.h, os.fsencode(path)))


def row_width(a):
    """Bytes per tuple of a row-major (n, ...) array, also when n == 0."""
    return int(a.itemsize * int(np.prod(a.shape[1:]))) if a.ndim > 1 else int(a.itemsize)


def kernel_launches():
    return lib().pg_kernel_launches()
