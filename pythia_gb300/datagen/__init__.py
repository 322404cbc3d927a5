"""Seeded synthetic relations (ctypes over libpythia_datagen.so).

Rows use the reference's packed tuple layout: (long key, long payload) and
(long key, dec value) are both 16-byte rows, returned here as ``(n, 2)``
int64 arrays (a double column is the same bytes viewed as float64).

Relation seeds follow one convention: ``SEED_BASE + relation_id``.
"""
import ctypes
import os

import numpy as np

SEED_BASE = 0x5059544849410000
_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def seed_for(relation_id: int) -> int:
    return (SEED_BASE + relation_id) & 0xFFFFFFFFFFFFFFFF


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libpythia_datagen.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build() first")
        lib = ctypes.CDLL(path)
        u64, i64, dbl, vp, ci = (ctypes.c_uint64, ctypes.c_int64, ctypes.c_double,
                                 ctypes.c_void_p, ctypes.c_int)
        lib.pgd_gen_build.argtypes = [u64, u64, i64, vp, ci]
        lib.pgd_gen_probe_uniform.argtypes = [u64, u64, vp, u64, vp, ci]
        lib.pgd_gen_probe_zipf.argtypes = [u64, u64, dbl, vp, u64, vp, ci]
        lib.pgd_gen_uniform_keys.argtypes = [u64, u64, u64, vp, ci]
        lib.pgd_gen_zipf_keys.argtypes = [u64, u64, u64, dbl, vp, ci]
        lib.pgd_gen_groupby.argtypes = [u64, u64, u64, dbl, vp, ci]
        lib.pgd_raw_words.argtypes = [u64, u64, u64, vp]
        lib.pgd_raw_bounded.argtypes = [u64, u64, u64, u64, vp]
        for f in (lib.pgd_gen_build, lib.pgd_gen_probe_uniform, lib.pgd_gen_probe_zipf,
                  lib.pgd_gen_uniform_keys, lib.pgd_gen_zipf_keys, lib.pgd_gen_groupby,
                  lib.pgd_raw_words, lib.pgd_raw_bounded):
            f.restype = None
        _LIB = lib
    return _LIB


def _threads(t):
    return t if t else max(1, min(64, os.cpu_count() or 1))


def _out(n, out):
    if out is None:
        return np.empty((n, 2), dtype=np.int64)
    assert out.dtype == np.int64 and out.shape == (n, 2) and out.flags.c_contiguous
    return out


def build_relation(n, seed, key_base=1, threads=None, out=None):
    """Unique keys: a random permutation of key_base..key_base+n-1; payload U[0,2^31)."""
    o = _out(n, out)
    _lib().pgd_gen_build(seed, n, key_base, o.ctypes.data, _threads(threads))
    return o


def probe_uniform(n, build, seed, threads=None, out=None):
    """Foreign keys drawn uniformly over ``build``'s keys; payload U[0,2^31)."""
    o = _out(n, out)
    b = np.ascontiguousarray(build)
    _lib().pgd_gen_probe_uniform(seed, n, b.ctypes.data, b.shape[0], o.ctypes.data,
                                 _threads(threads))
    return o


def probe_zipf(n, s, build, seed, threads=None, out=None):
    """Foreign keys with Zipf(s) ranks mapped through ``build``'s key order."""
    o = _out(n, out)
    b = np.ascontiguousarray(build)
    _lib().pgd_gen_probe_zipf(seed, n, float(s), b.ctypes.data, b.shape[0], o.ctypes.data,
                              _threads(threads))
    return o


def uniform_keys(n, key_range, seed, threads=None, out=None):
    """Keys uniform in [0, key_range); payload U[0,2^31)."""
    o = _out(n, out)
    _lib().pgd_gen_uniform_keys(seed, n, key_range, o.ctypes.data, _threads(threads))
    return o


def zipf_keys(n, key_range, s, seed, threads=None, out=None):
    """Keys = Zipf(s) rank - 1 over [0, key_range); payload U[0,2^31)."""
    o = _out(n, out)
    _lib().pgd_gen_zipf_keys(seed, n, key_range, float(s), o.ctypes.data, _threads(threads))
    return o


def groupby_rows(n, groups, vmax, seed, threads=None, out=None):
    """(long key U[0,groups), dec value U[0,vmax)); column 1 holds float64 bits."""
    o = _out(n, out)
    _lib().pgd_gen_groupby(seed, n, groups, float(vmax), o.ctypes.data, _threads(threads))
    return o


def raw_words(seed, stream, n):
    o = np.empty(n, dtype=np.uint64)
    _lib().pgd_raw_words(seed, stream, n, o.ctypes.data)
    return o


def raw_bounded(seed, stream, key_range, n):
    o = np.empty(n, dtype=np.uint64)
    _lib().pgd_raw_bounded(seed, stream, key_range, n, o.ctypes.data)
    return o
