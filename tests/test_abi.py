"""CPU-side checks of the drop-in boundary: the C ABI library loads and
exports every function include/pythia_gpu.h declares (no compute calls), and
the reference's hash-function known answers (unit_tests/testhash.cpp)."""
import ctypes
import os
import re
import subprocess

import numpy as np

from oracle import oracle as orc
from pythia_gb300 import gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", text)))


def test_gpu_library_exports_every_declared_symbol():
    names = declared("pythia_gpu.h")
    assert len(names) >= 20
    lib = ctypes.CDLL(gpu.lib_path())
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(gpu.SYMBOLS)
    nm = subprocess.run(["nm", "-D", "--defined-only", gpu.lib_path()], capture_output=True, text=True).stdout
    for n in names:
        assert re.search(rf"\bT {n}\b", nm), n


def test_getlogarithm_and_generate_known_answers():
    # testhash.cpp:53-69: ParameterizedModuloValueHasher(0, 1024, 2).generate(3)
    # splits ten radix bits into passes of 8, 8 and 16 buckets.
    L = orc.lib()
    assert [L.or_getlogarithm(k) for k in (1, 2, 3, 4, 5, 1024, 1025)] == [0, 1, 2, 2, 3, 10, 11]
    f = orc.hashfn(orc.hashcfg("parammodulo", 1024, skipbits=2))
    out = (orc.HashFn * 3)()
    assert L.or_parammodulo_generate(ctypes.byref(f), 3, out) == 0
    assert [out[i].nbuckets for i in range(3)] == [8, 8, 16]
    assert [out[i].skipbits for i in range(3)] == [9, 6, 2]


def test_exactrange_bucket_edges():
    # testhash.cpp:120-144: hash(minimumforbucket(j)) == j for every bucket.
    for lo, hi, b in ((0, 999, 7), (-50, 50, 3), (1, 1 << 20, 127)):
        cfg = orc.hashcfg("exactrange", b, lo, hi)
        f = orc.hashfn(cfg)
        for j in range(b):
            m = orc.lib().or_exactrange_minimumforbucket(ctypes.byref(f), j)
            v = np.array([[m, 0]], dtype=np.int64)
            assert orc.hash_column(cfg, v)[0] == j
            if m > lo:
                assert orc.hash_column(cfg, np.array([[m - 1, 0]], dtype=np.int64))[0] == j - 1


def test_modulo_bounds_and_alwayszero():
    # testhash.cpp:96-118: modulo stays below buckets(); alwayszero is one bucket.
    keys = np.random.default_rng(0).integers(-1 << 40, 1 << 40, size=(20000, 2))
    for b in (1, 2, 3, 100, 1024):
        cfg = orc.hashcfg("modulo", b)
        assert orc.hash_column(cfg, keys).max() < orc.hashfn(cfg).nbuckets
    z = orc.hashcfg("alwayszero")
    assert orc.hashfn(z).nbuckets == 1 and orc.hash_column(z, keys).max() == 0
