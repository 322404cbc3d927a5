"""The exact dec-sum arithmetic of the group-by kernels
(pythia_gb300/csrc/pg_fixsum.h), checked on the host against exact
fractions: quantisation to units 2^s rounds to nearest (ties to even), the
table adds (one word at a time, carries and signed overflows from the old
words, as the kernels' atomics do) hold the exact sum of the counts in any
order, a 256-bit count converts back to the correctly rounded double
(normal, subnormal, overflow), and a sum of values within the exact range
equals math.fsum bit for bit in any order."""
import ctypes
import math
import os
import shutil
import struct
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
U64 = ctypes.c_uint64


@pytest.fixture(scope="module")
def fx(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    so = str(tmp_path_factory.mktemp("fx") / "libfxshim.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I" + os.path.join(ROOT, "pythia_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "fixsum_shim.cpp"), "-o", so], check=True)
    L = ctypes.CDLL(so)
    L.fx_unit.argtypes, L.fx_unit.restype = [ctypes.c_int], ctypes.c_int
    L.fx_field.argtypes, L.fx_field.restype = [ctypes.c_double], ctypes.c_int
    L.fx_sum.argtypes = [ctypes.POINTER(ctypes.c_double), U64, ctypes.c_int, ctypes.POINTER(U64)]
    L.fx_sum.restype = ctypes.c_double
    L.fx_quant.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.POINTER(U64)]
    L.fx_double.argtypes, L.fx_double.restype = [ctypes.POINTER(U64), ctypes.c_int], ctypes.c_double
    L.fx_table_add.argtypes, L.fx_table_add.restype = [ctypes.POINTER(U64), ctypes.POINTER(U64)], ctypes.c_int
    L.fx_table_count.argtypes = [ctypes.POINTER(U64), ctypes.POINTER(U64)]
    L.fx_words.restype = ctypes.c_int
    L.fx_chain_add.argtypes = [ctypes.POINTER(U64), ctypes.POINTER(U64)]
    L.fx_chain_count.argtypes = [ctypes.POINTER(U64), ctypes.POINTER(U64)]
    L.fx_special_bits.argtypes, L.fx_special_bits.restype = [ctypes.c_uint32], U64
    return L


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def signed192(w):
    v = w[0] | (w[1] << 64) | (w[2] << 128)
    return v - (1 << 192) if v >> 191 else v


def signed256(w):
    v = sum(int(w[k]) << (64 * k) for k in range(4))
    return v - (1 << 256) if v >> 255 else v


def words(v):
    u = v & ((1 << 256) - 1)
    return (U64 * 4)(*[(u >> (64 * k)) & (2 ** 64 - 1) for k in range(4)])


def unit_of(L, xs):
    field = max((L.fx_field(float(x)) for x in xs), default=0)
    return L.fx_unit(field)


def table(L):
    return (U64 * L.fx_words())()


def table_total(L, t):
    w = (U64 * 4)()
    L.fx_table_count(t, w)
    return signed256(w)


def exact_quant(x, s):
    return round(Fraction(x) / Fraction(2) ** s)          # round half to even


def scale(s):
    return Fraction(2) ** s


def test_quantise_rounds_to_nearest_even(fx):
    rng = np.random.default_rng(5)
    w = (U64 * 3)()
    for s in (-1200, -1100, -1074, -200, -60, -1, 0, 3, 40, 900):
        for x in list(rng.standard_normal(40) * 2.0 ** rng.integers(-30, 30, 40)) + [0.0, -0.0, 5e-324, -5e-324,
                                                                                    2.0 ** -1022, 1.5, -2.5, 3.5]:
            x = float(x)
            if x != 0 and math.floor(math.log2(abs(x))) - s > 187:
                continue                                  # above the bound a unit allows (2^188 units)
            fx.fx_quant(x, s, w)
            assert signed192(list(w)) == exact_quant(x, s), (x, s)
    # exact ties go to the even count
    for m in range(-9, 10):
        x = m + 0.5
        fx.fx_quant(x, 0, w)
        assert signed192(list(w)) == round(Fraction(x))


def test_count_to_double_is_correctly_rounded(fx):
    rng = np.random.default_rng(6)
    cases = []
    for _ in range(4000):
        nb = int(rng.integers(1, 255))
        v = sum(int(rng.integers(0, 1 << 62)) << (64 * k) for k in range(4))
        v &= (1 << nb) - 1
        v = v or 1
        if rng.random() < 0.5:
            v = -v
        cases.append((v, int(rng.integers(-1200, 960))))
    # halfway points and carries into the next binade
    for s in (-1100, -1074, -1080, 0, 7):
        for v in ((1 << 53) + 1, (1 << 54) + 2, (1 << 54) + 6, (1 << 60) - 1, (1 << 126) - 1, (1 << 190) - 1,
                  (1 << 117) + (1 << 64), ((1 << 53) + 1) << 120, 3, 1, (1 << 254) + (1 << 190) + 1,
                  ((1 << 53) + 1) << 200, (1 << 192) - 1):
            cases += [(v, s), (-v, s)]
    for v, s in cases:
        got = fx.fx_double(words(v), s)
        exact = Fraction(v) * scale(s)
        try:
            want = float(exact)                           # correctly rounded
        except OverflowError:
            want = math.inf if v > 0 else -math.inf
        assert bits(got) == bits(want), (v, s, got, want)
    assert bits(fx.fx_double(words(0), 5)) == bits(0.0)


def test_sums_equal_fsum_in_any_order(fx):
    rng = np.random.default_rng(7)
    w = table(fx)
    for trial in range(60):
        n = int(rng.integers(1, 3000))
        spread = int(rng.integers(0, 100))
        xs = rng.standard_normal(n) * 2.0 ** rng.integers(-spread, 1, n) * 10.0 ** rng.integers(-5, 6)
        if trial % 3 == 0:
            xs = np.concatenate([xs, -xs[: n // 2]])      # cancellation
        s = unit_of(fx, xs)
        want = math.fsum(xs.tolist())
        exact = sum(exact_quant(float(x), s) for x in xs)
        for order in range(3):
            arr = np.ascontiguousarray(rng.permutation(xs) if order else xs, dtype=np.float64)
            got = fx.fx_sum(arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(arr), s, w)
            assert bits(got) == bits(want), (trial, order, got, want)
            assert table_total(fx, w) == exact


def test_values_below_the_exact_range_are_rounded_to_the_unit(fx):
    xs = np.array([1.0e30, 3.0e-30, -1.0e30, 7.0e-31], dtype=np.float64)
    s = unit_of(fx, xs)
    w = table(fx)
    got = fx.fx_sum(xs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(xs), s, w)
    want = sum(exact_quant(float(x), s) for x in xs) * scale(s)
    assert got == float(want)
    assert abs(got - math.fsum(xs.tolist())) <= 4 * 2.0 ** s


def test_table_adds_hold_the_exact_sum(fx):
    # Values at the top of the bound's binade overflow the signed word t2
    # every few adds (one add into t3); values far below the largest add
    # 28-bit chunks into the lazy words; runs of one sign, cancellation and
    # wide sums (warp-combined counts) end on the exact total in any order, in
    # the global tables' form and in the chained form of shared-memory tables.
    rng = np.random.default_rng(8)
    top = 1 << 188
    for trial in range(40):
        n = int(rng.integers(1, 2000))
        kind = trial % 4
        if kind == 0:                                     # near the bound, one sign
            vs = [top - 1 - int(rng.integers(0, 1 << 62)) for _ in range(n)]
        elif kind == 1:                                   # near the bound, both signs
            vs = [(top - 1 - int(rng.integers(0, 1 << 62))) * (1 if rng.random() < 0.5 else -1) for _ in range(n)]
        elif kind == 2:                                   # every scale: low words and carries
            vs = [int(rng.integers(0, 1 << 62)) << int(rng.integers(0, 126)) for _ in range(n)]
            vs = [v if rng.random() < 0.6 else -v for v in vs]
        else:                                             # sums of up to 32 values, then more
            vs = [sum(top - 1 - int(rng.integers(0, 1 << 40)) for _ in range(int(rng.integers(1, 33))))
                  * (1 if rng.random() < 0.7 else -1) for _ in range(n)]
        want = sum(vs)
        for order in range(2):
            t = table(fx)
            seq = vs if order == 0 else [vs[i] for i in rng.permutation(n)]
            marks = [fx.fx_table_add(t, words(v)) for v in seq]
            assert table_total(fx, t) == want, (trial, order)
            assert marks[0] == 1                          # the first add returns the initial 0 (or makes none)
            c, w = (U64 * 4)(), (U64 * 4)()               # the chained form of shared-memory tables
            for v in seq:
                fx.fx_chain_add(c, words(v))
            fx.fx_chain_count(c, w)
            assert signed256(w) == want, (trial, order)


def test_special_results(fx):
    assert fx.fx_special_bits(1) == bits(math.inf)
    assert fx.fx_special_bits(2) == bits(-math.inf)
    for f in (3, 4, 5, 6, 7):
        assert math.isnan(struct.unpack("<d", struct.pack("<Q", fx.fx_special_bits(f)))[0])
