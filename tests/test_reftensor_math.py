"""CPU tests of the reference-tensor contraction's arithmetic (florence_gb300/csrc/
fl_reftensor_math.cuh, built for the host through tests/reftensor_host_shim.cpp): the digit planes
are exact BF16 values within their bounds and sum to the split value, the integer int64 -> FP64
conversion rounds exactly like Python's correctly rounded int -> float, and one emulated GEMM
entry (digit planes, exact level sums, FP32 accumulation of the shared levels 4-5, exact
recombination) matches the exact dot product to within 2^-51 K max|a| max|b|, the Ozaki bound of
seven 8-bit digits per operand scaled per row and per column (plus the FP32 rounding of the shared
levels)."""
import ctypes
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("rt") / "rt_shim.so")
    subprocess.check_call(["g++", "-O2", "-shared", "-fPIC", "-o", so, os.path.join(HERE, "reftensor_host_shim.cpp")])
    L = ctypes.CDLL(so)
    f, d, i, P = ctypes.c_float, ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    L.rt_digits_c.argtypes = [f, f, f, P]
    L.rt_digits_f64_c.argtypes = [d, P]
    L.rt_i64_to_f64_c.argtypes = [ctypes.c_longlong, i]
    L.rt_i64_to_f64_c.restype = d
    L.rt_combine_c.argtypes = [P, i]
    L.rt_combine_c.restype = d
    L.rt_pair_c.argtypes = [i, P, P]
    L.rt_row_scale_c.argtypes = [f, P, P]
    L.rt_sym9_c.argtypes = [i, i]
    L.rt_dot_c.argtypes = [i, P, P, P]
    L.rt_dot_c.restype = d
    return L


def _bf16_exact(x):
    """x (float32) has no bits below the BF16 significand."""
    return (np.asarray(x, np.float32).view(np.uint32) & 0xFFFF) == 0


def _pair(x):
    h = np.float32(x)
    return h, np.float32(x - float(h))


def test_digits_of_float_pairs(shim):
    rng = np.random.default_rng(0)
    out = np.zeros(7, np.float32)
    for _ in range(4000):
        x = rng.uniform(-1, 1) * 2.0 ** rng.integers(-30, 7)       # |x| < 128
        h, l = _pair(x)
        shim.rt_digits_c(h, l, 1.0, out.ctypes.data)
        for s in range(7):
            assert abs(float(out[s])) <= 128.0 * 2.0 ** (-8 * s) * (1 + 1e-12)
            assert float(out[s]) * 2.0 ** (8 * s) == round(float(out[s]) * 2.0 ** (8 * s))  # multiple of 2^-8s
        assert _bf16_exact(out).all()
        exact = Fraction(float(h)) + Fraction(float(l))
        got = sum(Fraction(float(v)) for v in out)
        assert abs(float(got - exact)) <= 2.0 ** -48


def test_digits_of_fp64_values(shim):
    rng = np.random.default_rng(1)
    out = np.zeros(7, np.float32)
    for _ in range(2000):
        y = rng.uniform(-128, 128) * (2.0 ** -rng.integers(0, 20))
        shim.rt_digits_f64_c(y, out.ctypes.data)
        assert _bf16_exact(out).all()
        for s in range(7):
            assert abs(float(out[s])) <= 128.0 * 2.0 ** (-8 * s)
        assert abs(float(sum(Fraction(float(v)) for v in out) - Fraction(y))) <= 2.0 ** -48


def test_int64_to_double_is_correctly_rounded(shim):
    rng = np.random.default_rng(2)
    vals = [0, 1, -1, 2 ** 53 + 1, 2 ** 53 + 3, -(2 ** 60) - 5, 2 ** 62 - 1, 12345678901234567]
    vals += [int(v) for v in rng.integers(-2 ** 62, 2 ** 62, 2000)]
    for z in vals:
        for e2 in (-60, -40, 0, 7):
            assert shim.rt_i64_to_f64_c(z, e2) == float(Fraction(z) * Fraction(2) ** e2), (z, e2)


def test_row_scale_bounds(shim):
    E = ctypes.c_int(0)
    sc = ctypes.c_float(0)
    for amax in (1e-3, 0.5, 0.99, 1.0, 3.0, 127.9, 1e20, 2.0 ** -99):
        shim.rt_row_scale_c(amax, ctypes.byref(E), ctypes.byref(sc))
        assert amax < 2.0 ** E.value and amax * sc.value < 128.0 and amax * sc.value >= 32.0
    shim.rt_row_scale_c(0.0, ctypes.byref(E), ctypes.byref(sc))
    assert sc.value == 0.0


def test_pair_index_and_symmetric_packing(shim):
    a, b = ctypes.c_int(), ctypes.c_int()
    n = 0
    for bb in range(20):
        for aa in range(bb + 1):
            shim.rt_pair_c(n, ctypes.byref(a), ctypes.byref(b))
            assert (a.value, b.value) == (aa, bb)
            n += 1
    seen = set()
    for I in range(9):
        for K in range(I, 9):
            v = shim.rt_sym9_c(I, K)
            assert v == shim.rt_sym9_c(K, I) and 0 <= v < 45
            seen.add(v)
    assert len(seen) == 45


@pytest.mark.parametrize("K", [9, 126, 256])
def test_emulated_gemm_entry_is_fp64_accurate(shim, K):
    """sum_k a_k b_k with a_k float pairs (the pulled-back tangent) and b_k FP64 products of
    shape-function gradients, spread over several binades and with cancellation."""
    rng = np.random.default_rng(K)
    for trial in range(200):
        a = rng.standard_normal(K) * np.exp(rng.uniform(-6, 6, K))
        b = rng.standard_normal(K) * np.exp(rng.uniform(-4, 4, K)) * 10.0 ** rng.integers(-3, 3)
        ah = a.astype(np.float32)
        al = (a - ah.astype(np.float64)).astype(np.float32)
        got = shim.rt_dot_c(K, ah.ctypes.data, al.ctypes.data, b.ctypes.data)
        exact = sum(Fraction(float(x)) * Fraction(float(y)) + Fraction(float(z)) * Fraction(float(y))
                    for x, z, y in zip(ah, al, b))
        bound = 2.0 ** -51 * K * float(np.abs(a).max()) * float(np.abs(b).max())
        assert abs(got - float(exact)) <= bound, (trial, got, float(exact), bound)
