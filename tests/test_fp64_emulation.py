"""The integer FP64 add, multiply and divide (tea_emu.cuh) against IEEE
arithmetic.

The stencil kernels move part of their FP64 multiplies and their divisions
to integer instructions; the solve stays bit-exact only if those
give the correctly rounded result for every operand pair.  The header is built for the host
here and compared bit for bit with numpy's float64 + and * on random
operands over the whole exponent range, on the hard cases of each
algorithm (cancellation, exact ties, carries out of the rounding) and on
zeros, subnormals, infinities and NaNs (which take the fallback).
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "tealeaf_opencl_gb300", "csrc")
P = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    out = str(tmp_path_factory.mktemp("emu") / "emu.so")
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC,
                    os.path.join(HERE, "native", "emu_harness.cpp"), "-o", out], check=True)
    return ctypes.CDLL(out)


def call(fn, a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    o = np.empty_like(a)
    fn(a.ctypes.data_as(P), b.ctypes.data_as(P), o.ctypes.data_as(P), ctypes.c_long(a.size))
    return o


def mismatches(want, got):
    both_nan = np.isnan(want) & np.isnan(got)
    return int(np.sum((want.view(np.uint64) != got.view(np.uint64)) & ~both_nan))


def rand_bits(rng, n, elo, ehi, low_zero_bits=0):
    s = rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    e = rng.integers(elo, ehi + 1, n, dtype=np.uint64) << np.uint64(52)
    m = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    m &= ~np.uint64((1 << low_zero_bits) - 1)
    return (s | e | m).view(np.float64)


def operand_sets(seed=7, n=400_000):
    rng = np.random.default_rng(seed)
    yield "whole range", rand_bits(rng, n, 1, 2046), rand_bits(rng, n, 1, 2046)
    yield "close exponents", rand_bits(rng, n, 1000, 1050), rand_bits(rng, n, 1000, 1050)
    a = rand_bits(rng, n, 1015, 1030)
    near = (a.view(np.uint64) + rng.integers(-3, 4, n).astype(np.uint64)).view(np.float64)
    yield "cancellation", a, -near
    yield "ties", rand_bits(rng, n, 1020, 1025, 26), rand_bits(rng, n, 1020, 1025, 26)
    yield "short b", rand_bits(rng, n, 1020, 1025), rand_bits(rng, n, 1020, 1025, 30)
    yield "tiny", rand_bits(rng, n, 1, 130), rand_bits(rng, n, 1, 130)
    yield "huge", rand_bits(rng, n, 1990, 2046), rand_bits(rng, n, 1, 2046)
    ones = np.full(n, 1.0) + rng.integers(0, 1 << 20, n) * 2.0 ** -52
    yield "carries", ones, 2.0 - ones
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324,
                   2.2250738585072014e-308, -2.2250738585072014e-308,
                   1.7976931348623157e308, -1.7976931348623157e308, 1.0, -1.0,
                   0.5, 3.0, 2.0 ** 64, 2.0 ** -1000, -(2.0 ** -1021)])
    A, B = np.meshgrid(sp, sp)
    yield "special values", A.ravel(), B.ravel()


@pytest.mark.parametrize("op", ["add", "mul"])
def test_integer_fp64_matches_ieee(emu, op):
    fn = emu.emu_add_n if op == "add" else emu.emu_mul_n
    for name, a, b in operand_sets():
        with np.errstate(all="ignore"):
            want = a + b if op == "add" else a * b
        assert mismatches(want, call(fn, a, b)) == 0, name
        assert mismatches(want, call(fn, b, a)) == 0, name + " (swapped)"


def test_integer_division_by_invariant_divisor_matches_ieee(emu):
    emu.emu_div_n.argtypes = [P, ctypes.c_double, P, ctypes.c_long]
    rng = np.random.default_rng(11)
    divisors = list(rand_bits(rng, 30, 1, 2046)) + list(rand_bits(rng, 30, 1010, 1040))
    divisors += [1.0, 3.0, 0.1, 7.0, -1.5, 1.0000000000000002, 1.9999999999999998,
                 5e-324, 0.0, -0.0, np.inf, np.nan, 2.2250738585072014e-308,
                 1.7976931348623157e308]
    for y in divisors:
        for xs in (rand_bits(rng, 40_000, 1, 2046), rand_bits(rng, 40_000, 1000, 1050),
                   rand_bits(rng, 5_000, 1, 60), rand_bits(rng, 5_000, 1990, 2046),
                   np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 1.0, y, -y, 2 * y])):
            xs = np.ascontiguousarray(xs)
            got = np.empty_like(xs)
            emu.emu_div_n(xs.ctypes.data_as(P), float(y), got.ctypes.data_as(P), xs.size)
            with np.errstate(all="ignore"):
                want = xs / y
            assert mismatches(want, got) == 0, y


def test_integer_division_by_varying_divisor_matches_ieee(emu):
    """emu_ddiv_var: every element its own divisor (Jacobi, init_common,
    block_init, finalise, the exact form's strip sweep)."""
    emu.emu_divv_n.argtypes = [P, P, P, ctypes.c_long]
    rng = np.random.default_rng(13)
    sets = [rand_bits(rng, 300_000, 1, 2046), rand_bits(rng, 300_000, 1000, 1050),
            rand_bits(rng, 100_000, 1, 100), rand_bits(rng, 100_000, 1900, 2046),
            rand_bits(rng, 100_000, 1000, 1050, 30)]
    pairs = [(a, b) for a in sets[:2] for b in sets[:2]] + [(sets[2], sets[3]), (sets[3], sets[2]),
                                                            (sets[4], sets[4][::-1].copy())]
    # divisor significands at and next to the ends of the binade
    frac = np.concatenate([np.arange(0, 2000, dtype=np.uint64),
                           np.uint64((1 << 52) - 1) - np.arange(0, 2000, dtype=np.uint64)])
    ys = (frac | (np.uint64(1023) << np.uint64(52))).view(np.float64)
    for x in (1.0, 1.5, 1.9999999999999998, 1.0000000000000002, 0.1, -3.0):
        pairs.append((np.full(ys.size, x), ys))
    y = rand_bits(rng, 100_000, 1015, 1030)
    near = (y.view(np.uint64) + rng.integers(-3, 4, y.size).astype(np.uint64)).view(np.float64)
    pairs.append((near, y))
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 2.2250738585072014e-308,
                   1.7976931348623157e308, 1.0, -7.5, 2.0 ** -1022, 2.0 ** 1023])
    A, B = np.meshgrid(sp, sp)
    pairs.append((A.ravel(), B.ravel()))
    for a, b in pairs:
        with np.errstate(all="ignore"):
            want = a / b
        assert mismatches(want, call(emu.emu_divv_n, a, b)) == 0


def test_integer_fp64_long_random_sweep(emu):
    """Ten million random operand pairs per operation, exponents near 1 and
    over the whole range, against numpy."""
    emu.emu_divv_n.argtypes = [P, P, P, ctypes.c_long]
    emu.emu_div_n.argtypes = [P, ctypes.c_double, P, ctypes.c_long]
    rng = np.random.default_rng(2024)
    for _ in range(5):
        for elo, ehi in ((1000, 1050), (1, 2046)):
            a = rand_bits(rng, 1_000_000, elo, ehi)
            b = rand_bits(rng, 1_000_000, elo, ehi)
            with np.errstate(all="ignore"):
                assert mismatches(a + b, call(emu.emu_add_n, a, b)) == 0
                assert mismatches(a * b, call(emu.emu_mul_n, a, b)) == 0
                assert mismatches(a / b, call(emu.emu_divv_n, a, b)) == 0
                y = float(b[0])
                got = np.empty_like(a)
                emu.emu_div_n(a.ctypes.data_as(P), y, got.ctypes.data_as(P), a.size)
                assert mismatches(a / y, got) == 0
