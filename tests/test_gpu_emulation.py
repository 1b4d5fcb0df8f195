"""The integer-pipe FP64 arithmetic (tea_emu.cuh) on the GPU against the
GPU's own FP64 instructions.

tests/test_fp64_emulation.py checks the host build of the header against
numpy.  The solver kernels run the device build, so here the same operand
sets (hard cases of each algorithm, special values) and ten million random
operand pairs per operation go through tea_gb300_emu_check, which runs the
emulated operation and __dmul_rn / __ddiv_rn / __dadd_rn side by side on
the GPU and counts the results whose bits differ.  Zero is the only pass.
"""
import ctypes

import numpy as np
import pytest

from tealeaf_opencl_gb300 import lib
from tests.test_fp64_emulation import operand_sets, rand_bits

pytestmark = pytest.mark.gpu
MUL, DIV_INVARIANT, DIV, ADD = 0, 1, 2, 3


def gpu_check(op, a, b=None, divisor=0.0):
    import torch
    ta = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    tb = torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).cuda() if b is not None else None
    bad, first = ctypes.c_longlong(), ctypes.c_longlong()
    rc = lib.load().tea_gb300_emu_check(op, ta.data_ptr(), tb.data_ptr() if tb is not None else None,
                                        ta.numel(), float(divisor), ctypes.byref(bad),
                                        ctypes.byref(first))
    assert rc == 0
    return bad.value, first.value


@pytest.mark.parametrize("op", [MUL, ADD, DIV])
def test_hard_cases_match_the_gpu_instruction(op):
    for name, a, b in operand_sets():
        for x, y in ((a, b), (b, a)):
            bad, first = gpu_check(op, x, y)
            assert bad == 0, (name, first, x[first], y[first])


def test_invariant_divisor_matches_the_gpu_instruction():
    rng = np.random.default_rng(11)
    divisors = list(rand_bits(rng, 20, 1, 2046)) + list(rand_bits(rng, 20, 1010, 1040))
    divisors += [1.0, 3.0, 0.1, 7.0, -1.5, 1.0000000000000002, 1.9999999999999998,
                 5e-324, 0.0, -0.0, np.inf, np.nan, 2.2250738585072014e-308,
                 1.7976931348623157e308]
    for y in divisors:
        xs = np.concatenate([rand_bits(rng, 100_000, 1, 2046), rand_bits(rng, 100_000, 1000, 1050),
                             np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 1.0, y, -y])])
        bad, first = gpu_check(DIV_INVARIANT, xs, divisor=y)
        assert bad == 0, (y, first)


def test_ten_million_random_pairs_per_operation():
    rng = np.random.default_rng(2024)
    for _ in range(5):
        for elo, ehi in ((1000, 1050), (1, 2046)):
            a = rand_bits(rng, 1_000_000, elo, ehi)
            b = rand_bits(rng, 1_000_000, elo, ehi)
            for op in (MUL, DIV, ADD):
                assert gpu_check(op, a, b)[0] == 0, (op, elo, ehi)
            assert gpu_check(DIV_INVARIANT, a, divisor=b[0])[0] == 0
