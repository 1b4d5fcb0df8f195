"""Failure detection, without a GPU fault.

The reference runs on silently when CG breaks down and DIEs on every other
error (tea_solve.f90:270-330, ocl_errors.cpp:175-194).  The library keeps
that by default and adds, on request, error returns for a breakdown and for
a step that used up tl_max_iters.  The failures are made on the host: a NaN
written into an input field, or a tiny iteration budget.  The persistent
loop's grid barrier is tested by a wait that is bound to run out (it waits
for one block more than the grid has) under a short poll limit: the kernel
returns, the call reports error 25, and the context stays usable.
"""
import math

import numpy as np
import pytest

from tealeaf_opencl_gb300 import decks, lib

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def no_abort():
    L = lib.load()
    L.tea_gb300_set_abort_on_error(0)
    L.tea_gb300_last_error(None, 0)  # start from a clear record
    yield L
    L.tea_gb300_set_resident_mode(0)
    L.tea_gb300_set_barrier_limits(1 << 26, 0)
    L.tea_gb300_last_error(None, 0)


def last_error(L):
    import ctypes
    buf = ctypes.create_string_buffer(512)
    return L.tea_gb300_last_error(buf, 512), buf.value.decode()


def cg_deck(**kw):
    args = dict(solver="cg", prec="jac_diag", steps=2, eps=1e-15, max_iters=5000,
                summary_frequency=0)
    args.update(kw)
    return decks.five_state_deck(96, **args)


def poison_density(drv):
    d = lib.read_field("density")
    d[40, 50] = np.nan
    lib.write_field("density", d)


@pytest.mark.parametrize("mode", [lib.DRIVER_PER_CALL, lib.DRIVER_RESIDENT])
@pytest.mark.parametrize("solver", ["cg", "ppcg"])
def test_nan_input_is_a_breakdown_error_when_checked(no_abort, mode, solver):
    L = no_abort
    kw = dict(solver=solver, prec="jac_block", halo=2, inner_steps=6, presteps=10) \
        if solver == "ppcg" else {}
    drv = lib.Driver(cg_deck(**kw), mode=mode, checks=lib.CHECK_BREAKDOWN)
    poison_density(drv)
    info = lib.StepInfo()
    assert L.tea_gb300_driver_step(info) == -1
    code, msg = last_error(L)
    assert code == 70, msg
    assert "breakdown" in msg
    drv.close()


def test_nan_input_runs_on_silently_by_default(no_abort):
    """Without the check the library does what the reference does."""
    L = no_abort
    drv = lib.Driver(cg_deck(steps=1), mode=lib.DRIVER_PER_CALL, max_iters_cap=30)
    poison_density(drv)
    info = drv.step()
    assert info is not None and info.iterations == 30
    assert math.isnan(info.conduction_error)
    assert last_error(L)[0] == 0
    drv.close()


@pytest.mark.parametrize("mode", [lib.DRIVER_PER_CALL, lib.DRIVER_RESIDENT])
def test_exhausted_iteration_budget_is_an_error_when_checked(no_abort, mode):
    L = no_abort
    deck = cg_deck(steps=1, max_iters=7)
    steps = lib.run_deck(deck, mode=mode)  # unchecked: completes, 7 iterations
    assert steps[-1].iterations == 7
    drv = lib.Driver(deck, mode=mode, checks=lib.CHECK_MAX_ITERS)
    info = lib.StepInfo()
    assert L.tea_gb300_driver_step(info) == -1
    code, msg = last_error(L)
    assert code == 72, msg
    drv.close()
    # a budget that suffices passes the same check
    ok = lib.run_deck(cg_deck(steps=1, eps=1e-8), mode=mode, checks=lib.CHECK_MAX_ITERS)
    assert ok[-1].iterations < 5000


def test_persistent_barrier_time_out_returns_an_error(no_abort):
    L = no_abort
    deck = cg_deck(steps=1)
    good = lib.run_deck(deck, mode=lib.DRIVER_RESIDENT)
    assert L.tea_gb300_set_resident_mode(2) == 0
    # at most 4096 polls of about 64 ns each: a few ms, then every block returns
    assert L.tea_gb300_set_barrier_limits(1 << 12, 1) == 0
    drv = lib.Driver(deck, mode=lib.DRIVER_RESIDENT)
    info = lib.StepInfo()
    assert L.tea_gb300_driver_step(info) == -1
    code, msg = last_error(L)
    assert code == 25, msg
    drv.close()
    # the context is still usable: the same deck with the normal barrier
    assert L.tea_gb300_set_barrier_limits(1 << 26, 0) == 0
    again = lib.run_deck(deck, mode=lib.DRIVER_RESIDENT)
    assert [s.iterations for s in again] == [s.iterations for s in good]
    assert again[-1].temp == good[-1].temp
