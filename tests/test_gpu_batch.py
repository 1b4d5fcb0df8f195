"""Batched solves on the GPU against single-chunk runs of the same problems.

Every problem of a batch must give what the single-chunk driver gives for
it (tea_solve.f90's CG loop through the C ABI, itself pinned to the oracle
by test_gpu_runs.py): the same iteration count in every timestep and the
same field_summary values, bit for bit.  The launch geometry (blocks per
SM, supertiles per work unit, iterations per graph replay) and the
autotuner must not change any result.
"""
import numpy as np
import pytest

from oracle import oracle
from tealeaf_opencl_gb300 import decks, lib

pytestmark = pytest.mark.gpu

STEPS = 3
EPS = 1e-12
DT = 0.004


def single_chunk(problem, prec, mode, steps=STEPS, eps=EPS, max_iters=5000):
    """(density, energy1 after set-up, iterations per step, final summary)."""
    deck = decks.batch_deck(problem, steps=steps, eps=eps, max_iters=max_iters,
                            prec=prec, arithmetic=mode)
    drv = lib.Driver(deck, mode=lib.DRIVER_RESIDENT)
    try:
        dens = lib.read_field("density")
        en = lib.read_field("energy1")
        infos = []
        while True:
            info = drv.step()
            if info is None:
                break
            infos.append(info)
            if info.complete:
                break
    finally:
        drv.close()
    last = infos[-1]
    return dens, en, [s.iterations for s in infos], (last.vol, last.mass, last.ie, last.temp)


def make_batch(problems, fields, prec, mode):
    lib.load().tea_gb300_set_arithmetic(lib.arithmetic_form(mode))
    b = lib.Batch([(p["x"], p["y"]) for p in problems], prec=prec)
    for i, (d, e) in enumerate(fields):
        b.set_fields(i, d, e)
    return b


def bits(t):
    return np.array(t, dtype=np.float64).view(np.int64).tolist()


def problem_set():
    ps = decks.batch_problems(9, seed=11, side=(64, 300))
    # ragged shapes: narrower than a tile, one row of supertiles, odd sizes
    ps += decks.batch_problems(1, seed=12, side=(5, 31))
    ps.append(dict(x=700, y=37, states=ps[0]["states"]))
    ps.append(dict(x=33, y=513, states=ps[1]["states"]))
    return ps


@pytest.mark.parametrize("prec,mode", [("jac_diag", "fused"), ("jac_diag", "exact"),
                                       ("jac_diag", "chain"), ("none", "fused"),
                                       ("jac_block", "fused")])
def test_batch_matches_single_chunk_runs(prec, mode):
    problems = problem_set()
    ref = [single_chunk(p, prec, mode) for p in problems]
    b = make_batch(problems, [(r[0], r[1]) for r in ref], prec, mode)
    try:
        st = b.run(STEPS, DT, EPS, 5000)
        for i, r in enumerate(ref):
            assert b.iterations(i) == r[2], (i, problems[i]["x"], problems[i]["y"])
            assert bits(b.summary(i)) == bits(r[3]), i
        # the chain to the oracle, for the problems it finishes in seconds
        if prec == "jac_diag":
            for i in (9, 11):
                deck = decks.batch_deck(problems[i], steps=STEPS, eps=EPS, prec=prec,
                                        arithmetic=mode)
                res = oracle.run_deck(deck)
                assert b.iterations(i) == list(res.iterations[:res.n_steps])
                assert bits(b.summary(i)) == bits(res.summaries()[-1][[1, 2, 4, 5]])
        assert st.steps == STEPS
        assert st.max_iterations == max(max(r[2]) for r in ref)
        assert st.iterations == sum(sum(r[2]) for r in ref)
        assert st.kernel_launches > 0 and st.graph_launches > 0
    finally:
        b.free()


def test_launch_geometry_and_autotune_do_not_change_results():
    problems = decks.batch_problems(6, seed=5, side=(64, 400))
    fields = [decks.paint(p) for p in problems]
    b = make_batch(problems, fields, "jac_diag", "fused")
    try:
        base = None
        # the last three: one persistent (cooperative) launch per replay
        geoms = [(1, 1, 1, 0), (2, 5, 3, 0), (b.launch()["blocks_per_sm"], 16, 8, 0),
                 (1, 1, 1, 1), (2, 7, 2, 1), (b.launch()["blocks_per_sm"], 16, 4, 1)]
        for bps, gi, g, pers in geoms:
            for i, f in enumerate(fields):
                b.set_fields(i, *f)
            b.set_launch(bps, gi, g, pers)
            b.run(2, DT, EPS, 5000)
            got = [(b.iterations(i), bits(b.summary(i))) for i in range(len(problems))]
            if base is None:
                base = got
            assert got == base, (bps, gi, g, pers)
        for i, f in enumerate(fields):
            b.set_fields(i, *f)
        best = b.autotune()
        assert 1 <= best["blocks_per_sm"] and 1 <= best["supertiles_per_unit"] <= 8
        b.run(2, DT, EPS, 5000)
        assert [(b.iterations(i), bits(b.summary(i))) for i in range(len(problems))] == base
    finally:
        b.free()


def test_tall_tile_problem_in_a_batch():
    """A problem large enough for 16-row reduction tiles beside small ones."""
    problems = [dict(x=2048, y=2432, states=decks.batch_problems(1, seed=3)[0]["states"])]
    problems += decks.batch_problems(3, seed=4, side=(64, 128))
    assert lib.load().tea_gb300_reduction_rows(2048, 2432) == 16
    ref = [single_chunk(p, "jac_diag", "fused", steps=1) for p in problems]
    b = make_batch(problems, [(r[0], r[1]) for r in ref], "jac_diag", "fused")
    try:
        b.run(1, DT, EPS, 5000)
        for i, r in enumerate(ref):
            assert b.iterations(i) == r[2]
            assert bits(b.summary(i)) == bits(r[3])
    finally:
        b.free()


def test_iteration_cap_and_fields():
    """max_iters caps every problem as tl_max_iters does; energy1 and u are
    readable and energy1 = u / density after a step."""
    problems = decks.batch_problems(3, seed=9, side=(64, 200))
    ref = [single_chunk(p, "jac_diag", "fused", steps=2, max_iters=7) for p in problems]
    b = make_batch(problems, [(r[0], r[1]) for r in ref], "jac_diag", "fused")
    try:
        b.run(2, DT, EPS, 7)
        for i, r in enumerate(ref):
            assert b.iterations(i) == r[2] == [7, 7]
            assert bits(b.summary(i)) == bits(r[3])
            u, e, d = b.read(i, "u"), b.read(i, "energy1"), b.read(i, "density")
            assert np.array_equal(e, u / d)
    finally:
        b.free()


def test_batch_errors():
    L = lib.load()
    with pytest.raises(lib.TeaError):
        lib.Batch([(0, 5)])
    with pytest.raises(lib.TeaError):
        lib.Batch([(8, 8)], prec=7)
    b = lib.Batch([(40, 30), (20, 10)])
    try:
        with pytest.raises(lib.TeaError):
            b.summary(0)  # no run yet
        with pytest.raises(lib.TeaError):
            b.run(0, DT, EPS, 10)
        with pytest.raises(lib.TeaError):
            b.set_launch(1000)
        out = np.zeros(40 * 30)
        assert L.tea_gb300_batch_read_field(5, 4, out.ctypes.data_as(lib.PD)) == -1
        with pytest.raises(lib.TeaError):
            lib.check()
        with pytest.raises(lib.TeaError):
            b.read(0, "w")
    finally:
        b.free()
    with pytest.raises(lib.TeaError):
        b.summary(0)  # freed
    assert L.tea_gb300_batch_run(1, DT, EPS, 10, None) == -1
    with pytest.raises(lib.TeaError):
        lib.check()
