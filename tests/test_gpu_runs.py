"""Whole tea.in decks on the GPU: reference goldens and oracle parity.

The C++ driver restates the reference's Fortran driver on top of the C ABI.
Each run must (a) pass the reference's own test-problem check
(field_summary.f90:88-106, 0.001 %) where the deck is a test problem and
(b) match the oracle's run of the same deck bit for bit: the same iteration
count in every timestep and the same field_summary values.
"""
import json
import os
from pathlib import Path

import pytest

from oracle import oracle
from tealeaf_opencl_gb300 import decks, lib

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def problem(tp):
    meta = json.loads(Path(os.path.join(GOLD, "test_problems.json")).read_text())
    p = meta["problems"][str(tp)]
    return Path(os.path.join(GOLD, p["deck"])).read_text(), p["temp"]


def pins(mode):
    name = "oracle_pins.json" if mode == "exact" else "oracle_pins_%s.json" % mode
    path = os.path.join(GOLD, name)
    return json.loads(Path(path).read_text()) if os.path.exists(path) else {}


def with_arithmetic(deck, mode):
    return deck.replace("*endtea", "tl_arithmetic %s\n*endtea" % mode, 1)


def gpu_run(deck, mode=lib.DRIVER_PER_CALL):
    steps = lib.run_deck(deck, mode=mode)
    assert steps and steps[-1].complete
    return steps


def assert_matches_oracle(steps, res):
    assert len(steps) == res.n_steps
    assert [s.iterations for s in steps] == list(res.iterations[:res.n_steps])
    assert [s.inner_iterations for s in steps] == list(res.inner_iterations[:res.n_steps])
    last = steps[-1]
    final = res.summaries()[-1]
    assert (last.vol, last.mass, last.ie, last.temp) == tuple(final[[1, 2, 4, 5]])


@pytest.mark.parametrize("mode", ["exact", "fused", "chain"])
@pytest.mark.parametrize("tp", [1, 6])
def test_test_problem_matches_golden_and_oracle(tp, mode):
    deck, temp = problem(tp)
    deck = with_arithmetic(deck, mode)
    steps = gpu_run(deck)
    assert steps[-1].qa_passed == 1, steps[-1].qa_diff
    assert abs(100.0 * steps[-1].temp / temp - 100.0) < 0.001
    assert_matches_oracle(steps, oracle.run_deck(deck))


@pytest.mark.parametrize("mode", ["exact", "fused", "chain"])
@pytest.mark.parametrize("tp", [2, 3])
def test_cg_test_problem_matches_golden_and_oracle_pin(tp, mode):
    deck, temp = problem(tp)
    steps = gpu_run(with_arithmetic(deck, mode), mode=lib.DRIVER_RESIDENT)
    assert steps[-1].qa_passed == 1, steps[-1].qa_diff
    pin = pins(mode).get(str(tp))
    if pin is None:
        pytest.skip("no oracle pin recorded for test problem %d (%s)" % (tp, mode))
    assert pin["arithmetic"] == mode if "arithmetic" in pin else mode == "exact"
    assert [s.iterations for s in steps] == pin["iterations"]
    assert steps[-1].temp == float.fromhex(pin["temp_hex"])


@pytest.mark.parametrize("tp", [4, 5])
def test_long_cg_test_problems_match_golden(tp):
    deck, temp = problem(tp)
    steps = gpu_run(deck, mode=lib.DRIVER_RESIDENT)
    assert steps[-1].qa_passed == 1, steps[-1].qa_diff


@pytest.mark.parametrize("mode", ["exact", "fused", "chain"])
def test_c1_512_cg_jac_diag_matches_oracle(mode):
    """512x512 CG + diagonal Jacobi, eps 1e-15, 10 steps."""
    deck = decks.five_state_deck(512, solver="cg", prec="jac_diag", steps=10,
                                 eps=1e-15, max_iters=5000,
                                 extra="tl_arithmetic %s" % mode)
    res = oracle.run_deck(deck)
    per_call = gpu_run(deck)
    assert_matches_oracle(per_call, res)
    resident = gpu_run(deck, mode=lib.DRIVER_RESIDENT)
    assert_matches_oracle(resident, res)


@pytest.mark.parametrize("solver,prec", [("chebyshev", "jac_block"), ("ppcg", "jac_block"),
                                         ("chebyshev", "jac_diag"), ("ppcg", "none")])
@pytest.mark.parametrize("mode", ["fused", "chain"])
def test_cheby_ppcg_decks_match_oracle(solver, prec, mode):
    deck = decks.five_state_deck(256, solver=solver, prec=prec, steps=4, eps=1e-15,
                                 max_iters=5000, halo=2, inner_steps=10, presteps=20,
                                 extra="tl_arithmetic %s" % mode)
    res = oracle.run_deck(deck)
    assert_matches_oracle(gpu_run(deck), res)
    if solver == "ppcg":
        # the device-resident PPCG loop (fused calc_ur + init_sd, scalars on
        # the device) stops at the same iteration with the same bits
        assert_matches_oracle(gpu_run(deck, mode=lib.DRIVER_RESIDENT), res)


@pytest.mark.parametrize("prec,eps,steps", [("jac_block", 1e-10, 3), ("jac_diag", 1e-15, 2),
                                            ("none", 1e-8, 3)])
def test_resident_ppcg_matches_per_call(prec, eps, steps):
    """Converging and capped PPCG runs, tall tiles: resident = per-call."""
    deck = decks.five_state_deck(2048, solver="ppcg", prec=prec, steps=steps, eps=eps,
                                 max_iters=300, y_cells=2440, inner_steps=8, presteps=15,
                                 summary_frequency=0, extra="tl_arithmetic chain")
    a = gpu_run(deck)
    b = gpu_run(deck, mode=lib.DRIVER_RESIDENT)
    assert [s.iterations for s in a] == [s.iterations for s in b]
    assert [s.inner_iterations for s in a] == [s.inner_iterations for s in b]
    assert (a[-1].vol, a[-1].mass, a[-1].ie, a[-1].temp) == \
        (b[-1].vol, b[-1].mass, b[-1].ie, b[-1].temp)


@pytest.mark.parametrize("prec,mode,inner,reflective",
                         [("jac_block", "chain", 7, False), ("jac_block", "exact", 9, True),
                          ("jac_diag", "fused", 5, True), ("none", "chain", 3, False),
                          ("jac_block", "fused", 6, True)])
def test_resident_ppcg_inner_steps(prec, mode, inner, reflective):
    """Odd and even inner-step counts, strips cut by the top edge
    (y_cells % 4 != 0) and reflective faces (whose operator reads the sd
    halo) give the per-call results and the oracle's in the resident loop."""
    deck = decks.five_state_deck(157, solver="ppcg", prec=prec, steps=3, eps=1e-13,
                                 max_iters=2000, y_cells=143, inner_steps=inner,
                                 presteps=12, reflective=reflective,
                                 extra="tl_arithmetic %s" % mode)
    res = oracle.run_deck(deck)
    assert_matches_oracle(gpu_run(deck), res)
    resident = gpu_run(deck, mode=lib.DRIVER_RESIDENT)
    assert_matches_oracle(resident, res)
    assert all(s.inner_iterations > 0 for s in resident)


def test_reflective_check_result_deck_matches_oracle():
    deck = decks.five_state_deck(123, solver="cg", prec="jac_block", steps=3, eps=1e-12,
                                 y_cells=99, reflective=True, check_result=True,
                                 coefficient="inverse")
    steps = gpu_run(deck)
    res = oracle.run_deck(deck)
    assert_matches_oracle(steps, res)
    assert [s.exact_error for s in steps] == list(res.exact_error[:res.n_steps])


@pytest.mark.parametrize("cells,y_cells,prec,mode", [(512, 512, "jac_diag", "chain"),
                                                    (300, 211, "jac_block", "fused"),
                                                    (2048, 2440, "none", "exact")])
def test_persistent_and_graph_resident_loops_agree(cells, y_cells, prec, mode):
    """The resident CG loop as one cooperative launch (grid barriers between
    its phases) gives the same iteration counts and field summaries, bit for
    bit, as the graph-replayed three-kernel loop; small decks also against
    the oracle."""
    L = lib.load()
    deck = decks.five_state_deck(cells, solver="cg", prec=prec, steps=3, eps=1e-15,
                                 max_iters=5000, y_cells=y_cells,
                                 extra="tl_arithmetic %s" % mode)
    try:
        L.tea_gb300_set_resident_mode(1)
        graph = gpu_run(deck, mode=lib.DRIVER_RESIDENT)
        L.tea_gb300_set_resident_mode(2)
        persistent = gpu_run(deck, mode=lib.DRIVER_RESIDENT)
    finally:
        L.tea_gb300_set_resident_mode(0)
    assert [s.iterations for s in graph] == [s.iterations for s in persistent]
    a, b = graph[-1], persistent[-1]
    assert (a.vol, a.mass, a.ie, a.temp) == (b.vol, b.mass, b.ie, b.temp)
    if cells * y_cells <= 512 * 512:
        assert_matches_oracle(persistent, oracle.run_deck(deck))
