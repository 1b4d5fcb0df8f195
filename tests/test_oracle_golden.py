"""Pins the CPU oracle to the reference's own known answers.

The reference's only self-checks are its built-in test problems: the final
field_summary temperature must lie within 0.001 % of a constant
(field_summary.f90:88-106).  The decks and constants are fixtures generated
from the reference tree by tests/golden/make_golden.py.
"""
import json
import os
from pathlib import Path

import pytest

from oracle import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def problem(tp):
    meta = json.loads(Path(os.path.join(GOLD, "test_problems.json")).read_text())
    p = meta["problems"][str(tp)]
    return Path(os.path.join(GOLD, p["deck"])).read_text(), p["temp"]


def check(tp, mode="fused"):
    deck, temp = problem(tp)
    deck = deck.replace("*endtea", "tl_arithmetic %s\n*endtea" % mode, 1)
    res = oracle.run_deck(deck)
    qa = abs(100.0 * (res.final_temp / temp) - 100.0)
    assert qa < 0.001, (tp, res.final_temp, temp, qa)
    assert res.qa_passed == 1
    return res


@pytest.mark.parametrize("mode", ["exact", "fused", "chain"])
def test_tp1_jacobi_10x10(mode):
    res = check(1, mode)
    assert res.n_steps == 10
    # every step exits well before tl_max_iters
    assert all(0 < res.iterations[i] < 1000 for i in range(10))


@pytest.mark.parametrize("mode", ["exact", "fused", "chain"])
def test_tp6_ppcg_500x500_halo4(mode):
    res = check(6, mode)
    assert res.n_steps == 20
    # 88 inner steps per outer PPCG iteration: tl_ppcg_inner_steps defaults
    # to 4*INT(SQRT(SQRT(500*500))) (read_input.f90:293-297)
    assert all(res.inner_iterations[i] % 88 == 0 for i in range(20))
    assert res.inner_iterations[1] > 0


@pytest.mark.slow
@pytest.mark.parametrize("mode", ["exact", "fused", "chain"])
def test_tp2_cg_960x960(mode):
    check(2, mode)


@pytest.mark.slow
def test_tp3_cg_3840x3840():
    check(3)


@pytest.mark.parametrize("other", ["fused", "chain"])
@pytest.mark.parametrize("solver,prec", [("cg", "jac_diag"), ("ppcg", "jac_block")])
def test_arithmetic_forms_agree_within_tolerance(other, solver, prec):
    """The fused and chain forms differ from the exact one only by rounding:
    on a 64^2 run the field summaries agree to 1e-12 and the iteration
    counts to 1."""
    from tealeaf_opencl_gb300 import decks
    out = {}
    for mode in ("exact", other):
        deck = decks.five_state_deck(64, solver=solver, prec=prec, steps=5, eps=1e-15,
                                     inner_steps=8 if solver == "ppcg" else None,
                                     presteps=20 if solver == "ppcg" else None,
                                     extra="tl_arithmetic %s" % mode)
        out[mode] = oracle.run_deck(deck)
    a, b = out["exact"], out[other]
    sa, sb = a.summaries()[-1], b.summaries()[-1]
    assert max(abs(sa[i] - sb[i]) / abs(sa[i]) for i in (1, 2, 4, 5)) < 1e-12
    assert all(abs(a.iterations[i] - b.iterations[i]) <= 1 for i in range(5))


HEADLINE_PINS = os.path.join(GOLD, "oracle_pins_headline.json")


@pytest.mark.parametrize("workload", ["ppcg4096", "cheby4096"])
def test_headline_pins_are_the_bench_decks_and_forms_agree(workload):
    """The oracle pins of the benchmark's 4096^2 decks (recorded by
    make_oracle_pins.py) hold the exact deck bench.py times, in the exact
    and chain forms; on the oracle the two forms agree to 1e-12 in the
    field summary and to 1 in every iteration count."""
    import bench
    pins = json.loads(Path(HEADLINE_PINS).read_text())
    got = {}
    for form in ("exact", "chain"):
        p = pins["%s/%s" % (workload, form)]
        saved = bench.ARITHMETIC
        bench.ARITHMETIC = form
        try:
            assert p["deck"] == bench.deck_for(workload, len(p["iterations"]))
        finally:
            bench.ARITHMETIC = saved
        assert p["switch_iteration"][0] >= 20  # past the CG pre-steps
        assert all(s > 0 for s in p["switch_iteration"])
        got[form] = p
    a, b = got["exact"], got["chain"]
    assert all(abs(x - y) <= 1 for x, y in zip(a["iterations"], b["iterations"]))
    for k, v in a["summary_hex"].items():
        x, y = float.fromhex(v), float.fromhex(b["summary_hex"][k])
        assert abs(x - y) <= 1e-12 * abs(x), k


def test_largest_grid_pins_are_the_ppcg_deck_at_8192_and_forms_agree():
    """The 8192^2 pins hold bench.py's PPCG deck at that grid (one
    timestep), in the exact and chain forms, past the switch from CG.  On
    the oracle the two forms take the same iterations; their field summaries
    agree to 2.0e-12 relative (ie) and 1.0e-13 (temp).  The step ends 5
    iterations after the switch at CG iteration 785, far from convergence,
    and at 8192^2 the operator's condition number is 4 times that of the
    4096^2 grid (where the forms agree to 3.7e-14), so the bar here is
    1e-11."""
    from tests.golden.make_oracle_pins import LARGE_CAP, large_deck
    pins = json.loads(Path(HEADLINE_PINS).read_text())
    got = {}
    for form in ("exact", "chain"):
        p = pins["ppcg8192/%s" % form]
        assert p["deck"] == large_deck(8192, form)
        assert p["cap_after_switch"] == LARGE_CAP
        assert p["switch_iteration"][0] >= 20
        got[form] = p
    a, b = got["exact"], got["chain"]
    assert all(abs(x - y) <= 1 for x, y in zip(a["iterations"], b["iterations"]))
    for k, v in a["summary_hex"].items():
        x, y = float.fromhex(v), float.fromhex(b["summary_hex"][k])
        assert abs(x - y) <= 1e-11 * abs(x), k


def test_mixed_tall_pin_is_its_deck():
    """The mixed-precision pin at 2048x2440 holds the deck
    make_oracle_pins.py builds for it, and its solve reached 1e-8."""
    from tests.golden.make_oracle_pins import mixed_tall_deck
    p = json.loads(Path(HEADLINE_PINS).read_text())["mixed2048x2440"]
    assert p["deck"] == mixed_tall_deck()
    assert all(float.fromhex(v) <= 1e-8 for v in p["relative_residual_hex"])
    assert all(c >= 1 for c in p["outer_corrections"])


@pytest.mark.parametrize("solver", ["ppcg", "chebyshev"])
def test_cap_after_switch_bounds_the_polynomial_phase(solver):
    """max_after_switch ends a step that many iterations after its switch,
    the switch's own iteration counted; steps after the first PPCG step
    switch at iteration 2 (tea_solve.f90:153-155)."""
    from tealeaf_opencl_gb300 import decks
    deck = decks.five_state_deck(64, solver=solver, prec="jac_block", steps=3, eps=1e-15,
                                 halo=2, inner_steps=10, presteps=20, summary_frequency=0)
    full = oracle.run_deck(deck)
    cap = 3
    res = oracle.run_deck(deck, max_after_switch=cap)
    for i in range(3):
        sw = res.switch_iteration[i]
        assert sw >= (20 if (i == 0 or solver == "chebyshev") else 2)
        assert res.iterations[i] == sw - 1 + cap
        if solver == "ppcg":
            assert res.inner_iterations[i] == 10 * cap
    assert res.switch_iteration[0] == full.switch_iteration[0]
    if solver == "ppcg":
        assert list(res.switch_iteration[1:3]) == [2, 2]
