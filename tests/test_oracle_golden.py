"""Pins the CPU oracle to the reference's own known answers.

The reference's only self-checks are its built-in test problems: the final
field_summary temperature must lie within 0.001 % of a constant
(field_summary.f90:88-106).  The decks and constants are fixtures generated
from the reference tree by tests/golden/make_golden.py.
"""
import json
import os

import pytest

from oracle import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def problem(tp):
    meta = json.load(open(os.path.join(GOLD, "test_problems.json")))
    p = meta["problems"][str(tp)]
    return open(os.path.join(GOLD, p["deck"])).read(), p["temp"]


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
