"""Mixed precision: FP32 inner CG in FP64 defect correction.

The GPU solve is compared bit for bit with the oracle's restatement
(oracle_mixed_solve): per-step FP32 iteration counts, FP64 corrections,
final relative residuals and field summaries.  Its answer is compared with
the FP64 solve to the same true relative residual, within the accuracy that
residual implies.
"""
import numpy as np
import pytest

from oracle import oracle
from tealeaf_opencl_gb300 import decks, lib

pytestmark = pytest.mark.gpu


def mixed_deck(cells, steps=3, eps=1e-10, inner=1e-5, y_cells=None, extra="",
               solver="cg", inner_steps=None, presteps=None):
    return decks.five_state_deck(cells, solver=solver, prec="jac_diag", steps=steps, eps=eps,
                                 max_iters=20000, y_cells=y_cells, inner_steps=inner_steps,
                                 presteps=presteps,
                                 extra="tl_mixed_precision\ntl_mixed_inner_eps %g\n%s"
                                 % (inner, extra))


@pytest.mark.parametrize("cells,y_cells,inner", [(130, 129, 1e-5), (257, 131, 1e-4),
                                                 (64, 64, 1e-6)])
def test_mixed_matches_oracle(cells, y_cells, inner):
    deck = mixed_deck(cells, y_cells=y_cells, inner=inner)
    steps = lib.run_deck(deck)
    res = oracle.run_deck(deck)
    n = res.n_steps
    assert [s.iterations for s in steps] == list(res.iterations[:n])
    assert [s.outer_corrections for s in steps] == list(res.outer_corrections[:n])
    assert [s.relative_residual for s in steps] == list(res.relative_residual[:n])
    final = res.summaries()[-1]
    last = steps[-1]
    assert (last.vol, last.mass, last.ie, last.temp) == tuple(final[[1, 2, 4, 5]])
    assert all(s.relative_residual <= 1e-10 for s in steps)


def test_mixed_tall_tiles_match_oracle_pin():
    """2048x2440, the smallest grid with 16-row reduction tiles, one
    timestep to 1e-8: iteration counts, corrections, residual and field
    summary bit for bit against the oracle's run of the same deck
    (tests/golden/oracle_pins_headline.json, made by make_oracle_pins.py
    --mixed-tall; the oracle needs minutes for it)."""
    import json
    import os
    from pathlib import Path
    path = os.path.join(os.path.dirname(__file__), "golden", "oracle_pins_headline.json")
    p = json.loads(Path(path).read_text()).get("mixed2048x2440")
    if p is None:
        pytest.skip("no mixed 2048x2440 pin")
    assert lib.load().tea_gb300_reduction_rows(2048, 2440) == 16
    steps = lib.run_deck(p["deck"])
    assert [s.iterations for s in steps] == p["iterations"]
    assert [s.outer_corrections for s in steps] == p["outer_corrections"]
    assert [float(s.relative_residual).hex() for s in steps] == p["relative_residual_hex"]
    last = steps[-1]
    got = dict(vol=last.vol, mass=last.mass, ie=last.ie, temp=last.temp)
    assert {k: float(v).hex() for k, v in got.items()} == p["summary_hex"]


def test_mixed_answer_agrees_with_fp64():
    """Both solves stop at a true relative residual of 1e-10."""
    cells = 512
    fp64 = lib.run_deck(decks.five_state_deck(
        cells, solver="cg", prec="jac_diag", steps=4, eps=1e-10, max_iters=20000,
        extra="tl_exit_true_residual"), mode=lib.DRIVER_RESIDENT)
    mixed = lib.run_deck(mixed_deck(cells, steps=4))
    a, b = fp64[-1], mixed[-1]
    for k in ("mass", "ie", "temp"):
        assert abs(getattr(a, k) - getattr(b, k)) <= 1e-8 * abs(getattr(a, k)), k
    assert all(s.relative_residual <= 1e-10 for s in mixed)


def test_true_residual_exit_reaches_target():
    cells = 256
    deck = decks.five_state_deck(cells, solver="cg", prec="jac_diag", steps=2, eps=1e-10,
                                 max_iters=20000, check_result=True,
                                 extra="tl_exit_true_residual")
    steps = lib.run_deck(deck, mode=lib.DRIVER_RESIDENT)
    plain = lib.run_deck(deck.replace("tl_exit_true_residual\n", ""),
                         mode=lib.DRIVER_RESIDENT)
    for s, p in zip(steps, plain):
        assert s.exact_error < 1.1e-10          # recurrence vs recomputed residual
        assert s.iterations >= p.iterations     # a stricter test on this problem


@pytest.mark.parametrize("cells,y_cells,inner,inner_steps,presteps",
                         [(130, 129, 1e-5, 10, 25), (200, 97, 1e-4, 6, 12)])
def test_mixed_ppcg_matches_oracle(cells, y_cells, inner, inner_steps, presteps):
    """FP32 PPCG inner solver: CG presteps, eigenvalue range, Chebyshev
    inner steps; bit for bit against the oracle's restatement."""
    deck = mixed_deck(cells, y_cells=y_cells, inner=inner, solver="ppcg",
                      inner_steps=inner_steps, presteps=presteps)
    steps = lib.run_deck(deck)
    res = oracle.run_deck(deck)
    n = res.n_steps
    assert [s.iterations for s in steps] == list(res.iterations[:n])
    assert [s.inner_iterations for s in steps] == list(res.inner_iterations[:n])
    assert all(s.inner_iterations > 0 for s in steps)  # the PPCG phase ran
    assert [s.outer_corrections for s in steps] == list(res.outer_corrections[:n])
    assert [s.relative_residual for s in steps] == list(res.relative_residual[:n])
    final = res.summaries()[-1]
    last = steps[-1]
    assert (last.vol, last.mass, last.ie, last.temp) == tuple(final[[1, 2, 4, 5]])
    assert all(s.relative_residual <= 1e-10 for s in steps)
