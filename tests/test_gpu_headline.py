"""The benchmark's own 4096^2 configurations, pinned.

bench.py times PPCG (and, as a second workload, Chebyshev) at 4096^2 with
the block-Jacobi preconditioner, halo depth 2, 20 CG steps before the
switch and tl_eps 1e-15, in the chain arithmetic form: the 5-point
operator as one chain of fused multiply-adds, which re-associates the
reference's expression (tea_leaf_ppcg_cl.cl:77-83, tea_leaf_cheby_cl.cl).
Here the same decks run for two timesteps, each ended 20 iterations after
its switch from CG (the first step switches at CG iteration 361), and

  * each form matches the oracle's run of the same deck bit for bit
    (tests/golden/oracle_pins_headline.json, made by make_oracle_pins.py);
  * the chain form agrees with the exact one, the reference's own
    association, within the bar of the reference's plain FP64 path:
    field_summary within 1e-12 relative and iteration counts within +-1.
"""
import json
import os
from pathlib import Path

import pytest

from tealeaf_opencl_gb300 import lib

pytestmark = pytest.mark.gpu
PINS = os.path.join(os.path.dirname(__file__), "golden", "oracle_pins_headline.json")
REL_TOL = 1e-12  # field_summary, relative
ITER_TOL = 1     # iteration counts


def pin(workload, form):
    return json.loads(Path(PINS).read_text())["%s/%s" % (workload, form)]


def run(p, mode):
    return lib.run_deck(p["deck"], mode=mode, cap_after_switch=p["cap_after_switch"])


def summary(step):
    return dict(vol=step.vol, mass=step.mass, ie=step.ie, temp=step.temp)


def assert_matches_pin(steps, p):
    assert [s.iterations for s in steps] == p["iterations"]
    assert [s.inner_iterations for s in steps] == p["inner_iterations"]
    assert [s.switch_iteration for s in steps] == p["switch_iteration"]
    got = summary(steps[-1])
    assert {k: float(v).hex() for k, v in got.items()} == p["summary_hex"]


@pytest.mark.parametrize("workload", ["ppcg4096", "cheby4096"])
def test_headline_deck_matches_oracle_and_exact_form(workload):
    runs = {}
    for form in ("exact", "chain"):
        p = pin(workload, form)
        steps = run(p, lib.DRIVER_RESIDENT)  # the bench's mode
        assert all(s.switch_iteration > 0 for s in steps)
        assert_matches_pin(steps, p)
        runs[form] = steps
    print("%s switch iterations %s, iterations %s"
          % (workload, [s.switch_iteration for s in runs["chain"]],
             [s.iterations for s in runs["chain"]]))
    ex, ch = runs["exact"], runs["chain"]
    for a, b in zip(ex, ch):
        assert abs(a.iterations - b.iterations) <= ITER_TOL
        assert abs(a.inner_iterations - b.inner_iterations) <= ITER_TOL * 10
    se, sc = summary(ex[-1]), summary(ch[-1])
    for k in se:
        assert abs(se[k] - sc[k]) <= REL_TOL * abs(se[k]), (k, se[k], sc[k])


def test_headline_ppcg_per_call_matches_pin():
    """The per-call C ABI (bench.py's e2e path) gives the pinned bits too."""
    p = pin("ppcg4096", "chain")
    assert_matches_pin(run(p, lib.DRIVER_PER_CALL), p)


@pytest.mark.parametrize("form", ["exact", "chain"])
def test_headline_ppcg_with_fused_inner_pairs_matches_pin(form):
    """The TMA-fed pair of inner steps (tea_gb300_set_inner_pairs(1)) gives
    the pinned bits at the benchmark's own size, resident and per call."""
    L = lib.load()
    p = pin("ppcg4096", form)
    L.tea_gb300_set_inner_pairs(1)
    try:
        assert_matches_pin(run(p, lib.DRIVER_RESIDENT), p)
        assert_matches_pin(run(p, lib.DRIVER_PER_CALL), p)
    finally:
        L.tea_gb300_set_inner_pairs(0)
