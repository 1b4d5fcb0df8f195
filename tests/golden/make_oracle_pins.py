"""Records the CPU oracle's results for runs too long for the CPU test suite.

Test problems.  tests/test_gpu_runs.py compares the GPU runs of test
problems 2 and 3 (960^2 and 3840^2 CG, tens of thousands of iterations)
with these records bit for bit: per-step iteration counts and the final
temperature (as a hex float).  The oracle takes minutes to hours on a CPU
for these, so the results are kept as a fixture: oracle_pins.json for the
exact arithmetic form, oracle_pins_fused.json and oracle_pins_chain.json
for the others.

    make_oracle_pins.py [--fused | --chain] TP [TP ...]

Benchmark workloads.  tests/test_gpu_headline.py runs the benchmark's own
4096^2 decks (bench.py's deck_for: five states, block Jacobi, halo depth 2,
20 CG steps before the switch, tl_eps 1e-15) for two timesteps, each ended
CAP iterations after its switch from CG to PPCG or Chebyshev, and compares
them with these records bit for bit.  The deck text is stored with the
record, so the pin says exactly what it pins.

    make_oracle_pins.py --workload ppcg4096|cheby4096 [--exact|--chain] [--cap N]

Largest grid.  tests/test_gpu_large.py runs the same PPCG deck at 8192^2
(the grid of the mixed-precision configuration) for one timestep, ended
LARGE_CAP iterations after its switch from CG, against these records.

    make_oracle_pins.py --large 8192 [--exact|--chain]

Mixed precision with 16-row reduction tiles.  tests/test_gpu_mixed.py runs
the FP32-inner / FP64-corrected CG solve at 2048x2440 (the smallest grid
with 16-row tiles) for one timestep to a 1e-8 relative residual against
this record.

    make_oracle_pins.py --mixed-tall
"""
import json
import os
import sys
import time
from pathlib import Path

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402

HEADLINE_FILE = os.path.join(HERE, "oracle_pins_headline.json")
HEADLINE_STEPS = 2
HEADLINE_CAP = 20
LARGE_CAP = 5


def headline_deck(workload, form, steps=HEADLINE_STEPS):
    """The deck bench.py times for `workload`, in arithmetic form `form`."""
    import bench
    saved = bench.ARITHMETIC
    try:
        bench.ARITHMETIC = form
        return bench.deck_for(workload, steps)
    finally:
        bench.ARITHMETIC = saved


def large_deck(cells, form):
    """bench.py's ppcg4096 deck (five states, PPCG, block Jacobi, halo depth
    2, 10 inner steps, 20 CG steps before the switch, tl_eps 1e-15,
    tl_max_iters 1000) at cells^2, one timestep."""
    from tealeaf_opencl_gb300 import decks
    return decks.five_state_deck(cells, solver="ppcg", prec="jac_block", steps=1,
                                 eps=1e-15, max_iters=1000, halo=2, inner_steps=10,
                                 presteps=20, summary_frequency=0,
                                 extra="tl_arithmetic %s" % form)


def mixed_tall_deck():
    """Mixed precision (FP32 inner CG, diagonal Jacobi) at 2048x2440, one
    timestep to 1e-8, inner tolerance 1e-4."""
    from tealeaf_opencl_gb300 import decks
    return decks.five_state_deck(2048, solver="cg", prec="jac_diag", steps=1, eps=1e-8,
                                 max_iters=20000, y_cells=2440,
                                 extra="tl_mixed_precision\ntl_mixed_inner_eps 1e-4\n")


def pin_mixed_tall():
    pins = json.loads(Path(HEADLINE_FILE).read_text()) if os.path.exists(HEADLINE_FILE) else {}
    deck = mixed_tall_deck()
    t0 = time.time()
    res = oracle.run_deck(deck)
    n = res.n_steps
    final = res.summaries()[-1]
    pins["mixed2048x2440"] = {
        "deck": deck,
        "iterations": list(res.iterations[:n]),
        "outer_corrections": list(res.outer_corrections[:n]),
        "relative_residual_hex": [float(v).hex() for v in res.relative_residual[:n]],
        "summary_hex": {k: float(final[i]).hex()
                        for k, i in (("vol", 1), ("mass", 2), ("ie", 4), ("temp", 5))},
        "oracle_threads": oracle.lib().oracle_num_threads(),
        "oracle_seconds": round(time.time() - t0, 1),
    }
    Path(HEADLINE_FILE).write_text(json.dumps(pins, indent=1, sort_keys=True))
    print("mixed2048x2440", list(res.iterations[:n]), list(res.outer_corrections[:n]),
          list(res.relative_residual[:n]), flush=True)


def pin_headline(workload, form, cap, deck=None):
    pins = json.loads(Path(HEADLINE_FILE).read_text()) if os.path.exists(HEADLINE_FILE) else {}
    deck = deck or headline_deck(workload, form)
    t0 = time.time()
    res = oracle.run_deck(deck, max_after_switch=cap)
    n = res.n_steps
    final = res.summaries()[-1]
    pins["%s/%s" % (workload, form)] = {
        "workload": workload,
        "arithmetic": form,
        "deck": deck,
        "cap_after_switch": cap,
        "iterations": list(res.iterations[:n]),
        "inner_iterations": list(res.inner_iterations[:n]),
        "switch_iteration": list(res.switch_iteration[:n]),
        "summary_hex": {k: float(final[i]).hex()
                        for k, i in (("vol", 1), ("mass", 2), ("ie", 4), ("temp", 5))},
        "oracle_threads": oracle.lib().oracle_num_threads(),
        "oracle_seconds": round(time.time() - t0, 1),
    }
    Path(HEADLINE_FILE).write_text(json.dumps(pins, indent=1, sort_keys=True))
    print(workload, form, list(res.iterations[:n]), list(res.switch_iteration[:n]),
          final[5], flush=True)


def main(tps, form):
    path = os.path.join(HERE, "oracle_pins.json" if form == "exact"
                        else "oracle_pins_%s.json" % form)
    pins = json.loads(Path(path).read_text()) if os.path.exists(path) else {}
    meta = json.loads(Path(os.path.join(HERE, "test_problems.json")).read_text())
    for tp in tps:
        p = meta["problems"][str(tp)]
        deck = Path(os.path.join(HERE, p["deck"])).read_text()
        deck = deck.replace("*endtea", "tl_arithmetic %s\n*endtea" % form, 1)
        t0 = time.time()
        res = oracle.run_deck(deck)
        pins[str(tp)] = {
            "deck": p["deck"],
            "arithmetic": form,
            "temp": res.final_temp,
            "temp_hex": float(res.final_temp).hex(),
            "golden_temp": p["temp"],
            "qa_diff_percent": res.qa_diff,
            "iterations": list(res.iterations[:res.n_steps]),
            "oracle_threads": oracle.lib().oracle_num_threads(),
            "oracle_seconds": round(time.time() - t0, 1),
        }
        Path(path).write_text(json.dumps(pins, indent=1, sort_keys=True))
        print(tp, res.final_temp, res.qa_diff, flush=True)


if __name__ == "__main__":
    args = sys.argv[1:]
    form = "fused" if "--fused" in args else "chain" if "--chain" in args else "exact"
    if "--mixed-tall" in args:
        pin_mixed_tall()
    elif "--large" in args:
        cells = int(args[args.index("--large") + 1])
        pin_headline("ppcg%d" % cells, form, LARGE_CAP, large_deck(cells, form))
    elif "--workload" in args:
        wl = args[args.index("--workload") + 1]
        cap = int(args[args.index("--cap") + 1]) if "--cap" in args else HEADLINE_CAP
        pin_headline(wl, form, cap)
    else:
        main([int(a) for a in args if not a.startswith("--")] or [2], form)
