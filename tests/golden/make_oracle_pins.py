"""Records the CPU oracle's results for the long CG test problems.

tests/test_gpu_runs.py compares the GPU runs of test problems 2 and 3
(960^2 and 3840^2 CG, tens of thousands of iterations) with these records
bit for bit: per-step iteration counts and the final temperature (as a hex
float).  The oracle takes minutes to hours on a CPU for these, so the
results are kept as a fixture: oracle_pins.json for the exact arithmetic
form, oracle_pins_fused.json and oracle_pins_chain.json for the others.
Usage: make_oracle_pins.py [--fused | --chain] TP [TP ...]
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle  # noqa: E402


def main(tps, form):
    path = os.path.join(HERE, "oracle_pins.json" if form == "exact"
                        else "oracle_pins_%s.json" % form)
    pins = json.load(open(path)) if os.path.exists(path) else {}
    meta = json.load(open(os.path.join(HERE, "test_problems.json")))
    for tp in tps:
        p = meta["problems"][str(tp)]
        deck = open(os.path.join(HERE, p["deck"])).read()
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
        json.dump(pins, open(path, "w"), indent=1, sort_keys=True)
        print(tp, res.final_temp, res.qa_diff, flush=True)


if __name__ == "__main__":
    args = sys.argv[1:]
    form = "fused" if "--fused" in args else "chain" if "--chain" in args else "exact"
    main([int(a) for a in args if not a.startswith("--")] or [2], form)
