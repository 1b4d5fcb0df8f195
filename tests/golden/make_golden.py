"""Regenerates the golden fixtures in tests/golden/ from the reference tree.

Run where the reference tree is available; its location is the one
required argument:

    python tests/golden/make_golden.py <path of the reference tree>

It copies the reference's input decks,
writes the built-in test-problem-1 deck that initialise.f90:67-92 generates
when tea.in is missing, and extracts the known-answer temperatures of
field_summary.f90:88-106.  Nothing at test time reads the reference.
"""
import json
import os
import re
import sys
from pathlib import Path

REF = None  # the reference tree, from the command line
HERE = os.path.dirname(os.path.abspath(__file__))

DECKS = {2: "tea_bm_short.in", 3: "tea_bm16_short.in", 4: "tea_bm.in",
         5: "tea_bm16.in", 6: "tea.in"}


def default_deck():
    """The deck initialise.f90 writes when no tea.in exists (test problem 1)."""
    src = Path(os.path.join(REF, "initialise.f90")).read_text()
    lines = re.findall(r"WRITE\(out_unit,'\(A\)'\)'(.*)'", src)
    return "\n".join(lines) + "\n"


def goldens():
    src = Path(os.path.join(REF, "field_summary.f90")).read_text()
    out = {}
    for tp, val in re.findall(
            r"IF\(test_problem\.EQ\.(\d)\) qa_diff=ABS\(\(100\.0_8\*\(temp/([0-9.]+)_8\)\)", src):
        out[int(tp)] = float(val)
    return out


def main():
    g = goldens()
    meta = {"source": "field_summary.f90:88-106 (temp known answers), "
                      "initialise.f90:67-92 (test problem 1 deck)",
            "criterion_percent": 0.001, "problems": {}}
    with open(os.path.join(HERE, "tp1.in"), "w") as f:
        f.write(default_deck())
    meta["problems"]["1"] = {"deck": "tp1.in", "temp": g[1]}
    for tp, name in DECKS.items():
        text = Path(os.path.join(REF, name)).read_text()
        out = "tp%d.in" % tp
        with open(os.path.join(HERE, out), "w") as f:
            f.write(text)
        meta["problems"][str(tp)] = {"deck": out, "temp": g[tp], "reference_file": name}
    with open(os.path.join(HERE, "test_problems.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print(json.dumps(meta, indent=1, sort_keys=True))


if __name__ == "__main__":
    if len(sys.argv) != 2 or not os.path.isdir(sys.argv[1]):
        sys.exit("usage: make_golden.py <path of the reference tree>")
    REF = sys.argv[1]
    main()
