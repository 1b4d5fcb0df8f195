"""The driver's text outputs in the reference's formats.

tea.out (tea_gb300_driver_open's log): the field summary block of
field_summary.f90:40-45 and :79-81 -- a header '(a13,5a26)' and the values
'(a6,i7,5e26.17)', where Fortran's E editing prints 0.d1...d17E+ee --, the
test-problem lines of :97-104, and the solver lines of tea_solve.f90:202-203
and :356-370.  17 significant digits identify a double, so the logged
values must read back as the step's own field summary, bit for bit.

The profiling report (print_opencl_profiling_info_, ocl_errors.cpp:196-232):
one row per launched kernel, '%30s : %10.3f ms (%.2f us avg. over %d
calls)', with nonzero totals.
"""
import json
import os
import re
from pathlib import Path

import pytest

from tealeaf_opencl_gb300 import decks, lib

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")

E26 = r"(?: {3}0\.\d{17}E[+-]\d{2}| {2}-0\.\d{17}E[+-]\d{2})"
STEP_LINE = re.compile(r"^ step:[ \d]{7}(%s)(%s)(%s)(%s)(%s)$" % ((E26,) * 5))
HEADER = "%13s%26s%26s%26s%26s%26s" % ("", "Volume", "Mass", "Density", "Energy", "U")


def fortran_float(s):
    return float(s.strip())


def test_problem_1_log_has_the_reference_layout(tmp_path):
    meta = json.loads(Path(os.path.join(GOLD, "test_problems.json")).read_text())
    deck = Path(os.path.join(GOLD, meta["problems"]["1"]["deck"])).read_text()
    log = str(tmp_path / "tea.out")
    steps = lib.run_deck(deck, log_path=log)
    text = Path(log).read_text().splitlines()
    # the first summary (start.f90) and the last (diffuse.f90's final call)
    step_lines = [ln for ln in text if ln.startswith(" step:")]
    assert len(step_lines) >= 2
    assert sum(1 for ln in text if ln == HEADER) == len(step_lines)
    for ln in step_lines:
        assert STEP_LINE.match(ln), repr(ln)
    m = STEP_LINE.match(step_lines[-1])
    vol, mass, dens, ie, temp = (fortran_float(g) for g in m.groups())
    last = steps[-1]
    assert (vol, mass, ie, temp) == (last.vol, last.mass, last.ie, last.temp)
    assert dens == last.mass / last.vol
    assert int(step_lines[-1][6:13]) == last.step
    qa = [ln for ln in text if ln.startswith("Test problem")]
    assert len(qa) == 1
    assert re.match(r"^Test problem   1 is within {3}0\.\d{7}E[+-]\d{2}% of the expected "
                    r"solution$", qa[0]), repr(qa[0])
    # e16.7 keeps 7 significant digits
    assert abs(fortran_float(qa[0][26:42]) - last.qa_diff) <= 5e-7 * last.qa_diff
    assert " This test is considered PASSED" in text
    its = [int(ln[16:]) for ln in text if ln.startswith("Iteration count ")]
    assert its == [s.iterations - 1 for s in steps] or its == [s.iterations for s in steps]
    for ln in text:
        if ln.startswith("Conduction error "):
            # e14.7: 13 characters for a positive value, one blank before it
            assert re.match(r"^Conduction error (?: 0\.\d{7}E[+-]\d{2}|-0\.\d{7}E[+-]\d{2})$",
                            ln), repr(ln)


def test_ppcg_log_reports_the_switch_in_the_reference_layout(tmp_path):
    deck = decks.five_state_deck(64, solver="ppcg", prec="jac_block", steps=2, eps=1e-12,
                                 halo=2, inner_steps=8, presteps=20)
    log = str(tmp_path / "tea.out")
    steps = lib.run_deck(deck, log_path=log)
    text = Path(log).read_text().splitlines()
    sw = [ln for ln in text if ln.startswith("Switching after")]
    assert len(sw) == 2
    # '(a,i3,a,e15.7)': "Switching after ", i3, " CG its, error ", e15.7
    # (13 characters for a positive value, two blanks before it)
    m = re.match(r"^Switching after ([ \d]{3}) CG its, error ( {2}0\.\d{7}E[+-]\d{2})$", sw[0])
    assert m, repr(sw[0])
    assert int(m.group(1)) == steps[0].switch_iteration
    eig = [ln for ln in text if ln.startswith("Eigen min")]
    e14 = r"(?: {2}0\.\d{6}E[+-]\d{2}| -0\.\d{6}E[+-]\d{2})"
    assert re.match(r"^Eigen min%s Eigen max%s Condition number[ \d.]{14} Error%s$"
                    % (e14, e14, e14), eig[0]), repr(eig[0])
    tot = [ln for ln in text if ln.startswith("PPCG Iteration count")]
    for ln, s in zip(tot, steps):
        # FORMAT 103: 'PPCG Iteration count', i8, ' (Total ', i8, ')'
        m = re.match(r"^PPCG Iteration count([ \d]{8}) \(Total ([ \d]{8})\)$", ln)
        assert m, repr(ln)
        assert int(m.group(1)) == s.inner_iterations


def test_profiling_report_has_one_row_per_launched_kernel(capfd):
    n = 64
    ch = lib.Chunk(n, n, 1, "cg", "jac_diag", profiler=True)
    decks.setup_five_state(ch, n)
    ch.common_init(1, 0.004)
    ch.calc_residual()
    rro = ch.cg_init()
    for _ in range(3):
        pw = ch.cg_calc_w()
        rrn = ch.cg_calc_ur(rro / pw)
        ch.cg_calc_p(rrn / rro)
        rro = rrn
    ch.finalise()
    ch.field_summary()
    capfd.readouterr()
    lib.load().print_opencl_profiling_info_()
    out = capfd.readouterr().out.splitlines()
    assert out[0] == "@@@@@ CUDA Profiling information @@@@@"
    row = re.compile(r"^ *(\S+) : +(\d+\.\d{3}) ms \((\d+\.\d{2}) μs avg\. over (\d+) calls\)$")
    rows = {}
    for ln in out[1:]:
        m = row.match(ln)
        assert m, repr(ln)
        assert len(ln.split(" : ")[0]) == 30
        rows[m.group(1)] = (float(m.group(2)), int(m.group(4)))
    for name, calls in (("tea_leaf_cg_solve_calc_w", 3), ("tea_leaf_cg_solve_calc_ur", 3),
                        ("tea_leaf_cg_solve_calc_p", 3), ("tea_leaf_finalise", 1),
                        ("field_summary", 1), ("tea_leaf_calc_residual", 1)):
        assert name in rows, name
        ms, n_calls = rows[name]
        assert n_calls >= calls and ms > 0.0, (name, rows[name])
    lib.load().tea_gb300_finalise()
