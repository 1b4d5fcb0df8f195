"""tea.in deck text for the benchmark and test workloads.

The five-state layout is the one of the reference's own decks (tea.in,
tea_bm*.in): a density-100 background, a density-0.1 source block at
x in [0,1], y in [1,2] with energy 25, and three density-0.1 channels of
energy 0.1, on the domain [0,10]^2.
"""

FIVE_STATES = """state 1 density=100.0 energy=0.0001
state 2 density=0.1 energy=25.0 geometry=rectangle xmin=0.0 xmax=1.0 ymin=1.0 ymax=2.0
state 3 density=0.1 energy=0.1 geometry=rectangle xmin=1.0 xmax=6.0 ymin=1.0 ymax=2.0
state 4 density=0.1 energy=0.1 geometry=rectangle xmin=5.0 xmax=6.0 ymin=1.0 ymax=8.0
state 5 density=0.1 energy=0.1 geometry=rectangle xmin=5.0 xmax=10.0 ymin=7.0 ymax=8.0
"""


def five_state_deck(cells, solver="cg", prec="none", steps=10, eps=1e-15,
                    max_iters=5000, halo=1, dt=0.004, inner_steps=None,
                    presteps=None, summary_frequency=10, extra="", y_cells=None,
                    test_problem=None, check_result=False, reflective=False,
                    coefficient=None):
    y = cells if y_cells is None else y_cells
    lines = ["*tea", FIVE_STATES.rstrip("\n"),
             "x_cells=%d" % cells, "y_cells=%d" % y,
             "xmin=0.0", "ymin=0.0", "xmax=10.0", "ymax=10.0",
             "initial_timestep=%r" % dt, "end_step=%d" % steps,
             "tl_max_iters=%d" % max_iters, "tl_use_%s" % solver,
             "tl_eps=%r" % eps, "halo_depth=%d" % halo,
             "summary_frequency=%d" % summary_frequency]
    if prec != "none":
        lines.append("tl_preconditioner_type=%s" % prec)
    if inner_steps is not None:
        lines.append("tl_ppcg_inner_steps=%d" % inner_steps)
    if presteps is not None:
        lines.append("tl_ch_cg_presteps=%d" % presteps)
    if test_problem is not None:
        lines.append("test_problem %d" % test_problem)
    if check_result:
        lines.append("tl_check_result")
    if reflective:
        lines.append("reflective_boundary")
    if coefficient == "inverse":
        lines.append("tl_coefficient_inverse_density")
    if extra:
        lines.append(extra.rstrip("\n"))
    lines.append("*endtea")
    return "\n".join(lines) + "\n"
