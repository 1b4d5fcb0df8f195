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


FIVE_STATE_TABLE = dict(density=[100.0, 0.1, 0.1, 0.1, 0.1],
                        energy=[1e-4, 25.0, 0.1, 0.1, 0.1],
                        xmin=[0.0, 0.0, 1.0, 5.0, 5.0], xmax=[0.0, 1.0, 6.0, 6.0, 10.0],
                        ymin=[0.0, 1.0, 1.0, 1.0, 7.0], ymax=[0.0, 2.0, 2.0, 8.0, 8.0],
                        radius=[0.0] * 5, geometry=[0, 1, 1, 1, 1])


def setup_five_state(chunk, x_cells, y_cells=None, width=10.0):
    """Set up the five-state problem on a chunk through the C-ABI entry
    points, as start.f90 does: mesh, states (boxes shrunk by a hundredth of
    a cell, read_input.f90:314-327), energy1 = energy0."""
    y_cells = x_cells if y_cells is None else y_cells
    dx, dy = width / x_cells, width / y_cells
    s = {k: list(v) for k, v in FIVE_STATE_TABLE.items()}
    for n in range(1, 5):
        s["xmin"][n] += dx / 100.0
        s["ymin"][n] += dy / 100.0
        s["xmax"][n] -= dx / 100.0
        s["ymax"][n] -= dy / 100.0
    chunk.initialise_chunk(0.0, 0.0, dx, dy)
    chunk.generate_chunk(s["density"], s["energy"], s["xmin"], s["xmax"], s["ymin"],
                         s["ymax"], s["radius"], s["geometry"])
    chunk.set_field()


def chebyshev_coefficients(eigmin, eigmax, n):
    """tea_calc_ch_coefs (tea_leaf_cheby.f90:145-172)."""
    theta = (eigmax + eigmin) / 2
    delta = (eigmax - eigmin) / 2
    sigma = theta / delta
    rho_old = 1.0 / sigma
    alphas, betas = [], []
    for _ in range(n):
        rho_new = 1.0 / (2.0 * sigma - rho_old)
        alphas.append(rho_new * rho_old)
        betas.append(2.0 * rho_new / delta)
        rho_old = rho_new
    return alphas, betas, theta


# ---------------------------------------------------------------------------
# batched workloads: many independent problems of uneven size
# ---------------------------------------------------------------------------

BATCH_BACKGROUND = dict(density=100.0, energy=1e-4)


def batch_problems(n, seed=0, side=(64, 1024), rects=(2, 6), extent=10.0):
    """n seeded random problems on [0,extent]^2: x and y cell counts drawn
    uniformly from `side`, each with 2-6 axis-aligned rectangles of density
    log-uniform in [0.05, 200] and energy uniform in [1e-4, 25] painted over
    the density-100, energy-1e-4 background."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        x = int(rng.integers(side[0], side[1] + 1))
        y = int(rng.integers(side[0], side[1] + 1))
        k = int(rng.integers(rects[0], rects[1] + 1))
        states = []
        for _ in range(k):
            x0, x1 = sorted(float(v) for v in rng.uniform(0.0, extent, 2))
            y0, y1 = sorted(float(v) for v in rng.uniform(0.0, extent, 2))
            dens = float(np.exp(rng.uniform(np.log(0.05), np.log(200.0))))
            en = float(rng.uniform(1e-4, 25.0))
            states.append(dict(density=dens, energy=en, xmin=x0, xmax=x1, ymin=y0, ymax=y1))
        out.append(dict(x=x, y=y, states=states))
    return out


def batch_deck(problem, steps=5, eps=1e-12, max_iters=5000, prec="jac_diag",
               dt=0.004, arithmetic=None, extent=10.0):
    """tea.in deck of one batched problem for a single-chunk CG run."""
    lines = ["*tea", "state 1 density=%r energy=%r" % (BATCH_BACKGROUND["density"],
                                                       BATCH_BACKGROUND["energy"])]
    for k, s in enumerate(problem["states"]):
        lines.append("state %d density=%r energy=%r geometry=rectangle xmin=%r xmax=%r "
                     "ymin=%r ymax=%r" % (k + 2, s["density"], s["energy"], s["xmin"],
                                          s["xmax"], s["ymin"], s["ymax"]))
    lines += ["x_cells=%d" % problem["x"], "y_cells=%d" % problem["y"],
              "xmin=0.0", "ymin=0.0", "xmax=%r" % extent, "ymax=%r" % extent,
              "initial_timestep=%r" % dt, "end_step=%d" % steps,
              "tl_max_iters=%d" % max_iters, "tl_use_cg", "tl_eps=%r" % eps,
              "halo_depth=1", "summary_frequency=0"]
    if prec != "none":
        lines.append("tl_preconditioner_type=%s" % prec)
    if arithmetic:
        lines.append("tl_arithmetic %s" % arithmetic)
    lines.append("*endtea")
    return "\n".join(lines) + "\n"


def paint(problem, extent=10.0):
    """(density, energy) arrays (y, x) of a batched problem: a cell takes
    the last state whose rectangle holds its centre."""
    import numpy as np
    x, y = problem["x"], problem["y"]
    xc = (np.arange(x) + 0.5) * (extent / x)
    yc = (np.arange(y) + 0.5) * (extent / y)
    dens = np.full((y, x), BATCH_BACKGROUND["density"])
    en = np.full((y, x), BATCH_BACKGROUND["energy"])
    for s in problem["states"]:
        mx = (xc >= s["xmin"]) & (xc < s["xmax"])
        my = (yc >= s["ymin"]) & (yc < s["ymax"])
        m = my[:, None] & mx[None, :]
        dens[m] = s["density"]
        en[m] = s["energy"]
    return dens, en
