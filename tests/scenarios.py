"""Call sequences run identically on the oracle chunk and the GPU chunk.

Each scenario drives the reference's entry points in the order its Fortran
driver uses them and records every returned scalar and selected fields, so
that two backends can be compared record by record.
"""
import numpy as np

FIVE = dict(density=[100.0, 0.1, 0.1, 0.1, 0.1],
            energy=[1e-4, 25.0, 0.1, 0.1, 0.1],
            xmin=[0.0, 0.0, 1.0, 5.0, 5.0], xmax=[0.0, 1.0, 6.0, 6.0, 10.0],
            ymin=[0.0, 1.0, 1.0, 1.0, 7.0], ymax=[0.0, 2.0, 2.0, 8.0, 8.0],
            radius=[0.0] * 5, geometry=[0, 1, 1, 1, 1])
# circle and point geometries as well
SHAPES = dict(density=[10.0, 0.5, 2.0, 0.2], energy=[1.0, 3.0, 0.5, 9.0],
              xmin=[0.0, 2.5, 6.0, 4.0], xmax=[0.0, 7.0, 0.0, 0.0],
              ymin=[0.0, 2.5, 6.0, 4.0], ymax=[0.0, 4.0, 0.0, 0.0],
              radius=[0.0, 0.0, 2.2, 0.0], geometry=[0, 1, 2, 3])

FIELDS = ["u", "u0", "r", "p", "w", "z", "sd", "energy1", "density", "Kx", "Ky"]


def shrink(states, x_cells, y_cells, width=10.0):
    """read_input.f90:314-327: state boxes shrunk by a hundredth of a cell."""
    s = {k: list(v) for k, v in states.items()}
    dx, dy = width / x_cells, width / y_cells
    for n in range(1, len(s["density"])):
        s["xmin"][n] += dx / 100.0
        s["ymin"][n] += dy / 100.0
        s["xmax"][n] -= dx / 100.0
        s["ymax"][n] -= dy / 100.0
    return s


def setup(ch, x, y, states=FIVE, lognormal_seed=None, reflective=False, halo=1):
    dx, dy = 10.0 / x, 10.0 / y
    ch.initialise_chunk(0.0, 0.0, dx, dy)
    s = shrink(states, x, y)
    ch.generate_chunk(s["density"], s["energy"], s["xmin"], s["xmax"], s["ymin"],
                      s["ymax"], s["radius"], s["geometry"])
    if lognormal_seed is not None:
        rng = np.random.default_rng(lognormal_seed)
        d = ch.read("density") * np.exp(0.5 * rng.standard_normal((y, x)))
        ch.write("density", d)
    if reflective:
        ch.update_halo([1, 1, 1, 0, 0, 0, 0], halo)
    ch.set_field()


def ch_coefs(eigmin, eigmax, n):
    """tea_calc_ch_coefs with fixed eigenvalue bounds."""
    theta = (eigmax + eigmin) / 2
    delta = (eigmax - eigmin) / 2
    sigma = theta / delta
    rho_old = 1.0 / sigma
    a, b = [], []
    for _ in range(n):
        rho_new = 1.0 / (2.0 * sigma - rho_old)
        a.append(rho_new * rho_old)
        b.append(2.0 * rho_new / delta)
        rho_old = rho_new
    return np.array(a), np.array(b), theta


def run(ch, x, y, solver, prec, halo=1, reflective=False, coef=1, cg_iters=6,
        cheby_iters=4, inner=5, jacobi_iters=4, dt=0.004, lognormal_seed=None,
        states=FIVE, snapshots=True, fused=True):
    rec = []
    ch.set_arithmetic(fused)

    def snap(tag):
        if snapshots:
            for f in FIELDS:
                rec.append((tag + ":" + f, ch.read(f)))

    setup(ch, x, y, states, lognormal_seed, reflective, halo)
    rec.append(("summary0", np.array(ch.field_summary())))
    rx, ry = ch.common_init(coef, dt, (1, 1, 1, 1), 1 if reflective else 0)
    rec.append(("rxry", np.array([rx, ry])))
    rec.append(("Kx_padded", ch.read_padded("Kx")))
    rec.append(("Ky_padded", ch.read_padded("Ky")))
    ch.calc_residual()
    rec.append(("r0", np.array([ch.calc_2norm(1)])))
    rec.append(("bb", np.array([ch.calc_2norm(0)])))
    if solver == "jacobi":
        for _ in range(jacobi_iters):
            rec.append(("jac_err", np.array([ch.jacobi_solve()])))
        snap("jacobi")
    else:
        rro = ch.cg_init()
        rec.append(("rro", np.array([rro])))
        snap("cg_init")
        for _ in range(cg_iters):
            pw = ch.cg_calc_w()
            alpha = rro / pw
            rrn = ch.cg_calc_ur(alpha)
            beta = rrn / rro
            ch.cg_calc_p(beta)
            rec.append(("cg", np.array([pw, rrn])))
            rro = rrn
        snap("cg")
        if solver == "chebyshev":
            a, b, theta = ch_coefs(0.9, 40.0, cheby_iters + 4)
            ch.cheby_init(a, b, theta)
            for s in range(1, cheby_iters + 1):
                ch.cheby_iterate(s)
            rec.append(("cheby_rr", np.array([ch.calc_2norm(1)])))
            snap("cheby")
        elif solver == "ppcg":
            a, b, theta = ch_coefs(0.9, 40.0, inner)
            ch.ppcg_init(a, b, theta)
            pw = ch.cg_calc_w()
            alpha = rro / pw
            ch.cg_calc_ur(alpha)
            ch.ppcg_init_sd()
            for s in range(1, inner + 1):
                ch.ppcg_inner(s)
            rrn = ch.calc_2norm(2)
            ch.cg_calc_p(rrn / rro)
            rec.append(("ppcg", np.array([pw, rrn])))
            snap("ppcg")
    ch.finalise()
    if reflective:
        ch.update_halo([0, 0, 1, 0, 0, 0, 0], 1)
    rec.append(("summary1", np.array(ch.field_summary())))
    snap("final")
    if reflective:
        rec.append(("energy1_padded", ch.read_padded("energy1")))
        rec.append(("density_padded", ch.read_padded("density")))
    return rec


def compare(rec_a, rec_b):
    """Return the names of records that differ bit-for-bit."""
    assert [k for k, _ in rec_a] == [k for k, _ in rec_b]
    bad = []
    for (k, a), (_, b) in zip(rec_a, rec_b):
        if a.shape != b.shape or not np.array_equal(a.view(np.int64), b.view(np.int64)):
            bad.append(k)
    return bad
