"""Bit-exact parity of every C-ABI entry point with the CPU oracle.

The same call sequence (the Fortran driver's order) runs on the GPU chunk
and on the oracle chunk; every returned scalar and every field snapshot must
agree bit for bit.  Both sides evaluate each cell's expression in the
reference's operation order without fused multiply-adds and sum in the same
fixed order, so equality is exact, not approximate.
"""
import numpy as np
import pytest

from oracle import oracle
from tests import scenarios

pytestmark = pytest.mark.gpu


def pair(x, y, H, solver, prec, **kw):
    from tealeaf_opencl_gb300 import lib
    sol = {"jacobi": 1, "cg": 2, "chebyshev": 3, "ppcg": 4}[solver]
    pr = {"none": 1, "jac_diag": 2, "jac_block": 3}[prec]
    g = lib.Chunk(x, y, H, sol, pr)
    rec_g = scenarios.run(g, x, y, solver, prec, halo=H, **kw)
    o = oracle.Chunk(x, y, H, sol, pr)
    rec_o = scenarios.run(o, x, y, solver, prec, halo=H, **kw)
    return rec_g, rec_o


CASES = [
    # (x, y, halo, solver, prec, extra)
    (37, 29, 1, "cg", "none", {}),
    (37, 29, 1, "cg", "jac_diag", {}),
    (37, 29, 1, "cg", "jac_block", {}),
    (64, 61, 2, "cg", "jac_block", {"lognormal_seed": 5}),
    (130, 129, 1, "chebyshev", "jac_diag", {}),
    (130, 129, 1, "chebyshev", "jac_block", {}),
    (67, 66, 2, "chebyshev", "none", {"coef": 2}),
    (96, 95, 1, "ppcg", "jac_diag", {}),
    (96, 95, 2, "ppcg", "jac_block", {"lognormal_seed": 11}),
    (300, 67, 3, "ppcg", "none", {}),
    (300, 67, 3, "cg", "jac_block", {}),
    (10, 10, 1, "jacobi", "none", {}),
    (45, 33, 2, "jacobi", "none", {"lognormal_seed": 2}),
    # one cell: A = I, r = 0 after the first residual, so no CG iteration is
    # defined (p.w = 0); the set-up, norms and summaries are still compared
    (1, 1, 1, "cg", "jac_diag", {"cg_iters": 0}),
    (3, 5, 2, "ppcg", "jac_block", {}),
    # odd width (a last single column in calc_sd's two-column walk) and, with
    # halo 1, a top strip of 3 interior rows that BLOCK_TOP counts as 4
    (97, 67, 1, "ppcg", "jac_block", {}),
    # Chebyshev with block Jacobi writes u to a second buffer, halo ring
    # included; halo depth 3 and a width and height that are not multiples
    # of the tiles
    (45, 37, 3, "chebyshev", "jac_block", {}),
    (33, 17, 1, "cg", "jac_block", {"reflective": True}),
    (33, 18, 2, "chebyshev", "jac_block", {"reflective": True}),
    (40, 23, 1, "jacobi", "none", {"reflective": True, "coef": 2}),
    (50, 41, 3, "ppcg", "jac_diag", {"reflective": True, "states": scenarios.SHAPES}),
    (257, 131, 1, "cg", "jac_diag", {"states": scenarios.SHAPES}),
]


@pytest.mark.parametrize("fused", [1, 0, 2], ids=["fused", "exact", "chain"])
@pytest.mark.parametrize("x,y,H,solver,prec,kw", CASES,
                         ids=["%dx%d-h%d-%s-%s%s" % (c[0], c[1], c[2], c[3], c[4],
                                                      "-" + "-".join(sorted(c[5])) if c[5] else "")
                              for c in CASES])
def test_entry_points_bit_exact(x, y, H, solver, prec, kw, fused):
    rec_g, rec_o = pair(x, y, H, solver, prec, fused=fused, **kw)
    bad = scenarios.compare(rec_g, rec_o)
    assert not bad, bad


@pytest.mark.parametrize("fused", [1, 0, 2], ids=["fused", "exact", "chain"])
def test_tall_tiles_bit_exact(fused):
    """A grid large enough for 16-row reduction tiles."""
    from tealeaf_opencl_gb300 import lib
    assert lib.load().tea_gb300_reduction_rows(2048, 2440) == 16
    rec_g, rec_o = pair(2048, 2440, 2, "ppcg", "jac_block", cg_iters=3, inner=3,
                        snapshots=False, lognormal_seed=1, fused=fused)
    bad = scenarios.compare(rec_g, rec_o)
    assert not bad, bad


def test_deterministic_run_to_run():
    from tealeaf_opencl_gb300 import lib
    recs = []
    for _ in range(2):
        g = lib.Chunk(130, 129, 1, 2, 2)
        recs.append(scenarios.run(g, 130, 129, "cg", "jac_diag", cg_iters=10))
    assert not scenarios.compare(*recs)


def test_poisoned_halo_leaves_interior_unchanged():
    """Finite garbage in the u/p halo meets zeroed boundary faces only."""
    from tealeaf_opencl_gb300 import lib
    x, y, H = 41, 37, 2
    outs = []
    for poison in (False, True):
        g = lib.Chunk(x, y, H, 2, 2)
        g.set_arithmetic(True)
        scenarios.setup(g, x, y)
        g.common_init(1, 0.004)
        if poison:
            rng = np.random.default_rng(0)
            for f in ("u", "p"):
                a = g.read_padded(f)
                mask = np.ones_like(a, dtype=bool)
                mask[H:H + y, H:H + x] = False
                a[mask] = rng.uniform(-1e6, 1e6, mask.sum())
                g.write_padded(f, a)
        g.calc_residual()
        rro = g.cg_init()
        for _ in range(5):
            pw = g.cg_calc_w()
            rrn = g.cg_calc_ur(rro / pw)
            g.cg_calc_p(rrn / rro)
            rro = rrn
        outs.append((g.read("u"), rro))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert outs[0][1] == outs[1][1]


def test_invalid_calls_report_errors():
    from tealeaf_opencl_gb300 import lib
    g = lib.Chunk(16, 16, 1, 2, 1)
    with pytest.raises(lib.TeaError):
        g.calc_2norm(7)
    g.neighbours[:] = [-1, 5, -1, -1]
    with pytest.raises(lib.TeaError):
        g.update_halo([1, 0, 0, 0, 0, 0, 0], 1)
    g.neighbours[:] = -1
    with pytest.raises(lib.TeaError):
        g.common_init(3, 0.004)
