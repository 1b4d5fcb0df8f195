"""Checks of the oracle's building blocks against independent restatements."""
import numpy as np
import pytest

from oracle import oracle
from tests import scenarios


def py_reduce(a):
    """The fixed summation order, restated in Python (oracle_reduce's doc)."""
    Y, X = a.shape
    TH = 16 if ((X + 255) // 256) * ((Y + 15) // 16) >= 1216 else 4
    ntx = (X + 31) // 32
    nty = (Y + TH - 1) // TH
    nsx = (ntx + 7) // 8

    def bfly(v):
        v = list(v)
        for off in (16, 8, 4, 2, 1):
            v = [v[l] + v[l ^ off] for l in range(32)]
        return v[0]

    S = []
    for sy in range(nty):
        for sx in range(nsx):
            t8 = []
            for w in range(8):
                tx = 8 * sx + w
                if tx >= ntx:
                    t8.append(0.0)
                    continue
                lanes = []
                for l in range(32):
                    col = 32 * tx + l
                    acc = 0.0
                    for j in range(TH):
                        row = TH * sy + j
                        acc = acc + (float(a[row, col]) if col < X and row < Y else 0.0)
                    lanes.append(acc)
                t8.append(bfly(lanes))
            S.append(bfly(t8 + [0.0] * 24))
    lanes = []
    for i in range(256):
        acc = 0.0
        for k in range(i, len(S), 256):
            acc = acc + S[k]
        lanes.append(acc)
    w8 = [bfly(lanes[32 * w:32 * w + 32]) for w in range(8)]
    return bfly(w8 + [0.0] * 24)


@pytest.mark.parametrize("shape", [(1, 1), (7, 5), (29, 37), (61, 300), (33, 17)])
def test_reduce_order_matches_python_restatement(shape):
    rng = np.random.default_rng(7)
    a = rng.standard_normal(shape) * np.exp(rng.uniform(-20, 20, shape))
    assert oracle.reduce(a) == py_reduce(a)


def test_reduce_pairs_unfused_is_reduce_of_products():
    rng = np.random.default_rng(3)
    a = rng.standard_normal((37, 61))
    b = rng.standard_normal((37, 61))
    assert oracle.reduce_pairs(a, b, 0) == oracle.reduce(a * b)
    assert abs(oracle.reduce_pairs(a, b, 1) - oracle.reduce(a * b)) < 1e-12


def test_reduce_exact_on_integers():
    a = np.arange(64 * 300, dtype=np.float64).reshape(64, 300)
    assert oracle.reduce(a) == a.sum()


def reflect_reference(a, H, d, x_max, y_max):
    """update_halo_{bottom,top,left,right} (update_halo_cl.cl:3-69) in order."""
    a = a.copy()
    for row in range(H - d, H):
        for col in range(H - d, x_max + H + d):
            a[row, col] = a[row + 1 + (H - row - 1) * 2, col]
    for row in range(H - d, H):
        for col in range(H - d, x_max + H + d):
            a[row + y_max + (H - row - 1) * 2 + 1, col] = a[row + y_max, col]
    for row in range(H - d, y_max + H + d):
        for col in range(H - d, H):
            a[row, col] = a[row, col + 1 + (H - col - 1) * 2]
    for row in range(H - d, y_max + H + d):
        for col in range(H - d, H):
            a[row, col + x_max + (H - col - 1) * 2 + 1] = a[row, col + x_max]
    return a


@pytest.mark.parametrize("H,d", [(1, 1), (2, 1), (2, 2), (4, 3)])
def test_update_halo_matches_four_pass_reflection(H, d):
    x, y = 13, 9
    ch = oracle.Chunk(x, y, H, 2, 1)
    rng = np.random.default_rng(H * 10 + d)
    a = rng.standard_normal((y + 2 * H, x + 2 * H))
    ch.write_padded("density", a)
    ch.update_halo([1, 0, 0, 0, 0, 0, 0], d)
    assert np.array_equal(ch.read_padded("density"), reflect_reference(a, H, d, x, y))


@pytest.mark.parametrize("x,y,H", [(9, 12, 1), (9, 11, 2), (6, 7, 1)])
def test_block_jacobi_solves_each_strip(x, y, H):
    """z = M^-1 r with M the 4-row tridiagonal strips of the operator."""
    ch = oracle.Chunk(x, y, H, 2, 3)
    ch.set_arithmetic(True)
    scenarios.setup(ch, x, y, lognormal_seed=3)
    ch.common_init(1, 0.004)
    rng = np.random.default_rng(1)
    r = rng.standard_normal((y, x))
    ch.write("r", r)
    ch.cg_init()
    z = ch.read("z")
    Kx = ch.read_padded("Kx")
    Ky = ch.read_padded("Ky")
    top = y if y % 4 == 0 else None
    for g in range(0, y, 4):
        n = min(4, y - g)
        # with H == 1 the reference's strip takes one halo row when y % 4 != 0;
        # that row has zero couplings and zero residual, so it does not change z
        for col in range(x):
            c = col + H
            M = np.zeros((n, n))
            for k in range(n):
                row = g + k + H
                M[k, k] = 1.0 + Ky[row + 1, c] + Ky[row, c] + Kx[row, c + 1] + Kx[row, c]
                if k > 0:
                    M[k, k - 1] = -Ky[row, c]
                if k < n - 1:
                    M[k, k + 1] = -Ky[row + 1, c]
            zz = np.linalg.solve(M, r[g:g + n, col])
            np.testing.assert_allclose(z[g:g + n, col], zz, rtol=1e-13, atol=1e-300)
    assert top is None or top == y


def test_cg_converges_and_check_result():
    x = y = 24
    ch = oracle.Chunk(x, y, 1, 2, 2)
    scenarios.setup(ch, x, y)
    ch.common_init(1, 0.004)
    ch.calc_residual()
    r0 = ch.calc_2norm(1)
    rro = ch.cg_init()
    for _ in range(200):
        pw = ch.cg_calc_w()
        rrn = ch.cg_calc_ur(rro / pw)
        ch.cg_calc_p(rrn / rro)
        rro = rrn
        if np.sqrt(abs(rrn)) < 1e-14 * np.sqrt(r0):
            break
    ch.calc_residual()
    assert np.sqrt(ch.calc_2norm(1)) < 1e-10 * np.sqrt(r0)


def test_reduction_rows_rule():
    assert oracle.lib().oracle_reduction_rows(4096, 4096) == 16
    assert oracle.lib().oracle_reduction_rows(512, 512) == 4
    assert oracle.lib().oracle_reduction_rows(3840, 3840) == 16


@pytest.mark.parametrize("solver", ["cg", "ppcg"])
def test_mixed_solve_reaches_fp64_tolerance(solver):
    """The oracle's mixed-precision solve (FP32 CG or PPCG inner, FP64
    defect correction) reaches the FP64 relative residual it is asked for,
    and its answer agrees with the FP64 CG solve to the accuracy that
    residual implies."""
    from tealeaf_opencl_gb300 import decks
    extra = "tl_mixed_precision\ntl_mixed_inner_eps 1e-5"
    kw = dict(solver=solver, prec="jac_diag", steps=2, eps=1e-10, max_iters=20000,
              summary_frequency=0, y_cells=61)
    if solver == "ppcg":
        kw.update(inner_steps=8, presteps=15)
    mixed = oracle.run_deck(decks.five_state_deck(72, extra=extra, **kw))
    kw["solver"] = "cg"
    kw.pop("inner_steps", None)
    kw.pop("presteps", None)
    fp64 = oracle.run_deck(decks.five_state_deck(72, **kw))
    n = mixed.n_steps
    assert all(r <= 1e-10 for r in mixed.relative_residual[:n])
    if solver == "ppcg":
        assert all(k > 0 for k in mixed.inner_iterations[:n])
    a, b = mixed.summaries()[-1], fp64.summaries()[-1]
    assert abs(a[5] - b[5]) <= 1e-8 * abs(b[5])
