"""PPCG inner steps run in fused pairs (tea_ppcg_tb.cu) give the oracle's
results bit for bit.

With the block-Jacobi preconditioner the library runs two inner steps of
tea_leaf_ppcg_solve_update_r + tea_leaf_ppcg_solve_calc_sd
(tea_leaf_ppcg_cl.cl:62-155) as one TMA-fed pass: in the resident loop
directly, and through the per-call C ABI by holding a step back until the
next one arrives.  These decks cover odd and even inner-step counts, halo
depths 1-3, the three arithmetic forms, reflective faces (whose operator
reads the sd halo), inverse-density coefficients and strips cut by the top
edge; each must match the oracle and must actually have launched the pair
kernel.
"""
import ctypes

import pytest

from oracle import oracle
from tealeaf_opencl_gb300 import decks, lib

pytestmark = pytest.mark.gpu
PAIR = b"tea_leaf_ppcg_solve_inner_pair"


@pytest.fixture(autouse=True)
def pairs_on():
    """The fused pairs are off by default (slower on GB300); these tests
    switch them on."""
    L = lib.load()
    assert L.tea_gb300_set_inner_pairs(1) == 0
    yield
    L.tea_gb300_set_inner_pairs(0)


def run_counting_pairs(deck, mode):
    L = lib.load()
    L.tea_gb300_kernel_timer_select(PAIR)
    try:
        steps = lib.run_deck(deck, mode=mode)
        ms, n = ctypes.c_double(), ctypes.c_longlong()
        L.tea_gb300_kernel_timer_read_name(PAIR, ctypes.byref(ms), ctypes.byref(n))
    finally:
        L.tea_gb300_kernel_timer_select(b"")
    return steps, n.value


def assert_matches_oracle(steps, res):
    assert [s.iterations for s in steps] == list(res.iterations[:res.n_steps])
    assert [s.inner_iterations for s in steps] == list(res.inner_iterations[:res.n_steps])
    last, final = steps[-1], res.summaries()[-1]
    assert (last.vol, last.mass, last.ie, last.temp) == tuple(final[[1, 2, 4, 5]])


@pytest.mark.parametrize("x,y,halo,mode,inner,reflective,coef", [
    (157, 143, 1, "chain", 5, False, None),
    (300, 67, 2, "exact", 6, True, None),
    (257, 131, 3, "fused", 4, False, "inverse"),
    (130, 64, 2, "chain", 10, True, None),
    (640, 258, 1, "fused", 7, False, None),
])
def test_fused_pairs_match_oracle(x, y, halo, mode, inner, reflective, coef):
    deck = decks.five_state_deck(x, solver="ppcg", prec="jac_block", steps=3, eps=1e-13,
                                 max_iters=2000, y_cells=y, halo=halo, inner_steps=inner,
                                 presteps=12, reflective=reflective, coefficient=coef,
                                 extra="tl_arithmetic %s" % mode)
    res = oracle.run_deck(deck)
    per_call, n_per_call = run_counting_pairs(deck, lib.DRIVER_PER_CALL)
    assert n_per_call > 0
    assert_matches_oracle(per_call, res)
    resident, _ = run_counting_pairs(deck, lib.DRIVER_RESIDENT)
    assert_matches_oracle(resident, res)


def test_held_step_is_launched_before_a_field_read():
    """A per-call step held back for pairing runs before anything reads the
    fields: step 1 alone, then r and sd read, equals the oracle's state
    after step 1."""
    from tests import scenarios
    x, y, H = 190, 77, 2
    recs = []
    for backend in ("gpu", "oracle"):
        ch = lib.Chunk(x, y, H, 4, 3) if backend == "gpu" else oracle.Chunk(x, y, H, 4, 3)
        scenarios.setup(ch, x, y, halo=H)
        ch.common_init(1, 0.004)
        ch.calc_residual()
        ch.cg_init()
        a, b, theta = scenarios.ch_coefs(0.9, 40.0, 6)
        ch.ppcg_init(a, b, theta)
        ch.ppcg_init_sd()
        ch.ppcg_inner(1)  # held back on the GPU: a second step may follow
        recs.append((ch.read("r"), ch.read("sd"), ch.read("u")))
        ch.ppcg_inner(2)  # alone now: the held step already ran
        ch.ppcg_inner(3)
        ch.ppcg_inner(4)  # paired with 3
        recs[-1] += (ch.read("r"), ch.read("sd"), ch.read("u"))
    for g, o in zip(*recs):
        assert (g.view("u8") == o.view("u8")).all()


@pytest.mark.parametrize("prec", [3, 2, 1])
def test_calc_ur_forms_sd_ahead_without_showing_it(prec):
    """In a PPCG chunk tea_leaf_cg_calc_ur_kernel_ocl_ also forms init_sd's
    sd into a spare buffer; init_sd uses it only when it directly follows.
    A read in between sees the old sd, and both orders give the oracle's
    fields."""
    from tests import scenarios
    x, y, H = 130, 97, 2
    out = []
    for backend in ("gpu", "oracle"):
        mk = lib.Chunk if backend == "gpu" else oracle.Chunk
        ch = mk(x, y, H, 4, prec)
        scenarios.setup(ch, x, y, halo=H)
        ch.common_init(1, 0.004)
        ch.calc_residual()
        rro = ch.cg_init()
        a, b, theta = scenarios.ch_coefs(0.9, 40.0, 4)
        ch.ppcg_init(a, b, theta)
        rec = []
        pw = ch.cg_calc_w()
        rrn = ch.cg_calc_ur(rro / pw)
        rec.append(ch.read("sd"))  # between calc_ur and init_sd
        ch.ppcg_init_sd()
        rec.append(ch.read("sd"))
        for s in range(1, 5):
            ch.ppcg_inner(s)
        rro = ch.calc_2norm(2)
        ch.cg_calc_p(rro / rrn)
        pw = ch.cg_calc_w()
        ch.cg_calc_ur(rro / pw)
        ch.ppcg_init_sd()  # directly after calc_ur
        rec += [ch.read("sd"), ch.read("r"), ch.read("u"), ch.read("z")]
        out.append(rec)
    for g, o in zip(*out):
        assert (g.view("u8") == o.view("u8")).all()
