"""The CUDA adjoint of the time-stepped solve (tea_gb300_adjoint_*).

- Its forward model is the single-chunk driver's CG timestep: the same
  iteration counts and the same final u, bit for bit.
- Its gradient w.r.t. log-density matches an independent FP64 reference
  (torch autograd through dense direct solves, tests/adjoint_reference.py).
- It matches central finite differences of its own forward model along
  random directions, through the torch.autograd.Function.
- The checkpoint interval changes no bit of the gradient.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
from tealeaf_opencl_gb300 import adjoint, decks, lib  # noqa: E402
from tests import adjoint_reference as ref  # noqa: E402

pytestmark = pytest.mark.gpu
DT = 0.004


def cuda(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def observed(adj, density, energy0, steps, seed, eps=1e-13):
    """u_obs from a forward run with a seeded smooth perturbation of density."""
    y, x = density.shape
    dens_obs = cuda(density.cpu().numpy() * np.exp(ref.smooth_field((y, x), seed)))
    u_obs = torch.empty_like(density)
    adj.forward(dens_obs, energy0, u_final=u_obs, cfg=adj.config(steps, DT, eps, 20000, 4))
    return u_obs


def test_forward_matches_single_chunk_driver():
    p = decks.batch_problems(1, seed=21, side=(150, 260))[0]
    steps = 5
    deck = decks.batch_deck(p, steps=steps, eps=1e-12, max_iters=5000, prec="jac_diag",
                            arithmetic="fused")
    drv = lib.Driver(deck, mode=lib.DRIVER_RESIDENT)
    dens, en = lib.read_field("density"), lib.read_field("energy1")
    iters = []
    while True:
        info = drv.step()
        if info is None:
            break
        iters.append(info.iterations)
        if info.complete:
            break
    u_drv = lib.read_field("u")
    drv.close()
    lib.load().tea_gb300_set_arithmetic(1)
    adj = lib.Adjoint(p["x"], p["y"])
    try:
        u = torch.empty((p["y"], p["x"]), dtype=torch.float64, device="cuda")
        _, st = adj.forward(cuda(dens), cuda(en), u_final=u,
                            cfg=adj.config(steps, DT, 1e-12, 5000, 2))
        assert st.forward_iterations == sum(iters)
        assert np.array_equal(u.cpu().numpy().view(np.int64), u_drv.view(np.int64))
    finally:
        adj.free()


@pytest.mark.parametrize("coefficient", [1, 2])
def test_gradient_matches_fp64_reference(coefficient):
    shape = (20, 24)
    rng = np.random.default_rng(4)
    density = np.exp(rng.uniform(np.log(0.1), np.log(100.0), shape))
    energy0 = rng.uniform(1e-4, 25.0, shape)
    steps = 6
    lib.load().tea_gb300_set_arithmetic(1)
    adj = lib.Adjoint(shape[1], shape[0], coefficient=coefficient)
    try:
        d, e = cuda(density), cuda(energy0)
        u_obs = observed(adj, d, e, steps, seed=9, eps=1e-15)
        cfg = adj.config(steps, DT, 1e-15, 20000, 4)
        loss, st = adj.forward(d, e, u_obs, cfg=cfg)
        g = torch.empty_like(d)
        st = adj.backward(g)
        assert st.checkpoints == 2 and st.recompute_iterations > 0
        loss_ref, g_ref = ref.loss_and_gradient(density, energy0, u_obs.cpu().numpy(), steps,
                                                DT, coefficient)
        assert abs(loss - loss_ref) <= 1e-10 * loss_ref
        gn = g.cpu().numpy()
        assert np.abs(gn - g_ref).max() <= 1e-8 * np.abs(g_ref).max()
    finally:
        adj.free()


def test_checkpoint_interval_changes_no_bit():
    p = decks.batch_problems(1, seed=8, side=(60, 90))[0]
    density, energy0 = decks.paint(p)
    steps = 7
    lib.load().tea_gb300_set_arithmetic(1)
    adj = lib.Adjoint(p["x"], p["y"])
    try:
        d, e = cuda(density), cuda(energy0)
        u_obs = observed(adj, d, e, steps, seed=2)
        grads = []
        for ce in (1, 3, 4, 7, 10):
            adj.forward(d, e, u_obs, cfg=adj.config(steps, DT, 1e-13, 20000, ce))
            g = torch.empty_like(d)
            adj.backward(g)
            grads.append(g.cpu().numpy().view(np.int64).copy())
        for g in grads[1:]:
            assert np.array_equal(g, grads[0])
    finally:
        adj.free()


def test_autograd_function_matches_finite_differences():
    p = decks.batch_problems(1, seed=13, side=(100, 140))[0]
    density, energy0 = decks.paint(p)
    steps = 8
    lib.load().tea_gb300_set_arithmetic(1)
    adj = lib.Adjoint(p["x"], p["y"])
    try:
        e = cuda(energy0)
        theta = torch.log(cuda(density)).requires_grad_(True)
        u_obs = observed(adj, cuda(density), e, steps, seed=5)
        cfg = adj.config(steps, DT, 1e-14, 20000, 4)
        loss = adjoint.time_stepped_loss(theta, e, u_obs, adj, cfg)
        loss.backward()
        g = theta.grad.detach()
        gen = torch.Generator(device="cuda").manual_seed(1)
        h = 1e-4
        for _ in range(4):
            v = torch.randn(theta.shape, dtype=torch.float64, device="cuda", generator=gen)
            v /= v.norm()
            with torch.no_grad():
                lp = adjoint.time_stepped_loss(theta + h * v, e, u_obs, adj, cfg)
                lm = adjoint.time_stepped_loss(theta - h * v, e, u_obs, adj, cfg)
            fd = float((lp - lm) / (2 * h))
            gv = float((g * v).sum())
            assert abs(fd - gv) <= 1e-5 * abs(fd), (fd, gv)
    finally:
        adj.free()


def test_adjoint_errors():
    L = lib.load()
    with pytest.raises(lib.TeaError):
        lib.Adjoint(1, 5)
    with pytest.raises(lib.TeaError):
        lib.Adjoint(8, 8, prec="jac_block")
    adj = lib.Adjoint(16, 12)
    try:
        g = torch.empty((12, 16), dtype=torch.float64, device="cuda")
        with pytest.raises(lib.TeaError):
            adj.backward(g)  # no forward pass yet
        d = torch.ones_like(g)
        with pytest.raises(lib.TeaError):
            adj.forward(d, d, cfg=adj.config(0))
        adj.forward(d, d, cfg=adj.config(2))  # without u_obs: nothing kept
        with pytest.raises(lib.TeaError):
            adj.backward(g)
    finally:
        adj.free()
    assert L.tea_gb300_adjoint_backward(None, None) == -1
    with pytest.raises(lib.TeaError):
        lib.check()
