"""CPU checks of the adjoint's mathematics (no GPU).

The torch-autograd reference gradient of the time-stepped solve must agree
with central finite differences of its own loss, and the adjoint rule that
the CUDA kernels implement (restated with numpy) must agree with it.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
from tests import adjoint_reference as ref  # noqa: E402


def problem(shape=(9, 11), seed=3, coefficient=1):
    rng = np.random.default_rng(seed)
    density = np.exp(rng.uniform(np.log(0.1), np.log(100.0), shape))
    energy0 = rng.uniform(1e-4, 25.0, shape)
    dens_obs = density * np.exp(ref.smooth_field(shape, seed + 1))
    with torch.no_grad():
        u_obs = ref.forward(torch.tensor(np.log(dens_obs)), torch.tensor(energy0), 5, 0.004,
                            coefficient).numpy()
    return density, energy0, u_obs


@pytest.mark.parametrize("coefficient", [1, 2])
def test_reference_gradient_matches_finite_differences(coefficient):
    density, energy0, u_obs = problem(coefficient=coefficient)
    steps, dt = 5, 0.004
    _, g = ref.loss_and_gradient(density, energy0, u_obs, steps, dt, coefficient)
    rng = np.random.default_rng(7)
    for _ in range(3):
        v = rng.standard_normal(density.shape)
        h = 1e-5
        lp = ref.loss_only(density * np.exp(h * v), energy0, u_obs, steps, dt, coefficient)
        lm = ref.loss_only(density * np.exp(-h * v), energy0, u_obs, steps, dt, coefficient)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - (g * v).sum()) <= 1e-6 * abs(fd)


@pytest.mark.parametrize("coefficient", [1, 2])
def test_adjoint_rule_matches_autograd(coefficient):
    density, energy0, u_obs = problem(shape=(7, 12), seed=5, coefficient=coefficient)
    _, g = ref.loss_and_gradient(density, energy0, u_obs, 4, 0.004, coefficient)
    a = ref.adjoint_formula(density, energy0, u_obs, 4, 0.004, coefficient)
    np.testing.assert_allclose(a, g, rtol=1e-9, atol=1e-12 * np.abs(g).max())
