"""FP64 reference gradient for the time-stepped solve, by torch autograd.

An independent statement of the forward model, small enough for dense
matrices: the TeaLeaf operator A = I + sum_f K_f (e_a - e_b)(e_a - e_b)^T
with the face coefficients of init_common (tea_leaf_common_cl.cl,
K_f = r (w_a + w_b) / (2 w_a w_b), w = density or 1/density, boundary faces
zeroed), u_0 = density * energy_0, u_{n+1} = A^-1 u_n (direct dense solves),
loss = 0.5*||u_T - u_obs||^2.  torch differentiates it with respect to
log(density); nothing here shares code with the CUDA adjoint.  Test
infrastructure only.
"""
import numpy as np
import torch


def operator(log_density, dt, extent=(0.0, 10.0, 0.0, 10.0), coefficient=1):
    """Dense A (N x N, N = y*x, x fastest) as a differentiable function of
    log_density (y, x)."""
    y, x = log_density.shape
    dx = (extent[1] - extent[0]) / float(np.float32(x))
    dy = (extent[3] - extent[2]) / float(np.float32(y))
    rx, ry = dt / (dx * dx), dt / (dy * dy)
    rho = torch.exp(log_density)
    w = rho if coefficient == 1 else 1.0 / rho
    kx = rx * (w[:, :-1] + w[:, 1:]) / (2.0 * w[:, :-1] * w[:, 1:])  # (y, x-1)
    ky = ry * (w[:-1, :] + w[1:, :]) / (2.0 * w[:-1, :] * w[1:, :])  # (y-1, x)
    n = x * y
    idx = torch.arange(n).reshape(y, x)
    A = torch.eye(n, dtype=torch.float64)
    for k, a, b in ((kx, idx[:, :-1], idx[:, 1:]), (ky, idx[:-1, :], idx[1:, :])):
        a, b, k = a.reshape(-1), b.reshape(-1), k.reshape(-1)
        A = A.index_put((a, a), k, accumulate=True)
        A = A.index_put((b, b), k, accumulate=True)
        A = A.index_put((a, b), -k, accumulate=True)
        A = A.index_put((b, a), -k, accumulate=True)
    return A


def forward(log_density, energy0, steps, dt, coefficient=1):
    """u_T (y, x)."""
    A = operator(log_density, dt, coefficient=coefficient)
    u = (torch.exp(log_density) * energy0).reshape(-1, 1)
    lu, piv = torch.linalg.lu_factor(A)
    for _ in range(steps):
        u = torch.linalg.lu_solve(lu, piv, u)
    return u.reshape(log_density.shape)


def loss_and_gradient(density, energy0, u_obs, steps, dt, coefficient=1):
    """(loss, d loss / d log(density)) as numpy, all FP64 on the CPU."""
    theta = torch.tensor(np.log(density), dtype=torch.float64, requires_grad=True)
    e0 = torch.tensor(energy0, dtype=torch.float64)
    uo = torch.tensor(u_obs, dtype=torch.float64)
    u = forward(theta, e0, steps, dt, coefficient)
    loss = 0.5 * ((u - uo) ** 2).sum()
    loss.backward()
    return loss.item(), theta.grad.numpy().copy()


def loss_only(density, energy0, u_obs, steps, dt, coefficient=1):
    with torch.no_grad():
        theta = torch.tensor(np.log(density), dtype=torch.float64)
        u = forward(theta, torch.tensor(energy0, dtype=torch.float64), steps, dt, coefficient)
        return float(0.5 * ((u - torch.tensor(u_obs)) ** 2).sum())


def smooth_field(shape, seed, sigma=0.3, corr=3.0):
    """Seeded smooth Gaussian field (spectral filter), scaled by sigma."""
    rng = np.random.Generator(np.random.Philox(seed))
    y, x = shape
    w = rng.standard_normal(shape)
    kx, ky = np.fft.fftfreq(x), np.fft.fftfreq(y)
    s = corr / np.sqrt(2.0)
    g = np.exp(-2.0 * (np.pi * s) ** 2 * (ky[:, None] ** 2 + kx[None, :] ** 2))
    f = np.fft.ifft2(np.fft.fft2(w) * g).real
    return sigma * (f - f.mean()) / f.std()


def adjoint_formula(density, energy0, u_obs, steps, dt, coefficient=1):
    """The adjoint rule the CUDA kernels implement, restated with numpy and
    direct solves: lambda_T = u_T - u_obs; per step backwards A mu =
    lambda_{n+1}, face gradients -(mu_a - mu_b)(u_a - u_b) times the cell's
    share of dK_f/dlog(density), lambda_n = mu; plus lambda_0 * u_0."""
    y, x = density.shape
    with torch.no_grad():
        A = operator(torch.tensor(np.log(density)), dt, coefficient=coefficient).numpy()
    dx, dy = 10.0 / float(np.float32(x)), 10.0 / float(np.float32(y))
    rx, ry = dt / (dx * dx), dt / (dy * dy)
    us = [(density * energy0).reshape(-1)]
    for _ in range(steps):
        us.append(np.linalg.solve(A, us[-1]))
    lam = us[-1] - u_obs.reshape(-1)
    grad = np.zeros((y, x))
    if coefficient == 1:
        sx, sy = -rx / (2.0 * density), -ry / (2.0 * density)
    else:
        sx, sy = 0.5 * rx * density, 0.5 * ry * density
    for n in range(steps - 1, -1, -1):
        mu = np.linalg.solve(A, lam).reshape(y, x)
        u = us[n + 1].reshape(y, x)
        gx_face = -(mu[:, :-1] - mu[:, 1:]) * (u[:, :-1] - u[:, 1:])  # (y, x-1)
        gy_face = -(mu[:-1, :] - mu[1:, :]) * (u[:-1, :] - u[1:, :])
        gx = np.zeros((y, x))
        gy = np.zeros((y, x))
        gx[:, :-1] += gx_face
        gx[:, 1:] += gx_face
        gy[:-1, :] += gy_face
        gy[1:, :] += gy_face
        grad += sx * gx + sy * gy
        lam = mu.reshape(-1)
    grad += lam.reshape(y, x) * us[0].reshape(y, x)
    return grad
