"""Shared helpers of the differentiable-raycast tests: se(3) exponential in FP64, the Huber loss
of the rendered depth, and central finite differences over the twist."""
import math

import numpy as np

HUBER_DELTA = 0.02


def se3_exp(xi):
    """exp([rho; omega]) as a 4x4 FP64 matrix (rotation by Rodrigues, translation V rho)."""
    xi = np.asarray(xi, np.float64)
    rho, w = xi[:3], xi[3:]
    th = float(np.linalg.norm(w))
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-12:
        R = np.eye(3) + K
        V = np.eye(3) + 0.5 * K
    else:
        R = np.eye(3) + math.sin(th) / th * K + (1 - math.cos(th)) / th ** 2 * K @ K
        V = np.eye(3) + (1 - math.cos(th)) / th ** 2 * K + (th - math.sin(th)) / th ** 3 * K @ K
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = V @ rho
    return T


def perturb(T, xi):
    """Left perturbation exp(xi) T."""
    return se3_exp(xi) @ np.asarray(T, np.float64)


def huber(r, delta=HUBER_DELTA):
    a = np.abs(r)
    return np.where(a <= delta, 0.5 * r * r, delta * (a - 0.5 * delta))


def huber_grad(r, delta=HUBER_DELTA):
    return np.clip(r, -delta, delta)


def twist_fd(render, T0, obs, mask, h=1e-4, smooth_tol=2e-5):
    """Central differences of sum(huber(render(exp(xi) T0) - obs)) over mask, and the mask used:
    pixels that render in every evaluation and are smooth in every twist direction,
    |d(+h) - 2 d(0) + d(-h)| < smooth_tol metres. The render has no derivative where a pixel
    moves from one surface to another (silhouettes, a second zero crossing inside the last
    march step); there the second difference is the size of the jump, while on a smooth surface
    it is of order h^2 (below 1e-5 m for 95 % of the pixels at h = 1e-4)."""
    d0 = render(T0)
    grads = np.zeros(6)
    depths = []
    for j in range(6):
        e = np.zeros(6)
        e[j] = h
        depths += [render(perturb(T0, e)), render(perturb(T0, -e))]
    full = mask & (d0 > 0)
    for d in depths:
        full &= d > 0
    for j in range(6):
        full &= np.abs(depths[2 * j] - 2.0 * d0 + depths[2 * j + 1]) < smooth_tol
    for j in range(6):
        dp, dm = depths[2 * j], depths[2 * j + 1]
        lp = huber(dp[full] - obs[full]).sum()
        lm = huber(dm[full] - obs[full]).sum()
        grads[j] = (lp - lm) / (2 * h)
    return grads, full


def rel_err(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-30))
