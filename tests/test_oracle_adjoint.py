"""The oracle's FP64 differentiable render and its adjoint (the checker of the GPU adjoint).

The analytic gradients (implicit function theorem at the trilinear root) must match central
finite differences of the FP64 render with h = 1e-4 to a relative error <= 1e-3 (the twist,
over the pixels where the render is smooth, and single voxels); and the per-pixel twist rows must be the ICP's point-to-plane
Jacobian [n, p x n] (icp_impl.hpp:92-99) scaled by -n_z / (n . d).
"""
import numpy as np
import pytest

from tests.adjoint_util import huber, huber_grad, perturb, rel_err, twist_fd


@pytest.fixture(scope="module")
def scene(oracle):
    from supereight2_gb300 import synthetic as syn
    sensor, _, poses, frames = syn.dataset("tsdf320", 6)
    spec = dict(width=sensor.width, height=sensor.height, fx=sensor.fx, fy=sensor.fy,
                cx=sensor.cx, cy=sensor.cy, near_plane=sensor.near_plane,
                far_plane=sensor.far_plane)
    s = oracle.pinhole(**spec)
    m = oracle.OracleMap(10.24, 0.02)
    for i, (T, d) in enumerate(zip(poses[:5], frames[:5])):
        m.integrate_depth(d, s, T.astype(np.float32), i)
    # held-out frame 5, start pose perturbed by a small twist
    T0 = perturb(poses[5], [0.01, -0.008, 0.005, 0.004, -0.006, 0.003])
    return dict(m=m, s=s, T0=T0, obs=frames[5].astype(np.float64), T_gt=poses[5])


def test_render_is_near_the_raycast(scene):
    d = scene["m"].render_depth_f64(scene["s"], scene["T0"])
    pts, _, _ = scene["m"].raycast(scene["s"], scene["T0"].astype(np.float32))
    hit = (pts != 0).any(-1) & (d > 0)
    Tinv = np.linalg.inv(scene["T0"])
    z = (pts.reshape(-1, 3).astype(np.float64) @ Tinv[:3, :3].T + Tinv[:3, 3])[:, 2].reshape(d.shape)
    assert hit.mean() > 0.8
    # a raycast hit needs no interpolation at its last samples; the render does
    assert (d > 0).sum() >= 0.9 * (pts != 0).any(-1).sum()
    # the raycast's one-step secant estimate and the exact root agree to about a voxel (2 cm)
    err = np.abs(z[hit] - d[hit])
    assert np.median(err) < 0.002 and np.quantile(err, 0.99) < 0.03


def test_twist_gradient_matches_finite_differences(scene):
    m, s, T0, obs = scene["m"], scene["s"], scene["T0"], scene["obs"]
    base = m.render_depth_f64(s, T0)
    mask = (base > 0) & (obs > 0)
    fd, full = twist_fd(lambda T: m.render_depth_f64(s, T), T0, obs, mask)
    g = np.where(full, huber_grad(base - obs), 0.0)
    tw, _, _ = m.adjoint_f64(s, T0, g)
    assert full.sum() > 0.8 * mask.sum()
    assert rel_err(tw, fd) <= 1e-3, (tw, fd)


def test_voxel_gradient_matches_finite_differences(scene):
    m, s, T0, obs = scene["m"], scene["s"], scene["T0"], scene["obs"]
    base = m.render_depth_f64(s, T0)
    mask = (base > 0) & (obs > 0)
    g = np.where(mask, huber_grad(base - obs), 0.0)
    _, vg, _ = m.adjoint_f64(s, T0, g, voxel_grad=True)
    keys, coords, tsdf, weight, _ = m.blocks()
    h = 1e-4
    checked = 0
    for idx in np.argsort(-np.abs(vg).ravel())[:40]:
        if checked == 4:
            break
        b, v = divmod(int(idx), 512)
        c = coords[b] + np.array([v % 8, (v // 8) % 8, v // 64], np.int32)
        t0, w0 = float(tsdf[b, v]), float(weight[b, v])
        # the perturbation is applied to a float32 voxel: use its exact size
        tp, tm = np.float32(t0 + h), np.float32(t0 - h)
        m.set_voxel(c, tp, w0)
        dp = m.render_depth_f64(s, T0)
        m.set_voxel(c, tm, w0)
        dm = m.render_depth_f64(s, T0)
        m.set_voxel(c, np.float32(t0), w0)
        # pixels where the render is smooth in this voxel (see twist_fd)
        ok = mask & (dp > 0) & (dm > 0) & (np.abs(dp - 2 * base + dm) < 2e-5)
        fd = (huber(dp[ok] - obs[ok]).sum() - huber(dm[ok] - obs[ok]).sum()) / (float(tp) - float(tm))
        _, vg_ok, _ = m.adjoint_f64(s, T0, np.where(ok, g, 0.0), voxel_grad=True)
        if abs(vg_ok[b, v]) < 1e-3:
            continue  # every pixel this voxel moves jumps (a silhouette): no derivative to check
        assert abs(fd - vg_ok[b, v]) <= 1e-3 * abs(vg_ok[b, v]), (fd, vg_ok[b, v])
        checked += 1
    assert checked == 4


def test_twist_rows_are_the_icp_jacobian(scene):
    """d depth / d xi = -n_z / (n . d) [n, p x n]: the ICP point-to-plane Jacobian row of
    icp::trackKernel (icp_impl.hpp:92-99) at the rendered point, with the raycast's normal."""
    m, s, T0 = scene["m"], scene["s"], scene["T0"]
    depth = m.render_depth_f64(s, T0)
    _, _, jac = m.adjoint_f64(s, T0, None, jac=True)
    _, nrm, _ = m.raycast(s, T0.astype(np.float32))
    ok = (np.abs(jac).sum(-1) > 0) & (nrm != 0).any(-1)
    assert ok.mean() > 0.8
    H, W = depth.shape
    v, u = np.mgrid[0:H, 0:W]
    ray = np.stack([(u - s.cx) / s.fx, (v - s.cy) / s.fy, np.ones_like(u, dtype=np.float64)], -1)
    p_C = ray * depth[..., None]
    p = (p_C @ T0[:3, :3].T + T0[:3, 3])[ok]
    d = ray / np.linalg.norm(ray, axis=-1, keepdims=True)
    nz = d[..., 2][ok]
    d_W = (d @ T0[:3, :3].T)[ok]
    n = nrm[ok].astype(np.float64)
    J_icp = np.concatenate([n, np.cross(p, n)], -1)  # icp::trackKernel's J for normal n at p
    # structure: the rotational part is p x (translational part), as in the ICP row
    r = np.cross(p, jac[ok][:, :3])
    assert np.max(np.linalg.norm(r - jac[ok][:, 3:], axis=-1) / np.linalg.norm(r, axis=-1)) < 1e-9
    # direction and scale against the ICP row built from the raycast's normal (the 32-sample
    # central difference, which smooths the noisy trilinear gradient over +-1 voxel)
    pred = (-nz / np.sum(n * d_W, -1))[:, None] * J_icp
    cos = np.sum(jac[ok] * pred, -1) / (np.linalg.norm(jac[ok], axis=-1) * np.linalg.norm(pred, axis=-1))
    assert np.median(cos) > 0.95 and (cos > 0.9).mean() > 0.6
    ratio = np.linalg.norm(jac[ok], axis=-1) / np.linalg.norm(pred, axis=-1)
    assert 0.9 < np.median(ratio) < 1.1
