"""The GPU's differentiable depth render and its adjoint (se_gpu_render_depth,
se_gpu_raycast_adjoint), checked against the FP64 oracle and against central finite
differences (h = 1e-4) of the FP64 render, to a relative error <= 1e-3; wrapped in a
torch.autograd.Function (here, in the test harness only) and used for Gauss-Newton pose
refinement against a held-out frame.
"""
import numpy as np
import pytest

from tests.adjoint_util import huber_grad, perturb, rel_err, twist_fd

pytestmark = pytest.mark.gpu

DEPTH_TOL_M = 1e-4


@pytest.fixture(scope="module")
def scene(oracle, gpu):
    import torch
    from supereight2_gb300 import synthetic as syn
    sensor, _, poses, frames = syn.dataset("tsdf320", 6)
    spec = dict(width=sensor.width, height=sensor.height, fx=sensor.fx, fy=sensor.fy,
                cx=sensor.cx, cy=sensor.cy, near_plane=sensor.near_plane,
                far_plane=sensor.far_plane)
    s = oracle.pinhole(**spec)
    om = oracle.OracleMap(10.24, 0.02)
    gm = gpu.Map(10.24, 0.02, max_blocks=1 << 16)
    gs = gpu.PinholeCamera(**spec)
    integ = gpu.MapIntegrator(gm)
    for i, (T, d) in enumerate(zip(poses[:5], frames[:5])):
        om.integrate_depth(d, s, T.astype(np.float32), i)
        integ.integrateDepth(i, torch.from_numpy(d).cuda(), gs, T.astype(np.float32))
    gm.check()
    T0 = perturb(poses[5], [0.01, -0.008, 0.005, 0.004, -0.006, 0.003])
    return dict(om=om, gm=gm, s=s, gs=gs, T0=T0, obs=frames[5].astype(np.float64),
                T_gt=poses[5], obs_t=torch.from_numpy(frames[5]).cuda())


def test_render_matches_fp64_oracle(scene, gpu):
    d_o = scene["om"].render_depth_f64(scene["s"], scene["T0"])
    d_g = gpu.render_depth(scene["gm"], scene["gs"], scene["T0"]).cpu().numpy().astype(np.float64)
    vo, vg = d_o > 0, d_g > 0
    # the FP32 and FP64 marches can stop in different steps where a ray grazes a surface
    assert (vo == vg).mean() >= 0.998
    both = vo & vg
    assert both.mean() > 0.8
    assert (np.abs(d_o - d_g)[both] <= DEPTH_TOL_M).mean() >= 0.999


def test_twist_adjoint_matches_fd_and_fp64(scene, gpu):
    import torch
    om, s, T0, obs = scene["om"], scene["s"], scene["T0"], scene["obs"]
    base = om.render_depth_f64(s, T0)
    d_g = gpu.render_depth(scene["gm"], scene["gs"], T0).cpu().numpy().astype(np.float64)
    mask = (base > 0) & (obs > 0) & (d_g > 0)
    fd, full = twist_fd(lambda T: om.render_depth_f64(s, T), T0, obs, mask)
    # the loss gradient with respect to the rendered depth, at the GPU's own render
    g = np.where(full, huber_grad(d_g - obs), 0.0).astype(np.float32)
    tw = gpu.raycast_adjoint(scene["gm"], scene["gs"], T0, torch.from_numpy(g).cuda()).cpu().numpy()
    tw_o, _, _ = om.adjoint_f64(s, T0, g.astype(np.float64))
    assert rel_err(tw, tw_o) <= 1e-4, (tw, tw_o)
    assert rel_err(tw, fd) <= 1e-3, (tw, fd)


def test_voxel_adjoint_matches_fp64(scene, gpu):
    import torch
    om, s, T0, obs = scene["om"], scene["s"], scene["T0"], scene["obs"]
    gm = scene["gm"]
    d_g = gpu.render_depth(gm, scene["gs"], T0).cpu().numpy().astype(np.float64)
    d_o = om.render_depth_f64(s, T0)
    # pixels where both renders find the same root: a pixel that stops on another surface in
    # FP32 moves its whole gradient to other voxels
    same = (d_g > 0) & (d_o > 0) & (np.abs(d_g - d_o) <= DEPTH_TOL_M)
    g = np.where(same & (obs > 0), huber_grad(d_g - obs), 0.0).astype(np.float32)
    vg = torch.zeros((gm.max_blocks, 512), dtype=torch.float32, device="cuda")
    gpu.raycast_adjoint(gm, scene["gs"], T0, torch.from_numpy(g).cuda(), voxel_grad=vg)
    keys_g = gm.download_blocks(voxels=False)[0]
    vg = vg.cpu().numpy()[: len(keys_g)]
    _, vg_o, _ = om.adjoint_f64(s, T0, g.astype(np.float64), voxel_grad=True)
    keys_o = om.blocks()[0]
    vg_g = vg[np.argsort(keys_g)]
    vg_o = vg_o[np.argsort(keys_o)]
    assert np.array_equal(np.sort(keys_g), np.sort(keys_o))
    assert np.count_nonzero(vg_o) > 1000
    assert rel_err(vg_g, vg_o) <= 1e-3


def test_jacobian_rows_match_fp64(scene, gpu):
    import torch
    gs = scene["gs"]
    jac = torch.zeros((gs.height, gs.width, 6), dtype=torch.float32, device="cuda")
    gpu.raycast_adjoint(scene["gm"], gs, scene["T0"], None, jac=jac)
    jac = jac.cpu().numpy().astype(np.float64)
    _, _, jo = scene["om"].adjoint_f64(scene["s"], scene["T0"], None, jac=True)
    ok = (np.abs(jac).sum(-1) > 0) & (np.abs(jo).sum(-1) > 0)
    rel = np.linalg.norm(jac[ok] - jo[ok], axis=-1) / np.linalg.norm(jo[ok], axis=-1)
    assert np.median(rel) < 1e-4 and np.quantile(rel, 0.99) < 1e-2


def _autograd_render(gpu, torch):
    class RenderDepth(torch.autograd.Function):
        """depth = render(exp(xi) T); the gradient is taken at xi = 0 (left perturbation)."""

        @staticmethod
        def forward(ctx, xi, map_, sensor, T):
            ctx.map, ctx.sensor, ctx.T = map_, sensor, T
            return gpu.render_depth(map_, sensor, T)

        @staticmethod
        def backward(ctx, grad_depth):
            tw = gpu.raycast_adjoint(ctx.map, ctx.sensor, ctx.T, grad_depth.contiguous())
            return tw, None, None, None

    return RenderDepth


def test_gauss_newton_refinement_recovers_the_pose(scene, gpu):
    """Refine a pose perturbed by 0.05 m / 3 deg against the held-out frame: 50 Gauss-Newton
    steps on the Huber loss with the adjoint's gradient and Jacobian rows."""
    import torch
    gs, gm = scene["gs"], scene["gm"]
    Render = _autograd_render(gpu, torch)
    rng = np.random.default_rng(5)
    a = rng.normal(size=3)
    w = rng.normal(size=3)
    xi0 = np.concatenate([0.05 * a / np.linalg.norm(a), np.deg2rad(3.0) * w / np.linalg.norm(w)])
    T = perturb(scene["T_gt"], xi0)
    obs = scene["obs_t"].to(torch.float64)
    jac = torch.zeros((gs.height, gs.width, 6), dtype=torch.float32, device="cuda")
    for _ in range(50):
        xi = torch.zeros(6, dtype=torch.float64, device="cuda", requires_grad=True)
        depth = Render.apply(xi, gm, gs, T).to(torch.float64)
        valid = (depth > 0) & (obs > 0)
        r = torch.where(valid, depth - obs, torch.zeros_like(depth))
        loss = torch.where(r.abs() <= 0.02, 0.5 * r * r, 0.02 * (r.abs() - 0.01)).sum()
        loss.backward()
        g = xi.grad
        jac.zero_()
        gpu.raycast_adjoint(gm, gs, T, None, jac=jac)
        J = jac.reshape(-1, 6).to(torch.float64)[valid.reshape(-1)]
        ra = r.detach().abs().reshape(-1)[valid.reshape(-1)]
        wgt = torch.clamp(0.02 / ra.clamp_min(1e-12), max=1.0)  # Huber IRLS weights
        Hm = (J * wgt[:, None]).T @ J
        Hm = Hm + 1e-6 * torch.trace(Hm) * torch.eye(6, dtype=torch.float64, device="cuda")
        step = -torch.linalg.solve(Hm, g)
        T = perturb(T, step.cpu().numpy())
    dT = np.linalg.inv(scene["T_gt"]) @ T
    t_err = np.linalg.norm(dT[:3, 3])
    r_err = np.degrees(np.arccos(np.clip((np.trace(dT[:3, :3]) - 1) / 2, -1, 1)))
    assert t_err < 0.01 and r_err < 0.5, (t_err, r_err)
