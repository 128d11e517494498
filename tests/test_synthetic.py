"""The seeded synthetic room: deterministic, with the documented noise and dropout."""
import numpy as np

from supereight2_gb300 import synthetic as syn


def test_scene_is_deterministic():
    a = syn.make_scene(7)
    b = syn.make_scene(7)
    assert np.array_equal(a.sphere_c, b.sphere_c) and np.array_equal(a.box_R, b.box_R)
    assert len(a.sphere_r) == 12 and len(a.box_c) == 8
    assert (a.sphere_r >= 0.1).all() and (a.sphere_r <= 0.6).all()


def test_render_depth_statistics():
    scene = syn.make_scene(3)
    poses = syn.circle_trajectory(2)
    d0 = syn.render_depth(scene, syn.SENSOR_320, poses[0], 11)
    d1 = syn.render_depth(scene, syn.SENSOR_320, poses[0], 11)
    assert d0.dtype == np.float32 and d0.shape == (240, 320)
    assert np.array_equal(d0, d1)
    zero = (d0 == 0).mean()
    assert 0.01 < zero < 0.04  # 2 % dropout
    assert d0.max() < 8.0 and np.median(d0[d0 > 0]) > 0.5
    clean = syn.render_depth(scene, syn.SENSOR_320, poses[0], 11, noise=False)
    valid = d0 > 0
    resid = (d0 - clean)[valid] / (0.0015 * clean[valid] ** 2)
    assert abs(resid.std() - 1.0) < 0.05


def test_trajectories():
    c = syn.circle_trajectory(20, step_m=0.05)
    steps = [np.linalg.norm(c[i + 1][:3, 3] - c[i][:3, 3]) for i in range(19)]
    assert np.allclose(steps, 0.05, atol=2e-3)
    r = syn.random_walk_trajectory(50, seed=1)
    for T in r:
        assert np.allclose(T[:3, :3] @ T[:3, :3].T, np.eye(3), atol=1e-9)
        assert abs(T[0, 3]) < 3.0 and abs(T[1, 3]) < 2.5
    steps = [np.linalg.norm(r[i + 1][:3, 3] - r[i][:3, 3]) for i in range(49)]
    assert max(steps) < 0.06
