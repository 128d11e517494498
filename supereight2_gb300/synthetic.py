"""Seeded synthetic scenes and trajectories (input data for tests and the benchmark).

The scene stands in for the datasets the reference reports on (they are not available here):
an axis-aligned 6 x 5 x 3 m room seen from the inside, 12 random spheres (radius 0.1-0.6 m)
and 8 randomly oriented boxes, ray traced analytically in float64 and stored as float32 depth
(z, metres). Per-pixel noise N(0, (0.0015 z^2)^2) is added and 2 % of the pixels are zeroed.
Pinhole camera frame: x right, y down, z forward. Poses are T_WC (camera to world), 4x4.

Rendering runs with torch on any device; noise and dropout come from a numpy generator seeded
per frame, so a frame's bytes do not depend on the device it was rendered on except for
float64 rounding in the ray tracing.
"""
from dataclasses import dataclass, field
import math

import numpy as np
import torch

ROOM_HALF = (3.0, 2.5, 1.5)


@dataclass
class PinholeSpec:
    width: int
    height: int
    fx: float
    fy: float
    cx: float
    cy: float
    near_plane: float = 0.4
    far_plane: float = 6.0


# The camera set-ups of the benchmark configurations.
SENSOR_320 = PinholeSpec(320, 240, 262.5, 262.5, 159.5, 119.5, 0.4, 6.0)
SENSOR_640 = PinholeSpec(640, 480, 525.0, 525.0, 319.5, 239.5, 0.4, 6.0)
# A wide, coarse camera for multi-resolution tests: at 2 cm voxels a pixel covers z / 1.6
# voxels, so the reference's pixel/voxel ratios {1.5, 3, 6} select scales 0-2 within the room.
SENSOR_160W = PinholeSpec(160, 120, 80.0, 80.0, 79.5, 59.5, 0.4, 6.0)


@dataclass
class Scene:
    sphere_c: np.ndarray  # [12, 3]
    sphere_r: np.ndarray  # [12]
    box_c: np.ndarray     # [8, 3]
    box_R: np.ndarray     # [8, 3, 3] box-to-world rotation
    box_h: np.ndarray     # [8, 3] half extents
    seed: int = 0
    room_half: tuple = field(default=ROOM_HALF)


def _rot_zyx(yaw, pitch, roll):
    cy, sy = math.cos(yaw), math.sin(yaw)
    cp, sp = math.cos(pitch), math.sin(pitch)
    cr, sr = math.cos(roll), math.sin(roll)
    Rz = np.array([[cy, -sy, 0], [sy, cy, 0], [0, 0, 1]])
    Ry = np.array([[cp, 0, sp], [0, 1, 0], [-sp, 0, cp]])
    Rx = np.array([[1, 0, 0], [0, cr, -sr], [0, sr, cr]])
    return Rz @ Ry @ Rx


def make_scene(seed: int, keep_out_radius=(0.9, 2.1)) -> Scene:
    """12 spheres and 8 oriented boxes, kept out of the annulus the cameras move in."""
    rng = np.random.default_rng(seed)
    hx, hy, hz = ROOM_HALF

    def place(extent):
        for _ in range(10000):
            c = np.array([rng.uniform(-hx + extent, hx - extent),
                          rng.uniform(-hy + extent, hy - extent),
                          rng.uniform(-hz + extent, hz - extent)])
            rxy = math.hypot(c[0], c[1])
            if rxy + extent < keep_out_radius[0] or rxy - extent > keep_out_radius[1]:
                return c
        raise RuntimeError("could not place object")

    sr = rng.uniform(0.1, 0.6, size=12)
    sr = np.minimum(sr, 0.6)
    sc = np.stack([place(r) for r in sr])
    bh = rng.uniform(0.1, 0.4, size=(8, 3))
    bR = np.stack([_rot_zyx(*rng.uniform(-math.pi, math.pi, size=3)) for _ in range(8)])
    bc = np.stack([place(float(np.linalg.norm(h))) for h in bh])
    return Scene(sc, sr, bc, bR, bh, seed)


def look_at(eye, target, up=(0.0, 0.0, 1.0)) -> np.ndarray:
    """T_WC of a z-forward, y-down camera at eye looking at target."""
    eye = np.asarray(eye, np.float64)
    z = np.asarray(target, np.float64) - eye
    z /= np.linalg.norm(z)
    x = np.cross(z, np.asarray(up, np.float64))
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    T = np.eye(4)
    T[:3, 0], T[:3, 1], T[:3, 2], T[:3, 3] = x, y, z, eye
    return T


def _axis_angle(axis, angle):
    axis = np.asarray(axis, np.float64)
    axis = axis / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + math.sin(angle) * K + (1 - math.cos(angle)) * K @ K


def circle_trajectory(n_frames: int, radius=1.5, step_m=0.05, height=0.1) -> list:
    """Frames on a horizontal circle, looking at the room centre, step_m apart."""
    dtheta = step_m / radius
    poses = []
    for i in range(n_frames):
        th = i * dtheta
        eye = (radius * math.cos(th), radius * math.sin(th), height)
        poses.append(look_at(eye, (0.0, 0.0, -0.2)))
    return poses


def random_walk_trajectory(n_frames: int, seed: int, sigma_m=0.02, sigma_deg=1.0,
                           radius=1.5) -> list:
    """Random-walk velocity around the circle: translation steps with std sigma_m and
    orientation jitter of sigma_deg per frame about the inward-looking direction."""
    rng = np.random.default_rng(seed)
    th = 0.0
    vel = np.zeros(3)
    pos = np.array([radius, 0.0, 0.1])
    yaw_off = pitch_off = 0.0
    poses = []
    for _ in range(n_frames):
        base = look_at(pos, (0.0, 0.0, -0.2))
        R = base[:3, :3] @ _axis_angle((0, 1, 0), yaw_off) @ _axis_angle((1, 0, 0), pitch_off)
        T = np.eye(4)
        T[:3, :3], T[:3, 3] = R, pos
        poses.append(T)
        # velocity: random walk plus a pull back onto the circle and along its tangent
        th = math.atan2(pos[1], pos[0])
        target = np.array([radius * math.cos(th + 0.015), radius * math.sin(th + 0.015), 0.1])
        vel = 0.7 * vel + 0.3 * (target - pos) + rng.normal(0.0, sigma_m * 0.5, size=3)
        n = np.linalg.norm(vel)
        if n > 2.5 * sigma_m:
            vel *= 2.5 * sigma_m / n
        pos = pos + vel
        yaw_off = float(np.clip(0.8 * yaw_off + math.radians(rng.normal(0, sigma_deg)), -0.15, 0.15))
        pitch_off = float(np.clip(0.8 * pitch_off + math.radians(rng.normal(0, sigma_deg)), -0.1, 0.1))
    return poses


def dolly_trajectory(n_frames: int, x_far=-2.0, x_near=1.8) -> list:
    """Frames looking along +x at the room's end wall: the first 70 % move from x_far to
    x_near (5 m to 1.2 m from the wall), the rest move back, with a small sideways wobble."""
    n_in = max(2, int(math.ceil(0.7 * n_frames)))
    poses = []
    for i in range(n_frames):
        if i < n_in:
            x = x_far + (x_near - x_far) * i / (n_in - 1)
        else:
            x = x_near - (x_near - x_far) * 0.6 * (i - n_in + 1) / max(1, n_frames - n_in)
        eye = np.array([x, 0.3 * math.sin(0.4 * i), 0.1])
        target = eye + np.array([1.0, 0.1 * math.cos(0.3 * i), -0.05])
        poses.append(look_at(eye, target))
    return poses


def render_depth(scene: Scene, sensor: PinholeSpec, T_WC, frame_seed: int, device="cpu",
                 noise=True) -> np.ndarray:
    """Ray trace one float32 depth image (metres of z) with noise and 2 % dropout."""
    dt = torch.float64
    dev = torch.device(device)
    W, H = sensor.width, sensor.height
    v, u = torch.meshgrid(torch.arange(H, dtype=dt, device=dev),
                          torch.arange(W, dtype=dt, device=dev), indexing="ij")
    d_C = torch.stack([(u - sensor.cx) / sensor.fx, (v - sensor.cy) / sensor.fy,
                       torch.ones_like(u)], -1).reshape(-1, 3)
    T = torch.as_tensor(np.asarray(T_WC, np.float64), dtype=dt, device=dev)
    R, o = T[:3, :3], T[:3, 3]
    d = d_C @ R.T  # world direction; the ray parameter equals the camera z-depth
    inf = torch.full((d.shape[0],), float("inf"), dtype=dt, device=dev)

    # room interior: exit distance of the box
    half = torch.as_tensor(scene.room_half, dtype=dt, device=dev)
    safe_d = torch.where(d.abs() < 1e-12, torch.full_like(d, 1e-12), d)
    bound = torch.where(d > 0, half, -half)
    t_room = ((bound - o) / safe_d).amin(-1)
    best = torch.where(t_room > 0, t_room, inf)

    for c, r in zip(scene.sphere_c, scene.sphere_r):
        c = torch.as_tensor(c, dtype=dt, device=dev)
        oc = o - c
        a = (d * d).sum(-1)
        b = (d * oc).sum(-1)
        cc = (oc * oc).sum() - float(r) ** 2
        disc = b * b - a * cc
        sq = torch.sqrt(torch.clamp(disc, min=0.0))
        t0 = (-b - sq) / a
        t1 = (-b + sq) / a
        t = torch.where(t0 > 1e-6, t0, t1)
        hit = (disc >= 0) & (t > 1e-6)
        best = torch.where(hit & (t < best), t, best)

    for c, Rb, hb in zip(scene.box_c, scene.box_R, scene.box_h):
        c = torch.as_tensor(c, dtype=dt, device=dev)
        Rb = torch.as_tensor(Rb, dtype=dt, device=dev)
        hb = torch.as_tensor(hb, dtype=dt, device=dev)
        ol = (o - c) @ Rb
        dl = d @ Rb
        dl = torch.where(dl.abs() < 1e-12, torch.full_like(dl, 1e-12), dl)
        ta = (-hb - ol) / dl
        tb = (hb - ol) / dl
        tn = torch.minimum(ta, tb).amax(-1)
        tf = torch.maximum(ta, tb).amin(-1)
        hit = (tn <= tf) & (tf > 1e-6)
        t = torch.where(tn > 1e-6, tn, tf)
        best = torch.where(hit & (t < best), t, best)

    z = best.reshape(H, W).cpu().numpy()
    z = np.where(np.isfinite(z), z, 0.0)
    rng = np.random.default_rng(frame_seed)
    if noise:
        z = z + rng.standard_normal(z.shape) * (0.0015 * z * z)
        drop = rng.random(z.shape) < 0.02
        z = np.where(drop, 0.0, z)
    return z.astype(np.float32)


def dataset(config: str, n_frames: int, device="cpu", seed=None):
    """(sensor, scene, poses, depth frames) for a named benchmark configuration.

    config "tsdf320": 320x240, circle of 0.05 m / ~2 deg steps, ground-truth poses.
    config "tsdf640": 640x480, random-walk velocity (0.02 m, 1 deg per frame).
    config "mr160": 160x120 wide camera dollying towards and away from the end wall (multi-res
    integration scales 0-2 at 2 cm voxels); objects kept out of the central 2.2 m.
    """
    if config == "tsdf320":
        seed = 1001 if seed is None else seed
        sensor = SENSOR_320
        poses = circle_trajectory(n_frames, radius=1.5, step_m=0.05)
    elif config == "tsdf640":
        seed = 1002 if seed is None else seed
        sensor = SENSOR_640
        poses = random_walk_trajectory(n_frames, seed=seed * 31 + 7)
    elif config == "mr160":
        seed = 1003 if seed is None else seed
        sensor = SENSOR_160W
        poses = dolly_trajectory(n_frames)
        scene = make_scene(seed, keep_out_radius=(0.0, 2.2))
    else:
        raise ValueError(config)
    if config != "mr160":
        scene = make_scene(seed)
    frames = [render_depth(scene, sensor, T, seed * 7919 + i, device=device)
              for i, T in enumerate(poses)]
    return sensor, scene, poses, frames


# --------------------------------------------------------------------- outdoor LiDAR --
# A seeded outdoor scene for the spinning LiDAR: the ground plane z = 0 plus 100 boxes (yawed,
# standing on the ground) and 100 vertical cylinders over 100 x 100 m, kept out of 8 east-west
# roads (y = -35, -25, ..., 35; 3 m either side) that the sensors drive along 1.8 m above the
# ground. Ranges are ray traced in float64 and stored as float32 metres, with N(0, 0.01^2)
# range noise; rays without a hit within the far plane (or nearer than the near plane) are 0.


@dataclass
class LidarSpec:
    width: int = 1024
    height: int = 64
    elevation_min_deg: float = -22.5
    elevation_max_deg: float = 22.5
    near_plane: float = 0.5
    far_plane: float = 60.0


LIDAR_64 = LidarSpec()
ROADS_Y = tuple(-35.0 + 10.0 * k for k in range(8))


@dataclass
class OutdoorScene:
    box_c: np.ndarray    # [Nb, 3] centres (z = half height)
    box_yaw: np.ndarray  # [Nb]
    box_h: np.ndarray    # [Nb, 3] half extents
    cyl_c: np.ndarray    # [Nc, 2]
    cyl_r: np.ndarray    # [Nc]
    cyl_top: np.ndarray  # [Nc] heights
    seed: int = 0


def make_outdoor_scene(seed: int, n_boxes=100, n_cylinders=100, half=50.0, road_half=3.0) -> OutdoorScene:
    rng = np.random.default_rng(seed)
    roads = np.asarray(ROADS_Y)

    def place(radius):
        for _ in range(10000):
            c = rng.uniform(-half + radius, half - radius, size=2)
            if np.min(np.abs(c[1] - roads)) > road_half + radius:
                return c
        raise RuntimeError("could not place object")

    bh = np.stack([rng.uniform(0.5, 2.0, n_boxes), rng.uniform(0.5, 2.0, n_boxes),
                   rng.uniform(0.5, 5.0, n_boxes)], -1)
    bxy = np.stack([place(float(np.hypot(h[0], h[1]))) for h in bh])
    bc = np.concatenate([bxy, bh[:, 2:3]], -1)
    byaw = rng.uniform(-math.pi, math.pi, n_boxes)
    cr = rng.uniform(0.3, 1.5, n_cylinders)
    cc = np.stack([place(float(r)) for r in cr])
    ct = rng.uniform(1.0, 10.0, n_cylinders)
    return OutdoorScene(bc, byaw, bh, cc, cr, ct, seed)


def lidar_directions(spec: LidarSpec) -> np.ndarray:
    """Unit ray directions [height, width, 3] in the sensor frame (x forward, z up) through the
    pixel centres of the equiangular model: az = pi - (u + 0.5) 2 pi / width, el linear from
    elevation_max_deg (row 0) to elevation_min_deg."""
    u = np.arange(spec.width, dtype=np.float64)
    v = np.arange(spec.height, dtype=np.float64)
    az = math.pi - (u + 0.5) * (2.0 * math.pi / spec.width)
    el_max, el_min = math.radians(spec.elevation_max_deg), math.radians(spec.elevation_min_deg)
    el = el_max - v * (el_max - el_min) / (spec.height - 1)
    ce, se = np.cos(el)[:, None], np.sin(el)[:, None]
    return np.stack([ce * np.cos(az)[None, :], ce * np.sin(az)[None, :],
                     np.broadcast_to(se, (spec.height, spec.width))], -1)


def road_trajectory(k: int, n_frames: int, step_m=1.0, height=1.8, phase=0.0) -> list:
    """T_WS of a sensor driving along road k (even k eastwards from x = -45, odd k westwards
    from x = 45), weaving 1 m across the road, heading along the motion."""
    y0 = ROADS_Y[k % len(ROADS_Y)]
    sgn = 1.0 if k % 2 == 0 else -1.0
    poses = []
    for i in range(n_frames):
        s = i * step_m
        x = sgn * (-45.0 + s)
        y = y0 + math.sin(0.15 * s + phase)
        dy = 0.15 * math.cos(0.15 * s + phase)
        yaw = math.atan2(dy, sgn)
        T = np.eye(4)
        T[:3, :3] = _rot_zyx(yaw, 0.0, 0.0)
        T[:3, 3] = (x, y, height)
        poses.append(T)
    return poses


def render_range(scene: OutdoorScene, spec: LidarSpec, T_WS, frame_seed: int, keep=1.0, device="cpu",
                 noise=True) -> np.ndarray:
    """Ray trace one float32 range image [height, width] (metres, 0 = no return); a fraction
    1 - keep of the returns is dropped at random."""
    dt = torch.float64
    dev = torch.device(device)
    T = torch.as_tensor(np.asarray(T_WS, np.float64), dtype=dt, device=dev)
    d = torch.as_tensor(lidar_directions(spec), dtype=dt, device=dev).reshape(-1, 3) @ T[:3, :3].T
    o = T[:3, 3]
    inf = torch.full((d.shape[0],), float("inf"), dtype=dt, device=dev)
    best = inf.clone()
    # ground
    tg = -o[2] / torch.where(d[:, 2] < -1e-12, d[:, 2], torch.full_like(d[:, 2], -1e-12))
    best = torch.where((d[:, 2] < -1e-12) & (tg > 0), tg, best)
    # boxes (yawed): slabs in the box frame
    bc = torch.as_tensor(scene.box_c, dtype=dt, device=dev)
    bh = torch.as_tensor(scene.box_h, dtype=dt, device=dev)
    cy_, sy_ = torch.cos(torch.as_tensor(scene.box_yaw, dtype=dt, device=dev)), torch.sin(
        torch.as_tensor(scene.box_yaw, dtype=dt, device=dev))
    ol = o[None, :] - bc                                                   # [Nb, 3]
    olx = cy_ * ol[:, 0] + sy_ * ol[:, 1]
    oly = -sy_ * ol[:, 0] + cy_ * ol[:, 1]
    dlx = d[:, None, 0] * cy_[None] + d[:, None, 1] * sy_[None]            # [R, Nb]
    dly = -d[:, None, 0] * sy_[None] + d[:, None, 1] * cy_[None]
    dlz = d[:, None, 2].expand_as(dlx)
    tn = torch.full_like(dlx, -float("inf"))
    tf = torch.full_like(dlx, float("inf"))
    for oc, dc, hc in ((olx, dlx, bh[:, 0]), (oly, dly, bh[:, 1]), (ol[:, 2], dlz, bh[:, 2])):
        dc = torch.where(dc.abs() < 1e-12, torch.full_like(dc, 1e-12), dc)
        ta = (-hc[None] - oc[None]) / dc
        tb = (hc[None] - oc[None]) / dc
        tn = torch.maximum(tn, torch.minimum(ta, tb))
        tf = torch.minimum(tf, torch.maximum(ta, tb))
    hit = (tn <= tf) & (tn > 1e-6)
    tbox = torch.where(hit, tn, torch.full_like(tn, float("inf"))).amin(-1)
    best = torch.minimum(best, tbox)
    # vertical cylinders with a top cap
    cc = torch.as_tensor(scene.cyl_c, dtype=dt, device=dev)
    cr = torch.as_tensor(scene.cyl_r, dtype=dt, device=dev)
    ct = torch.as_tensor(scene.cyl_top, dtype=dt, device=dev)
    ox, oy = o[0] - cc[:, 0], o[1] - cc[:, 1]                              # [Nc]
    a = d[:, None, 0] ** 2 + d[:, None, 1] ** 2                            # [R, 1]
    b = d[:, None, 0] * ox[None] + d[:, None, 1] * oy[None]                # [R, Nc]
    c = (ox * ox + oy * oy - cr * cr)[None]
    disc = b * b - a * c
    sq = torch.sqrt(torch.clamp(disc, min=0.0))
    a_safe = torch.where(a < 1e-12, torch.full_like(a, 1e-12), a)
    t0 = (-b - sq) / a_safe
    z0 = o[2] + t0 * d[:, None, 2]
    side = (disc >= 0) & (a >= 1e-12) & (t0 > 1e-6) & (z0 >= 0) & (z0 <= ct[None])
    tcyl = torch.where(side, t0, torch.full_like(t0, float("inf")))
    dz = d[:, None, 2]
    dz_safe = torch.where(dz.abs() < 1e-12, torch.full_like(dz, -1e-12), dz)
    tc = (ct[None] - o[2]) / dz_safe
    px, py = ox[None] + tc * d[:, None, 0], oy[None] + tc * d[:, None, 1]
    cap = (dz < -1e-12) & (tc > 1e-6) & (px * px + py * py <= (cr * cr)[None])
    tcyl = torch.minimum(tcyl, torch.where(cap, tc, torch.full_like(tc, float("inf"))))
    best = torch.minimum(best, tcyl.amin(-1))
    r = best.reshape(spec.height, spec.width).cpu().numpy()
    r = np.where(np.isfinite(r) & (r >= spec.near_plane) & (r <= spec.far_plane), r, 0.0)
    rng = np.random.default_rng(frame_seed)
    if noise:
        r = np.where(r > 0, r + rng.standard_normal(r.shape) * 0.01, 0.0)
    if keep < 1.0:
        r = np.where(rng.random(r.shape) < keep, r, 0.0)
    return r.astype(np.float32)


def lidar_dataset(n_maps: int, n_frames: int, seed=1004, device="cpu", spec: LidarSpec = LIDAR_64):
    """(spec, scene, poses[map][frame], ranges[map][frame], keep[map]) for the batched LiDAR
    workload: map k drives road k with its own weave phase and keeps a fraction
    0.40 + 0.55 k / (n_maps - 1) of its returns (40 % to 95 %)."""
    scene = make_outdoor_scene(seed)
    keep = [0.40 + 0.55 * k / max(n_maps - 1, 1) for k in range(n_maps)]
    poses = [road_trajectory(k, n_frames, phase=0.7 * k) for k in range(n_maps)]
    ranges = [[render_range(scene, spec, T, seed * 7919 + 1000 * k + i, keep=keep[k], device=device)
               for i, T in enumerate(poses[k])] for k in range(n_maps)]
    return spec, scene, poses, ranges, keep


def wall_rays(d=10.0, lo=-15.0, res=0.1, n=300) -> np.ndarray:
    """Ray batch of a LeicaLidar facing a wall d metres away along x: n x n rays over [lo, lo + n
    res) degrees of elevation and azimuth (the batch of the reference's RayIntegrator.Propagation
    test, test/integrator/ray_integrator_unittest.cpp, angles accumulated in float as there)."""
    deg = np.float32(np.pi / 180.0)
    rays = []
    el = np.float32(lo)
    for _ in range(n):
        z = np.float32(d * np.tan(np.float32(el * deg)))
        az = np.float32(lo)
        for _ in range(n):
            y = np.float32(d * np.tan(np.float32(az * deg)))
            rays.append((d, y, z))
            az = np.float32(az + np.float32(res))
        el = np.float32(el + np.float32(res))
    return np.array(rays, np.float32)
