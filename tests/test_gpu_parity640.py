"""Parity of the CUDA path with the CPU oracle on the tracked 640x480 workload the benchmark
measures: 640x480 pinhole (fx = fy = 525), TSDF single-res 1024^3 at 1 cm, the bilateral
pre-filter (5x5, 4 px, 0.03 m) on the tracking input, 3-level ICP {10, 5, 4}, integration and
raycast per frame, on 12 consecutive frames of the seeded random-walk trajectory.

Every frame the GPU is handed the oracle's pose and the oracle's raycast images (the tracking
reference), so that a difference in one frame does not carry into the next and each frame is
checked on its own:
  - the bilateral-filtered input and the tracker's pyramid (half-sampled depth, point cloud and
    normals at all three levels) are bit-identical;
  - the tracked pose is within 1e-5 m / 1e-5 rad of the oracle's track (tracker_impl.hpp:30-116,
    icp.cpp:45-246), acceptance equal, inlier counts within 1e-4, iterations per level within one
    of the range the oracle's own variants (other start poses and summation orders) run (where
    the convergence test |x| < 1e-5 falls the other way, against the oracle run for the GPU's
    iteration counts); on a frame where the ICP sits at its convergence floor (the two stop
    a level one iteration apart, or the oracle's own results from start poses one float step away,
    or with its sums in other orders, spread by more than half the bar) within two threshold-sized
    updates and twice that spread;
  - the integration counters are equal each frame; after the last frame the allocated block-key
    set and integer weights are bit-exact and the TSDF values within 1e-5 * truncation;
  - the raycast depth is within 1e-4 m on >= 99.9 % of the pixels both hit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_FRAMES = 12
TSDF_TOL = 1e-5
DEPTH_TOL_M = 1e-4
DEPTH_FRAC = 0.999
POSE_TOL_M = 1e-5
POSE_TOL_RAD = 1e-5
BL = dict(radius=2, sigma_space=4.0, sigma_range=0.03)


def _rot_angle(R):
    """Rotation angle of R: atan2 of the skew part's norm and (trace - 1) / 2. Near the identity
    arccos((trace - 1) / 2) is dominated by the rounding of float32 rotation matrices (a trace
    off by 1e-7 reads as 4.5e-4 rad); the skew part carries the small angle itself."""
    s = 0.5 * float(np.linalg.norm([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]))
    c = (float(np.trace(R)) - 1.0) / 2.0
    return float(np.arctan2(s, c))


def _cam_depth(pts, T_WS):
    Tinv = np.linalg.inv(T_WS.astype(np.float64))
    p = pts.reshape(-1, 3).astype(np.float64) @ Tinv[:3, :3].T + Tinv[:3, 3]
    return p[:, 2].reshape(pts.shape[:2])


@pytest.fixture(scope="module")
def run640(oracle, gpu):
    import torch
    from supereight2_gb300 import synthetic as syn
    spec, _, poses, frames = syn.dataset("tsdf640", N_FRAMES)
    os_ = oracle.pinhole(spec.width, spec.height, spec.fx, spec.fy, spec.cx, spec.cy,
                         spec.near_plane, spec.far_plane)
    gs = gpu.PinholeCamera.from_spec(spec)
    om = oracle.OracleMap(10.24, 0.01)
    gm = gpu.Map(10.24, 0.01, max_blocks=1 << 17)
    integ = gpu.MapIntegrator(gm)
    tracker = gpu.Tracker(gm, gs, gpu.TrackerConfig())
    cfg_o = oracle.tracker_config()
    H, W = spec.height, spec.width
    pts = torch.zeros((H, W, 3), dtype=torch.float32, device="cuda")
    nrm = torch.zeros_like(pts)
    sc = torch.zeros((H, W), dtype=torch.int8, device="cuda")
    rec = dict(filter=[], pyramid=[], track=[], counters=[], raycast=[])
    T_o = poses[0].astype(np.float32)
    op = on = None
    for k in range(N_FRAMES):
        d = frames[k]
        dd = torch.from_numpy(d).cuda()
        if k > 0:
            fo = oracle.bilateral_filter(d, **BL)
            fg = gpu.bilateral_filter(dd, **BL)
            fg_h = fg.cpu().numpy()
            rec["filter"].append(np.array_equal(fg_h, fo))
            acc_o, T_new, st_o = oracle.track(os_, cfg_o, fo, T_o, op, on)
            # the oracle's own sensitivity: its results from start poses one float step away in
            # each translation component, and with its ICP sums in other orders (other thread
            # counts: the GPU's reductions sum in yet another order)
            spread_t = spread_r = 0.0
            its_var = [list(st_o.converged_iterations)]
            for a in range(3):
                for direction in (np.inf, -np.inf):
                    T_p = T_o.copy()
                    T_p[a, 3] = np.nextafter(T_p[a, 3], np.float32(direction))
                    _, T_q, st_q = oracle.track(os_, cfg_o, fo, T_p, op, on)
                    dt_q, dr_q = _pose_diff(T_q, T_new)
                    spread_t, spread_r = max(spread_t, dt_q), max(spread_r, dr_q)
                    its_var.append(list(st_q.converged_iterations))
            n_threads = oracle.num_threads()
            for nt in (1, 2, 3, 4, 6, 12, 16):
                oracle.set_num_threads(nt)
                _, T_q, st_q = oracle.track(os_, cfg_o, fo, T_o, op, on)
                dt_q, dr_q = _pose_diff(T_q, T_new)
                spread_t, spread_r = max(spread_t, dt_q), max(spread_r, dr_q)
                its_var.append(list(st_q.converged_iterations))
            oracle.set_num_threads(n_threads)
            # the GPU tracks from the same start pose against the oracle's reference images
            pts.copy_(torch.from_numpy(op))
            nrm.copy_(torch.from_numpy(on))
            T_g = T_o.copy()
            acc_g = tracker.track(fg, T_g, pts, nrm)
            red_g, its_g = tracker.last_reduction()
            its_o = list(st_o.converged_iterations)
            T_cmp, red_cmp = T_new, st_o.reduction
            if list(its_g) != its_o:
                # the convergence test fell the other way on one side: the oracle run for exactly
                # the GPU's iteration counts (no early exit) is the pose to compare with
                cfg_f = oracle.tracker_config(iterations=tuple(its_g), icp_threshold=0.0)
                _, T_cmp, st_f = oracle.track(os_, cfg_f, fo, T_o, op, on)
                red_cmp = st_f.reduction
            rec["track"].append(dict(frame=k, acc=(acc_g, acc_o), T=(T_g, T_cmp.astype(np.float32)),
                                     T_oracle=T_new.astype(np.float32), spread=(spread_t, spread_r),
                                     its=(list(its_g), its_o), its_oracle_range=(
                                         [min(v[l] for v in its_var) for l in range(3)],
                                         [max(v[l] for v in its_var) for l in range(3)]),
                                     inliers=(float(red_g[28]), float(red_cmp[28]))))
            pyr_o = oracle.tracker_pyramid(os_, fo, 3)
            levels = []
            for lvl, (do, po, no) in enumerate(pyr_o):
                dg, pg, ng = tracker.level_images(lvl)
                levels.append(((dg.cpu().numpy() if dg is not None else do), pg.cpu().numpy(),
                               ng.cpu().numpy(), do, po, no))
            rec["pyramid"].append(levels)
            T_o = T_new.astype(np.float32)
        ost = om.integrate_depth(d, os_, T_o, k)
        integ.integrateDepth(k, dd, gs, T_o)
        rec["counters"].append((ost, gm.integrate_stats()))
        op, on, _ = om.raycast(os_, T_o)
        gpu.raycast_volume(gm, gs, T_o, pts, nrm, sc)
        torch.cuda.synchronize()
        rec["raycast"].append((T_o.copy(), op, on, pts.cpu().numpy(), nrm.cpu().numpy()))
    gm.check()
    rec.update(om=om, gm=gm)
    return rec


def test_bilateral_input_bit_identical(run640):
    assert len(run640["filter"]) == N_FRAMES - 1
    assert all(run640["filter"])


def test_pyramid_images_bit_identical(run640):
    for levels in run640["pyramid"]:
        assert len(levels) == 3
        for dg, pg, ng, do, po, no in levels:
            assert np.array_equal(dg, do)
            assert np.array_equal(pg, po)
            assert np.array_equal(ng, no)
            assert (no != 0).any(-1).mean() > 0.3  # the images are not trivially empty


def _pose_diff(A, Bm):
    dt = float(np.max(np.abs(A[:3, 3].astype(np.float64) - Bm[:3, 3].astype(np.float64))))
    return dt, _rot_angle(A[:3, :3].astype(np.float64) @ Bm[:3, :3].astype(np.float64).T)


def test_tracked_pose_per_frame(run640):
    """Bar: 1e-5 m / 1e-5 rad against the oracle. Projective ICP re-associates pixels every
    iteration (rounded projections), and a level stops once its update x = [rho; omega] has
    |x| < 1e-5: its last updates are of that size, and one of them moves the camera position by
    up to (1 + |t|) 1e-5 m (omega rotates about the world origin, |t| ~ 1.5 m here). A frame is at
    this floor when the GPU and the oracle stop a level one iteration apart (the test |x| < 1e-5
    falling either side between FP64 and FP32 solves), or when the oracle's own results from
    start poses one float step away (or with its sums in other orders) spread by more than half
    the bar; there the GPU (exact
    reductions, FP64 solve and pose update) must lie within two such updates (and twice that
    spread) of the oracle; every other frame is held to the bar itself."""
    assert len(run640["track"]) == N_FRAMES - 1
    floor_frames = 0
    for t in run640["track"]:
        T_g, T_o = t["T"]
        assert t["acc"][0] == t["acc"][1], t["frame"]
        spread_t, spread_r = t["spread"]
        # the last iteration's reduction is taken at poses up to the bar apart: the pixels whose
        # projection lies that close to a rounding boundary change their association (a few in 1e5)
        tol_t, tol_r, tol_in = POSE_TOL_M, POSE_TOL_RAD, max(2.0, 1e-4 * t["inliers"][1])
        if (t["its"][0] != t["its"][1] or spread_t > 0.5 * POSE_TOL_M or spread_r > 0.5 * POSE_TOL_RAD):
            floor_frames += 1
            step_t = (1.0 + float(np.linalg.norm(T_o[:3, 3]))) * 1e-5
            tol_t = max(tol_t, 2 * spread_t, 2 * step_t)
            tol_r = max(tol_r, 2 * spread_r, 2 * 1e-5)
            # the last iteration's reduction is then taken at poses ~1e-5 m apart: a few pixels
            # of ~1e5 change their association
            tol_in = 1e-3 * t["inliers"][1]
        assert abs(t["inliers"][0] - t["inliers"][1]) <= tol_in, (t["frame"], t["inliers"])
        dt, dr = _pose_diff(T_g, T_o)
        assert dt <= tol_t, (t["frame"], dt, spread_t)
        assert dr <= tol_r, (t["frame"], dr, spread_r)
        # the convergence test |x| < 1e-5 can fall either side of the threshold between the
        # FP64 solve and the oracle's FP32 one: then the level runs a different number of
        # iterations and T_o above is the oracle run for the GPU's iteration counts. At the floor
        # the oracle's own count moves with its summation order (frame 1 of this trajectory
        # stops level 0 after 3 to 7 iterations with 1 to 16 threads): the GPU's count lies
        # within one of the range of the oracle's own variants
        lo, hi = t["its_oracle_range"]
        assert all(lo[l] - 1 <= t["its"][0][l] <= hi[l] + 1 for l in range(3)), (t["frame"], t["its"], lo, hi)
    # the floor is decided by the oracle's own sensitivity (its thread count changes its sums) and
    # by iteration-count flips, never by the GPU's pose error; several frames stay on the bar itself
    assert len(run640["track"]) - floor_frames >= 3, floor_frames


def test_integration_counters_per_frame(run640):
    for ost, gst in run640["counters"]:
        assert gst["n_valid_pixels"] == ost.n_valid_pixels
        assert gst["n_new_blocks"] == ost.n_new_blocks
        assert gst["n_listed_blocks"] == ost.n_new_blocks + ost.n_frustum_blocks
        assert gst["n_updated_voxels"] == ost.n_updated_voxels


def test_block_keys_weights_tsdf(run640):
    ok, oc, ot, ow, ots = run640["om"].blocks()
    gk, gc, gt, gw, gts = run640["gm"].download_blocks()
    oo, go = np.argsort(ok), np.argsort(gk)
    assert len(gk) == len(ok) > 1000
    assert np.array_equal(gk[go], ok[oo])        # bit-exact key set
    assert np.array_equal(gc[go], oc[oo])
    assert np.array_equal(gw[go], ow[oo])        # bit-exact integer weights
    assert np.array_equal(gts[go], ots[oo])
    assert np.max(np.abs(gt[go] - ot[oo])) <= TSDF_TOL


def test_raycast_depth_per_frame(run640):
    for T, op, on, gp, gn in run640["raycast"]:
        ohit = (op != 0).any(-1)
        ghit = (gp != 0).any(-1)
        assert (ohit == ghit).mean() >= DEPTH_FRAC
        both = ohit & ghit
        assert both.mean() > 0.5
        dz = np.abs(_cam_depth(gp, T) - _cam_depth(op, T))[both]
        assert (dz <= DEPTH_TOL_M).mean() >= DEPTH_FRAC, np.quantile(dz, [0.5, 0.999, 1.0])
        n_ok = (on != 0).any(-1) & both
        assert (np.sum(gn[n_ok] * on[n_ok], -1) > 1 - 1e-6).mean() >= DEPTH_FRAC
