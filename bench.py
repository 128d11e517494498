#!/usr/bin/env python3
"""Frames/s of supereight2's per-frame dense-mapping path (track + integrate + raycast).

Workload (config "tsdf640"): 640x480 pinhole (fx = fy = 525, cx = 319.5, cy = 239.5), a
single-resolution TSDF map of 1024^3 voxels at 1 cm, a seeded synthetic room trajectory with
random-walk velocity (0.02 m, 1 deg per frame). One step is one frame: the bilateral pre-filter
of the tracking input (5x5, 4 px, 0.03 m), 3-level ICP {10, 5, 4} against the previous raycast,
integration of the raw depth at the tracked pose, raycast at that pose.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). ``value``: frames/s with the depth images resident in HBM, the
device time of the K steps measured with CUDA events on the launching stream and L2 flushed
(256 MiB write) between steps outside the timed pairs. ``e2e``: the same through the public API
with each frame's depth copied from pinned host memory and its pose read back into pinned
memory (read on the host while the next frame runs), host clock over consecutive frames with
no L2 flush between them.
``--impl reference`` times the CPU oracle (the restatement of the reference's OpenMP code) on
all host cores. Under torchrun every rank runs an independent replica (the path does not
shard); the value is the sum of frames over the max time across ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MAP_DIM = 10.24
MAP_RES = 0.01
CONFIG = "tsdf640"
METRIC = "frames/s 640x480 TSDF integrate+raycast+ICP"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# Bench kernel names -> the kernel names of the committed DRAM-traffic capture of this workload
_TRAFFIC_NAMES = {"icp_iter": "icp_persistent_kernel", "update": "update_kernel<0, 4>",
                  "raycast": "raycast_kernel<0, 0, 0>", "mr_update": "mr_update_kernel<0>"}


def _traffic(kernel):
    """DRAM bytes (read + write) per launch of `kernel` from the committed ncu captures of this
    workload, one kernel each (profiles/dram_traffic_per_kernel_tsdf640.txt), or None."""
    p = os.path.join(ROOT, "profiles", "dram_traffic_per_kernel_tsdf640.txt")
    name = _TRAFFIC_NAMES.get(kernel)
    if not name or not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            parts = line.split()
            # name (may hold spaces), launches, read, write, total bytes per launch, us per launch
            if len(parts) >= 6 and not line.startswith("#") and " ".join(parts[:-5]) == name:
                return float(parts[-2])
    return None


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None

    def start(self):
        """Start polling every 20 ms and return once the first sample is in, so that the timed
        region that follows is covered (nvidia-smi takes ~0.1 s to start)."""
        self.first = ""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.first = self.proc.stdout.readline()
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.05)  # one more sample after the timed region's last step
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        out = self.first + out
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_data(n_frames, device):
    from supereight2_gb300 import synthetic as syn
    return syn.dataset(CONFIG, n_frames, device=device)


# ----------------------------------------------------------------------------- GPU arm --

TUNE_FRAMES = 12  # the frame pipeline's autotuner runs (part of the untimed frames)


def _variant(se, torch, dev, sensor, poses, depth_dev, first, steps, warmup, path, storage, max_blocks,
             flush, profile=False, clocks=None, res_type="single"):
    """Run frame 0 and frames 1..first-1 untimed, then time `steps` frames (CUDA events per
    step on the launching stream, L2 flushed between steps outside the timed pairs).
    path "plain": the blocking reference-style calls (track with host pose readback, integrate,
    raycast); path "graph": the captured whole-frame pipeline with the pose on the device, whose
    first TUNE_FRAMES untimed frames are its autotuner's runs."""
    import ctypes as C
    W, H = sensor.width, sensor.height
    m = se.Map(MAP_DIM, MAP_RES, max_blocks=max_blocks, storage=storage, res_type=res_type)
    tracker = se.Tracker(m, sensor, se.TrackerConfig())
    stream = torch.cuda.current_stream(dev)
    T0 = poses[0].astype(np.float32).copy()
    if path == "plain":
        integ = se.MapIntegrator(m)
        pts = torch.zeros((H, W, 3), dtype=torch.float32, device=dev)
        nrm = torch.zeros_like(pts)
        scale = torch.zeros((H, W), dtype=torch.int8, device=dev)
        state = {"T": T0}
        filt = torch.empty((H, W), dtype=torch.float32, device=dev)

        def step(i, depth):
            se.bilateral_filter(depth, out=filt, **se.BILATERAL_DEFAULTS)
            tracker.track(filt, state["T"], pts, nrm)
            integ.integrateDepth(i, depth, sensor, state["T"])
            se.raycast_volume(m, sensor, state["T"], pts, nrm, scale)

        integ.integrateDepth(0, depth_dev[0], sensor, T0)
        se.raycast_volume(m, sensor, T0, pts, nrm, scale)
        fp = None
    else:
        fp = se.FramePipeline(m, sensor, tracker)
        fp.set_bilateral(**se.BILATERAL_DEFAULTS)
        fp.set_pose(T0, 0)
        fp.depth.copy_(depth_dev[0])
        fp.run(track=False)
        fp.autotune(TUNE_FRAMES)

        def step(i, depth):
            fp.depth.copy_(depth, non_blocking=True)
            fp.run(track=True)

    for i in range(1, first):
        step(i, depth_dev[i])
    torch.cuda.synchronize()
    m.check()
    tiles = fp.tiles()[0] if fp is not None else None

    L = se.library()
    n_prof = L.se_gpu_profiling_count()
    names = [L.se_gpu_profiling_name(i).decode() for i in range(n_prof)]
    if profile:
        L.se_gpu_profiling_read(0, None, None, 1)
        L.se_gpu_profiling_enable(1)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    stats = []
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    wall0 = time.perf_counter()
    for k in range(steps):
        flush.zero_()
        ev[k][0].record(stream)
        step(first + k, depth_dev[first + k])
        ev[k][1].record(stream)
        if profile:
            st_k = m.integrate_stats()
            st_k["icp_iterations"] = tracker.last_reduction()[1]
            stats.append(st_k)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clk = clocks.stop() if clocks else None
    kernel_ms, kernel_launches = {}, {}
    if profile:
        L.se_gpu_profiling_enable(0)
        tot = (C.c_double * n_prof)()
        cnt = (C.c_int64 * n_prof)()
        L.se_gpu_profiling_read(n_prof, tot, cnt, 1)
        kernel_ms = {names[i]: float(tot[i]) for i in range(n_prof) if cnt[i]}
        kernel_launches = {names[i]: int(cnt[i]) for i in range(n_prof) if cnt[i]}
    m.check()
    dev_ms = float(sum(a.elapsed_time(b) for a, b in ev))
    return {"dev_ms": dev_ms, "wall_s": wall, "stats": stats, "kernel_ms": kernel_ms,
            "kernel_launches": kernel_launches, "clocks": clk, "map": m, "fp": fp,
            "tracker": tracker, "num_blocks": m.num_blocks(), "tiles": tiles}


def run_ours(args, ws, rank, local):
    import torch
    import supereight2_gb300 as se

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n_frames = 1 + TUNE_FRAMES + args.warmup + 2 * args.steps + 1  # the last frame is held out (adjoint)
    t0 = time.perf_counter()
    sensor_spec, scene, poses, frames = make_data(n_frames, dev)
    gen_s = time.perf_counter() - t0
    sensor = se.PinholeCamera.from_spec(sensor_spec)
    W, H = sensor.width, sensor.height
    depth_dev = [torch.from_numpy(f).to(dev) for f in frames]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    first = 1 + TUNE_FRAMES + args.warmup
    K = args.steps

    # plain FP32 (blocking calls) with per-kernel events: the roofline and kernel breakdown
    plain = _variant(se, torch, dev, sensor, poses, depth_dev, first, K, args.warmup, "plain", "f32",
                     args.max_blocks, flush, profile=True)
    del plain["map"], plain["tracker"]
    # captured graph, FP16 storage
    g16 = _variant(se, torch, dev, sensor, poses, depth_dev, first, K, args.warmup, "graph", "f16",
                   args.max_blocks, flush)
    del g16["map"], g16["tracker"], g16["fp"]
    # captured graph, FP32 storage: the headline; clocks sampled during its timed region
    if ws > 1:
        torch.distributed.barrier()
    g32 = _variant(se, torch, dev, sensor, poses, depth_dev, first, K, args.warmup, "graph", "f32",
                   args.max_blocks, flush, clocks=Clocks(local))
    if ws > 1:
        torch.distributed.barrier()

    # e2e through the public API: pinned host depth copied in every step, pose read back
    fp = g32["fp"]
    host_frames = [torch.from_numpy(f).pin_memory() for f in frames]
    first_e2e = first + K
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    # each frame's pose (48 + 4 bytes device -> host) is read while the next frame runs
    bufs = [(torch.zeros(12, dtype=torch.float32).pin_memory(), torch.zeros(1, dtype=torch.int32).pin_memory(),
             torch.cuda.Event()) for _ in range(2)]
    e2e_poses = []
    for k in range(K):
        fp.run(track=True, depth=host_frames[first_e2e + k])  # host depth copied in on the stream
        pose12, acc, ev = bufs[k % 2]
        fp.pose_async(pose12, acc)
        ev.record()
        if k > 0:
            p_prev, a_prev, ev_prev = bufs[(k - 1) % 2]
            ev_prev.synchronize()
            e2e_poses.append((p_prev.numpy().copy(), int(a_prev[0])))
    torch.cuda.synchronize()
    e2e_poses.append((bufs[(K - 1) % 2][0].numpy().copy(), int(bufs[(K - 1) % 2][1][0])))
    e2e_s = time.perf_counter() - e0
    assert len(e2e_poses) == K and all(np.isfinite(p).all() for p, _ in e2e_poses)
    g32["map"].check()

    # differentiable render + adjoint on the map after all integrated frames, against the
    # held-out frame
    adjoint = _adjoint_bench(se, torch, g32["map"], sensor, poses[-1], depth_dev[-1], flush)

    # multi-resolution TSDF map (the reference's MultiresTSDF), FP32 and FP16 storage, same
    # frames through the captured pipeline
    mr = {}
    for st in ("f32", "f16"):
        v = _variant(se, torch, dev, sensor, poses, depth_dev, first, K, args.warmup, "graph", st,
                     args.max_blocks, flush, res_type="multi")
        mr[st] = {"value": K / (v["dev_ms"] * 1e-3), "ms_per_step": v["dev_ms"] / K}
        del v["map"], v["tracker"], v["fp"]

    # the multi-res update's own time per frame (blocking calls, per-kernel events) and the
    # integration scales of the blocks it updates, for its roofline
    mr_roof = _mr_update_roofline(se, torch, dev, sensor, poses, depth_dev, first, K, args.warmup,
                                  args.max_blocks, flush, W, H)

    # eight LiDAR occupancy maps in one batch
    lidar = _lidar_bench(se, torch, dev, args.lidar_steps, args.warmup, flush)
    lidar_data = lidar.pop("_data")

    # the ray integrator (integrateRayBatch, LeicaLidar) on the reference's wall batch
    ray_batch = _ray_batch_bench(se, torch, dev)

    times = torch.tensor([g32["dev_ms"], e2e_s, plain["dev_ms"], g16["dev_ms"]], dtype=torch.float64,
                         device=dev)
    if ws > 1:
        torch.distributed.all_reduce(times, op=torch.distributed.ReduceOp.MAX)
    g32_ms, e2e_max, plain_ms, g16_ms = [float(v) for v in times.cpu()]

    # ---- roofline of the dominant kernel (per-kernel CUDA events, plain run)
    hbm_peak, peak_kind = _peaks()
    kms, kl = plain["kernel_ms"], plain["kernel_launches"]
    dom = max(kms, key=kms.get)
    S_v = 8
    algo = None
    if dom == "update":
        b = [st["n_updated_voxels"] * 2 * S_v + st["n_listed_blocks"] * 8 + W * H * 4 for st in plain["stats"]]
        algo = float(np.mean(b))
    elif dom == "icp_iter":
        # per launch: 48 B per pixel of every iteration the launch ran (the persistent ICP runs
        # all iterations of a frame in one launch; converged levels stop early)
        npx = [sum((W >> l) * (H >> l) * it for l, it in enumerate(st["icp_iterations"])) for st in plain["stats"]]
        launches_per_frame = kl[dom] / max(len(plain["stats"]), 1)
        algo = float(np.mean(npx)) * 48.0 / launches_per_frame
    elif dom == "raycast":
        # outputs only here; with the CPU baseline run, the voxels the oracle's raycast reads are
        # added below (W H 25 + N_touched S_v)
        algo = W * H * 25.0
    avg_launch_ms = kms[dom] / max(kl[dom], 1)
    achieved = (algo / (avg_launch_ms * 1e-3) / 1e9) if algo else None
    upd = [st["n_updated_voxels"] for st in plain["stats"]]
    ub = [st["n_updated_voxels"] * 2 * S_v + st["n_listed_blocks"] * 8 + W * H * 4 for st in plain["stats"]]
    upd_ms = kms.get("update", 0.0) / max(kl.get("update", 1), 1)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": (achieved / hbm_peak) if achieved else None, "traffic": _traffic(dom),
                "traffic_source": "profiles/dram_traffic_per_kernel_tsdf640.txt (ncu, one kernel per capture, --cache-control none)",
                "peak_kind": peak_kind, "algorithmic_bytes_per_launch": algo,
                "avg_launch_us": avg_launch_ms * 1e3,
                "integration": {"kernel": "update", "avg_launch_us": upd_ms * 1e3,
                                "algorithmic_bytes_per_launch": float(np.mean(ub)),
                                "achieved_GBps": float(np.mean(ub)) / (upd_ms * 1e-3) / 1e9 if upd_ms else None,
                                "frac": float(np.mean(ub)) / (upd_ms * 1e-3) / 1e9 / hbm_peak if upd_ms else None,
                                "traffic": _traffic("update")}}
    if mr_roof:
        mr_roof["achieved_GBps"] = mr_roof["algorithmic_bytes_per_launch"] / (mr_roof["avg_launch_us"] * 1e-6) / 1e9
        mr_roof["frac"] = mr_roof["achieved_GBps"] / hbm_peak
        mr_roof["traffic"] = _traffic("mr_update")
        roofline["multires_update"] = mr_roof
    icp_ms = kms.get("icp_iter", 0.0) / max(kl.get("icp_iter", 1), 1)
    if icp_ms:
        # 48 B per pixel of every iteration a tracked frame ran (its working set stays in L2)
        ib = float(np.mean([sum((W >> l) * (H >> l) * it for l, it in enumerate(st["icp_iterations"]))
                            for st in plain["stats"]])) * 48.0 / (kl["icp_iter"] / max(len(plain["stats"]), 1))
        roofline["icp"] = {"kernel": "icp_persistent_kernel", "avg_launch_us": icp_ms * 1e3,
                           "algorithmic_bytes_per_launch": ib, "achieved_GBps": ib / (icp_ms * 1e-3) / 1e9,
                           "frac": ib / (icp_ms * 1e-3) / 1e9 / hbm_peak, "traffic": _traffic("icp_iter"),
                           "iterations_per_frame": float(np.mean([sum(st["icp_iterations"])
                                                                   for st in plain["stats"]]))}

    value = ws * K / (g32_ms * 1e-3)
    out = {
        "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": ws,
        "steps": K, "warmup": args.warmup, "ms_per_step": g32_ms / K,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded room: 6x5x3 m box, 12 spheres, 8 boxes; depth noise "
                "N(0,(0.0015 z^2)^2), 2% dropout)",
        "config": {"workload": "tsdf640: 640x480 pinhole, TSDF single-res 1024^3 @ 1 cm, "
                               "bilateral-filtered tracking input (5x5, 4 px, 0.03 m), "
                               "ICP 3 levels {10,5,4}, integrate + raycast per frame",
                   "map_res_m": MAP_RES, "map_voxels": 1024, "storage": "f32",
                   "path": "captured CUDA graph per frame, pose on the device",
                   "parallelism": f"replicas x{ws}", "l2": "flushed (256 MiB write) between steps",
                   "untimed_frames": f"frame 0, {TUNE_FRAMES} autotuner runs of the graph variants, "
                                     f"{args.warmup} warm-up frames"},
        "variants": {
            "plain_f32": {"value": ws * K / (plain_ms * 1e-3), "ms_per_step": plain_ms / K,
                          "api": "blocking se:: calls: track (host pose), integrateDepth, raycast_volume"},
            "graph_f32": {"value": value, "ms_per_step": g32_ms / K, "tiles": g32["tiles"]},
            "graph_f16": {"value": ws * K / (g16_ms * 1e-3), "ms_per_step": g16_ms / K, "tiles": g16["tiles"],
                          "storage": "FP16 tsdf with 8 guard bits + 8-bit weight (4 B per voxel), FP32 arithmetic"},
            "graph_vs_plain": plain_ms / g32_ms, "graph_f16_vs_plain": plain_ms / g16_ms},
        "roofline": roofline,
        "e2e": {"value": ws * K / e2e_max, "unit": "frames/s", "h2d_bytes_per_step": W * H * 4,
                "d2h_bytes_per_step": 52,
                "api": "FramePipeline.run(depth=pinned host frame) + pose_async; frame k's pose is "
                       "read on the host while frame k+1 runs",
                "l2": "not flushed: wall clock of consecutive frames as an application runs them"},
        # per tracked frame: bilateral 1 + track 3 (state init with the depth pyramid, points
        # with normals, the persistent ICP with its pose check) + integrate 4 (prep, carve,
        # frustum, update) + raycast 2 (prep, raycast)
        "gpu_launches": 10 * K,
        "kernel_ms_per_frame_plain": {k: v / K for k, v in kms.items()},
        "kernel_launches": kl,
        "voxels_per_s": float(np.mean(upd)) * K / (g32_ms * 1e-3),
        "updated_voxels_per_frame": float(np.mean(upd)),
        "num_blocks": g32["num_blocks"],
        "multires": {"workload": "the same frames into a MultiresTSDF map (1024^3 at 1 cm, 8^3 blocks "
                                 "with the 585-entry voxel pyramid), captured graph per frame",
                     "graph_f32": mr["f32"], "graph_f16": mr["f16"]},
        "adjoint": adjoint,
        "lidar_batch": lidar,
        "ray_batch": ray_batch,
        "gen_s": gen_s,
        "clocks": g32["clocks"],
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(frames, poses, sensor_spec, first - 1, 2 * K, args.cpu_budget_s)
        touched = out["cpu_baseline"].pop("raycast_voxels_touched", None)
        rc_ms = kms.get("raycast", 0.0) / max(kl.get("raycast", 1), 1)
        if touched and rc_ms:
            rb = W * H * 25.0 + touched * S_v
            rc = {"kernel": "raycast", "avg_launch_us": rc_ms * 1e3, "algorithmic_bytes_per_launch": rb,
                  "voxels_touched": touched, "achieved_GBps": rb / (rc_ms * 1e-3) / 1e9,
                  "frac": rb / (rc_ms * 1e-3) / 1e9 / hbm_peak, "traffic": _traffic("raycast")}
            out["roofline"]["raycast"] = rc
            if dom == "raycast":
                out["roofline"].update(achieved=rc["achieved_GBps"], frac=rc["frac"],
                                       algorithmic_bytes_per_launch=rb)
        out["lidar_batch"]["cpu_baseline"] = lidar_cpu_baseline(lidar_data)
        out["ray_batch"]["cpu_baseline"] = ray_batch_cpu_baseline()
        if args.precision_frames > 0:
            out["precision_vs_f64"] = _precision_report(se, torch, torch.device("cuda", local),
                                                        args.precision_frames, args.max_blocks)
    return out


def _mr_update_roofline(se, torch, dev, sensor, poses, depth_dev, first, K, warmup, max_blocks, flush, W, H):
    """Algorithmic bytes of the multi-res TSDF update (both launches: scale selection with down-
    propagation, then the update with up-propagation) against its time in the blocking FP32 path.
    Per listed block at integration scale s: its (8 >> s)^3 entries read and written (16 B each,
    data and past data), and every coarser entry written by the up-propagation and read back;
    a new block also writes its 585 default entries; plus the depth image. The scale mix is the
    one of the blocks the last timed frame updated; the block counts are the timed frames' mean."""
    v = _variant(se, torch, dev, sensor, poses, depth_dev, first, K, warmup, "plain", "f32", max_blocks, flush,
                 profile=True, res_type="multi")
    kms, kl = v["kernel_ms"], v["kernel_launches"]
    if not kms.get("update"):
        return None
    m = v["map"]
    keys, _, _, _, ts = m.download_blocks(voxels=False)
    mk, _, _, _, _, _, sc = m.download_multires()
    scale_of = dict(zip(mk.tolist(), sc[:, 0].tolist()))
    last = int(ts.max())
    cur = [scale_of[k] for k, t in zip(keys.tolist(), ts.tolist()) if t == last]
    entries = {0: 512, 1: 64, 2: 8, 3: 1}
    coarser = {0: 73, 1: 9, 2: 1, 3: 0}
    E = 16
    per_block = float(np.mean([2 * E * (entries[s] + coarser[s]) for s in cur])) if cur else 0.0
    n_list = float(np.mean([st["n_listed_blocks"] for st in v["stats"]]))
    n_new = float(np.mean([st["n_new_blocks"] for st in v["stats"]]))
    algo = n_list * per_block + n_new * 585 * E + W * H * 4
    hist = {int(s): int(c) for s, c in zip(*np.unique(np.asarray(cur), return_counts=True))} if cur else {}
    out = {"kernel": "mr_scale_down_kernel + mr_update_kernel (FP32)",
           "avg_launch_us": kms["update"] / kl["update"] * 1e3, "algorithmic_bytes_per_launch": algo,
           "listed_blocks": n_list, "new_blocks": n_new, "scale_histogram_last_frame": hist,
           "bytes_per_listed_block": per_block}
    del v["map"], v["tracker"], v["fp"]
    return out


def _se3_exp(xi):
    xi = np.asarray(xi, np.float64)
    rho, w = xi[:3], xi[3:]
    th = float(np.linalg.norm(w))
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-12:
        R, V = np.eye(3) + K, np.eye(3) + 0.5 * K
    else:
        R = np.eye(3) + np.sin(th) / th * K + (1 - np.cos(th)) / th ** 2 * K @ K
        V = np.eye(3) + (1 - np.cos(th)) / th ** 2 * K + (th - np.sin(th)) / th ** 3 * K @ K
    T = np.eye(4)
    T[:3, :3], T[:3, 3] = R, V @ rho
    return T


def _adjoint_bench(se, torch, m, sensor, T_gt, obs, flush, reps=20, gn_steps=50, delta=0.02):
    """Differentiable render + adjoint against a held-out frame whose pose is perturbed by a
    seeded 0.05 m / 3 deg twist: the forward + backward time (render, Huber gradient, adjoint
    into the twist and every TSDF voxel), a central-difference check of the twist gradient with
    the FP32 render (h = 1e-4, pixels where the render is smooth), and the pose error after
    Gauss-Newton refinement with the adjoint's Jacobian rows."""
    rng = np.random.default_rng(1005)
    a, w = rng.normal(size=3), rng.normal(size=3)
    xi0 = np.concatenate([0.05 * a / np.linalg.norm(a), np.deg2rad(3.0) * w / np.linalg.norm(w)])
    T = _se3_exp(xi0) @ T_gt
    H, W = sensor.height, sensor.width
    obs64 = obs.to(torch.float64)
    vg = torch.zeros((m.max_blocks, 512), dtype=torch.float32, device="cuda")
    tw = torch.zeros(6, dtype=torch.float64, device="cuda")
    depth = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def fwd_bwd(Tp):
        se.render_depth(m, sensor, Tp, out=depth)
        r = torch.where((depth > 0) & (obs > 0), depth - obs, torch.zeros_like(depth))
        g = torch.clamp(r, -delta, delta).contiguous()
        tw.zero_()
        vg.zero_()
        se.raycast_adjoint(m, sensor, Tp, g, twist_grad=tw, voxel_grad=vg)

    for _ in range(3):
        fwd_bwd(T)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for e0, e1 in ev:
        flush.zero_()
        e0.record(stream)
        fwd_bwd(T)
        e1.record(stream)
    torch.cuda.synchronize()
    ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ev]))

    def loss_of(d):
        r = torch.where(mask, d.to(torch.float64) - obs64, torch.zeros_like(obs64))
        a_ = r.abs()
        return float(torch.where(a_ <= delta, 0.5 * r * r, delta * (a_ - 0.5 * delta)).sum())

    # central differences over the twist with the FP32 render
    h = 1e-4
    base = se.render_depth(m, sensor, T).clone()
    ds = []
    for j in range(6):
        e = np.zeros(6)
        e[j] = h
        ds.append((se.render_depth(m, sensor, _se3_exp(e) @ T).clone(),
                   se.render_depth(m, sensor, _se3_exp(-e) @ T).clone()))
    mask = (base > 0) & (obs > 0)
    for dp, dm in ds:
        mask &= (dp > 0) & (dm > 0) & ((dp.double() - 2 * base.double() + dm.double()).abs() < 2e-5)
    fd = np.array([(loss_of(dp) - loss_of(dm)) / (2 * h) for dp, dm in ds])
    g = torch.where(mask, torch.clamp(base - obs, -delta, delta), torch.zeros_like(base)).contiguous()
    tw.zero_()
    se.raycast_adjoint(m, sensor, T, g, twist_grad=tw)
    adj = tw.cpu().numpy()
    fd_rel = float(np.linalg.norm(adj - fd) / max(np.linalg.norm(fd), 1e-30))

    # Gauss-Newton refinement (Huber IRLS weights) with the adjoint's per-pixel rows
    jac = torch.zeros((H, W, 6), dtype=torch.float32, device="cuda")
    Tk = T.copy()
    for _ in range(gn_steps):
        d = se.render_depth(m, sensor, Tk)
        valid = ((d > 0) & (obs > 0)).reshape(-1)
        r = (d.double() - obs64).reshape(-1)[valid]
        jac.zero_()
        se.raycast_adjoint(m, sensor, Tk, None, twist_grad=tw, jac=jac)
        J = jac.reshape(-1, 6).double()[valid]
        wgt = torch.clamp(delta / r.abs().clamp_min(1e-12), max=1.0)
        Hm = (J * wgt[:, None]).T @ J
        Hm = Hm + 1e-6 * torch.trace(Hm) * torch.eye(6, dtype=torch.float64, device="cuda")
        b = J.T @ torch.clamp(r, -delta, delta)
        Tk = _se3_exp(-np.linalg.solve(Hm.cpu().numpy(), b.cpu().numpy())) @ Tk  # 6x6 on the host

    def pose_err(Ta):
        dT = np.linalg.inv(T_gt) @ Ta
        return float(np.linalg.norm(dT[:3, 3])), _rot_deg(dT[:3, :3], np.eye(3))

    t0, r0 = pose_err(T)
    t1, r1 = pose_err(Tk)
    return {"workload": "640x480 differentiable depth render of the headline map after all its frames, "
                        "Huber (0.02 m) loss against the next (held-out) frame, start pose perturbed by "
                        "0.05 m / 3 deg",
            "fwd_bwd_ms": ms, "fwd_bwd_per_s": 1e3 / ms,
            "fd_rel_err": fd_rel, "fd_h": h, "fd_pixels": int(mask.sum()),
            "gn_steps": gn_steps, "pose_err_start": {"m": t0, "deg": r0},
            "pose_err_final": {"m": t1, "deg": r1}}


# ------------------------------------------------------- precision against an FP64 run --

def _rot_deg(Ra, Rb):
    """Angle of Ra Rb^T in degrees: atan2 of the skew part's norm and (trace - 1) / 2, which keeps
    small angles that arccos of (trace - 1) / 2 loses to the rounding of float32 rotations."""
    R = np.asarray(Ra, np.float64) @ np.asarray(Rb, np.float64).T
    s = 0.5 * float(np.linalg.norm([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]))
    return float(np.degrees(np.arctan2(s, (float(np.trace(R)) - 1.0) / 2.0)))


def _precision_report(se, torch, dev, n_frames, max_blocks):
    """The multi-res TSDF pipeline (bilateral-filtered tracking input, 3-level ICP, integration,
    raycast) on n_frames of the seeded trajectory, on the GPU with FP32 and with FP16 storage and
    in the FP64 run of the oracle, each tracking on its own. Reports, against the FP64 run: the
    per-frame pose, the trajectory error (ATE: RMSE of the positions against ground truth), the
    TSDF of the blocks both hold at scale 0 after the last frame, and the raycast depth of both
    maps at the FP64 run's last pose; these include the effect of each run's own tracked poses.
    "identical_poses" then gives the kernels' own errors: all three integrate at the
    ground-truth poses and raycast at the last one."""
    from oracle import pyoracle64 as o64
    spec, scene, poses_gt, frames = make_data(n_frames, dev)
    sensor = se.PinholeCamera.from_spec(spec)
    H, W = sensor.height, sensor.width
    t0 = time.perf_counter()
    o64.set_num_threads(os.cpu_count() or 1)
    s64 = o64.pinhole(spec.width, spec.height, spec.fx, spec.fy, spec.cx, spec.cy, spec.near_plane, spec.far_plane)
    cfg64 = o64.tracker_config()
    m64 = o64.OracleMap64(MAP_DIM, MAP_RES, multires=True)
    T = poses_gt[0].astype(np.float32).astype(np.float64)
    traj64 = [T.copy()]
    m64.integrate_depth(frames[0], s64, T, 0)
    pts, nrm, _ = m64.raycast(s64, T)
    for i in range(1, n_frames):
        _, T, _ = o64.track(s64, cfg64, o64.bilateral_filter(frames[i], **se.BILATERAL_DEFAULTS), T, pts, nrm)
        m64.integrate_depth(frames[i], s64, T, i)
        pts, nrm, _ = m64.raycast(s64, T)
        traj64.append(T.copy())
    f64_s = time.perf_counter() - t0
    keys64, _, t64, w64, _, _, sc64 = m64.mr_blocks()
    T_last = traj64[-1]
    pts64 = pts
    gt = np.stack([P[:3, 3] for P in poses_gt])
    ate = lambda tr: float(np.sqrt(np.mean(np.sum((np.stack([P[:3, 3] for P in tr]) - gt) ** 2, -1))))  # noqa: E731
    out = {"workload": f"{n_frames} frames of the tsdf640 trajectory, MultiresTSDF 1024^3 at 1 cm, "
                       "bilateral-filtered tracking input, track + integrate + raycast, each run tracking on its own",
           "f64_oracle_s": f64_s, "ate_m": {"f64_oracle": ate(traj64)}}
    for st in ("f32", "f16"):
        m = se.Map(MAP_DIM, MAP_RES, max_blocks=max_blocks, storage=st, res_type="multi")
        tr = se.Tracker(m, sensor, se.TrackerConfig())
        fp = se.FramePipeline(m, sensor, tr)
        fp.set_bilateral(**se.BILATERAL_DEFAULTS)
        fp.set_pose(poses_gt[0].astype(np.float32), 0)
        traj = []
        for i in range(n_frames):
            fp.depth.copy_(torch.from_numpy(frames[i]).to(dev))
            fp.run(track=i > 0)
            traj.append(fp.pose()[0].astype(np.float64))
        m.check()
        dt = [float(np.linalg.norm(a[:3, 3] - b[:3, 3])) for a, b in zip(traj, traj64)]
        dr = [_rot_deg(a[:3, :3], b[:3, :3]) for a, b in zip(traj, traj64)]
        keys, _, tsdf, weight, _, _, sc = m.download_multires()
        common, ia, ib = np.intersect1d(keys, keys64, return_indices=True)
        same0 = (sc[ia, 0] == 0) & (sc64[ib, 0] == 0)
        ta, tb = tsdf[ia][same0][:, :512], t64[ib][same0][:, :512]
        both = (weight[ia][same0][:, :512] > 0) & (w64[ib][same0][:, :512] > 0)
        e = np.abs(ta[both].astype(np.float64) - tb[both])
        rp = torch.zeros((H, W, 3), dtype=torch.float32, device=dev)
        rn = torch.zeros_like(rp)
        se.raycast_volume(m, sensor, T_last.astype(np.float32), rp, rn)
        rp = rp.cpu().numpy().astype(np.float64)
        R, t = T_last[:3, :3], T_last[:3, 3]
        z = lambda P: ((P - t) @ R)[..., 2]  # noqa: E731
        hit = (rp != 0).any(-1) & (pts64 != 0).any(-1)
        ez = np.abs(z(rp)[hit] - z(pts64)[hit])
        q = lambda a, p: float(np.quantile(a, p)) if len(a) else None  # noqa: E731
        out[st] = {
            "pose_err_vs_f64": {"max_m": max(dt), "mean_m": float(np.mean(dt)), "max_deg": max(dr),
                                "mean_deg": float(np.mean(dr))},
            "tsdf_err_vs_f64_trunc_units": {"median": q(e, 0.5), "p99": q(e, 0.99), "p999": q(e, 0.999),
                                            "max": float(e.max()) if len(e) else None, "voxels": int(len(e)),
                                            "blocks_same_scale0": int(same0.sum()), "blocks_common": int(len(common))},
            "raycast_depth_err_vs_f64_m": {"median": q(ez, 0.5), "p99": q(ez, 0.99), "p999": q(ez, 0.999),
                                           "pixels": int(hit.sum())},
        }
        out["ate_m"][st] = ate(traj)
        del fp, tr, m

    # the kernels' own error: the FP64 oracle and the GPU with FP32 and FP16 storage all integrate
    # every frame at its ground-truth pose and raycast at the last one (no tracking, so no pose
    # drift enters the figures)
    t0 = time.perf_counter()
    m64g = o64.OracleMap64(MAP_DIM, MAP_RES, multires=True)
    for i in range(n_frames):
        m64g.integrate_depth(frames[i], s64, poses_gt[i].astype(np.float32).astype(np.float64), i)
    T_gt = poses_gt[-1].astype(np.float32)
    pts64g, _, _ = m64g.raycast(s64, T_gt.astype(np.float64))
    keys64g, _, t64g, w64g, _, _, sc64g = m64g.mr_blocks()
    ident = {"workload": f"{n_frames} frames of the tsdf640 trajectory integrated at their ground-truth poses into "
                         "MultiresTSDF maps (1024^3 at 1 cm), raycast at the last pose",
             "f64_oracle_s": time.perf_counter() - t0}
    for st in ("f32", "f16"):
        m = se.Map(MAP_DIM, MAP_RES, max_blocks=max_blocks, storage=st, res_type="multi")
        integ = se.MapIntegrator(m)
        for i in range(n_frames):
            integ.integrateDepth(i, torch.from_numpy(frames[i]).to(dev), sensor, poses_gt[i].astype(np.float32))
        m.check()
        keys, _, tsdf, weight, _, _, sc = m.download_multires()
        common, ia, ib = np.intersect1d(keys, keys64g, return_indices=True)
        same0 = (sc[ia, 0] == 0) & (sc64g[ib, 0] == 0)
        ta, tb = tsdf[ia][same0][:, :512], t64g[ib][same0][:, :512]
        both = (weight[ia][same0][:, :512] > 0) & (w64g[ib][same0][:, :512] > 0)
        e = np.abs(ta[both].astype(np.float64) - tb[both])
        wa, wb = weight[ia][same0][:, :512], w64g[ib][same0][:, :512]
        rp = torch.zeros((H, W, 3), dtype=torch.float32, device=dev)
        rn = torch.zeros_like(rp)
        se.raycast_volume(m, sensor, T_gt, rp, rn)
        rp = rp.cpu().numpy().astype(np.float64)
        R, t = T_gt[:3, :3].astype(np.float64), T_gt[:3, 3].astype(np.float64)
        z = lambda P: ((P - t) @ R)[..., 2]  # noqa: E731
        hit = (rp != 0).any(-1) & (pts64g != 0).any(-1)
        ez = np.abs(z(rp)[hit] - z(pts64g)[hit])
        q = lambda a, p: float(np.quantile(a, p)) if len(a) else None  # noqa: E731
        ident[st] = {
            "tsdf_err_vs_f64_trunc_units": {"median": q(e, 0.5), "p99": q(e, 0.99), "p999": q(e, 0.999),
                                            "max": float(e.max()) if len(e) else None, "voxels": int(len(e)),
                                            "blocks_same_scale0": int(same0.sum()),
                                            "blocks_common": int(len(common)),
                                            "blocks_only_gpu": int(len(keys) - len(common)),
                                            "blocks_only_f64": int(len(keys64g) - len(common))},
            "weights_equal_fraction": float(np.mean(wa == wb)) if wa.size else None,
            "raycast_depth_err_vs_f64_m": {"median": q(ez, 0.5), "p99": q(ez, 0.99), "p999": q(ez, 0.999),
                                           "max": float(ez.max()) if len(ez) else None,
                                           "within_1e-4_m": float(np.mean(ez <= 1e-4)) if len(ez) else None,
                                           "pixels": int(hit.sum())},
        }
        del integ, m
    out["identical_poses"] = ident
    return out


# ------------------------------------------------------------------ 8-map LiDAR batch --

LIDAR_MAPS = 8
LIDAR_RES = 0.4
LIDAR_MAX_BLOCKS = 1 << 16


def _lidar_maps(se, n):
    T_MW = np.eye(4, dtype=np.float32)
    T_MW[:3, 3] = (51.2, 51.2, 12.8)
    return [se.Map(102.4, LIDAR_RES, res_type="multi", field="occupancy", max_blocks=LIDAR_MAX_BLOCKS,
                   T_MW=T_MW) for _ in range(n)]


def _lidar_bench(se, torch, dev, K, warmup, flush):
    """Scans/s of 8 occupancy maps, each driving its own road with its own LiDAR stream, every
    call integrating one scan into each map. Variants: batched launches replayed from a captured
    CUDA graph after autotuning (the headline), batched launches without the graph, one map per
    call (the reference's API shape), and the graph end to end from pinned host memory."""
    from supereight2_gb300 import synthetic as syn
    tune = 16  # the autotuner's calls (four untimed, then three rounds of four candidates), part of the warm-up
    W = max(warmup, 3) + tune
    n_frames = W + K
    t0 = time.perf_counter()
    spec, scene, poses, ranges, keep = syn.lidar_dataset(LIDAR_MAPS, n_frames, device=dev)
    gen_s = time.perf_counter() - t0
    sensor = se.OusterLidar.from_spec(spec)
    imgs = [torch.from_numpy(np.stack([ranges[k][i] for k in range(LIDAR_MAPS)])).to(dev) for i in range(n_frames)]
    Ts = [np.stack([poses[k][i] for k in range(LIDAR_MAPS)]).astype(np.float32) for i in range(n_frames)]
    valid = [float(np.mean([(ranges[k][i] > 0).mean() for i in range(n_frames)])) for k in range(LIDAR_MAPS)]

    def timed(step):
        ev = []
        for i in range(W):
            step(i)
        torch.cuda.synchronize()
        for i in range(W, W + K):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            step(i)
            b.record()
            ev.append((a, b))
        torch.cuda.synchronize()
        return float(sum(a.elapsed_time(b) for a, b in ev))

    res = {}
    # batched + graph + autotuned
    maps = _lidar_maps(se, LIDAR_MAPS)
    batch = se.OccupancyBatch(maps, sensor, graph=True, autotune=True)
    ms_graph = timed(lambda i: batch.integrate(imgs[i], Ts[i], i))
    tiles, left = batch.tiles()
    for m in maps:
        m.check()
    blocks = [int(m.occupancy_stats()[0]) for m in maps]
    del batch, maps
    # batched, one persistent cooperative launch per step, in a captured graph, autotuned
    maps = _lidar_maps(se, LIDAR_MAPS)
    batch = se.OccupancyBatch(maps, sensor, graph=True, autotune=True, persistent=True)
    ms_persist = timed(lambda i: batch.integrate(imgs[i], Ts[i], i))
    ptiles, _ = batch.tiles()
    for m in maps:
        m.check()
    del batch, maps
    # batched, no graph, default geometry
    maps = _lidar_maps(se, LIDAR_MAPS)
    batch = se.OccupancyBatch(maps, sensor, graph=False)
    ms_batch = timed(lambda i: batch.integrate(imgs[i], Ts[i], i))
    for m in maps:
        m.check()
    del batch, maps
    # one map per call
    maps = _lidar_maps(se, LIDAR_MAPS)
    integ = [se.MapIntegrator(m) for m in maps]
    ms_single = timed(lambda i: [integ[k].integrateDepth(i, imgs[i][k], sensor, Ts[i][k]) for k in range(LIDAR_MAPS)])
    for m in maps:
        m.check()
    del integ, maps
    # end to end: pinned host scans copied in every call (on a copy stream into two staging
    # buffers, step i + 1's copy issued before step i's integration), the maps' counters read back
    maps = _lidar_maps(se, LIDAR_MAPS)
    batch = se.OccupancyBatch(maps, sensor, graph=True, autotune=True)
    host = [im.cpu().pin_memory() for im in imgs]
    stage = [torch.empty_like(imgs[0]) for _ in range(2)]
    main, copy = torch.cuda.current_stream(dev), torch.cuda.Stream(dev)
    copied = [torch.cuda.Event() for _ in range(2)]
    consumed = [torch.cuda.Event() for _ in range(2)]

    def fetch(i):
        slot = i % 2
        copy.wait_event(consumed[slot])
        with torch.cuda.stream(copy):
            stage[slot].copy_(host[i], non_blocking=True)
            copied[slot].record(copy)

    def integrate(i):
        slot = i % 2
        main.wait_event(copied[slot])
        batch.integrate(stage[slot], Ts[i], i)
        consumed[slot].record(main)

    for k in range(2):
        consumed[k].record(main)
    for i in range(W):
        fetch(i)
        integrate(i)
    # each step's counters (8 maps x 4 int32) come back on the stream and are read on the host
    # while the next step runs
    stats = [(torch.zeros((LIDAR_MAPS, 4), dtype=torch.int32).pin_memory(), torch.cuda.Event()) for _ in range(2)]
    read = []
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    fetch(W)
    for i in range(W, W + K):
        if i + 1 < W + K:
            fetch(i + 1)
        integrate(i)
        buf, ev = stats[i % 2]
        batch.stats_async(buf)
        ev.record(main)
        if i > W:
            pbuf, pev = stats[(i - 1) % 2]
            pev.synchronize()
            read.append(pbuf.numpy().copy())
    torch.cuda.synchronize()
    read.append(stats[(W + K - 1) % 2][0].numpy().copy())
    e2e_s = time.perf_counter() - e0
    assert len(read) == K and all(r[:, 0].min() > 0 for r in read)
    for m in maps:
        m.check()
    del batch, maps
    scans = LIDAR_MAPS * K
    bd = 5  # 256^3 voxels: blocks at depth 5
    levels = 6  # pooling levels of a 64-row image
    launches = 1 + 1 + (levels - 1) + 1 + bd + 1 + (bd + 1) + 2 + (bd - 1) + 1
    return {
        "workload": f"{LIDAR_MAPS} multi-res occupancy maps (256^3 voxels at {LIDAR_RES} m, 8^3 blocks), "
                    f"LiDAR {spec.height}x{spec.width} (+-22.5 deg, {spec.near_plane}-{spec.far_plane} m), "
                    "seeded outdoor scene (ground + 100 boxes + 100 cylinders over 100 x 100 m), each map "
                    "driving its own road at 1 m per scan; one step = one scan into every map",
        "metric": "scans/s", "value": scans / (ms_graph * 1e-3), "ms_per_step": ms_graph / K,
        "steps": K, "warmup": W, "kept_return_fraction": keep, "valid_pixel_fraction": valid,
        "blocks_listed_last_step": blocks,
        "variants": {
            "batched_graph_autotuned": {"value": scans / (ms_graph * 1e-3), "ms_per_step": ms_graph / K,
                                        "tiles_ctas_per_sm": {"carve": tiles[0], "lists": tiles[1],
                                                              "blocks": tiles[2]}},
            "batched_persistent_graph_autotuned": {"value": scans / (ms_persist * 1e-3), "ms_per_step": ms_persist / K,
                                                   "launches_per_step": 1, "ctas_per_sm": ptiles[0]},
            "batched_no_graph": {"value": scans / (ms_batch * 1e-3), "ms_per_step": ms_batch / K},
            "one_map_per_call": {"value": scans / (ms_single * 1e-3), "ms_per_step": ms_single / K},
        },
        "e2e": {"value": scans / e2e_s, "unit": "scans/s",
                "h2d_bytes_per_step": LIDAR_MAPS * spec.width * spec.height * 4,
                "d2h_bytes_per_step": LIDAR_MAPS * 4 * 4,
                "api": "OccupancyBatch.integrate from staging buffers filled on a copy stream + stats_async; "
                       "step k's counters are read on the host while step k + 1 runs"},
        "gpu_launches_per_step": launches,
        "gen_s": gen_s,
        "l2": "flushed (256 MiB write) between steps",
        "_data": (spec, poses, ranges, W, K),
    }


RAY_WALL = dict(width=360, height=180, near_plane=0.6, far_plane=30.0, elevation_resolution_deg=0.1,
                azimuth_resolution_deg=0.1)


def _ray_wall_batch():
    from supereight2_gb300.synthetic import wall_rays
    return wall_rays()


def _ray_batch_bench(se, torch, dev, reps=5):
    """integrateRayBatch of the reference's Propagation batch (300 x 300 rays at 0.1 degree onto a
    wall 10 m away, 25.6 m map at 5 cm) into a fresh map per repetition; host wall clock around
    the synchronous call (the first, untimed, builds the scratch)."""
    rays = torch.from_numpy(_ray_wall_batch()).to(dev)
    poses = torch.eye(4, dtype=torch.float32, device=dev).expand(rays.shape[0], 4, 4).contiguous()
    T_MW = np.eye(4, dtype=np.float32)
    T_MW[:3, 3] = 12.8
    sensor = se.LeicaLidar(**RAY_WALL)
    times, n_oct = [], 0
    for r in range(reps + 1):
        m = se.Map(25.6, 0.05, res_type="multi", field="occupancy", T_MW=T_MW, max_blocks=1 << 16)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        n_oct = se.integrate_ray_batch(m, 0, poses, rays, sensor, with_octants=False)
        torch.cuda.synchronize()
        if r > 0:
            times.append(time.perf_counter() - t0)
        del m
    ms = 1e3 * float(np.median(times))
    return {"workload": "integrateRayBatch, LeicaLidar 0.1 deg, 90000 rays (300 x 300 over +-15 deg) onto a "
                        "wall 10 m away, multi-res occupancy map 25.6 m at 5 cm (512^3), fresh map per batch",
            "value": rays.shape[0] / (ms * 1e-3), "unit": "rays/s", "ms_per_batch": ms,
            "updated_octants": int(n_oct), "timing": f"host wall clock around the synchronous call, median of {reps}"}


def ray_batch_cpu_baseline():
    """The oracle's serial ray integrator (the reference's loop is serial) on the same batch."""
    from oracle import pyoracle as o
    rays = _ray_wall_batch()
    T_MW = np.eye(4, dtype=np.float32)
    T_MW[:3, 3] = 12.8
    m = o.OracleOccMap(25.6, 0.05, T_MW=T_MW)
    t0 = time.perf_counter()
    m.integrate_ray_batch(o.leica(**RAY_WALL), np.eye(4, dtype=np.float32), rays, 0)
    dt = time.perf_counter() - t0
    return {"value": len(rays) / dt, "unit": "rays/s", "cores": 1, "kind": "port",
            "sample": f"the whole 90000-ray batch, {dt:.1f} s"}


def lidar_cpu_baseline(data, budget_s=20.0):
    """The oracle (all host threads) integrating the same scans: map k's scans in order, the
    GPU's timed scans (after its warm-up) timed, maps in turn until budget_s is spent."""
    from oracle import pyoracle as o
    spec, poses, ranges, W, K = data
    o.set_num_threads(os.cpu_count() or 1)
    T_MW = np.eye(4, dtype=np.float32)
    T_MW[:3, 3] = (51.2, 51.2, 12.8)
    L = o.lidar(spec.width, spec.height, spec.elevation_min_deg, spec.elevation_max_deg,
                spec.near_plane, spec.far_plane)
    times = []
    t_start = time.perf_counter()
    n_maps = 0
    for k in range(len(poses)):
        m = o.OracleOccMap(102.4, LIDAR_RES, T_MW=T_MW)
        for i in range(W + K):
            t0 = time.perf_counter()
            m.integrate_lidar(ranges[k][i], L, poses[k][i].astype(np.float32), i)
            if i >= W:
                times.append(time.perf_counter() - t0)
        n_maps += 1
        del m
        if time.perf_counter() - t_start > budget_s:
            break
    return {"value": len(times) / sum(times), "unit": "scans/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"scans {W}..{W + K - 1} of {n_maps} of the {len(poses)} maps (each map's scans "
                      f"0..{W - 1} integrated untimed first), {sum(times):.1f} s of CPU work"}


# --------------------------------------------------------------------- CPU oracle arm --

def _oracle_pipeline(frames, poses, spec, n_warm, n_steps, budget_s=None, touched=None, timed_threads=None):
    """Run the oracle (OpenMP, all host threads) pipeline: integrate frame 0, run frames
    1..n_warm untimed, then time up to n_steps frames (stopping once budget_s is spent), on
    timed_threads threads if given. Returns the per-frame seconds of the timed frames."""
    from oracle import pyoracle as o
    o.set_num_threads(os.cpu_count() or 1)
    m = o.OracleMap(MAP_DIM, MAP_RES)
    s = o.pinhole(spec.width, spec.height, spec.fx, spec.fy, spec.cx, spec.cy,
                  spec.near_plane, spec.far_plane)
    cfg = o.tracker_config()
    T = poses[0].astype(np.float32)
    bl = dict(radius=2, sigma_space=4.0, sigma_range=0.03)  # the bilateral pre-filter of the tracking input
    m.integrate_depth(frames[0], s, T, 0)
    pts, nrm, _ = m.raycast(s, T)
    times = []
    t_start = None
    last = min(len(frames) - 1, n_warm + n_steps)
    for i in range(1, last + 1):
        if i == n_warm + 1:
            if timed_threads:
                o.set_num_threads(timed_threads)
            t_start = time.perf_counter()
        t0 = time.perf_counter()
        _, T, _ = o.track(s, cfg, o.bilateral_filter(frames[i], **bl), T, pts, nrm)
        m.integrate_depth(frames[i], s, T, i)
        pts, nrm, _ = m.raycast(s, T)
        if i > n_warm:
            times.append(time.perf_counter() - t0)
            if budget_s is not None and time.perf_counter() - t_start > budget_s:
                break
    if touched is not None:
        # untimed: the distinct voxels the raycast of the last timed frame reads
        touched.append(m.raycast_touched(s, T))
    o.set_num_threads(os.cpu_count() or 1)
    return times


def cpu_baseline(frames, poses, spec, n_warm, n_max, budget_s):
    touched = []
    times = _oracle_pipeline(frames, poses, spec, n_warm, n_max, budget_s, touched)
    # the same frames on one host thread (a shorter sample: the first timed frames)
    one = _oracle_pipeline(frames, poses, spec, n_warm, n_max, budget_s / 2, timed_threads=1)
    return {"value": len(times) / sum(times), "unit": "frames/s", "cores": os.cpu_count(),
            "raycast_voxels_touched": touched[0] if touched else None,
            "kind": "port",
            "sample": f"{len(times)} frames ({n_warm + 1}..{n_warm + len(times)}: the GPU's timed "
                      f"frames) of the same trajectory, track+integrate+raycast, after replaying "
                      f"frames 0..{n_warm} untimed; {sum(times):.1f} s of CPU work",
            "one_thread": {"value": len(one) / sum(one), "unit": "frames/s", "cores": 1,
                           "sample": f"frames {n_warm + 1}..{n_warm + len(one)} on one thread "
                                     f"({sum(one):.1f} s of CPU work), the warm-up replayed on all threads"}}


def run_reference(args, ws, rank, local):
    if rank != 0:
        return None
    n_frames = 1 + args.warmup + args.steps
    sensor_spec, scene, poses, frames = make_data(n_frames, "cpu")
    from oracle import pyoracle as o
    o.set_num_threads(os.cpu_count() or 1)
    # warm-up frames are folded into the run (the map must grow the same way); the timed sample
    # is bounded to ~120 s of CPU work
    timed = _oracle_pipeline(frames, poses, sensor_spec, args.warmup, args.steps,
                             budget_s=args.reference_budget_s)
    value = len(timed) / sum(timed)
    return {
        "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": ws,
        "steps": len(timed), "warmup": args.warmup, "ms_per_step": 1e3 * sum(timed) / len(timed),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded room)", "impl": "reference",
        "config": {"workload": "tsdf640: 640x480 pinhole, TSDF single-res 1024^3 @ 1 cm, "
                               "bilateral-filtered tracking input (5x5, 4 px, 0.03 m), "
                               "ICP 3 levels {10,5,4}, integrate + raycast per frame",
                   "parallelism": "OpenMP, all host threads"},
        "cpu_baseline": {"value": value, "unit": "frames/s", "cores": os.cpu_count(),
                         "kind": "port",
                         "sample": f"{len(timed)} timed frames after {args.warmup} warm-up "
                                   f"frames (bounded to {args.reference_budget_s:.0f} s)"},
        "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--storage", choices=["f32", "f16"], default="f32")
    ap.add_argument("--max-blocks", type=int, default=1 << 19)
    ap.add_argument("--cpu-budget-s", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-budget-s", type=float, default=120.0)
    ap.add_argument("--lidar-steps", type=int, default=20)
    ap.add_argument("--precision-frames", type=int, default=300,
                    help="frames of the FP64 precision report (0: no report)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    ws, rank, local = _dist()
    if args.impl == "reference":
        # the CPU arm runs on rank 0 only; other ranks exit without work
        out = run_reference(args, ws, rank, local)
        if rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
        return
    if ws > 1:
        import torch
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    out = run_ours(args, ws, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
