"""Generates the committed golden fixtures of tests/golden/ (run in a checkout next to the
supereight2 sources; not needed to run the tests).

reference_pins.json — values the reference's own tests assert, extracted from their sources:
  test/map/map/map_unittest.cpp (Map.initialization: dim, res, octree size) and
  test/system/multires_ofusion/multires_ofusion_systemtest.cpp (the voxels its GetField and
  GetFieldInterpolation tests check, with the expected data); and the dual-corner partition
  that meshing::norm_dual_corner_idxs (include/se/map/algorithms/impl/marching_cube_impl.hpp)
  tabulates for the 26 block-boundary positions of a primal corner; and the marching-cubes case
  table (include/se/map/algorithms/edge_tables.hpp, triTable) that both libraries decode from
  supereight2_gb300/csrc/mc_case_table.inc.
oracle_fixtures.npz — small seeded inputs (stored: five 320x240 depth frames with their poses,
  one 64x1024 LiDAR scan with its pose) and the CPU oracle's outputs on them, as per-block
  CRC32s and raw arrays, so the oracle built on another machine and the GPU path are both
  checked against one committed record: a 4-frame 320x240 TSDF integration (block keys, CRC of tsdf and
  weight per block), a raycast (CRC of points and normals), one ICP track (pose, reduction
  count), a LiDAR occupancy scan (block coordinates and CRC of the mean pyramid, counts), the
  bilateral filter and downsample_depth of one frame (CRC), and the marching-cubes face count.

    python tests/golden/make_golden.py path/to/supereight2
"""
import json
import os
import re
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def crc(a) -> int:
    return zlib.crc32(np.ascontiguousarray(a).tobytes()) & 0xffffffff


def reference_pins(src):
    pins = {}
    txt = open(os.path.join(src, "test/map/map/map_unittest.cpp")).read()
    body = txt[txt.index("TEST(Map, initialization)"):]
    body = body[body.index("std::vector<TestData> data{"):]
    body = body[: body.index("};")]
    pins["map_sizes"] = [[float(a), float(b), int(c)]
                         for a, b, c in re.findall(r"\{([\d.]+)f,\s*([\d.]+)f,\s*(\d+)\}", body)]
    txt = open(os.path.join(src, "test/system/multires_ofusion/multires_ofusion_systemtest.cpp")).read()

    def section(name):
        start = txt.index("TEST(MultiResOFusionSystemTest, %s)" % name)
        end = txt.find("\nTEST(", start + 1)
        return txt[start:end if end > 0 else len(txt)]

    def coords(body):
        return {n: [int(a), int(b), int(c)]
                for n, a, b, c in re.findall(r"Eigen::Vector3i (voxel_coord_\w+)\((\d+),\s*(\d+),\s*(\d+)\)", body)}

    interp = section("GetFieldInterpolation")
    ci = coords(interp)
    pins["occupancy_interp_free"] = [ci[n] for n in re.findall(r"map\.voxelToPoint\((voxel_coord_free_\d)", interp)]
    pins["occupancy_interp_value"] = float(re.findall(r"EXPECT_FLOAT_EQ\((-?[\d.]+),", interp)[0])
    field = section("GetField")
    cf = coords(field)
    pins["occupancy_unknown"] = [cf[n] for n in sorted(cf) if "unknown" in n]
    pins["occupancy_free"] = [cf[n] for n in sorted(cf) if "free" in n]
    pins["occupancy_free_value"] = float(re.findall(r"EXPECT_FLOAT_EQ\((-?[\d.]+),", field)[0])
    pins["dual_corner_partition"] = dual_corner_partition(src)
    pins["mc_tri_table"] = mc_tri_table(src)
    return pins


def mc_tri_table(src):
    """The 256 x 16 rows of triTable (edge_tables.hpp), -1 padded."""
    txt = open(os.path.join(src, "include/se/map/algorithms/edge_tables.hpp")).read()
    body = txt[txt.index("triTable[256][16]"):]
    body = body[body.index("{") + 1:]
    rows = [[int(v) for v in r.split(",") if v.strip()] for r in re.findall(r"\{([-\d,\s]+)\}", body)[:256]]
    assert len(rows) == 256 and all(len(r) == 16 for r in rows)
    return rows


def dual_corner_partition(src):
    """meshing::norm_dual_corner_idxs (marching_cube_impl.hpp): for every boundary position of a
    primal corner (crossmask: upper x, y, z, lower x, y, z bits from high to low) the corners of
    each neighbouring block (first: the meshed block) and the representative corners of the blocks
    ranking below and above the meshed block."""
    txt = open(os.path.join(src, "include/se/map/algorithms/impl/marching_cube_impl.hpp")).read()
    body = txt[txt.index("switch (crossmask)"):]
    body = body[: body.index("template<typename OctreeT, typename DataT>")]
    out = {}
    for m in re.finditer(r"case (\d+):(.*?)(?=case \d+:|\Z)", body, re.S):
        code = m.group(2)

        def ints(t):
            return [int(v) for v in re.findall(r"\d+", t)]

        lower = re.search(r"lower_priority_neighbours = \{([^}]*)\}", code).group(1)
        higher = re.search(r"higher_priority_neighbours = \{([^}]*)\}", code).group(1)
        nbrs = re.search(r"(?<!_)neighbours = \{(.*?)\};", code, re.S).group(1)
        out[m.group(1)] = {"lower": ints(lower), "higher": ints(higher),
                           "groups": [ints(g) for g in re.findall(r"\{([^{}]*)\}", nbrs)]}
    return out


def oracle_fixtures():
    from oracle import pyoracle as o
    from supereight2_gb300 import synthetic as syn
    o.set_num_threads(4)  # the ICP sums depend on the thread count (tested within the pose bar)
    out = {}
    spec, scene, poses, frames = syn.dataset("tsdf320", 5)
    # the inputs themselves: the scene generator's float64 ray tracing may round differently on
    # another machine, so the fixtures carry the exact frames and poses they were computed from
    out["frames"] = np.stack(frames).astype(np.float32)
    out["poses"] = np.stack(poses).astype(np.float32)
    s = o.pinhole(spec.width, spec.height, spec.fx, spec.fy, spec.cx, spec.cy, spec.near_plane, spec.far_plane)
    m = o.OracleMap(10.24, 0.02)
    frames, poses = out["frames"], out["poses"]
    for i in range(4):
        m.integrate_depth(frames[i], s, poses[i], i)
    keys, coords, tsdf, weight, ts = m.blocks()
    order = np.argsort(keys)
    out["tsdf_keys"] = keys[order]
    out["tsdf_crc"] = np.array([crc(tsdf[i]) ^ (crc(weight[i]) << 1 & 0xffffffff) for i in order], np.uint64)
    T = poses[3]
    pts, nrm, _ = m.raycast(s, T)
    out["raycast_crc"] = np.array([crc(pts), crc(nrm)], np.uint64)
    acc, T4, st = o.track(s, o.tracker_config(), o.bilateral_filter(frames[4]), T, pts, nrm)
    out["track_pose"] = T4.astype(np.float32)
    out["track_accepted"] = np.array([int(acc)])
    out["bilateral_crc"] = np.array([crc(o.bilateral_filter(frames[4]))], np.uint64)
    ds, dmap = o.downsample_depth(frames[4], 2)
    out["downsample_crc"] = np.array([crc(ds), crc(dmap)], np.uint64)
    out["mc_faces"] = np.array([len(m.marching_cubes())])
    # one LiDAR scan into an occupancy map
    lspec = syn.LIDAR_64
    scan = syn.render_range(syn.make_outdoor_scene(1004), lspec, syn.road_trajectory(0, 1)[0], 5, keep=0.6)
    T_S = syn.road_trajectory(0, 1)[0].astype(np.float32)
    out["lidar_scan"] = scan
    out["lidar_pose"] = T_S
    T_MW = np.eye(4, dtype=np.float32)
    T_MW[:3, 3] = (51.2, 51.2, 12.8)
    om = o.OracleOccMap(102.4, 0.4, T_MW=T_MW)
    L = o.lidar(lspec.width, lspec.height, lspec.elevation_min_deg, lspec.elevation_max_deg, lspec.near_plane,
                lspec.far_plane)
    st = om.integrate_lidar(scan, L, T_S, 0)
    out["occ_counts"] = np.array([st.n_blocks_listed, st.n_nodes_listed, st.n_blocks_freed, st.n_nodes_pruned])
    c, sc, cnt, mean, mn, mx = om.blocks()
    key = (c[:, 0].astype(np.int64) << 40) | (c[:, 1].astype(np.int64) << 20) | c[:, 2]
    order = np.argsort(key)
    out["occ_coords"] = c[order]
    out["occ_crc"] = np.array([crc(mean[i]) for i in order], np.uint64)
    # weights and observed flags are integers; the occupancies also as per-block sums
    out["occ_crc_int"] = np.array([crc(mean[i][:, 1:]) for i in order], np.uint64)
    out["occ_sum"] = np.array([mean[i][:, 0].astype(np.float64).sum() for i in order])
    out["occ_scales"] = sc[order]
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <supereight2 source tree>")
    src = sys.argv[1]
    with open(os.path.join(HERE, "reference_pins.json"), "w") as f:
        json.dump(reference_pins(src), f, indent=1)
    np.savez_compressed(os.path.join(HERE, "oracle_fixtures.npz"), **oracle_fixtures())
    print("written", os.listdir(HERE))


if __name__ == "__main__":
    main()
