// oracle_dual_mc.hpp — dual marching cubes of multi-resolution maps, part of the CPU oracle
// (test infrastructure only). A restatement of
//   algorithms::dual_marching_cube_kernel   include/se/map/algorithms/impl/marching_cube_impl.hpp:895-975
//   meshing::compute_dual_index             :763-805
//   meshing::gather_dual_data (in a block)  :269-289
//   meshing::gather_dual_data (across)      :683-758, with norm_dual_corner_idxs :311-680
//   meshing::compute_dual_intersection      :208-219
//   meshing::checkVertex                    :814-818
//   isosurface::occupied                    :25-41
// for any multi-res block store (a View, below). The triangulation comes from this oracle's own
// case table (the single-res rule), passed in by the caller.
//
// Dual corner i of a primal corner p sits at the logical voxel p + L_i with L_i = corner_i - 1
// (corner_i the unit-cube corner of marching-cube corner i, so L matches the reference's
// logical_dual_offset) and in the normalised direction N_i = 2 corner_i - 1. On a block face,
// edge or corner the dual corners fall into up to 8 blocks. norm_dual_corner_idxs tabulates,
// for the 26 boundary positions, which corners share a block and whether each neighbouring
// block ranks below or above the block being meshed; this oracle derives the same partition from
// a rule instead of a table:
//   - block offset of corner i along an axis: -1 if the primal corner lies on the block's lower
//     face (relative coordinate 0) and L_i = -1 there, +1 if it lies on the upper face
//     (relative coordinate 8) and L_i = 0 there, else 0; corners with equal offsets share a block;
//   - corner value v_i = 4 [N_i.x > 0] + 2 [N_i.y > 0] + [N_i.z > 0]; a group's value is the
//     minimum over its corners; a neighbouring group ranks below the meshed block when its value
//     is below the value of the corners inside the meshed block, above otherwise.
// A block ranking below must integrate at a strictly coarser scale than the meshed block, one
// ranking above at the same or a coarser scale; otherwise (or with the block missing, or the
// corner outside the map) the cube is skipped. The tests compare this partition with the one the
// reference tabulates.
#pragma once

#include <cstdint>
#include <vector>

namespace dual_mc {

struct Groups {
    int group_of[8];    // 0 = inside the meshed block, 1.. = neighbouring groups
    int n_groups;       // including the inside group
    int offset[8][3];   // block offset of each group
    int above[8];       // per group: 1 ranks above, 0 below (inside group: -1)
};

inline int corner_bit(int i, int a)
{
    static const int c[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}};
    return c[i][a];
}

inline int corner_value(int i) { return 4 * corner_bit(i, 0) + 2 * corner_bit(i, 1) + corner_bit(i, 2); }

// rel: primal corner relative to the block coordinate, each in [0, block_size].
inline Groups dual_groups(const int rel[3], int block_size)
{
    Groups g;
    g.n_groups = 1; // group 0: the corners inside the meshed block
    g.offset[0][0] = g.offset[0][1] = g.offset[0][2] = 0;
    int minv[8] = {8, 8, 8, 8, 8, 8, 8, 8};
    for (int i = 0; i < 8; ++i) {
        int off[3];
        for (int a = 0; a < 3; ++a) {
            const int c = corner_bit(i, a);
            off[a] = (rel[a] == 0 && c == 0) ? -1 : ((rel[a] == block_size && c == 1) ? 1 : 0);
        }
        int k = -1;
        for (int j = 0; j < g.n_groups && k < 0; ++j)
            if (g.offset[j][0] == off[0] && g.offset[j][1] == off[1] && g.offset[j][2] == off[2])
                k = j;
        if (k < 0) {
            k = g.n_groups++;
            for (int a = 0; a < 3; ++a)
                g.offset[k][a] = off[a];
        }
        g.group_of[i] = k;
        const int v = corner_value(i);
        if (v < minv[k])
            minv[k] = v;
    }
    g.above[0] = -1;
    for (int j = 1; j < g.n_groups; ++j)
        g.above[j] = minv[j] > minv[0] ? 1 : 0;
    return g;
}

/* View interface:
 *   int size() const;                         octree size in voxels
 *   int num_blocks() const;                   block ids 0 .. num_blocks()-1
 *   bool live(int b) const;                   false for deleted blocks
 *   const int32_t* coord(int b) const;        block coordinate
 *   int current_scale(int b) const;
 *   int block_at(const int32_t c[3]) const;   fetcher::block: block id or -1
 *   bool data(int b, const int32_t c[3], int scale, float& field) const;
 *                                             BlockT::data(c, scale): get_field and is_valid
 *   bool inside(float field) const;           is_inside
 */
template <class View>
long long dual_marching_cubes(const View& v, int min_desired_scale, const int32_t* ntri, const int32_t* tri,
                              int tri_stride, float* faces, int8_t* scales, long long capacity)
{
    static const int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {0, 3}, {4, 5}, {5, 6},
                                     {6, 7}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
    const int size = v.size();
    const int nb = v.num_blocks();
    std::vector<std::vector<float>> per_block((size_t) nb);
    std::vector<std::vector<int8_t>> per_block_scale((size_t) nb);
#pragma omp parallel for schedule(dynamic, 8)
    for (int b = 0; b < nb; ++b) {
        if (!v.live(b))
            continue;
        std::vector<float>& out = per_block[(size_t) b];
        std::vector<int8_t>& out_s = per_block_scale[(size_t) b];
        const int cur = v.current_scale(b);
        // std::clamp(min_desired_scale, current_scale, max_scale)
        const int voxel_scale = min_desired_scale < cur ? cur : (min_desired_scale > 3 ? 3 : min_desired_scale);
        const int stride = 1 << voxel_scale;
        const int32_t* start = v.coord(b);
        int32_t last[3];
        for (int a = 0; a < 3; ++a)
            last[a] = start[a] + 8 < size - 1 ? start[a] + 8 : size - 1;
        for (int x = start[0]; x <= last[0]; x += stride)
            for (int y = start[1]; y <= last[1]; y += stride)
                for (int z = start[2]; z <= last[2]; z += stride) {
                    const int32_t p[3] = {x, y, z};
                    if (x == last[0] || y == last[1] || z == last[2])
                        if (v.block_at(p) < 0)
                            continue;
                    float val[8];
                    bool ok[8];
                    float pos[8][3];
                    for (int i = 0; i < 8; ++i) {
                        ok[i] = false;
                        val[i] = 0.0f;
                    }
                    const bool local = !(x % 8 == 0 || y % 8 == 0 || z % 8 == 0);
                    if (local) {
                        // gather_dual_data in the block: p + (stride / 2) N_i at voxel_scale
                        const float h = (float) stride / 2;
                        for (int i = 0; i < 8; ++i) {
                            int32_t c[3];
                            for (int a = 0; a < 3; ++a) {
                                pos[i][a] = (float) p[a] + h * (float) (2 * corner_bit(i, a) - 1);
                                c[a] = (int32_t) pos[i][a];
                            }
                            ok[i] = v.data(b, c, voxel_scale, val[i]);
                        }
                    }
                    else {
                        const int rel[3] = {x - start[0], y - start[1], z - start[2]};
                        const Groups g = dual_groups(rel, 8);
                        int gblock[8], gscale[8];
                        gblock[0] = b;
                        gscale[0] = voxel_scale;
                        bool skip = false;
                        for (int j = 1; j < g.n_groups && !skip; ++j) {
                            int rep = -1;
                            for (int i = 0; i < 8 && rep < 0; ++i)
                                if (g.group_of[i] == j)
                                    rep = i;
                            int32_t c[3];
                            bool in_map = true;
                            for (int a = 0; a < 3; ++a) {
                                c[a] = p[a] + corner_bit(rep, a) - 1;
                                in_map = in_map && c[a] >= 0 && c[a] < size;
                            }
                            const int n = in_map ? v.block_at(c) : -1;
                            if (n < 0 || (g.above[j] ? v.current_scale(n) < cur : v.current_scale(n) <= cur)) {
                                skip = true;
                                break;
                            }
                            gblock[j] = n;
                            gscale[j] = v.current_scale(n) > voxel_scale ? v.current_scale(n) : voxel_scale;
                        }
                        if (skip)
                            continue; // cell index 0: no faces
                        for (int i = 0; i < 8; ++i) {
                            const int j = g.group_of[i];
                            const int s = 1 << gscale[j];
                            int32_t c[3];
                            for (int a = 0; a < 3; ++a) {
                                const int d = p[a] + corner_bit(i, a) - 1;
                                pos[i][a] = (float) ((d / s) * s) + (float) s * 0.5f;
                                c[a] = (int32_t) pos[i][a];
                            }
                            ok[i] = v.data(gblock[j], c, gscale[j], val[i]);
                        }
                    }
                    // isosurface::occupied
                    int cfg = 0;
                    bool valid = true;
                    for (int i = 0; i < 8; ++i) {
                        valid = valid && ok[i];
                        if (v.inside(val[i]))
                            cfg |= 1 << i;
                    }
                    if (!valid)
                        continue;
                    for (int f = 0; f < ntri[cfg]; ++f) {
                        float vert[9];
                        bool keep = true;
                        for (int j = 0; j < 3; ++j) {
                            const int e = tri[cfg * tri_stride + 3 * f + j];
                            const int a = kEdge[e][0], bb = kEdge[e][1];
                            const float s = (0.0f - val[a]) / (val[bb] - val[a]);
                            for (int k = 0; k < 3; ++k)
                                vert[3 * j + k] = pos[a][k] + s * (pos[bb][k] - pos[a][k]);
                            for (int k = 0; k < 3; ++k)
                                if (vert[3 * j + k] <= 0.0f || vert[3 * j + k] > (float) size)
                                    keep = false;
                        }
                        if (!keep)
                            continue;
                        out.insert(out.end(), vert, vert + 9);
                        out_s.push_back((int8_t) voxel_scale);
                    }
                }
    }
    long long n = 0;
    for (int b = 0; b < nb; ++b) {
        const long long k = (long long) per_block_scale[(size_t) b].size();
        for (long long j = 0; j < k && n + j < capacity; ++j) {
            if (faces)
                for (int q = 0; q < 9; ++q)
                    faces[9 * (n + j) + q] = per_block[(size_t) b][(size_t) (9 * j + q)];
            if (scales)
                scales[n + j] = per_block_scale[(size_t) b][(size_t) j];
        }
        n += k;
    }
    return n;
}

} // namespace dual_mc
