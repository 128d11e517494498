// occupancy.cu — se::MapIntegrator::integrateDepth for multi-resolution occupancy maps and a
// pinhole camera (map_integrator_impl.hpp:90-130), as stream-ordered launches:
//   sigma          uncert::depth_sigma (uncertainty.cpp:12-34)
//   pooling        DensePoolingImage<PinholeCamera> of the depth and sigma images
//                  (dense_pooling_image_impl.hpp:56-213): one launch per level
//   carve          VolumeCarver (volume_carver_impl.hpp:46-310) breadth first: one launch per
//                  octree depth over that depth's octants; a split node allocates its 8 children
//                  (Octree::allocateChildren) and queues them for the next depth
//   free nodes     Updater::freeNodeRecurse (multires_ofusion_updater_impl.hpp:550-600) breadth
//                  first over the free-space nodes' subtrees, then freeBlock on the blocks below
//   update         Updater::updateBlock (:296-409) on the carver's blocks, one warp per block
//   propagate      propagate_block_to_coarsest_scale on updated and freed blocks, then
//                  propagateToRoot (:129-164) one depth per launch from the blocks' parents up,
//                  with pruning, and the root
// The reference's recursion and OpenMP loops visit independent octants; the breadth-first
// launches visit the same octants with the same per-octant computation, so the allocated
// octree, the block lists (as sets) and every voxel agree with a serial run.
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "occupancy.cuh"
#include "pipeline.cuh"
#include "profile.cuh"

namespace se_gpu {

struct OccFrame {
    Pinhole s;
    Tf T_WS, T_SW;
    int w, h, levels;
    float tau_min, tau_max, sigma_min, sigma_max;
    int frame_id;
};

struct OccScratch {
    int w = 0, h = 0, levels = 0;
    float* sigma = nullptr;
    float4* pool_depth = nullptr; // levels * w * h of (min, max, crossing, known)
    float4* pool_sigma = nullptr;
    float* max_value = nullptr;   // [0] max pooled depth, [1] max_depth_value
    int* frontier[2] = {nullptr, nullptr};
    int* block_list = nullptr;    // slot block index
    int* block_var = nullptr;     // 0 Constant, 1 Gradient, 2 Undefined
    int* block_inside = nullptr;
    int* node_list = nullptr;
    int* freed = nullptr;
    int2* work[2] = {nullptr, nullptr}; // (node, depth)
    int* sets = nullptr;          // per depth, node_capacity entries each
    int set_depths = 0;
};

} // namespace se_gpu

struct se_gpu_occ_map {
    se_gpu::OccDevice dev;
    se_gpu::OccScratch scratch;
    int frame_id;
};

namespace se_gpu {

// ------------------------------------------------------------------ per-pixel inputs --

__global__ void occ_sigma_kernel(const float* __restrict__ depth, int n, float smin, float smax, float k_sigma,
                                 float* __restrict__ sigma)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float d = depth[i];
    if (d <= 0.0f || isnan(d)) {
        sigma[i] = 0.0f;
        return;
    }
    const float v = k_sigma * d;
    sigma[i] = v < smin ? smin : (smax < v ? smax : v); // std::clamp
}

// Pixel::knownPixel / unknownPixel: min = FLT_MAX, max = FLT_MIN (the smallest normal float)
__global__ void pool_l0_kernel(const float* __restrict__ img, int w, int h, float4* __restrict__ L0)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h)
        return;
    const float d = img[i];
    L0[i] = d <= 0.0f ? make_float4(FLT_MAX, FLT_MIN, 0.0f, 2.0f) : make_float4(d, d, 0.0f, 0.0f);
}

__global__ void pool_l1_kernel(const float4* __restrict__ L0, int w, int h, float4* __restrict__ L1)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h)
        return;
    const int x = i % w, y = i / w;
    float4 p = make_float4(FLT_MAX, FLT_MIN, 1.0f, 0.0f); // crossingKnownPixel
    if (y >= 1 && y < h - 1 && x >= 1 && x < w - 1)
        p.z = 0.0f;
    const int top = y > 0 ? y - 1 : 0, bottom = y < h - 1 ? y + 1 : h - 1;
    const int left = x > 0 ? x - 1 : 0, right = x < w - 1 ? x + 1 : w - 1;
    const int xs[9] = {x, left, x, right, right, right, x, left, left};
    const int ys[9] = {y, top, top, top, y, bottom, bottom, bottom, y};
    float mn = FLT_MAX, mx = -FLT_MAX;
    int uf = 0;
    for (int k = 0; k < 9; ++k) {
        const float4 q = L0[xs[k] + ys[k] * w];
        mn = fminf(mn, q.x);
        mx = fmaxf(mx, q.y);
        uf += (int) q.w;
    }
    p.x = mn;
    p.y = mx;
    if (uf == 18)
        p.w = 2.0f;
    else if (uf > 0)
        p.w = 1.0f;
    L1[i] = p;
}

__global__ void pool_lk_kernel(const float4* __restrict__ P, int w, int h, int s, float4* __restrict__ L)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h)
        return;
    const int x = i % w, y = i / w;
    float4 p = make_float4(FLT_MAX, FLT_MIN, 1.0f, 0.0f);
    const int s_half = s / 2;
    int left, right, top, bottom;
    if (x - s_half < 0) {
        left = 0;
        p.z = 1.0f;
    }
    else
        left = x - s_half;
    if (x + s_half >= w) {
        right = w - 1;
        p.z = 1.0f;
    }
    else
        right = x + s_half;
    if (y - s_half < 0) {
        top = 0;
        p.z = 1.0f;
    }
    else
        top = y - s_half;
    if (y + s_half >= h) {
        bottom = h - 1;
        p.z = 1.0f;
    }
    else
        bottom = y + s_half;
    const float4 a = P[left + top * w], b = P[right + top * w], c = P[left + bottom * w], d = P[right + bottom * w];
    p.x = fminf(fminf(a.x, b.x), fminf(c.x, d.x));
    p.y = fmaxf(fmaxf(a.y, b.y), fmaxf(c.y, d.y));
    const int uf = (int) a.w + (int) b.w + (int) c.w + (int) d.w;
    if (uf == 8)
        p.w = 2.0f;
    else if (uf > 0)
        p.w = 1.0f;
    if (y >= s && y < h - s && x >= s && x < w - s)
        p.z = 0.0f;
    L[i] = p;
}

// DensePoolingImage::maxValue over the coarsest level, then VolumeCarver's max_depth_value
__global__ void pool_max_kernel(const float4* __restrict__ Lmax, int w, int h, int max_level, float far_plane,
                                float tau_max, float* out)
{
    const int s = 1 << (max_level - 1);
    float mv = 0.0f;
    for (int v = s; true; v += 2 * s) {
        if (v > h - s - 1)
            v = h - s - 1;
        for (int u = s; true; u += 2 * s) {
            if (u > w - s - 1)
                u = w - s - 1;
            const float m = Lmax[u + w * v].y;
            if (mv < m)
                mv = m;
            if (u == w - s - 1)
                break;
        }
        if (v == h - s - 1)
            break;
    }
    out[0] = mv;
    const float t = mv + tau_max;
    out[1] = far_plane < t ? far_plane : t;
}

struct PoolQuery {
    float min, max;
    int crossing, known;
};

// DensePoolingImage<PinholeCamera>::poolBoundingBox (dense_pooling_image_impl.hpp:218-290)
__device__ PoolQuery pool_bounding_box(const float4* __restrict__ pool, int w, int h, int max_level, int u_min,
                                       int u_max, int v_min, int v_max)
{
    const int min_side = min(u_max - u_min, v_max - v_min);
    const int half = min_side / 2;
    // log2(0) = -inf: the reference's clamps turn it into level 0
    int lc = INT_MIN;
    if (half > 0)
        lc = (int) ceil(log2((double) half));
    const int level = max(0, min(max_level, lc));
    const int s = level > 0 ? 1 << max(level - 1, 0) : 0;
    PoolQuery b{FLT_MAX, FLT_MIN, 0, 0};
    unsigned long long n = 0, n_unknown = 0, n_part = 0;
    const int step = 2 * s + 1;
    const float4* L = pool + (size_t) level * w * h;
    for (int v = v_min + s; true; v += step) {
        if (v > v_max - s)
            v = v_max - s;
        for (int u = u_min + s; true; u += step) {
            if (u > u_max - s)
                u = u_max - s;
            const float4 p = L[u + w * v];
            if (b.max < p.y)
                b.max = p.y;
            if (b.min > p.x)
                b.min = p.x;
            if (p.w == 2.0f) {
                ++n_unknown;
                ++n_part;
            }
            else if (p.w == 1.0f) {
                ++n_part;
            }
            ++n;
            if (u == u_max - s)
                break;
        }
        if (v == v_max - s)
            break;
    }
    if (n == n_unknown)
        b.known = 2;
    else if (n_part > 0)
        b.known = 1;
    return b;
}

// DensePoolingImage<PinholeCamera>::conservativeQuery (dense_pooling_image_impl.hpp:295-347)
__device__ PoolQuery conservative_query(const float4* __restrict__ pool, int w, int h, int max_level, int u_min,
                                        int v_min, int u_max, int v_max)
{
    bool u_in = true, u_out = false, v_in = true, v_out = false;
    const float wl = (float) (unsigned) (w - 1), hl = (float) (unsigned) (h - 1);
    if ((float) u_min < 0.0f) {
        u_in = false;
        u_min = 0;
        if ((float) u_max < 0.0f)
            u_out = true;
    }
    else if ((float) u_min > wl) {
        u_out = true;
    }
    if ((float) u_max > wl) {
        u_in = false;
        u_max = w - 1;
    }
    if ((float) v_min < 0.0f) {
        v_in = false;
        v_min = 0;
        if ((float) v_max < 0.0f)
            v_out = true;
    }
    else if ((float) v_min > hl) {
        v_out = true;
    }
    if ((float) v_max > hl) {
        v_in = false;
        v_max = h - 1;
    }
    if (u_out || v_out || u_min == u_max || v_min == v_max)
        return PoolQuery{0.0f, 0.0f, 2, 2};
    PoolQuery p = pool_bounding_box(pool, w, h, max_level, u_min, u_max, v_min, v_max);
    if (!u_in || !v_in)
        p.crossing = 1;
    return p;
}

// ---------------------------------------------------------------------- allocation --

__device__ __forceinline__ void occ_aabb_extend(const OccDevice& m, int x, int y, int z, int sz)
{
    atomicMin(&m.aabb[0], x);
    atomicMin(&m.aabb[1], y);
    atomicMin(&m.aabb[2], z);
    atomicMax(&m.aabb[3], x + sz - 1);
    atomicMax(&m.aabb[4], y + sz - 1);
    atomicMax(&m.aabb[5], z + sz - 1);
    m.aabb[6] = 0;
}

// Octree::allocateChildren (octree_impl.hpp:200-233); only the thread that owns node n calls it
__device__ void occ_allocate_children(const OccDevice& m, int n)
{
    const OccD init = node_data(m, n);
    const int4 nc = m.node_coord[n];
    const int csize = nc.w / 2;
    const bool blocks_below = nc.w == 16;
    int* child = m.node_child + 8 * (size_t) n;
    for (int i = 0; i < 8; ++i) {
        if (child[i] != -1)
            continue;
        const int cx = nc.x + csize * (i & 1), cy = nc.y + csize * ((i >> 1) & 1), cz = nc.z + csize * (i >> 2);
        if (blocks_below) {
            const int b = atomicAdd(&m.counters[kOccBlocks], 1);
            if (b >= m.block_capacity) {
                atomicOr(&m.counters[kOccError], kOccErrBlockPool);
                continue;
            }
            m.block_coord[3 * b] = cx;
            m.block_coord[3 * b + 1] = cy;
            m.block_coord[3 * b + 2] = cz;
            OccBlockState st;
            st.init_data = init;
            st.min_scale = -1;
            st.current_scale = kOccMaxScale;
            st.finest = kOccMaxScale;
            st.buffer_scale = -1;
            st.curr_integr = st.curr_obs = st.buf_integr = st.buf_obs = 0ull;
            st.parent = n;
            st.live = 1;
            m.block_state[b] = st;
            blk_mean(m, b, kOccMaxScale)[0] = init;
            child[i] = -2 - b;
        }
        else {
            const int c = atomicAdd(&m.counters[kOccNodes], 1);
            if (c >= m.node_capacity) {
                atomicOr(&m.counters[kOccError], kOccErrNodePool);
                continue;
            }
            m.node_coord[c] = make_int4(cx, cy, cz, csize);
            m.node_parent[c] = n;
            for (int k = 0; k < 8; ++k)
                m.node_child[8 * (size_t) c + k] = -1;
            m.node_min[c] = init;
            m.node_max[c] = init;
            m.node_mark[c] = -1;
            m.node_ts[c] = -1;
            child[i] = c;
        }
    }
    if (blocks_below)
        occ_aabb_extend(m, nc.x, nc.y, nc.z, nc.w);
}

__global__ void occ_carve_root_kernel(OccDevice m, int* frontier, int* frontier_n)
{
    occ_allocate_children(m, 0);
    int n = 0;
    for (int i = 0; i < 8; ++i)
        if (m.node_child[i] != -1)
            frontier[n++] = m.node_child[i];
    *frontier_n = n;
}

__device__ __forceinline__ int push(int* list, int* count, int cap, int v, int* err)
{
    const int k = atomicAdd(count, 1);
    if (k < cap)
        list[k] = v;
    else
        atomicOr(err, kOccErrList);
    return k;
}

// VolumeCarver<.., PinholeCamera>::operator()(octant) (volume_carver_impl.hpp:132-310)
__global__ void __launch_bounds__(128) occ_carve_kernel(OccDevice m, OccFrame f, const float4* __restrict__ pool_d,
                                                        const float4* __restrict__ pool_s,
                                                        const float* __restrict__ maxv, const int* __restrict__ in,
                                                        const int* __restrict__ in_n, int* out, int* out_n,
                                                        int* block_list, int* block_var, int* block_inside,
                                                        int* node_list, int depth)
{
    const int n_in = *in_n < (m.node_capacity + m.block_capacity) ? *in_n : (m.node_capacity + m.block_capacity);
    const float max_depth_value = maxv[1];
    int* err = &m.counters[kOccError];
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n_in; idx += gridDim.x * blockDim.x) {
        const int slot = in[idx];
        const bool is_block = slot_is_block(slot);
        int cx, cy, cz, size;
        if (is_block) {
            const int b = slot_block(slot);
            cx = m.block_coord[3 * b];
            cy = m.block_coord[3 * b + 1];
            cz = m.block_coord[3 * b + 2];
            size = 8;
        }
        else {
            const int4 nc = m.node_coord[slot];
            cx = nc.x;
            cy = nc.y;
            cz = nc.z;
            size = nc.w;
        }
        const float size_to_radius = sqrtf(3.0f) / 2.0f;
        const float zero_depth_band = 1.0e-6f;
        const float off = (float) size * 0.5f;
        const F3 centre_W =
            apply(m.T_WM, f3(((float) cx + off) * m.res, ((float) cy + off) * m.res, ((float) cz + off) * m.res));
        const F3 centre_S = apply(f.T_SW, centre_W);
        const float rad = (float) size * size_to_radius * m.res;
        if (centre_S.z - rad > max_depth_value || centre_S.z + rad < zero_depth_band)
            continue;
        F3 cS[8];
        int n_front = 0;
        for (int k = 0; k < 8; ++k) {
            const F3 p_M = f3(((float) size * (float) (k & 1) + (float) cx) * m.res,
                              ((float) size * (float) ((k >> 1) & 1) + (float) cy) * m.res,
                              ((float) size * (float) (k >> 2) + (float) cz) * m.res);
            cS[k] = apply(f.T_SW, apply(m.T_WM, p_M));
            if (!(cS[k].z < zero_depth_band))
                ++n_front;
        }
        if (n_front == 0)
            continue;
        float pu[8], pv[8];
        bool ok[8];
        for (int k = 0; k < 8; ++k) {
            const F3 p = cS[k];
            if (fabsf(p.z) < 1.0e-12f) {
                pu[k] = pv[k] = 0.0f;
                ok[k] = false;
                continue;
            }
            const float rz = 1.0f / p.z;
            pu[k] = f.s.fx * (p.x * rz) + f.s.cx;
            pv[k] = f.s.fy * (p.y * rz) + f.s.cy;
            ok[k] = p.z > 0.0f && pu[k] >= -0.5f && pu[k] < (float) f.s.w - 0.5f && pv[k] >= -0.5f
                && pv[k] < (float) f.s.h - 0.5f;
        }
        bool should_split = false, projects_inside = false;
        int var = 1; // Gradient
        if (n_front < 8) {
            // cameraInNode with pointToVoxel<Safe::On>
            float vx = -1.0f, vy = -1.0f, vz = -1.0f;
            const F3 p_M = apply(m.T_MW, f3(f.T_WS.t[0], f.T_WS.t[1], f.T_WS.t[2]));
            if (p_M.x >= 0.0f && p_M.x < m.dim && p_M.y >= 0.0f && p_M.y < m.dim && p_M.z >= 0.0f && p_M.z < m.dim) {
                vx = p_M.x / m.res;
                vy = p_M.y / m.res;
                vz = p_M.z / m.res;
            }
            const bool cam_in = vx >= (float) cx && vx <= (float) (cx + size) && vy >= (float) cy
                && vy <= (float) (cy + size) && vz >= (float) cz && vz <= (float) (cz + size);
            bool crosses = false;
            for (int k = 0; k < 8; ++k)
                crosses = crosses || ok[k];
            if (cam_in || crosses) {
                should_split = true;
            }
            else {
                bool in_f = true;
                for (int i = 0; i < 5; ++i) {
                    const float d = ((centre_S.x * f.s.planes[i][0] + centre_S.y * f.s.planes[i][1])
                                     + centre_S.z * f.s.planes[i][2])
                        + f.s.planes[i][3];
                    if (d < -rad)
                        in_f = false;
                }
                if (!in_f)
                    continue;
                should_split = true;
            }
        }
        else {
            float umin = 0.0f, umax = 0.0f, vmin = 0.0f, vmax = 0.0f, zmin = 0.0f, zmax = 0.0f;
            for (int k = 0; k < 8; ++k) {
                float u = pu[k] > 1e7f ? 1e7f : pu[k];
                float v = pv[k] > 1e7f ? 1e7f : pv[k];
                u = u < -1e7f ? -1e7f : u;
                v = v < -1e7f ? -1e7f : v;
                if (k == 0) {
                    umin = umax = u;
                    vmin = vmax = v;
                    zmin = zmax = cS[0].z;
                }
                else {
                    umin = fminf(umin, u);
                    umax = fmaxf(umax, u);
                    vmin = fminf(vmin, v);
                    vmax = fmaxf(vmax, v);
                    zmin = fminf(zmin, cS[k].z);
                    zmax = fmaxf(zmax, cS[k].z);
                }
            }
            const int bu0 = (int) umin, bv0 = (int) vmin, bu1 = (int) umax, bv1 = (int) vmax;
            const PoolQuery pp = conservative_query(pool_d, f.w, f.h, f.levels - 1, bu0, bv0, bu1, bv1);
            if (pp.known == 2)
                continue;
            if (zmin > pp.max + f.tau_max)
                continue;
            const PoolQuery sp = conservative_query(pool_s, f.w, f.h, f.levels - 1, bu0, bv0, bu1, bv1);
            // computeVariance (volume_carver_impl.hpp:100-126)
            {
                const float z_diff_max = zmax - pp.min;
                const float z_diff_min = zmin - pp.max;
                const float tv = m.cfg.k_tau * pp.max;
                const float tau_max = tv < f.tau_min ? f.tau_min : (f.tau_max < tv ? f.tau_max : tv);
                const float three_sigma_min = 3.0f * sp.max;
                if ((double) z_diff_min > 1.25 * (double) tau_max)
                    var = 2;
                else if ((double) z_diff_max < -1.25 * (double) three_sigma_min)
                    var = 0;
                else
                    var = 1;
            }
            if (var != 1) {
                OccD cd;
                if (is_block) {
                    const int b = slot_block(slot);
                    const OccBlockState& st = m.block_state[b];
                    cd = blk_max(m, b, st.finest, kOccMaxScale)[0];
                }
                else {
                    cd = node_data(m, slot);
                }
                if (cd.observed && (double) occ_field(cd) <= 0.95 * -100.0)
                    continue;
            }
            if (pp.crossing == 1)
                should_split = true;
            else if (pp.known == 1)
                should_split = true;
            else if (var == 1)
                should_split = true;
            projects_inside = pp.known == 0;
        }
        if (is_block) {
            const int k = push(block_list, &m.counters[kOccBlockListN], m.block_capacity, slot_block(slot), err);
            if (k < m.block_capacity) {
                block_var[k] = var;
                block_inside[k] = projects_inside ? 1 : 0;
            }
        }
        else if (should_split) {
            occ_allocate_children(m, slot);
            for (int i = 0; i < 8; ++i) {
                const int ch = m.node_child[8 * (size_t) slot + i];
                if (ch != -1) // -1 only when a pool ran out (latched in the error word)
                    push(out, out_n, m.node_capacity + m.block_capacity, ch, err);
            }
        }
        else if (var == 0) {
            push(node_list, &m.counters[kOccNodeListN], m.node_capacity, slot, err);
        }
    }
    (void) depth;
}

__global__ void occ_leaf_aabb_kernel(OccDevice m, const int* __restrict__ node_list)
{
    const int n = min(m.counters[kOccNodeListN], m.node_capacity);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int node = node_list[i];
        if (node_is_leaf(m, node)) {
            const int4 c = m.node_coord[node];
            occ_aabb_extend(m, c.x, c.y, c.z, c.w);
        }
    }
}

// ---------------------------------------------------------------- propagation sets --

__device__ __forceinline__ int occ_node_depth(const OccDevice& m, int n)
{
    return m.log2_size - (31 - __clz(m.node_coord[n].w));
}

// Insert node n into the propagation set of its depth (std::set semantics: once per frame).
__device__ __forceinline__ void occ_set_insert(const OccDevice& m, int* sets, int n, int frame_id)
{
    if (n < 0)
        return;
    if (atomicExch(&m.node_mark[n], frame_id) == frame_id)
        return;
    const int d = occ_node_depth(m, n);
    const int k = atomicAdd(&m.counters[kOccSetN + d], 1);
    if (k < m.node_capacity)
        sets[(size_t) d * m.node_capacity + k] = n;
    else
        atomicOr(&m.counters[kOccError], kOccErrList);
}

// ---------------------------------------------------------------- block state machine --

// Sums a per-lane flag over the warp.
__device__ __forceinline__ unsigned warp_count(bool b) { return __popc(__ballot_sync(0xffffffffu, b)); }

__device__ __forceinline__ void occ_update(OccD& d, float value, float max_weight)
{
    if (d.weight < max_weight)
        d.weight = d.weight + 1.0f;
    d.occ = (d.occ * (d.weight - 1.0f) + value) / d.weight;
    d.observed = 1;
}

__device__ __forceinline__ float clampf_std(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }

// computeIntegrationScaleImpl (pinhole_camera.cpp:115-152), default ratios {1.5, 3, 6}
__device__ int occ_integration_scale(const Pinhole& s, float z, float res, int last_scale, int min_scale)
{
    for (int pass = 0; pass < 2; ++pass) {
        const float pv = (z * s.inv_fx) / res;
        int scale = 0;
        if (pv >= 1.5f) {
            scale = 1;
            if (pv >= 3.0f) {
                scale = 2;
                if (pv >= 6.0f)
                    scale = 3;
            }
        }
        if (pass == 0 && min_scale != -1 && scale != last_scale) {
            z = scale > last_scale ? z - 0.25f : z + 0.25f;
            continue;
        }
        return scale;
    }
    return 0;
}

// allocateDownTo (block_impl.hpp:540-586) by a whole warp; st is lane 0's copy
__device__ void occ_allocate_down_to(const OccDevice& m, int b, OccBlockState& st, int new_min, int lane)
{
    if (new_min >= st.current_scale)
        return;
    for (int s = st.current_scale; s >= new_min; --s) {
        OccD* d = blk_mean(m, b, s);
        const int nv = (8 >> s) * (8 >> s) * (8 >> s);
        if (s != st.current_scale)
            for (int i = lane; i < nv; i += 32)
                d[i] = st.init_data;
        __syncwarp();
        if (s != new_min) {
            OccD* mn = m.block_min + (size_t) b * 585 + occ_scale_offset(s);
            OccD* mx = m.block_max + (size_t) b * 585 + occ_scale_offset(s);
            for (int i = lane; i < nv; i += 32) {
                mn[i] = d[i];
                mx[i] = d[i];
            }
        }
        __syncwarp();
    }
    st.finest = new_min;
    st.current_scale = new_min;
    st.min_scale = new_min;
}

// the buffer set-up of updateBlock / freeBlock when the recommended scale differs
__device__ void occ_prepare_buffer(const OccDevice& m, int b, OccBlockState& st, int rec, int last_scale, int lane)
{
    if (rec == st.buffer_scale)
        return;
    st.buffer_scale = rec; // initBuffer: resetBuffer then the new scale
    st.buf_integr = 0ull;
    st.buf_obs = 0ull;
    OccD* buf = blk_buffer(m, b, st);
    if (rec < st.current_scale) {
        const int nv = (8 >> rec) * (8 >> rec) * (8 >> rec);
        for (int i = lane; i < nv; i += 32)
            buf[i] = occ_default();
        __syncwarp();
    }
    if (rec < last_scale) {
        const unsigned np = 8u >> last_scale, np2 = np * np;
        const unsigned nb = np << 1, nb2 = nb * nb;
        const OccD* cur = blk_mean(m, b, st.current_scale);
        for (unsigned k = lane; k < np * np2 * 8; k += 32) {
            const unsigned pidx = k >> 3, c = k & 7;
            const unsigned x = pidx % np, y = (pidx / np) % np, z = pidx / np2;
            const unsigned i = c & 1, j = (c >> 1) & 1, kk = c >> 2;
            const OccD pd = cur[x + y * np + z * np2];
            OccD& bd = buf[(2 * x + i) + (2 * y + j) * nb + (2 * z + kk) * nb2];
            bd.occ = pd.occ;
            bd.weight = pd.weight;
            bd.observed = 0;
        }
        __syncwarp();
    }
}

// switchData (block_impl.hpp:718-780); returns true when the block switched scales
__device__ bool occ_switch_data(const OccDevice& m, int b, OccBlockState& st, int lane)
{
    const bool go = st.buf_integr >= 20ull
        && (double) (st.buf_obs * (unsigned long long) ((1 << st.buffer_scale) * (1 << st.buffer_scale)
                                                        * (1 << st.buffer_scale)))
            >= 0.9
                * (double) (st.curr_obs
                            * (unsigned long long) ((1 << st.current_scale) * (1 << st.current_scale)
                                                    * (1 << st.current_scale)));
    if (!go)
        return false;
    const int bs = st.buffer_scale;
    const int nv = (8 >> bs) * (8 >> bs) * (8 >> bs);
    if (bs < st.current_scale) {
        const OccD* buf = m.block_buffer + (size_t) b * 512;
        OccD* d = blk_mean(m, b, bs);
        for (int i = lane; i < nv; i += 32)
            d[i] = buf[i];
        const int nv1 = (8 >> (bs + 1)) * (8 >> (bs + 1)) * (8 >> (bs + 1));
        OccD* mn = m.block_min + (size_t) b * 585 + occ_scale_offset(bs + 1);
        OccD* mx = m.block_max + (size_t) b * 585 + occ_scale_offset(bs + 1);
        for (int i = lane; i < nv1; i += 32) {
            mn[i] = occ_default();
            mx[i] = occ_default();
        }
        st.finest = bs;
    }
    else if (!(bs <= st.min_scale || st.min_scale == -1)) { // deleteUpTo
        st.finest = bs;
        st.min_scale = bs;
    }
    __syncwarp();
    OccD* d = blk_mean(m, b, bs);
    unsigned long long added = 0;
    for (int base = 0; base < nv; base += 32) {
        const int i = base + lane;
        bool f = false;
        if (i < nv) {
            OccD e = d[i];
            if (e.weight > 0.0f && !e.observed) {
                e.observed = 1;
                d[i] = e;
                f = true;
            }
        }
        added += warp_count(f);
    }
    st.buf_obs += added;
    st.current_scale = bs;
    st.min_scale = bs;
    st.curr_integr = st.buf_integr;
    st.curr_obs = st.buf_obs;
    st.buffer_scale = -1;
    st.buf_integr = 0ull;
    st.buf_obs = 0ull;
    __syncwarp();
    return true;
}

__device__ __forceinline__ void occ_incr_buffer_integr(OccBlockState& st, bool do_increment)
{
    if (do_increment
        || (double) (st.buf_obs * (unsigned long long) ((1 << st.buffer_scale) * (1 << st.buffer_scale)
                                                        * (1 << st.buffer_scale)))
            >= 0.90
                * (double) (st.curr_obs
                            * (unsigned long long) ((1 << st.current_scale) * (1 << st.current_scale)
                                                    * (1 << st.current_scale))))
        ++st.buf_integr;
}

// updateBlockData<UpdateBuffer> (multires_ofusion_updater_impl.hpp:413-545) by a warp
__device__ void occ_update_block_data(const OccDevice& m, const OccFrame& f, const float* __restrict__ depth,
                                      const float* __restrict__ sigma, int b, OccBlockState& st, F3 centre_C,
                                      int scale, bool low_var, bool inside, bool to_buffer, int lane)
{
    const int stride = 1 << scale;
    const int n = 8 >> scale, n2 = n * n;
    const int cx = m.block_coord[3 * b], cy = m.block_coord[3 * b + 1], cz = m.block_coord[3 * b + 2];
    const float off = (float) stride * 0.5f;
    const F3 base_C = apply(f.T_SW, apply(m.T_WM, f3(((float) cx + off) * m.res, ((float) cy + off) * m.res,
                                                   ((float) cz + off) * m.res)));
    const float rs = m.res * (float) stride;
    float D[9];
    for (int i = 0; i < 9; ++i)
        D[i] = f.T_SW.R[i] * rs;
    const float tv = m.cfg.k_tau * centre_C.z;
    const float tau = clampf_std(tv, f.tau_min, f.tau_max);
    OccD* data = to_buffer ? blk_buffer(m, b, st) : blk_mean(m, b, st.current_scale);
    const float lom = m.cfg.log_odd_min, lomax = m.cfg.log_odd_max;
    unsigned long long newly_total = 0;
    for (int base = 0; base < n * n2; base += 32) {
        const int k = base + lane;
        bool newly = false;
        if (k < n * n2) {
            const int x = k % n, y = (k / n) % n, z = k / n2;
            const float fx = (float) x, fy = (float) y, fz = (float) z;
            const F3 dl = f3((D[0] * fx + D[1] * fy) + D[2] * fz, (D[3] * fx + D[4] * fy) + D[5] * fz,
                             (D[6] * fx + D[7] * fy) + D[8] * fz);
            const F3 p = add(base_C, dl);
            float u, v;
            if (project(f.s, p, u, v)) {
                const int px = (int) (u + 0.5f), py = (int) (v + 0.5f);
                const float dv = depth[px + py * f.s.w];
                if (!(dv < f.s.near_plane)) {
                    const float three_sigma = 3.0f * sigma[px + py * f.s.w];
                    OccD d = data[k];
                    bool count = true;
                    if (low_var) {
                        newly = !d.observed;
                        occ_update(d, lom, m.cfg.max_weight);
                        data[k] = d;
                    }
                    else {
                        const float pm = p.z;
                        const float range = sqrtf(dot(p, p));
                        const float range_diff = (pm - dv) * (range / pm);
                        float sample = 0.0f;
                        bool upd = true;
                        if (range_diff < -three_sigma)
                            sample = lom;
                        else if (range_diff < tau / 2)
                            sample = fminf(lom - lom / three_sigma * (range_diff + three_sigma), lomax);
                        else if (range_diff < tau)
                            sample = fminf(-lom * tau / (2 * three_sigma), lomax);
                        else
                            upd = false;
                        if (upd) {
                            newly = !d.observed;
                            occ_update(d, sample, m.cfg.max_weight);
                            data[k] = d;
                        }
                        if (dv > f.s.far_plane)
                            count = false;
                    }
                    newly = newly && count;
                }
            }
        }
        newly_total += warp_count(newly);
    }
    if (to_buffer) {
        st.buf_obs += newly_total;
        occ_incr_buffer_integr(st, inside);
    }
    else {
        st.curr_obs += newly_total;
        ++st.curr_integr;
    }
    __syncwarp();
}

__device__ __forceinline__ int occ_recommended_scale(const OccDevice& m, const OccFrame& f, int b,
                                                     const OccBlockState& st, F3 centre_C, bool free_min,
                                                     int& last_scale)
{
    last_scale = (st.min_scale == -1) ? 0 : st.current_scale;
    const int computed = occ_integration_scale(f.s, centre_C.z, m.res, last_scale, st.min_scale);
    const OccD mx = blk_max(m, b, st.finest, kOccMaxScale)[0];
    const int min_integr = (free_min && (st.min_scale == -1 || (double) mx.occ < 0.95 * (double) m.cfg.log_odd_min))
        ? m.cfg.fs_integr_scale
        : max(0, last_scale - 1);
    const int max_integr = (st.min_scale == -1) ? kOccMaxScale : min(kOccMaxScale, last_scale + 1);
    return min(max(min_integr, computed), max_integr);
}

__device__ __forceinline__ F3 occ_block_centre_C(const OccDevice& m, const OccFrame& f, int b)
{
    const float off = 8.0f * 0.5f;
    return apply(f.T_SW, apply(m.T_WM, f3(((float) m.block_coord[3 * b] + off) * m.res,
                                          ((float) m.block_coord[3 * b + 1] + off) * m.res,
                                          ((float) m.block_coord[3 * b + 2] + off) * m.res)));
}

// Updater::updateBlock (free == false) / Updater::freeBlock (free == true), one warp per block
__device__ void occ_process_block(const OccDevice& m, const OccFrame& f, const float* __restrict__ depth,
                                  const float* __restrict__ sigma, int b, bool low_var, bool inside, bool free,
                                  int lane)
{
    OccBlockState st = m.block_state[b];
    const F3 centre_C = occ_block_centre_C(m, f, b);
    int last_scale;
    const int rec = occ_recommended_scale(m, f, b, st, centre_C, free ? true : low_var, last_scale);
    int integration_scale = last_scale;
    bool done = false;
    if (st.min_scale == -1) {
        integration_scale = rec;
        occ_allocate_down_to(m, b, st, integration_scale, lane);
        st.current_scale = integration_scale;
        // initCurrCout
        if (st.init_data.observed) {
            st.curr_integr = (unsigned long long) st.init_data.weight;
            const int ns = 8 >> st.current_scale;
            st.curr_obs = (unsigned long long) (ns * ns * ns);
        }
        else {
            st.curr_integr = 0ull;
            st.curr_obs = 0ull;
        }
        st.init_data = occ_default();
    }
    else if (rec != last_scale) {
        occ_prepare_buffer(m, b, st, rec, last_scale, lane);
        if (free) {
            OccD* buf = blk_buffer(m, b, st);
            const int nv = (8 >> rec) * (8 >> rec) * (8 >> rec);
            unsigned long long cnt = 0;
            for (int base = 0; base < nv; base += 32) {
                const int i = base + lane;
                bool newly = false;
                if (i < nv) {
                    OccD d = buf[i];
                    newly = !d.observed;
                    occ_update(d, m.cfg.log_odd_min, m.cfg.max_weight);
                    buf[i] = d;
                }
                cnt += warp_count(newly);
            }
            st.buf_obs += cnt;
            occ_incr_buffer_integr(st, true);
            __syncwarp();
        }
        else {
            occ_update_block_data(m, f, depth, sigma, b, st, centre_C, rec, low_var, inside, true, lane);
        }
        done = occ_switch_data(m, b, st, lane);
    }
    else {
        st.buffer_scale = -1; // resetBuffer
        st.buf_integr = 0ull;
        st.buf_obs = 0ull;
    }
    if (!done) {
        if (free) {
            const int nv = (8 >> integration_scale) * (8 >> integration_scale) * (8 >> integration_scale);
            OccD* cur = blk_mean(m, b, st.current_scale);
            unsigned long long cnt = 0;
            for (int base = 0; base < nv; base += 32) {
                const int i = base + lane;
                bool newly = false;
                if (i < nv) {
                    OccD d = cur[i];
                    newly = !d.observed;
                    occ_update(d, m.cfg.log_odd_min, m.cfg.max_weight);
                    cur[i] = d;
                }
                cnt += warp_count(newly);
            }
            st.curr_obs += cnt;
            ++st.curr_integr;
            __syncwarp();
        }
        else {
            occ_update_block_data(m, f, depth, sigma, b, st, centre_C, integration_scale, low_var, inside, false,
                                  lane);
        }
    }
    if (lane == 0)
        m.block_state[b] = st;
    __syncwarp();
}

__global__ void __launch_bounds__(256) occ_update_blocks_kernel(OccDevice m, OccFrame f, const float* __restrict__ depth,
                                                                const float* __restrict__ sigma,
                                                                const int* __restrict__ block_list,
                                                                const int* __restrict__ block_var,
                                                                const int* __restrict__ block_inside)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int n_warps = (gridDim.x * blockDim.x) >> 5;
    const int n = min(m.counters[kOccBlockListN], m.block_capacity);
    for (int i = warp; i < n; i += n_warps)
        occ_process_block(m, f, depth, sigma, block_list[i], block_var[i] == 0, block_inside[i] != 0, false, lane);
}

__global__ void __launch_bounds__(256) occ_free_blocks_kernel(OccDevice m, OccFrame f, const float* __restrict__ depth,
                                                              const float* __restrict__ sigma,
                                                              const int* __restrict__ freed)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int n_warps = (gridDim.x * blockDim.x) >> 5;
    const int n = min(m.counters[kOccFreedN], m.block_capacity);
    for (int i = warp; i < n; i += n_warps)
        occ_process_block(m, f, depth, sigma, freed[i], true, true, true, lane);
}

// Updater::freeNodeRecurse, one level of the subtrees per launch
__global__ void occ_free_nodes_kernel(OccDevice m, int frame_id, const int2* __restrict__ in, const int* __restrict__ in_n,
                                      int2* out, int* out_n, int* freed, int* sets)
{
    const int n_in = min(*in_n, m.node_capacity);
    int* err = &m.counters[kOccError];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += gridDim.x * blockDim.x) {
        const int n = in[i].x, depth = in[i].y;
        if (node_is_leaf(m, n)) {
            OccD d = node_data(m, n);
            occ_update(d, m.cfg.log_odd_min, m.cfg.max_weight);
            m.node_min[n] = d;
            m.node_max[n] = d;
            occ_set_insert(m, sets, m.node_parent[n], frame_id);
        }
        else {
            for (int c = 0; c < 8; ++c) {
                const int ch = m.node_child[8 * (size_t) n + c];
                if (ch == -1)
                    continue;
                if (slot_is_block(ch)) {
                    occ_set_insert(m, sets, n, frame_id);
                    push(freed, &m.counters[kOccFreedN], m.block_capacity, slot_block(ch), err);
                }
                else {
                    const int k = atomicAdd(out_n, 1);
                    if (k < m.node_capacity)
                        out[k] = make_int2(ch, depth + 1);
                    else
                        atomicOr(err, kOccErrList);
                }
            }
        }
    }
}

__global__ void occ_seed_work_kernel(OccDevice m, const int* __restrict__ node_list, int2* work, int* work_n)
{
    const int n = min(m.counters[kOccNodeListN], m.node_capacity);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        work[i] = make_int2(node_list[i], occ_node_depth(m, node_list[i]));
    if (blockIdx.x == 0 && threadIdx.x == 0)
        *work_n = n;
}

// propagate_block_to_coarsest_scale (multires_ofusion_core_impl.hpp:120-276), one warp per block
__device__ void occ_up_best(OccD& parent, const OccD* ch, bool want_min)
{
    float best = want_min ? FLT_MAX : -FLT_MAX;
    int bi = 0, nv = 0, no = 0;
    for (int i = 0; i < 8; ++i) {
        if (occ_valid(ch[i])) {
            ++nv;
            no += ch[i].observed ? 1 : 0;
            const float fv = occ_field(ch[i]);
            if (want_min ? (fv < best) : (fv > best)) {
                best = fv;
                bi = i;
            }
        }
    }
    if (nv > 0) {
        parent = ch[bi];
        parent.observed = (no == 8) ? 1 : 0;
    }
}

__device__ void occ_up_mean(OccD& parent, const OccD* ch)
{
    float os = 0.0f, ws = 0.0f;
    int n = 0;
    for (int i = 0; i < 8; ++i)
        if (occ_valid(ch[i])) {
            ++n;
            os += ch[i].occ;
            ws += ch[i].weight;
        }
    if (n > 0) {
        parent.occ = os / (float) n;
        parent.weight = ceilf(ws / (float) n);
        parent.observed = 0;
    }
}

__device__ void occ_propagate_block(const OccDevice& m, int b, int lane)
{
    const OccBlockState st = m.block_state[b];
    if (st.current_scale == kOccMaxScale)
        return;
    int cs = st.current_scale;
    for (int ps = cs + 1; ps <= kOccMaxScale; ++ps) {
        cs = ps - 1;
        const int np = 8 >> ps, nc = 8 >> cs;
        OccD* pmin = blk_min(m, b, st.finest, ps);
        OccD* pmax = blk_max(m, b, st.finest, ps);
        OccD* pmean = blk_mean(m, b, ps);
        const OccD* cmean = blk_mean(m, b, cs);
        const OccD* cmin = blk_min(m, b, st.finest, cs);
        const OccD* cmax = blk_max(m, b, st.finest, cs);
        const bool first = ps == st.current_scale + 1;
        for (int k = lane; k < np * np * np; k += 32) {
            const int x = k % np, y = (k / np) % np, z = k / (np * np);
            OccD c0[8], c1[8], c2[8];
            for (int c = 0; c < 8; ++c) {
                const int ci = (2 * x + (c & 1)) + (2 * y + ((c >> 1) & 1)) * nc + (2 * z + (c >> 2)) * nc * nc;
                c0[c] = cmean[ci];
                c1[c] = first ? cmean[ci] : cmin[ci];
                c2[c] = first ? cmean[ci] : cmax[ci];
            }
            if (!(first && st.buffer_scale > st.current_scale))
                occ_up_mean(pmean[k], c0);
            occ_up_best(pmin[k], c1, true);
            occ_up_best(pmax[k], c2, false);
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(256) occ_propagate_blocks_kernel(OccDevice m, const int* __restrict__ list,
                                                                   int counter)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int n_warps = (gridDim.x * blockDim.x) >> 5;
    const int n = min(m.counters[counter], m.block_capacity);
    for (int i = warp; i < n; i += n_warps)
        occ_propagate_block(m, list[i], lane);
}

__global__ void occ_seed_sets_kernel(OccDevice m, int frame_id, const int* __restrict__ block_list, int* sets)
{
    const int n = min(m.counters[kOccBlockListN], m.block_capacity);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        occ_set_insert(m, sets, m.block_state[block_list[i]].parent, frame_id);
}

// updater::propagate_to_parent_node (multires_ofusion_core_impl.hpp:88-117)
__device__ OccD occ_propagate_node(const OccDevice& m, int n, int timestamp)
{
    m.node_ts[n] = timestamp;
    OccD cmin[8], cmax[8];
    for (int i = 0; i < 8; ++i) {
        const int c = m.node_child[8 * (size_t) n + i];
        if (c == -1) {
            cmin[i] = occ_default();
            cmax[i] = occ_default();
        }
        else if (slot_is_block(c)) {
            const int b = slot_block(c);
            const int fin = m.block_state[b].finest;
            cmin[i] = blk_min(m, b, fin, kOccMaxScale)[0];
            cmax[i] = blk_max(m, b, fin, kOccMaxScale)[0];
        }
        else {
            cmin[i] = m.node_min[c];
            cmax[i] = m.node_max[c];
        }
    }
    OccD mn = m.node_min[n], mx = m.node_max[n];
    occ_up_best(mn, cmin, true);
    occ_up_best(mx, cmax, false);
    m.node_min[n] = mn;
    m.node_max[n] = mx;
    return mx;
}

// Octree::deleteChildren: detach the subtree; its blocks stop being live
__device__ void occ_delete_children(const OccDevice& m, int n)
{
    int stack[64];
    int sp = 0;
    stack[sp++] = n;
    while (sp > 0) {
        const int q = stack[--sp];
        for (int i = 0; i < 8; ++i) {
            const int c = m.node_child[8 * (size_t) q + i];
            if (c == -1)
                continue;
            if (slot_is_block(c))
                m.block_state[slot_block(c)].live = 0;
            else if (sp < 64)
                stack[sp++] = c;
            else
                atomicOr(&m.counters[kOccError], kOccErrList);
            m.node_child[8 * (size_t) q + i] = -1;
        }
    }
}

__global__ void occ_propagate_nodes_kernel(OccDevice m, int frame_id, int timestamp, int depth, int* sets)
{
    const int n = min(m.counters[kOccSetN + depth], m.node_capacity);
    const int* list = sets + (size_t) depth * m.node_capacity;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int node = list[i];
        if (m.node_ts[node] == timestamp)
            continue;
        if (m.node_parent[node] < 0)
            continue;
        const OccD nd = occ_propagate_node(m, node, timestamp);
        occ_set_insert(m, sets, m.node_parent[node], frame_id);
        if (nd.observed && (double) occ_field(nd) <= 0.95 * -100.0) {
            occ_delete_children(m, node);
            atomicAdd(&m.counters[kOccPruned], 1);
        }
    }
}

__global__ void occ_propagate_root_kernel(OccDevice m, int timestamp) { occ_propagate_node(m, 0, timestamp); }

__global__ void occ_reset_frame_kernel(OccDevice m)
{
    const int i = threadIdx.x;
    if (i == kOccFrontierN0 || i == kOccFrontierN1 || i == kOccBlockListN || i == kOccNodeListN || i == kOccFreedN
        || i == kOccWorkN0 || i == kOccWorkN1 || i == kOccPruned || (i >= kOccSetN && i < kOccCounters))
        m.counters[i] = 0;
}

// ----------------------------------------------------------------- queries / raycast --

// fetcher::finest_octant (fetcher_impl.hpp:69-94) as a slot: the octant of size max(2^scale, 8)
// on the voxel's path, the deepest node when it has no children, or -1.
__device__ int occ_finest_octant(const OccDevice& m, int x, int y, int z, int scale_desired)
{
    const int size_desired = max(1 << scale_desired, 8);
    int n = 0, child = -1;
    for (int cs = m.size >> 1; cs >= size_desired; cs >>= 1) {
        const int idx = ((x & cs) > 0) + 2 * ((y & cs) > 0) + 4 * ((z & cs) > 0);
        child = m.node_child[8 * (size_t) n + idx];
        if (child == -1)
            return node_is_leaf(m, n) ? n : -1;
        if (slot_is_block(child))
            return child;
        n = child;
    }
    return child;
}

__device__ __forceinline__ int blk_voxel_idx(const OccDevice& m, int b, int x, int y, int z, int s)
{
    return occ_voxel_idx(x - m.block_coord[3 * b], y - m.block_coord[3 * b + 1], z - m.block_coord[3 * b + 2], s);
}

// visitor::getMaxData (visitor_impl.hpp:815-835)
__device__ OccD occ_max_data(const OccDevice& m, int x, int y, int z, int scale_desired)
{
    const int slot = occ_finest_octant(m, x, y, z, scale_desired);
    if (slot == -1)
        return occ_default();
    if (slot_is_block(slot)) {
        const int b = slot_block(slot);
        const OccBlockState& st = m.block_state[b];
        const int so = max(scale_desired, st.current_scale);
        return blk_max(m, b, st.finest, so)[blk_voxel_idx(m, b, x, y, z, so)];
    }
    return m.node_max[slot];
}

// visitor::getData(octree, voxel): a block's data at its current scale, a leaf node's data
__device__ OccD occ_get_data_voxel(const OccDevice& m, int x, int y, int z)
{
    const int slot = occ_leaf(m, x, y, z);
    if (slot == -1)
        return occ_default();
    if (slot_is_block(slot)) {
        const int b = slot_block(slot);
        const OccBlockState& st = m.block_state[b];
        return blk_mean(m, b, st.current_scale)[blk_voxel_idx(m, b, x, y, z, st.current_scale)];
    }
    return node_data(m, slot);
}

__device__ __forceinline__ F3 occ_to_voxel_f(const OccDevice& m, F3 p_W)
{
    const F3 p = apply(m.T_MW, p_W);
    return f3(p.x / m.res, p.y / m.res, p.z / m.res);
}

// Map::getData (Safe::Off)
__device__ __forceinline__ OccD occ_get_data(const OccDevice& m, F3 p_W)
{
    const F3 v = occ_to_voxel_f(m, p_W);
    return occ_get_data_voxel(m, (int) v.x, (int) v.y, (int) v.z);
}

__device__ __forceinline__ OccD occ_block_data_at(const OccDevice& m, int b, int x, int y, int z, int s)
{
    const OccBlockState& st = m.block_state[b];
    if (s < st.finest)
        return st.init_data;
    return blk_mean(m, b, s)[blk_voxel_idx(m, b, x, y, z, s)];
}

// visitor::getInterp multi-res with get_neighbours on an occupancy octree (leaf nodes take part)
__device__ bool occ_interp(const OccDevice& m, F3 vf, int desired_scale, float& out, int* returned_scale)
{
    const int q = occ_leaf(m, (int) vf.x, (int) vf.y, (int) vf.z);
    if (q == -1)
        return false;
    const bool q_block = slot_is_block(q);
    const int init = q_block ? max(m.block_state[slot_block(q)].current_scale, desired_scale) : 0;
#pragma unroll 1
    for (int scale = init; scale <= kOccMaxScale; ++scale) {
        const int stride = 1 << scale;
        const float inv = 1.0f / (float) stride;
        const F3 bf = f3(inv * vf.x - 0.5f, inv * vf.y - 0.5f, inv * vf.z - 0.5f);
        const int b0 = stride * (int) bf.x, b1 = stride * (int) bf.y, b2 = stride * (int) bf.z;
        if (m.aabb[6])
            return false;
        if (b0 < m.aabb[0] || b1 < m.aabb[1] || b2 < m.aabb[2] || b0 > m.aabb[3] || b1 > m.aabb[4] || b2 > m.aabb[5])
            return false;
        if (b0 + stride >= m.size || b1 + stride >= m.size || b2 + stride >= m.size || b0 < 0 || b1 < 0 || b2 < 0)
            continue;
        float f[8];
        bool ok = true, valid = true;
#pragma unroll 1
        for (int n = 0; n < 8; ++n) {
            const int cx = b0 + stride * (n & 1), cy = b1 + stride * ((n >> 1) & 1), cz = b2 + stride * (n >> 2);
            const int slot = occ_leaf(m, cx, cy, cz);
            if (slot == -1) {
                ok = false;
                break;
            }
            OccD d;
            if (slot_is_block(slot)) {
                const int b = slot_block(slot);
                if (m.block_state[b].current_scale > scale) {
                    ok = false;
                    break;
                }
                d = occ_block_data_at(m, b, cx, cy, cz, scale);
            }
            else {
                d = node_data(m, slot);
            }
            valid = valid && occ_valid(d);
            f[n] = occ_field(d);
        }
        if (!ok)
            continue;
        if (!valid)
            return false;
        if (returned_scale)
            *returned_scale = q_block ? scale : (31 - __clz(m.node_coord[q].w));
        const F3 t = f3(bf.x - floorf(bf.x), bf.y - floorf(bf.y), bf.z - floorf(bf.z));
        const F3 tc = f3(1.0f - t.x, 1.0f - t.y, 1.0f - t.z);
        out = ((f[0] * tc.x + f[1] * t.x) * tc.y + (f[2] * tc.x + f[3] * t.x) * t.y) * tc.z
            + ((f[4] * tc.x + f[5] * t.x) * tc.y + (f[6] * tc.x + f[7] * t.x) * t.y) * t.z;
        return true;
    }
    return false;
}

static __constant__ unsigned char kOccGradSel[32] = {
    0x14, 0x18, 0x24, 0x28, 0x11, 0x21, 0x05, 0x15, 0x25, 0x35, 0x09, 0x19, 0x29, 0x39, 0x1d, 0x2d,
    0x12, 0x22, 0x06, 0x16, 0x26, 0x36, 0x0a, 0x1a, 0x2a, 0x3a, 0x1e, 0x2e, 0x17, 0x1b, 0x27, 0x2b};

// visitor::getFieldGrad multi-res, desired scale 0 (visitor_impl.hpp:1257-1497), occupancy
__device__ bool occ_grad(const OccDevice& m, F3 vf, F3& g)
{
    const int q = occ_finest_octant(m, (int) vf.x, (int) vf.y, (int) vf.z, 0);
    if (q == -1)
        return false;
    if (!slot_is_block(q)) {
        if (occ_valid(node_data(m, q))) {
            g = f3(0.0f, 0.0f, 0.0f);
            return true;
        }
        return false;
    }
    const int qc = m.block_state[slot_block(q)].current_scale;
    const int init = qc > 0 ? qc : 0;
    const int top = m.size - 1;
#pragma unroll 1
    for (int scale = init; scale <= kOccMaxScale; ++scale) {
        const int stride = 1 << scale;
        const float inv = 1.0f / (float) stride;
        const F3 sv = f3(inv * vf.x - 0.5f, inv * vf.y - 0.5f, inv * vf.z - 0.5f);
        const F3 fac = f3(sv.x - floorf(sv.x), sv.y - floorf(sv.y), sv.z - floorf(sv.z));
        const int base[3] = {stride * (int) sv.x, stride * (int) sv.y, stride * (int) sv.z};
        int sel[3][4];
        for (int i = 0; i < 3; ++i) {
            sel[i][0] = max(base[i] - stride, 0);
            sel[i][1] = max(base[i], 0);
            sel[i][2] = min(base[i] + stride, top);
            sel[i][3] = min(base[i] + 2 * stride, top);
        }
        const int oct = occ_finest_octant(m, base[0], base[1], base[2], scale);
        if (oct == -1)
            continue;
        if (!slot_is_block(oct)) {
            if (node_is_leaf(m, oct) && occ_valid(node_data(m, oct))) {
                g = f3(0.0f, 0.0f, 0.0f);
                return true;
            }
            continue;
        }
        const int hb = slot_block(oct);
        const int hx = m.block_coord[3 * hb], hy = m.block_coord[3 * hb + 1], hz = m.block_coord[3 * hb + 2];
        float v[32];
        bool ok = true;
#pragma unroll 1
        for (int i = 0; i < 32; ++i) {
            const unsigned code = kOccGradSel[i];
            const int cx = sel[0][code & 3], cy = sel[1][(code >> 2) & 3], cz = sel[2][(code >> 4) & 3];
            int slot = oct;
            if (!(cx >= hx && cx <= hx + 7 && cy >= hy && cy <= hy + 7 && cz >= hz && cz <= hz + 7))
                slot = occ_leaf(m, cx, cy, cz);
            if (slot == -1) {
                ok = false;
                break;
            }
            OccD d;
            int rs;
            if (slot_is_block(slot)) {
                const int b = slot_block(slot);
                const OccBlockState& st = m.block_state[b];
                rs = max(scale, st.current_scale);
                d = blk_mean(m, b, rs)[blk_voxel_idx(m, b, cx, cy, cz, rs)];
            }
            else {
                rs = scale;
                d = node_data(m, slot);
            }
            if (!occ_valid(d) || rs != scale) {
                ok = false;
                break;
            }
            v[i] = occ_field(d);
        }
        if (!ok)
            continue;
        const float rx = 1.0f - fac.x, ry = 1.0f - fac.y, rz = 1.0f - fac.z;
        const float gx = (((v[19] - v[0]) * rx + (v[28] - v[7]) * fac.x) * ry
                          + ((v[23] - v[1]) * rx + (v[29] - v[11]) * fac.x) * fac.y) * rz
            + (((v[20] - v[2]) * rx + (v[30] - v[8]) * fac.x) * ry
               + ((v[24] - v[3]) * rx + (v[31] - v[12]) * fac.x) * fac.y) * fac.z;
        const float gy = (((v[11] - v[4]) * rx + (v[23] - v[16]) * fac.x) * ry
                          + ((v[14] - v[7]) * rx + (v[26] - v[19]) * fac.x) * fac.y) * rz
            + (((v[12] - v[5]) * rx + (v[24] - v[17]) * fac.x) * ry
               + ((v[15] - v[8]) * rx + (v[27] - v[20]) * fac.x) * fac.y) * fac.z;
        const float gz = (((v[8] - v[6]) * rx + (v[20] - v[18]) * fac.x) * ry
                          + ((v[12] - v[10]) * rx + (v[24] - v[22]) * fac.x) * fac.y) * rz
            + (((v[9] - v[7]) * rx + (v[21] - v[19]) * fac.x) * ry
               + ((v[13] - v[11]) * rx + (v[25] - v[23]) * fac.x) * fac.y) * fac.z;
        const float sf = (float) stride;
        g = f3((0.5f * gx) / sf, (0.5f * gy) / sf, (0.5f * gz) / sf);
        return true;
    }
    return false;
}

__device__ __forceinline__ bool occ_contains(const OccDevice& m, F3 p_W)
{
    const F3 p = apply(m.T_MW, p_W);
    return p.x >= 0.0f && p.x < m.dim && p.y >= 0.0f && p.y < m.dim && p.z >= 0.0f && p.z < m.dim;
}

// find_valid_point (raycaster_impl.hpp:32-70)
__device__ bool occ_find_valid_point(const OccDevice& m, F3 o, F3 d, float step, float t_max, float& t, F3& point_W,
                                     float& value)
{
    bool has = false;
    F3 p = add(o, mul(t, d));
    if (occ_contains(m, p) && occ_valid(occ_get_data(m, p)))
        has = occ_interp(m, occ_to_voxel_f(m, p), 0, value, nullptr);
#pragma unroll 1
    while (!has) {
        t += step;
        if (t > t_max)
            return false;
        p = add(o, mul(t, d));
        if (occ_contains(m, p) && occ_valid(occ_get_data(m, p)))
            has = occ_interp(m, occ_to_voxel_f(m, p), 0, value, nullptr);
    }
    point_W = p;
    return true;
}

// compute_map_intersection (raycaster_impl.hpp:85-173)
__device__ float occ_map_intersection(const OccDevice& m, F3 pos_W, F3 dir_W, float t_far, bool& valid)
{
    const F3 p = apply(m.T_MW, pos_W), dr = rot(m.T_MW, dir_W);
    const float pm[3] = {p.x, p.y, p.z}, dm[3] = {dr.x, dr.y, dr.z};
    const float mx = m.dim;
    bool inside = true;
    int quadrant[3];
    float cand[3] = {0.0f, 0.0f, 0.0f}, maxT[3];
    for (int i = 0; i < 3; ++i) {
        if (pm[i] < 0.0f) {
            quadrant[i] = 1;
            cand[i] = 0.0f;
            inside = false;
        }
        else if (pm[i] > mx) {
            quadrant[i] = 0;
            cand[i] = mx;
            inside = false;
        }
        else {
            quadrant[i] = 2;
        }
    }
    if (inside)
        return 0.0f;
    for (int i = 0; i < 3; ++i)
        maxT[i] = (quadrant[i] != 2 && dm[i] != 0.0f) ? (cand[i] - pm[i]) / dm[i] : -1.0f;
    int which = 0;
    for (int i = 1; i < 3; ++i)
        if (maxT[which] < maxT[i])
            which = i;
    if (maxT[which] < 0.0f) {
        valid = false;
        return 0.0f;
    }
    float hit[3];
    for (int i = 0; i < 3; ++i) {
        if (which != i) {
            hit[i] = pm[i] + maxT[which] * dm[i];
            if (hit[i] < 0.0f || hit[i] > mx) {
                valid = false;
                return 0.0f;
            }
        }
        else {
            hit[i] = cand[i];
        }
    }
    const F3 dh = f3(hit[0] - pm[0], hit[1] - pm[1], hit[2] - pm[2]);
    const float t = sqrtf(dot(dh, dh));
    if (t_far < t) {
        valid = false;
        return 0.0f;
    }
    return t;
}

__device__ __forceinline__ float occ_max_field(const OccDevice& m, F3 c, int s)
{
    return occ_field(occ_max_data(m, (int) c.x, (int) c.y, (int) c.z, s));
}

// advance_ray (raycaster_impl.hpp:189-338)
__device__ void occ_advance_ray(const OccDevice& m, F3 o, F3 d, float& t, float& t_far, int max_scale, bool& valid)
{
    const float voxel_dim = m.res;
    int scale = max_scale;
    float v_add = 0.0f;
    const float v = 1.0f / voxel_dim * t;
    float v_far = 1.0f / voxel_dim * t_far;
    F3 oc = f3(-1.0f, -1.0f, -1.0f);
    if (occ_contains(m, o))
        oc = occ_to_voxel_f(m, o);
    const float sz = (float) m.size;
    const float dv[3] = {d.x, d.y, d.z};
    const float ocv[3] = {oc.x, oc.y, oc.z};
    float vmap[3];
    for (int i = 0; i < 3; ++i) {
        const float dvm = sz / fabsf(dv[i]);
        const float frac = ocv[i] / sz;
        vmap[i] = dv[i] < 0 ? frac * dvm : (1 - frac) * dvm;
    }
    v_far = fminf(fminf(fminf(vmap[0], vmap[1]), vmap[2]) + v, v_far);
    t_far = voxel_dim * v_far;
    float f = occ_max_field(m, oc, scale);
    while (f > -0.2f && scale > 2) {
        scale -= 1;
        f = occ_max_field(m, oc, scale);
    }
    F3 rc = oc;
#pragma unroll 1
    for (int guard = 0; (v + v_add) < v_far && guard < (1 << 22); ++guard) {
        if (scale <= 2) {
            t = voxel_dim * (v + v_add - 4);
            return;
        }
        const int node_size = 1 << scale;
        const float rcv[3] = {rc.x, rc.y, rc.z};
        float Vmax[3];
        for (int i = 0; i < 3; ++i) {
            const int curr = node_size * (int) (floorf(rcv[i]) / (float) node_size);
            const float frac = (rcv[i] - (float) curr) / (float) node_size;
            const float dV = (float) node_size / fabsf(dv[i]);
            Vmax[i] = dv[i] < 0 ? frac * dV : (1 - frac) * dV;
            if (fabsf(dv[i]) < 1.0e-6f)
                Vmax[i] = __int_as_float(0x7f800000);
        }
        const float Vmin = fminf(fminf(Vmax[0], Vmax[1]), Vmax[2]);
        v_add = (float) ((double) v_add + ((double) Vmin + 0.01));
        rc = add(mul(v + v_add, d), oc);
        f = occ_max_field(m, rc, scale);
        if (f > -0.2f) {
            while (f > -0.2f && scale > 2) {
                scale -= 1;
                f = occ_max_field(m, rc, scale);
            }
        }
        else {
            for (int s = scale + 1; s <= max_scale; s++) {
                f = occ_max_field(m, rc, s);
                if (f > -0.2f)
                    break;
                scale += 1;
            }
        }
    }
    valid = false;
}

// raycast<Occupancy> (raycaster_impl.hpp:352-452)
__device__ bool occ_raycast(const OccDevice& m, F3 o, F3 d, float t_far, F3& hit, int& scale_out)
{
    bool valid = true;
    float t = occ_map_intersection(m, o, d, t_far, valid);
    if (!valid)
        return false;
    const int max_scale = min(7, m.log2_size - 1);
    occ_advance_ray(m, o, d, t, t_far, max_scale, valid);
    if (!valid)
        return false;
    const float step = m.res / 2;
    float value_t = 0.0f, value_tt = 0.0f;
    bool has_tt = false;
    F3 pt = f3(0.0f, 0.0f, 0.0f), ptt = f3(0.0f, 0.0f, 0.0f);
    int scale_tt = 0;
    if (!occ_find_valid_point(m, o, d, step, t_far, t, pt, value_t))
        return false;
    t += step;
    if (value_t <= 0.0f) {
#pragma unroll 1
        for (; t < t_far; t += step) {
            const F3 p = add(o, mul(d, t));
            const OccD data = occ_get_data(m, p);
            if (!occ_valid(data)) {
                t += step;
                if (!occ_find_valid_point(m, o, d, step, t_far, t, pt, value_t)) {
                    hit = f3(0.0f, 0.0f, 0.0f);
                    scale_out = 0;
                    return true;
                }
                if (value_t > 0.0f)
                    break;
                continue;
            }
            value_tt = occ_field(data);
            has_tt = true;
            ptt = p;
            if (value_tt > -0.2f) {
                float vi;
                int sc = scale_tt;
                if (occ_interp(m, occ_to_voxel_f(m, p), 0, vi, &sc)) {
                    value_tt = vi;
                    scale_tt = sc;
                }
                else {
                    has_tt = false;
                    t += step;
                    if (!occ_find_valid_point(m, o, d, step, t_far, t, pt, value_t))
                        return false;
                    if (value_t > 0.0f)
                        break;
                    continue;
                }
            }
            if (value_tt > 0.0f)
                break;
            value_t = value_tt;
            pt = ptt;
        }
        if (has_tt && value_tt > 0.0f && value_t < 0.0f) {
            const F3 dd = sub(ptt, pt);
            t = t - sqrtf(dot(dd, dd)) * (value_tt - 0.0f) / (value_tt - value_t);
            hit = add(o, mul(d, t));
            scale_out = scale_tt;
            return true;
        }
    }
    return false;
}

// raycaster::raycast_volume for occupancy maps: normals are -normalize(grad F)
__global__ void __launch_bounds__(128) occ_raycast_kernel(OccDevice m, Pinhole s, Tf T_WS, float* __restrict__ pts,
                                                          float* __restrict__ nrm, int8_t* __restrict__ scale)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
    if (x >= s.w || y >= s.h)
        return;
    const size_t idx = (size_t) x + (size_t) y * s.w;
    const F3 ray_S = back_project(s, (float) x, (float) y);
    const F3 nS = normalized(ray_S);
    const F3 dir_W = rot(T_WS, nS);
    const F3 origin = f3(T_WS.t[0], T_WS.t[1], T_WS.t[2]);
    F3 hit, p = f3(0.0f, 0.0f, 0.0f), n = f3(0.0f, 0.0f, 0.0f);
    int sc = 0;
    if (occ_raycast(m, origin, dir_W, s.far_plane / nS.z, hit, sc)) {
        p = hit;
        F3 g;
        if (occ_grad(m, occ_to_voxel_f(m, hit), g)) {
            g = f3(g.x / m.res, g.y / m.res, g.z / m.res);
            const float nn = sqrtf(dot(g, g));
            n = nn > 0.0f ? f3(-(g.x / nn), -(g.y / nn), -(g.z / nn)) : f3(-g.x, -g.y, -g.z);
        }
    }
    else {
        sc = 0;
    }
    pts[3 * idx + 0] = p.x;
    pts[3 * idx + 1] = p.y;
    pts[3 * idx + 2] = p.z;
    nrm[3 * idx + 0] = n.x;
    nrm[3 * idx + 1] = n.y;
    nrm[3 * idx + 2] = n.z;
    if (scale)
        scale[idx] = (int8_t) sc;
}

se_gpu_status occ_raycast_volume(const se_gpu_occ_map* om, const se_gpu_pinhole& sensor, const float* T_WS16,
                                 float* pts, float* nrm, int8_t* scale, cudaStream_t stream)
{
    const Pinhole s = make_pinhole(sensor);
    dim3 grid((s.w + 15) / 16, (s.h + 7) / 8);
    ProfScope ps(kProfRaycast, stream);
    occ_raycast_kernel<<<grid, 128, 0, stream>>>(om->dev, s, tf_from16(T_WS16), pts, nrm, scale);
    SE_CUDA_TRY(cudaGetLastError());
    return SE_GPU_OK;
}

} // namespace se_gpu

using namespace se_gpu;

// ------------------------------------------------------------------------ host side --

static se_gpu_status occ_scratch_reserve(se_gpu_occ_map* om, int w, int h)
{
    OccScratch& s = om->scratch;
    OccDevice& m = om->dev;
    if (s.w == w && s.h == h && s.sigma)
        return SE_GPU_OK;
    cudaFree(s.sigma);
    cudaFree(s.pool_depth);
    cudaFree(s.pool_sigma);
    s.sigma = nullptr;
    s.pool_depth = s.pool_sigma = nullptr;
    const int image_max_dim = w < h ? w : h;
    const int levels = (int) (std::log2((double) ((image_max_dim - 1) / 2)) + 2) - 1 + 1;
    const size_t npx = (size_t) w * h;
    SE_CUDA_TRY(cudaMalloc(&s.sigma, npx * sizeof(float)));
    SE_CUDA_TRY(cudaMalloc(&s.pool_depth, (size_t) levels * npx * sizeof(float4)));
    SE_CUDA_TRY(cudaMalloc(&s.pool_sigma, (size_t) levels * npx * sizeof(float4)));
    if (!s.max_value) {
        const size_t ncap = (size_t) m.node_capacity + m.block_capacity;
        SE_CUDA_TRY(cudaMalloc(&s.max_value, 2 * sizeof(float)));
        SE_CUDA_TRY(cudaMalloc(&s.frontier[0], ncap * sizeof(int)));
        SE_CUDA_TRY(cudaMalloc(&s.frontier[1], ncap * sizeof(int)));
        SE_CUDA_TRY(cudaMalloc(&s.block_list, (size_t) m.block_capacity * sizeof(int)));
        SE_CUDA_TRY(cudaMalloc(&s.block_var, (size_t) m.block_capacity * sizeof(int)));
        SE_CUDA_TRY(cudaMalloc(&s.block_inside, (size_t) m.block_capacity * sizeof(int)));
        SE_CUDA_TRY(cudaMalloc(&s.node_list, (size_t) m.node_capacity * sizeof(int)));
        SE_CUDA_TRY(cudaMalloc(&s.freed, (size_t) m.block_capacity * sizeof(int)));
        SE_CUDA_TRY(cudaMalloc(&s.work[0], (size_t) m.node_capacity * sizeof(int2)));
        SE_CUDA_TRY(cudaMalloc(&s.work[1], (size_t) m.node_capacity * sizeof(int2)));
        s.set_depths = m.block_depth + 1;
        SE_CUDA_TRY(cudaMalloc(&s.sets, (size_t) s.set_depths * m.node_capacity * sizeof(int)));
    }
    s.w = w;
    s.h = h;
    s.levels = levels;
    return SE_GPU_OK;
}

namespace se_gpu {

se_gpu_status occ_map_create(const se_gpu_map_config* cfg, const se_gpu_occupancy_config* occ, int size,
                             se_gpu_occ_map** out)
{
    se_gpu_occ_map* om = new se_gpu_occ_map();
    std::memset(&om->dev, 0, sizeof(om->dev));
    om->scratch = OccScratch();
    om->frame_id = 0;
    OccDevice& m = om->dev;
    m.size = size;
    m.log2_size = 0;
    while ((1 << m.log2_size) < size)
        ++m.log2_size;
    m.block_depth = m.log2_size - 3;
    m.res = cfg->res;
    m.dim = (float) size * cfg->res;
    if (cfg->has_T_MW) {
        m.T_MW = tf_from16(cfg->T_MW);
    }
    else {
        for (int i = 0; i < 9; ++i)
            m.T_MW.R[i] = (i % 4 == 0) ? 1.0f : 0.0f;
        m.T_MW.t[0] = cfg->dim[0] / 2.0f;
        m.T_MW.t[1] = cfg->dim[1] / 2.0f;
        m.T_MW.t[2] = cfg->dim[2] / 2.0f;
    }
    m.T_WM = inverse_iso(m.T_MW);
    se_gpu_occupancy_config c;
    if (occ) {
        c = *occ;
    }
    else {
        c.k_sigma = 0.052f;
        c.sigma_min_factor = 1.5f;
        c.sigma_max_factor = 6.0f;
        c.k_tau = 0.026f;
        c.tau_min_factor = 6.0f;
        c.tau_max_factor = 16.0f;
        c.log_odd_min = (float) -5.015;
        c.log_odd_max = (float) 5.015;
        c.fs_integr_scale = 1;
    }
    m.cfg.k_sigma = c.k_sigma;
    m.cfg.sigma_min_factor = c.sigma_min_factor;
    m.cfg.sigma_max_factor = c.sigma_max_factor;
    m.cfg.k_tau = c.k_tau;
    m.cfg.tau_min_factor = c.tau_min_factor;
    m.cfg.tau_max_factor = c.tau_max_factor;
    m.cfg.log_odd_min = c.log_odd_min;
    m.cfg.log_odd_max = c.log_odd_max;
    m.cfg.fs_integr_scale = c.fs_integr_scale;
    // FieldData<Occupancy>::Config::max_weight keeps its default (data_field.hpp:67): the YAML
    // reader does not recompute it from a configured log_odd_min
    m.cfg.max_weight = std::floor(std::fabs(-100.0f / (0.97f * (float) -5.015)));
    m.block_capacity = (int) cfg->max_blocks;
    // nodes per block stay below 0.3 in the tests' scenes; half the block capacity leaves margin
    m.node_capacity = (int) (cfg->max_blocks / 2 + 4096);
    auto fail = [&](cudaError_t e, const char* what) {
        se_gpu_status st = cuda_status(e, what);
        occ_map_destroy(om);
        return st;
    };
    cudaError_t e;
    const size_t nc = (size_t) m.node_capacity, bc = (size_t) m.block_capacity;
    if ((e = cudaMalloc(&m.node_coord, nc * sizeof(int4))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_parent, nc * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_child, nc * 8 * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_min, nc * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_max, nc * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_mark, nc * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_ts, nc * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.block_coord, bc * 3 * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.block_state, bc * sizeof(OccBlockState))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.block_mean, bc * 585 * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.block_min, bc * 585 * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.block_max, bc * 585 * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.block_buffer, bc * 512 * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.aabb, 8 * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(aabb)");
    if ((e = cudaMalloc(&m.counters, kOccCounters * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(counters)");
    {
        const int aabb[8] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN, 1, 0};
        if ((e = cudaMemcpy(m.aabb, aabb, sizeof(aabb), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "aabb");
        if ((e = cudaMemset(m.counters, 0, kOccCounters * sizeof(int))) != cudaSuccess) return fail(e, "counters");
        // the root: node 0
        const int one = 1;
        if ((e = cudaMemcpy(m.counters + kOccNodes, &one, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(e, "counters");
        const int4 rc = make_int4(0, 0, 0, size);
        const int minus1[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
        const int rp = -1;
        const OccD def = occ_default();
        if ((e = cudaMemcpy(m.node_coord, &rc, sizeof(rc), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_parent, &rp, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_child, minus1, sizeof(minus1), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_min, &def, sizeof(def), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_max, &def, sizeof(def), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_mark, &rp, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_ts, &rp, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e, "cudaDeviceSynchronize");
    *out = om;
    return SE_GPU_OK;
}

void occ_map_destroy(se_gpu_occ_map* om)
{
    if (!om)
        return;
    OccDevice& m = om->dev;
    cudaFree(m.node_coord);
    cudaFree(m.node_parent);
    cudaFree(m.node_child);
    cudaFree(m.node_min);
    cudaFree(m.node_max);
    cudaFree(m.node_mark);
    cudaFree(m.node_ts);
    cudaFree(m.block_coord);
    cudaFree(m.block_state);
    cudaFree(m.block_mean);
    cudaFree(m.block_min);
    cudaFree(m.block_max);
    cudaFree(m.block_buffer);
    cudaFree(m.aabb);
    cudaFree(m.counters);
    OccScratch& s = om->scratch;
    cudaFree(s.sigma);
    cudaFree(s.pool_depth);
    cudaFree(s.pool_sigma);
    cudaFree(s.max_value);
    cudaFree(s.frontier[0]);
    cudaFree(s.frontier[1]);
    cudaFree(s.block_list);
    cudaFree(s.block_var);
    cudaFree(s.block_inside);
    cudaFree(s.node_list);
    cudaFree(s.freed);
    cudaFree(s.work[0]);
    cudaFree(s.work[1]);
    cudaFree(s.sets);
    delete om;
}

se_gpu_status occ_integrate(se_gpu_occ_map* om, const float* depth_dev, const se_gpu_pinhole& sensor,
                            const float* T_WC16, int timestamp, cudaStream_t stream)
{
    se_gpu_status st = occ_scratch_reserve(om, sensor.width, sensor.height);
    if (st != SE_GPU_OK)
        return st;
    OccDevice& m = om->dev;
    OccScratch& s = om->scratch;
    OccFrame f;
    f.s = make_pinhole(sensor);
    f.T_WS = tf_from16(T_WC16);
    f.T_SW = inverse_iso(f.T_WS);
    f.w = sensor.width;
    f.h = sensor.height;
    f.levels = s.levels;
    f.tau_min = m.cfg.tau_min_factor * m.res;
    f.tau_max = m.cfg.tau_max_factor * m.res;
    f.sigma_min = m.cfg.sigma_min_factor * m.res;
    f.sigma_max = m.cfg.sigma_max_factor * m.res;
    f.frame_id = ++om->frame_id;
    const int npx = f.w * f.h;
    const int sms = device_sm_count();
    ProfScope ps(kProfUpdate, stream);
    occ_reset_frame_kernel<<<1, kOccCounters, 0, stream>>>(m);
    occ_sigma_kernel<<<(npx + 255) / 256, 256, 0, stream>>>(depth_dev, npx, f.sigma_min, f.sigma_max, m.cfg.k_sigma,
                                                           s.sigma);
    for (int img = 0; img < 2; ++img) {
        const float* src = img == 0 ? depth_dev : s.sigma;
        float4* P = img == 0 ? s.pool_depth : s.pool_sigma;
        pool_l0_kernel<<<(npx + 255) / 256, 256, 0, stream>>>(src, f.w, f.h, P);
        if (s.levels > 1)
            pool_l1_kernel<<<(npx + 255) / 256, 256, 0, stream>>>(P, f.w, f.h, P + (size_t) npx);
        for (int l = 2, sz = 2; l < s.levels; ++l, sz <<= 1)
            pool_lk_kernel<<<(npx + 255) / 256, 256, 0, stream>>>(P + (size_t) (l - 1) * npx, f.w, f.h, sz,
                                                                  P + (size_t) l * npx);
    }
    pool_max_kernel<<<1, 1, 0, stream>>>(s.pool_depth + (size_t) (s.levels - 1) * npx, f.w, f.h, s.levels - 1,
                                         f.s.far_plane, f.tau_max, s.max_value);
    // VolumeCarver, breadth first
    occ_carve_root_kernel<<<1, 1, 0, stream>>>(m, s.frontier[0], m.counters + kOccFrontierN0);
    for (int d = 1; d <= m.block_depth; ++d) {
        const int cur = (d - 1) & 1, nxt = d & 1;
        SE_CUDA_TRY(cudaMemsetAsync(m.counters + kOccFrontierN0 + nxt, 0, sizeof(int), stream));
        occ_carve_kernel<<<sms * 8, 128, 0, stream>>>(m, f, s.pool_depth, s.pool_sigma, s.max_value, s.frontier[cur],
                                                      m.counters + kOccFrontierN0 + cur, s.frontier[nxt],
                                                      m.counters + kOccFrontierN0 + nxt, s.block_list, s.block_var,
                                                      s.block_inside, s.node_list, d);
    }
    occ_leaf_aabb_kernel<<<sms, 256, 0, stream>>>(m, s.node_list);
    // Updater: free-space nodes (their subtrees breadth first), then the carver's blocks
    occ_seed_work_kernel<<<sms, 256, 0, stream>>>(m, s.node_list, s.work[0], m.counters + kOccWorkN0);
    for (int it = 0; it <= m.block_depth; ++it) {
        const int cur = it & 1, nxt = (it + 1) & 1;
        SE_CUDA_TRY(cudaMemsetAsync(m.counters + kOccWorkN0 + nxt, 0, sizeof(int), stream));
        occ_free_nodes_kernel<<<sms * 4, 256, 0, stream>>>(m, f.frame_id, s.work[cur], m.counters + kOccWorkN0 + cur,
                                                           s.work[nxt], m.counters + kOccWorkN0 + nxt, s.freed, s.sets);
    }
    occ_free_blocks_kernel<<<sms * 8, 256, 0, stream>>>(m, f, depth_dev, s.sigma, s.freed);
    occ_update_blocks_kernel<<<sms * 8, 256, 0, stream>>>(m, f, depth_dev, s.sigma, s.block_list, s.block_var,
                                                          s.block_inside);
    occ_propagate_blocks_kernel<<<sms * 8, 256, 0, stream>>>(m, s.block_list, kOccBlockListN);
    occ_propagate_blocks_kernel<<<sms * 8, 256, 0, stream>>>(m, s.freed, kOccFreedN);
    occ_seed_sets_kernel<<<sms, 256, 0, stream>>>(m, f.frame_id, s.block_list, s.sets);
    for (int d = m.block_depth - 1; d > 0; --d)
        occ_propagate_nodes_kernel<<<sms * 4, 256, 0, stream>>>(m, f.frame_id, timestamp, d, s.sets);
    occ_propagate_root_kernel<<<1, 1, 0, stream>>>(m, timestamp);
    SE_CUDA_TRY(cudaGetLastError());
    return SE_GPU_OK;
}

} // namespace se_gpu

namespace se_gpu {

se_gpu_status occ_check(se_gpu_occ_map* om)
{
    int err = 0;
    SE_CUDA_TRY(cudaMemcpy(&err, om->dev.counters + kOccError, sizeof(int), cudaMemcpyDeviceToHost));
    if (!err)
        return SE_GPU_OK;
    SE_CUDA_TRY(cudaMemset(om->dev.counters + kOccError, 0, sizeof(int)));
    if (err & kOccErrBlockPool) {
        set_last_error("occupancy block pool of %d blocks is full", om->dev.block_capacity);
        return SE_GPU_ERR_POOL_FULL;
    }
    if (err & kOccErrNodePool) {
        set_last_error("occupancy node pool of %d nodes is full", om->dev.node_capacity);
        return SE_GPU_ERR_POOL_FULL;
    }
    set_last_error("an occupancy work list overflowed");
    return SE_GPU_ERR_POOL_FULL;
}

se_gpu_status occ_aabb(const se_gpu_occ_map* om, int32_t mn[3], int32_t mx[3], int* empty)
{
    int a[8];
    SE_CUDA_TRY(cudaMemcpy(a, om->dev.aabb, sizeof(a), cudaMemcpyDeviceToHost));
    *empty = a[6];
    for (int i = 0; i < 3; ++i) {
        mn[i] = a[6] ? 0 : a[i];
        mx[i] = a[6] ? 0 : a[3 + i];
    }
    return SE_GPU_OK;
}

} // namespace se_gpu

static se_gpu_status occ_args(const se_gpu_map* map, const char* fn)
{
    if (!map) {
        set_last_error("%s: null map", fn);
        return SE_GPU_ERR_BAD_ARG;
    }
    if (!map->occ) {
        set_last_error("%s: not an occupancy map", fn);
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    return SE_GPU_OK;
}

extern "C" {

se_gpu_status se_gpu_map_occupancy_stats(se_gpu_map* map, int64_t stats[4])
{
    se_gpu_status st = occ_args(map, "se_gpu_map_occupancy_stats");
    if (st != SE_GPU_OK)
        return st;
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    int c[kOccCounters];
    SE_CUDA_TRY(cudaMemcpy(c, map->occ->dev.counters, sizeof(c), cudaMemcpyDeviceToHost));
    stats[0] = c[kOccBlockListN];
    stats[1] = c[kOccNodeListN];
    stats[2] = c[kOccFreedN];
    stats[3] = c[kOccPruned];
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_download_occupancy(const se_gpu_map* map, int64_t capacity, int32_t* coords, int32_t* scales,
                                            int64_t* counts, float* mean, float* min_data, float* max_data,
                                            int64_t* count)
{
    se_gpu_status st = occ_args(map, "se_gpu_map_download_occupancy");
    if (st != SE_GPU_OK)
        return st;
    if (capacity < 0) {
        set_last_error("se_gpu_map_download_occupancy: negative capacity");
        return SE_GPU_ERR_BAD_ARG;
    }
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    const OccDevice& m = map->occ->dev;
    int nb = 0;
    SE_CUDA_TRY(cudaMemcpy(&nb, m.counters + kOccBlocks, sizeof(int), cudaMemcpyDeviceToHost));
    nb = nb < m.block_capacity ? nb : m.block_capacity;
    std::vector<OccBlockState> states((size_t) nb);
    std::vector<int> bc((size_t) nb * 3);
    if (nb) {
        SE_CUDA_TRY(cudaMemcpy(states.data(), m.block_state, (size_t) nb * sizeof(OccBlockState), cudaMemcpyDeviceToHost));
        SE_CUDA_TRY(cudaMemcpy(bc.data(), m.block_coord, (size_t) nb * 3 * sizeof(int), cudaMemcpyDeviceToHost));
    }
    int64_t live = 0;
    for (int b = 0; b < nb; ++b)
        live += states[(size_t) b].live ? 1 : 0;
    if (count)
        *count = live;
    const bool want_data = mean || min_data || max_data;
    std::vector<OccD> hm, hn, hx;
    if (want_data && nb) {
        hm.resize((size_t) nb * 585);
        hn.resize((size_t) nb * 585);
        hx.resize((size_t) nb * 585);
        SE_CUDA_TRY(cudaMemcpy(hm.data(), m.block_mean, hm.size() * sizeof(OccD), cudaMemcpyDeviceToHost));
        SE_CUDA_TRY(cudaMemcpy(hn.data(), m.block_min, hn.size() * sizeof(OccD), cudaMemcpyDeviceToHost));
        SE_CUDA_TRY(cudaMemcpy(hx.data(), m.block_max, hx.size() * sizeof(OccD), cudaMemcpyDeviceToHost));
    }
    int64_t k = 0;
    for (int b = 0; b < nb && k < capacity; ++b) {
        const OccBlockState& s = states[(size_t) b];
        if (!s.live)
            continue;
        if (coords)
            for (int a = 0; a < 3; ++a)
                coords[3 * k + a] = bc[(size_t) b * 3 + a];
        if (scales) {
            scales[3 * k] = s.current_scale;
            scales[3 * k + 1] = s.min_scale;
            scales[3 * k + 2] = s.buffer_scale;
        }
        if (counts) {
            counts[4 * k] = (int64_t) s.curr_integr;
            counts[4 * k + 1] = (int64_t) s.curr_obs;
            counts[4 * k + 2] = (int64_t) s.buf_integr;
            counts[4 * k + 3] = (int64_t) s.buf_obs;
        }
        if (want_data) {
            for (int sc = 0; sc <= kOccMaxScale; ++sc) {
                const int nv = (8 >> sc) * (8 >> sc) * (8 >> sc);
                for (int v = 0; v < nv; ++v) {
                    const size_t src = (size_t) b * 585 + occ_scale_offset(sc) + v;
                    const size_t o = ((size_t) k * 585 + occ_scale_offset(sc) + v) * 3;
                    const OccD e = sc < s.finest ? s.init_data : hm[src];
                    const OccD mn = sc < s.finest ? s.init_data : (sc == s.finest ? hm[src] : hn[src]);
                    const OccD mx = sc < s.finest ? s.init_data : (sc == s.finest ? hm[src] : hx[src]);
                    const OccD* ds[3] = {&e, &mn, &mx};
                    float* outs[3] = {mean, min_data, max_data};
                    for (int q = 0; q < 3; ++q) {
                        if (!outs[q])
                            continue;
                        outs[q][o] = ds[q]->occ;
                        outs[q][o + 1] = ds[q]->weight;
                        outs[q][o + 2] = ds[q]->observed ? 1.0f : 0.0f;
                    }
                }
            }
        }
        ++k;
    }
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_download_nodes(const se_gpu_map* map, int64_t capacity, int32_t* coords, float* min_data,
                                        float* max_data, int32_t* leaf, int64_t* count)
{
    se_gpu_status st = occ_args(map, "se_gpu_map_download_nodes");
    if (st != SE_GPU_OK)
        return st;
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    const OccDevice& m = map->occ->dev;
    int nn = 0;
    SE_CUDA_TRY(cudaMemcpy(&nn, m.counters + kOccNodes, sizeof(int), cudaMemcpyDeviceToHost));
    nn = nn < m.node_capacity ? nn : m.node_capacity;
    std::vector<int4> nc((size_t) nn);
    std::vector<int> ch((size_t) nn * 8);
    std::vector<OccD> nmin((size_t) nn), nmax((size_t) nn);
    SE_CUDA_TRY(cudaMemcpy(nc.data(), m.node_coord, (size_t) nn * sizeof(int4), cudaMemcpyDeviceToHost));
    SE_CUDA_TRY(cudaMemcpy(ch.data(), m.node_child, (size_t) nn * 8 * sizeof(int), cudaMemcpyDeviceToHost));
    SE_CUDA_TRY(cudaMemcpy(nmin.data(), m.node_min, (size_t) nn * sizeof(OccD), cudaMemcpyDeviceToHost));
    SE_CUDA_TRY(cudaMemcpy(nmax.data(), m.node_max, (size_t) nn * sizeof(OccD), cudaMemcpyDeviceToHost));
    std::vector<int> stack{0};
    int64_t k = 0;
    while (!stack.empty()) {
        const int n = stack.back();
        stack.pop_back();
        if (k < capacity) {
            if (coords) {
                coords[4 * k] = nc[(size_t) n].x;
                coords[4 * k + 1] = nc[(size_t) n].y;
                coords[4 * k + 2] = nc[(size_t) n].z;
                coords[4 * k + 3] = nc[(size_t) n].w;
            }
            const OccD* ds[2] = {&nmin[(size_t) n], &nmax[(size_t) n]};
            float* outs[2] = {min_data, max_data};
            for (int q = 0; q < 2; ++q) {
                if (!outs[q])
                    continue;
                outs[q][3 * k] = ds[q]->occ;
                outs[q][3 * k + 1] = ds[q]->weight;
                outs[q][3 * k + 2] = ds[q]->observed ? 1.0f : 0.0f;
            }
            if (leaf) {
                bool is_leaf = true;
                for (int i = 0; i < 8; ++i)
                    is_leaf = is_leaf && ch[(size_t) n * 8 + i] == -1;
                leaf[k] = is_leaf ? 1 : 0;
            }
        }
        ++k;
        for (int i = 7; i >= 0; --i) {
            const int c = ch[(size_t) n * 8 + i];
            if (c >= 0)
                stack.push_back(c);
        }
    }
    if (count)
        *count = k;
    return SE_GPU_OK;
}

} // extern "C"
