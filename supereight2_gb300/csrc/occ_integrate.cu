// occ_integrate.cu — se::MapIntegrator::integrateDepth for multi-resolution occupancy maps
// (map_integrator_impl.hpp:90-130) with a pinhole camera or an OusterLidar, for one map or a
// batch of up to kOccMaxBatch maps. Every stage is one launch over all maps of the batch: the
// per-map work lists (carver frontiers, block lists, propagation sets) are laid end to end and
// the grid strides over their concatenation, so maps with uneven work share one grid.
//   begin      per-frame state of each map (pose, inverse pose, frame stamp), list counters
//   pixels     uncert::depth_sigma (uncertainty.cpp:12-34) and level 0 of both pooling images
//   pooling    DensePoolingImage<PinholeCamera | OusterLidar> levels 1.. of the depth and sigma
//              images (dense_pooling_image_impl.hpp:56-213, 395-598), one launch per level
//   root       DensePoolingImage::maxValue, VolumeCarver's max depth and the root's children
//   carve      VolumeCarver (volume_carver_impl.hpp:46-537) breadth first, one launch per octree
//              depth; a split node allocates its 8 children (Octree::allocateChildren) and queues
//              them for the next depth
//   nodes      the carver's free-space nodes: AABB of the leaves, seeds of freeNodeRecurse
//   free       Updater::freeNodeRecurse (multires_ofusion_updater_impl.hpp:550-600) one level of
//              the free nodes' subtrees per launch
//   blocks     Updater::freeBlock on the blocks below free nodes and Updater::updateBlock
//              (:168-409) on the carver's blocks, one warp per block
//   propagate  propagate_block_to_coarsest_scale on those blocks, then propagateToRoot (:129-164)
//              one depth per launch from the blocks' parents up, with pruning, and the root
// The reference's recursion and OpenMP loops visit independent octants; the breadth-first
// launches visit the same octants with the same per-octant computation, so the allocated
// octree, the block lists (as sets) and every voxel agree with a serial run.
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "occupancy.cuh"
#include "pipeline.cuh"
#include "profile.cuh"

namespace se_gpu {

// --------------------------------------------------------------------- batch indexing --

// Exclusive prefix sums of the per-map item counts into shared memory (pre[0..n]); every thread
// of the CTA gets the total. blockDim.x >= 32.
template <class Count>
__device__ __forceinline__ int batch_prefix(const OccLaunch& L, int* pre, Count count)
{
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const int c = lane < L.n ? count(L.job[lane]) : 0;
        int incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
                incl += t;
        }
        if (lane < L.n)
            pre[lane + 1] = incl;
        if (lane == 0)
            pre[0] = 0;
    }
    __syncthreads();
    return pre[L.n];
}

__device__ __forceinline__ int batch_find(const int* pre, int n, int idx)
{
    int j = 0;
    while (j + 1 < n && pre[j + 1] <= idx)
        ++j;
    return j;
}

__device__ __forceinline__ int clamp_count(int c, int cap) { return c < cap ? c : cap; }

__device__ __forceinline__ int push(int* list, int* count, int cap, int v, int* err)
{
    const int k = atomicAdd(count, 1);
    if (k < cap)
        list[k] = v;
    else
        atomicOr(err, kOccErrList);
    return k;
}

// -------------------------------------------------------------------------- begin --

__device__ __forceinline__ void occ_begin(const OccLaunch& L, const OccStep& step, int j)
{
    if (j >= L.n)
        return;
    const OccJob& J = L.job[j];
    for (int i = kOccFirstFrameCounter + threadIdx.x; i < kOccCounters; i += blockDim.x)
        J.m.counters[i] = 0;
    if (threadIdx.x == 0) {
        OccDyn d;
        d.T_WS = tf_from16(step.T_WS[j]);
        d.T_SW = inverse_iso(d.T_WS);
        d.depth = step.depth[j];
        d.frame_id = J.dyn->frame_id + 1;
        d.timestamp = step.timestamp[j];
        *J.dyn = d;
    }
}

// The frame's poses, images and timestamps by value (single-map calls) or from a device buffer
// that the call fills on the stream before the launches (batches: their captured graph then
// replays unchanged).
__global__ void occ_begin_kernel(const OccLaunch* __restrict__ Lp, const __grid_constant__ OccStep step)
{
    occ_begin(*Lp, step, blockIdx.x);
}
__global__ void occ_begin_dev_kernel(const OccLaunch* __restrict__ Lp, const OccStep* __restrict__ step)
{
    occ_begin(*Lp, *step, blockIdx.x);
}

// ------------------------------------------------------------------ per-pixel inputs --

// uncert::depth_sigma with the linear model, and level 0 of both pooling images
// (Pixel::knownPixel / unknownPixel: min = FLT_MAX, max = FLT_MIN, the smallest normal float)
__device__ __forceinline__ void occ_pixel(const OccLaunch& L, int j, int i)
{
    const OccJob& J = L.job[j];
    const float d = J.dyn->depth[i];
    float sg;
    if (d <= 0.0f || isnan(d)) {
        sg = 0.0f;
    }
    else {
        const float v = J.m.cfg.k_sigma * d;
        sg = v < J.sigma_min ? J.sigma_min : (J.sigma_max < v ? J.sigma_max : v); // std::clamp
    }
    J.sigma[i] = sg;
    J.pool_depth[i] = d <= 0.0f ? make_float4(FLT_MAX, FLT_MIN, 0.0f, 2.0f) : make_float4(d, d, 0.0f, 0.0f);
    J.pool_sigma[i] = sg <= 0.0f ? make_float4(FLT_MAX, FLT_MIN, 0.0f, 2.0f) : make_float4(sg, sg, 0.0f, 0.0f);
}

__global__ void occ_pixels_kernel(const OccLaunch* __restrict__ Lp)
{
    const OccLaunch& L = *Lp;
    const int npx = L.sensor.w * L.sensor.h;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= npx || j >= L.n)
        return;
    occ_pixel(L, j, i);
}

// Level 1 (3x3 windows, dense_pooling_image_impl.hpp:92-165 / 423-478) or level l >= 2 (the four
// overlapping windows of level l - 1, :167-213 / 480-565) of both images of every map; the LiDAR
// image wraps around in u.
__device__ __forceinline__ void occ_pool_pixel(const OccLaunch& L, int level, int j, int which, int i)
{
    const int w = L.sensor.w, h = L.sensor.h, npx = w * h;
    const bool wrap = L.sensor.lidar != 0;
    const OccJob& J = L.job[j];
    float4* base = which ? J.pool_sigma : J.pool_depth;
    const float4* P = base + (size_t) (level - 1) * npx;
    const int x = i % w, y = i / w;
    float4 p = make_float4(FLT_MAX, FLT_MIN, 1.0f, 0.0f); // crossingKnownPixel
    if (level == 1) {
        if (y >= 1 && y < h - 1 && (wrap || (x >= 1 && x < w - 1)))
            p.z = 0.0f;
        const int top = y > 0 ? y - 1 : 0, bottom = y < h - 1 ? y + 1 : h - 1;
        const int left = x > 0 ? x - 1 : (wrap ? w - 1 : 0);
        const int right = x < w - 1 ? x + 1 : (wrap ? 0 : w - 1);
        const int xs[9] = {x, left, x, right, right, right, x, left, left};
        const int ys[9] = {y, top, top, top, y, bottom, bottom, bottom, y};
        float mn = FLT_MAX, mx = -FLT_MAX;
        int uf = 0;
        for (int k = 0; k < 9; ++k) {
            const float4 q = P[xs[k] + ys[k] * w];
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
    }
    else {
        const int s = 1 << (level - 1);
        const int s_half = s / 2;
        int left, right, top, bottom;
        if (x - s_half < 0)
            left = wrap ? w + (x - s_half) : 0;
        else
            left = x - s_half;
        if (x + s_half >= w)
            right = wrap ? (x + s_half) - w : w - 1;
        else
            right = x + s_half;
        if (y - s_half < 0)
            top = 0;
        else
            top = y - s_half;
        if (y + s_half >= h)
            bottom = h - 1;
        else
            bottom = y + s_half;
        const float4 a = P[left + top * w], b = P[right + top * w], c = P[left + bottom * w],
                     d = P[right + bottom * w];
        p.x = fminf(fminf(a.x, b.x), fminf(c.x, d.x));
        p.y = fmaxf(fmaxf(a.y, b.y), fmaxf(c.y, d.y));
        const int uf = (int) a.w + (int) b.w + (int) c.w + (int) d.w;
        if (uf == 8)
            p.w = 2.0f;
        else if (uf > 0)
            p.w = 1.0f;
        // the window crossing the border stays crossing; windows inside are inside
        if (y >= s && y < h - s && x >= s && x < w - s)
            p.z = 0.0f;
    }
    base[(size_t) level * npx + i] = p;
}

__global__ void occ_pool_level_kernel(const OccLaunch* __restrict__ Lp, int level)
{
    const OccLaunch& L = *Lp;
    const int npx = L.sensor.w * L.sensor.h;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y >> 1;
    if (i >= npx || j >= L.n)
        return;
    occ_pool_pixel(L, level, j, blockIdx.y & 1, i);
}

struct PoolQuery {
    float min, max;
    int crossing, known;
};

// Number of positions the pooling loops visit between lo and hi: lo + s, lo + s + step, ...,
// the last one clamped to hi - s (a single position hi - s when the range is narrower than 2s).
__device__ __forceinline__ int visit_count(int lo, int hi, int s, int step)
{
    const int d = (hi - s) - (lo + s);
    return d <= 0 ? 1 : (d + step - 1) / step + 1;
}

// poolBoundingBox (dense_pooling_image_impl.hpp:218-290; Ouster: 607-731, columns outside the
// image fetched from the other side) of the depth and the sigma pyramids (w * h per level) over
// the same box, by a whole warp: the lanes share the visited pixels, two per lane in flight, then
// reduce. The reference's statistics only enter through "all visited pixels unknown" and "some
// visited pixel unknown or partly known", and min / max do not depend on the order, so the
// result equals the serial loops'. Only the sigma query's max is used by the carver.
struct PoolPair {
    PoolQuery d;
    float sigma_max;
};

__device__ __forceinline__ int pool_index(int k, int nu, int u_min, int u_max, int v_min, int v_max, int s, int step,
                                          int w, bool u_wrap)
{
    const int iu = k % nu, iv = k / nu;
    const int u = min(u_min + s + iu * step, u_max - s);
    const int v = min(v_min + s + iv * step, v_max - s);
    int uf = u;
    if (u_wrap) {
        if (u < 0)
            uf += w;
        else if (u > w - 1)
            uf -= w;
    }
    return uf + w * v;
}

__device__ PoolPair pool_bounding_box(const float4* __restrict__ pool_d, const float4* __restrict__ pool_s, int w,
                                      int h, int max_level, bool wrap, int u_min, int u_max, int v_min, int v_max,
                                      int lane)
{
    const int min_side = min(u_max - u_min, v_max - v_min);
    const int half = min_side / 2;
    // log2(0) = -inf: the reference's clamps turn it into level 0
    int lc = INT_MIN;
    if (half > 0)
        lc = (int) ceil(log2((double) half));
    const int level = max(0, min(max_level, lc));
    const int s = level > 0 ? 1 << max(level - 1, 0) : 0;
    const int step = 2 * s + 1;
    const bool u_wrap = wrap && (u_min < 0 || u_max > w - 1);
    const int nu = visit_count(u_min, u_max, s, step), nv = visit_count(v_min, v_max, s, step);
    const int n = nu * nv;
    const float4* Ld = pool_d + (size_t) level * w * h;
    const float* Ls = reinterpret_cast<const float*>(pool_s + (size_t) level * w * h) + 1; // .y = max
    float mn = FLT_MAX, mx = FLT_MIN, smx = FLT_MIN; // Pixel::knownPixel
    bool all_unknown = true, any_part = false;
    for (int k = lane; k < n; k += 64) {
        const int i0 = pool_index(k, nu, u_min, u_max, v_min, v_max, s, step, w, u_wrap);
        const bool two = k + 32 < n;
        const int i1 = two ? pool_index(k + 32, nu, u_min, u_max, v_min, v_max, s, step, w, u_wrap) : i0;
        const float4 p0 = Ld[i0], p1 = Ld[i1];
        const float s0 = Ls[4 * (size_t) i0], s1 = Ls[4 * (size_t) i1];
        if (mx < p0.y)
            mx = p0.y;
        if (mn > p0.x)
            mn = p0.x;
        if (mx < p1.y)
            mx = p1.y;
        if (mn > p1.x)
            mn = p1.x;
        if (smx < s0)
            smx = s0;
        if (smx < s1)
            smx = s1;
        all_unknown = all_unknown && p0.w == 2.0f && p1.w == 2.0f;
        any_part = any_part || p0.w >= 1.0f || p1.w >= 1.0f;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float omn = __shfl_xor_sync(0xffffffffu, mn, o), omx = __shfl_xor_sync(0xffffffffu, mx, o);
        const float osx = __shfl_xor_sync(0xffffffffu, smx, o);
        if (mn > omn)
            mn = omn;
        if (mx < omx)
            mx = omx;
        if (smx < osx)
            smx = osx;
    }
    PoolPair r;
    r.d = PoolQuery{mn, mx, 0, 0};
    if (__all_sync(0xffffffffu, all_unknown))
        r.d.known = 2;
    else if (__any_sync(0xffffffffu, any_part))
        r.d.known = 1;
    r.sigma_max = smx;
    return r;
}

// conservativeQuery (dense_pooling_image_impl.hpp:295-347; Ouster: 734-781 clips only v) of the
// depth and the sigma pyramids, by a whole warp with uniform arguments
__device__ PoolPair conservative_query(const float4* __restrict__ pool_d, const float4* __restrict__ pool_s, int w,
                                       int h, int max_level, bool wrap, int u_min, int v_min, int u_max, int v_max,
                                       int lane)
{
    bool u_in = true, u_out = false, v_in = true, v_out = false;
    const float wl = (float) (unsigned) (w - 1), hl = (float) (unsigned) (h - 1);
    if (!wrap) {
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
        return PoolPair{PoolQuery{0.0f, 0.0f, 2, 2}, 0.0f};
    PoolPair p = pool_bounding_box(pool_d, pool_s, w, h, max_level, wrap, u_min, u_max, v_min, v_max, lane);
    if (!u_in || !v_in)
        p.d.crossing = 1;
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
            m.block_ts[b] = -1;
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

// Octree::allocateChildren by a whole warp (uniform n): lane i < 8 initialises child slot i if it
// is empty, one atomic reserves the pool entries of all of them.
__device__ void occ_allocate_children_warp(const OccDevice& m, int n, int lane)
{
    const OccD init = node_data(m, n); // read before any child slot changes
    const int4 nc = m.node_coord[n];
    const int csize = nc.w / 2;
    const bool blocks_below = nc.w == 16;
    int* child = m.node_child + 8 * (size_t) n;
    const int i = lane & 7;
    const bool need = lane < 8 && child[i] == -1;
    const unsigned mask = __ballot_sync(0xffffffffu, need);
    const int cnt = __popc(mask);
    int base = 0;
    if (lane == 0 && cnt > 0)
        base = atomicAdd(&m.counters[blocks_below ? kOccBlocks : kOccNodes], cnt);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (need) {
        const int idx = base + __popc(mask & ((1u << lane) - 1u));
        const int cx = nc.x + csize * (i & 1), cy = nc.y + csize * ((i >> 1) & 1), cz = nc.z + csize * (i >> 2);
        if (blocks_below) {
            if (idx >= m.block_capacity) {
                atomicOr(&m.counters[kOccError], kOccErrBlockPool);
            }
            else {
                m.block_coord[3 * idx] = cx;
                m.block_coord[3 * idx + 1] = cy;
                m.block_coord[3 * idx + 2] = cz;
                OccBlockState st;
                st.init_data = init;
                st.min_scale = -1;
                st.current_scale = kOccMaxScale;
                st.finest = kOccMaxScale;
                st.buffer_scale = -1;
                st.curr_integr = st.curr_obs = st.buf_integr = st.buf_obs = 0ull;
                st.parent = n;
                st.live = 1;
                m.block_state[idx] = st;
                blk_mean(m, idx, kOccMaxScale)[0] = init;
                m.block_ts[idx] = -1;
                child[i] = -2 - idx;
            }
        }
        else {
            if (idx >= m.node_capacity) {
                atomicOr(&m.counters[kOccError], kOccErrNodePool);
            }
            else {
                m.node_coord[idx] = make_int4(cx, cy, cz, csize);
                m.node_parent[idx] = n;
                for (int k = 0; k < 8; ++k)
                    m.node_child[8 * (size_t) idx + k] = -1;
                m.node_min[idx] = init;
                m.node_max[idx] = init;
                m.node_mark[idx] = -1;
                m.node_ts[idx] = -1;
                child[i] = idx;
            }
        }
    }
    __syncwarp();
    if (blocks_below && lane == 0)
        occ_aabb_extend(m, nc.x, nc.y, nc.z, nc.w);
}

// DensePoolingImage::maxValue over the coarsest level (the lanes share the visited pixels) and
// VolumeCarver's max depth (volume_carver_impl.hpp:28-38), then the root's children as the first
// frontier; one warp per map.
__device__ void occ_root(const OccLaunch& L, int j, int lane)
{
    const OccJob& J = L.job[j];
    const int w = L.sensor.w, h = L.sensor.h;
    const int max_level = L.sensor.levels - 1;
    const float4* Lmax = J.pool_depth + (size_t) max_level * w * h;
    const int s = 1 << (max_level - 1);
    // rows s, 3s, ... and the last row h - s - 1; the same for the columns
    const int nv = visit_count(0, h - 1, s, 2 * s), nu = visit_count(0, w - 1, s, 2 * s);
    float mv = 0.0f;
    for (int k = lane; k < nu * nv; k += 32) {
        const int u = min(s + (k % nu) * 2 * s, w - s - 1), v = min(s + (k / nu) * 2 * s, h - s - 1);
        const float m = Lmax[u + w * v].y;
        if (mv < m)
            mv = m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float om = __shfl_xor_sync(0xffffffffu, mv, o);
        if (mv < om)
            mv = om;
    }
    if (lane != 0)
        return;
    J.max_value[0] = mv;
    const float t = mv + J.tau_max;
    J.max_value[1] = L.sensor.far_plane < t ? L.sensor.far_plane : t;
    const OccDevice& m = J.m;
    occ_allocate_children(m, 0);
    int n = 0;
    for (int i = 0; i < 8; ++i)
        if (m.node_child[i] != -1)
            J.frontier[1][n++] = m.node_child[i]; // depth 1 reads frontier[1]
    m.counters[kOccFrontierN + 1] = n;
}

__global__ void occ_root_kernel(const OccLaunch* __restrict__ Lp)
{
    const OccLaunch& L = *Lp;
    if (blockIdx.x >= L.n || threadIdx.x >= 32)
        return;
    occ_root(L, blockIdx.x, threadIdx.x & 31);
}

// cameraInNode with pointToVoxel<Safe::On> (volume_carver_impl.hpp:83-98)
__device__ __forceinline__ bool camera_in_node(const OccDevice& m, const Tf& T_WS, int cx, int cy, int cz, int size)
{
    float vx = -1.0f, vy = -1.0f, vz = -1.0f;
    const F3 p_M = apply(m.T_MW, f3(T_WS.t[0], T_WS.t[1], T_WS.t[2]));
    if (p_M.x >= 0.0f && p_M.x < m.dim && p_M.y >= 0.0f && p_M.y < m.dim && p_M.z >= 0.0f && p_M.z < m.dim) {
        vx = p_M.x / m.res;
        vy = p_M.y / m.res;
        vz = p_M.z / m.res;
    }
    return vx >= (float) cx && vx <= (float) (cx + size) && vy >= (float) cy && vy <= (float) (cy + size)
        && vz >= (float) cz && vz <= (float) (cz + size);
}

// computeVariance (volume_carver_impl.hpp:100-126): 0 Constant, 1 Gradient, 2 Undefined
__device__ __forceinline__ int compute_variance(const OccJob& J, float d_min, float d_max, float n_min, float n_max,
                                                float std_max)
{
    const float z_diff_max = n_max - d_min;
    const float z_diff_min = n_min - d_max;
    const float tv = J.m.cfg.k_tau * d_max;
    const float tau_max = tv < J.tau_min ? J.tau_min : (J.tau_max < tv ? J.tau_max : tv);
    const float three_sigma_min = 3.0f * std_max;
    if ((double) z_diff_min > 1.25 * (double) tau_max)
        return 2;
    if ((double) z_diff_max < -1.25 * (double) three_sigma_min)
        return 0;
    return 1;
}

// The octant's maximum data for the carver's redundancy test (maxData / NodeData::data()).
__device__ __forceinline__ OccD octant_max_data(const OccDevice& m, int slot)
{
    if (slot_is_block(slot)) {
        const int b = slot_block(slot);
        return blk_max(m, b, m.block_state[b].finest, kOccMaxScale)[0];
    }
    return node_data(m, slot);
}

// Min / max of a per-corner value over the 8 lanes of each 8-lane group (lane & 7 = corner);
// exact in any order.
__device__ __forceinline__ float corner_min(float v)
{
    for (int o = 1; o < 8; o <<= 1)
        v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float corner_max(float v)
{
    for (int o = 1; o < 8; o <<= 1)
        v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// The pooled-depth cases shared by both carvers; returns false when the octant is skipped.
__device__ __forceinline__ bool carve_pooled(const OccLaunch& L, const OccJob& J, int slot, int bu0, int bv0, int bu1,
                                             int bv1, float n_min, float n_max, bool& should_split, int& var,
                                             bool& projects_inside, int lane)
{
    const OccSensor& S = L.sensor;
    const bool wrap = S.lidar != 0;
    // both pyramids in one pass; the reference queries sigma only after the two early returns
    const PoolPair q =
        conservative_query(J.pool_depth, J.pool_sigma, S.w, S.h, S.levels - 1, wrap, bu0, bv0, bu1, bv1, lane);
    const PoolQuery& pp = q.d;
    if (pp.known == 2)
        return false;
    if (n_min > pp.max + J.tau_max)
        return false;
    var = compute_variance(J, pp.min, pp.max, n_min, n_max, q.sigma_max);
    if (var != 1) {
        const OccD cd = octant_max_data(J.m, slot);
        if (cd.observed && (double) occ_field(cd) <= 0.95 * -100.0)
            return false;
    }
    if (pp.crossing == 1)
        should_split = true;
    else if (pp.known == 1)
        should_split = true;
    else if (var == 1)
        should_split = true;
    projects_inside = pp.known == 0;
    return true;
}

__device__ __forceinline__ F3 corner_point(const OccDevice& m, const Tf& T_SW, int k, int cx, int cy, int cz, int size)
{
    const F3 p_M = f3(((float) size * (float) (k & 1) + (float) cx) * m.res,
                      ((float) size * (float) ((k >> 1) & 1) + (float) cy) * m.res,
                      ((float) size * (float) (k >> 2) + (float) cz) * m.res);
    return apply(T_SW, apply(m.T_WM, p_M));
}

// VolumeCarver<.., PinholeCamera>::operator()(octant) (volume_carver_impl.hpp:132-310) by a
// warp: lane & 7 projects corner lane & 7, the bounding box and the pooling queries are warp-wide.
__device__ bool carve_pinhole(const OccLaunch& L, const OccJob& J, const OccDyn& D, int slot, int cx, int cy, int cz,
                              int size, float max_depth_value, bool& should_split, int& var, bool& projects_inside,
                              int lane)
{
    const OccDevice& m = J.m;
    const Pinhole& ps = L.sensor.s;
    const float size_to_radius = sqrtf(3.0f) / 2.0f;
    const float zero_depth_band = 1.0e-6f;
    const float off = (float) size * 0.5f;
    const F3 centre_W =
        apply(m.T_WM, f3(((float) cx + off) * m.res, ((float) cy + off) * m.res, ((float) cz + off) * m.res));
    const F3 centre_S = apply(D.T_SW, centre_W);
    const float rad = (float) size * size_to_radius * m.res;
    if (centre_S.z - rad > max_depth_value || centre_S.z + rad < zero_depth_band)
        return false;
    const int k = lane & 7;
    const F3 p = corner_point(m, D.T_SW, k, cx, cy, cz, size);
    const bool front = !(p.z < zero_depth_band);
    const int n_front = __popc(__ballot_sync(0xffffffffu, front) & 0xffu);
    if (n_front == 0)
        return false;
    float pu = 0.0f, pv = 0.0f;
    bool ok = false;
    if (!(fabsf(p.z) < 1.0e-12f)) {
        const float rz = 1.0f / p.z;
        pu = ps.fx * (p.x * rz) + ps.cx;
        pv = ps.fy * (p.y * rz) + ps.cy;
        ok = p.z > 0.0f && pu >= -0.5f && pu < (float) ps.w - 0.5f && pv >= -0.5f && pv < (float) ps.h - 0.5f;
    }
    if (n_front < 8) {
        const bool crosses = (__ballot_sync(0xffffffffu, ok) & 0xffu) != 0u;
        if (camera_in_node(m, D.T_WS, cx, cy, cz, size) || crosses) {
            should_split = true;
            return true;
        }
        // sphereInFrustumInf: the frustum planes without the far one
        for (int i = 0; i < 5; ++i) {
            const float d =
                ((centre_S.x * ps.planes[i][0] + centre_S.y * ps.planes[i][1]) + centre_S.z * ps.planes[i][2])
                + ps.planes[i][3];
            if (d < -rad)
                return false;
        }
        should_split = true;
        return true;
    }
    float u = pu > 1e7f ? 1e7f : pu;
    float v = pv > 1e7f ? 1e7f : pv;
    u = u < -1e7f ? -1e7f : u;
    v = v < -1e7f ? -1e7f : v;
    const float umin = corner_min(u), umax = corner_max(u), vmin = corner_min(v), vmax = corner_max(v);
    const float zmin = corner_min(p.z), zmax = corner_max(p.z);
    return carve_pooled(L, J, slot, (int) umin, (int) vmin, (int) umax, (int) vmax, zmin, zmax, should_split, var,
                        projects_inside, lane);
}

// VolumeCarver<.., OusterLidar>::operator()(octant) (volume_carver_impl.hpp:339-537) by a warp:
// range bounds, camera-in-node first, corner columns unwrapped around the centre's column.
__device__ bool carve_lidar(const OccLaunch& L, const OccJob& J, const OccDyn& D, int slot, int cx, int cy, int cz,
                            int size, float max_depth_value, bool& should_split, int& var, bool& projects_inside,
                            int lane)
{
    const OccDevice& m = J.m;
    const Lidar& ld = L.sensor.L;
    const float size_to_radius = sqrtf(3.0f) / 2.0f;
    const float off = (float) size * 0.5f;
    const F3 centre_W =
        apply(m.T_WM, f3(((float) cx + off) * m.res, ((float) cy + off) * m.res, ((float) cz + off) * m.res));
    const F3 centre_S = apply(D.T_SW, centre_W);
    const float rad = (float) size * size_to_radius * m.res;
    const float range = norm(centre_S);
    const float approx_max = range + rad;
    const float approx_min = range - rad;
    if (approx_min > max_depth_value)
        return false;
    if (camera_in_node(m, D.T_WS, cx, cy, cz, size)) {
        should_split = true;
        return true;
    }
    float pu, pv;
    lidar_project(ld, corner_point(m, D.T_SW, lane & 7, cx, cy, cz, size), pu, pv);
    float cu, cv;
    lidar_project(ld, centre_S, cu, cv);
    const float W = (float) ld.w;
    float cu_comp = cu + (float) (ld.w / 2);
    if (cu_comp > W - 0.5f)
        cu_comp = cu_comp - W;
    if (cu < cu_comp && pu > cu && pu > cu_comp)
        pu = pu - W;
    else if (cu > cu_comp && pu < cu && pu < cu_comp)
        pu = pu + W;
    const float umin = corner_min(pu), umax = corner_max(pu), vmin = corner_min(pv), vmax = corner_max(pv);
    return carve_pooled(L, J, slot, (int) umin, (int) vmin, (int) umax, (int) vmax, approx_min, approx_max,
                        should_split, var, projects_inside, lane);
}

// One depth of the VolumeCarver over every map's frontier at that depth, one warp per octant;
// lane 0 lists the octant or allocates and queues its children.
__device__ void occ_carve_stage(const OccLaunch& L, int depth, int bid, int nbid)
{
    __shared__ int pre[kOccMaxBatch + 1];
    const int total = batch_prefix(L, pre, [depth](const OccJob& J) {
        return clamp_count(J.m.counters[kOccFrontierN + depth], J.m.node_capacity + J.m.block_capacity);
    });
    const int lane = threadIdx.x & 31;
    const int n_warps = (nbid * blockDim.x) >> 5;
    for (int idx = (bid * blockDim.x + threadIdx.x) >> 5; idx < total; idx += n_warps) {
        const int j = batch_find(pre, L.n, idx);
        const OccJob& J = L.job[j];
        const OccDevice& m = J.m;
        const OccDyn& D = *J.dyn;
        int* err = &m.counters[kOccError];
        const int slot = J.frontier[depth & 1][idx - pre[j]];
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
        bool should_split = false, projects_inside = false;
        int var = 1; // Gradient
        const float max_depth_value = J.max_value[1];
        const bool keep = L.sensor.lidar
            ? carve_lidar(L, J, D, slot, cx, cy, cz, size, max_depth_value, should_split, var, projects_inside, lane)
            : carve_pinhole(L, J, D, slot, cx, cy, cz, size, max_depth_value, should_split, var, projects_inside,
                            lane);
        if (keep && !is_block && should_split) {
            occ_allocate_children_warp(m, slot, lane);
            // queue the children: one atomic for all of them, lane i writes child i
            const int ch = lane < 8 ? m.node_child[8 * (size_t) slot + lane] : -1;
            const unsigned mask = __ballot_sync(0xffffffffu, ch != -1); // -1 only when a pool ran out
            int base = 0;
            if (lane == 0 && mask)
                base = atomicAdd(&m.counters[kOccFrontierN + depth + 1], __popc(mask));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (ch != -1) {
                const int k = base + __popc(mask & ((1u << lane) - 1u));
                if (k < m.node_capacity + m.block_capacity)
                    J.frontier[(depth + 1) & 1][k] = ch;
                else
                    atomicOr(err, kOccErrList);
            }
        }
        else if (keep && lane == 0) {
            if (is_block) {
                const int k = push(J.block_list, &m.counters[kOccBlockListN], m.block_capacity, slot_block(slot), err);
                if (k < m.block_capacity) {
                    J.block_var[k] = var;
                    J.block_inside[k] = projects_inside ? 1 : 0;
                }
            }
            else if (var == 0) {
                push(J.node_list, &m.counters[kOccNodeListN], m.node_capacity, slot, err);
            }
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(128) occ_carve_kernel(const OccLaunch* __restrict__ Lp, int depth)
{
    occ_carve_stage(*Lp, depth, blockIdx.x, gridDim.x);
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

// The carver's free-space nodes: the AABB grows by the leaves among them (Updater, multires_
// ofusion_updater_impl.hpp:70-78) and they seed level 0 of freeNodeRecurse.
__device__ void occ_nodes_stage(const OccLaunch& L, int bid, int nbid)
{
    __shared__ int pre[kOccMaxBatch + 1];
    const int total = batch_prefix(
        L, pre, [](const OccJob& J) { return clamp_count(J.m.counters[kOccNodeListN], J.m.node_capacity); });
    if (bid == 0 && threadIdx.x < L.n)
        L.job[threadIdx.x].m.counters[kOccWorkN] = pre[threadIdx.x + 1] - pre[threadIdx.x];
    for (int idx = bid * blockDim.x + threadIdx.x; idx < total; idx += nbid * blockDim.x) {
        const int j = batch_find(pre, L.n, idx);
        const OccJob& J = L.job[j];
        const OccDevice& m = J.m;
        const int i = idx - pre[j];
        const int node = J.node_list[i];
        if (node_is_leaf(m, node)) {
            const int4 c = m.node_coord[node];
            occ_aabb_extend(m, c.x, c.y, c.z, c.w);
        }
        J.work[0][i] = make_int2(node, occ_node_depth(m, node));
    }
}

__global__ void occ_nodes_kernel(const OccLaunch* __restrict__ Lp)
{
    occ_nodes_stage(*Lp, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void occ_update(OccD& d, float value, float max_weight)
{
    if (d.weight < max_weight)
        d.weight = d.weight + 1.0f;
    d.occ = (d.occ * (d.weight - 1.0f) + value) / d.weight;
    d.observed = 1;
}

// Updater::freeNodeRecurse, one level of the subtrees per launch: leaves are freed in place,
// blocks go to the freed list, inner nodes queue their children.
__device__ void occ_free_nodes_stage(const OccLaunch& L, int level, int bid, int nbid)
{
    __shared__ int pre[kOccMaxBatch + 1];
    const int total = batch_prefix(
        L, pre, [level](const OccJob& J) { return clamp_count(J.m.counters[kOccWorkN + level], J.m.node_capacity); });
    for (int idx = bid * blockDim.x + threadIdx.x; idx < total; idx += nbid * blockDim.x) {
        const int j = batch_find(pre, L.n, idx);
        const OccJob& J = L.job[j];
        const OccDevice& m = J.m;
        const int frame_id = J.dyn->frame_id;
        int* err = &m.counters[kOccError];
        const int2 it = J.work[level & 1][idx - pre[j]];
        const int n = it.x, depth = it.y;
        if (node_is_leaf(m, n)) {
            OccD d = node_data(m, n);
            occ_update(d, m.cfg.log_odd_min, m.cfg.max_weight);
            m.node_min[n] = d;
            m.node_max[n] = d;
            occ_set_insert(m, J.sets, m.node_parent[n], frame_id);
        }
        else {
            for (int c = 0; c < 8; ++c) {
                const int ch = m.node_child[8 * (size_t) n + c];
                if (ch == -1)
                    continue;
                if (slot_is_block(ch)) {
                    occ_set_insert(m, J.sets, n, frame_id);
                    push(J.freed, &m.counters[kOccFreedN], m.block_capacity, slot_block(ch), err);
                }
                else {
                    const int k = atomicAdd(&m.counters[kOccWorkN + level + 1], 1);
                    if (k < m.node_capacity)
                        J.work[(level + 1) & 1][k] = make_int2(ch, depth + 1);
                    else
                        atomicOr(err, kOccErrList);
                }
            }
        }
    }
}

__global__ void occ_free_nodes_kernel(const OccLaunch* __restrict__ Lp, int level)
{
    occ_free_nodes_stage(*Lp, level, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------- block state machine --

// Sums a per-lane flag over the warp.
__device__ __forceinline__ unsigned warp_count(bool b) { return __popc(__ballot_sync(0xffffffffu, b)); }

__device__ __forceinline__ float clampf_std(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }

// PinholeCamera::computeIntegrationScaleImpl (pinhole_camera.cpp:115-152), ratios {1.5, 3, 6}
__device__ int pinhole_integration_scale(const Pinhole& s, float z, float res, int last_scale, int min_scale)
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

// OusterLidar::computeIntegrationScaleImpl (ouster_lidar.cpp:107-146): the chord between
// neighbouring rays, 2 r tan(min_ray_angle / 2), against the voxel diagonal sqrt(3) res; the
// hysteresis moves the point 0.25 m along its ray.
__device__ int lidar_integration_scale(const Lidar& ld, F3 c, float res, int last_scale, int min_scale)
{
    for (int pass = 0; pass < 2; ++pass) {
        const float dist = norm(c);
        const float pixel_dim = 2.0f * dist * ld.tan_half_min_angle;
        const float pv = (float) ((double) pixel_dim / (sqrt(3.0) * (double) res));
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
            const F3 n = normalized(c);
            c = scale > last_scale ? sub(c, mul(0.25f, n)) : add(c, mul(0.25f, n));
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
            const unsigned ls = 3u - (unsigned) last_scale; // np = 2^ls
            const unsigned x = pidx & (np - 1u), y = (pidx >> ls) & (np - 1u), z = pidx >> (2u * ls);
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

// updateBlockData<UpdateBuffer> (multires_ofusion_updater_impl.hpp:413-545) by a warp; the
// measurement is the point's z for a pinhole camera and its range for a LiDAR.
__device__ void occ_update_block_data(const OccLaunch& L, const OccJob& J, const OccDyn& D, int b, OccBlockState& st,
                                      F3 centre_C, int scale, bool low_var, bool inside, bool to_buffer, int lane)
{
    const OccDevice& m = J.m;
    const OccSensor& S = L.sensor;
    const bool lidar = S.lidar != 0;
    const float* __restrict__ depth = D.depth;
    const float* __restrict__ sigma = J.sigma;
    const int stride = 1 << scale;
    const int n = 8 >> scale, n2 = n * n;
    const int cx = m.block_coord[3 * b], cy = m.block_coord[3 * b + 1], cz = m.block_coord[3 * b + 2];
    const float off = (float) stride * 0.5f;
    const F3 base_C = apply(D.T_SW, apply(m.T_WM, f3(((float) cx + off) * m.res, ((float) cy + off) * m.res,
                                                   ((float) cz + off) * m.res)));
    const float rs = m.res * (float) stride;
    float Dm[9];
    for (int i = 0; i < 9; ++i)
        Dm[i] = D.T_SW.R[i] * rs;
    const float tv = m.cfg.k_tau * (lidar ? norm(centre_C) : centre_C.z);
    const float tau = clampf_std(tv, J.tau_min, J.tau_max);
    OccD* data = to_buffer ? blk_buffer(m, b, st) : blk_mean(m, b, st.current_scale);
    const float lom = m.cfg.log_odd_min, lomax = m.cfg.log_odd_max;
    // four voxels per lane per round: all projections first, then every load of the round in
    // flight together, then the updates (the same per-voxel arithmetic as one at a time)
    constexpr int kU = 4;
    int newly_lane = 0;
    for (int base = 0; base < n * n2; base += 32 * kU) {
        F3 p[kU];
        int pix[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const int k = base + lane + 32 * u;
            pix[u] = -1;
            p[u] = f3(0.0f, 0.0f, 0.0f);
            if (k < n * n2) {
                const int x = k & (n - 1), y = (k >> (3 - scale)) & (n - 1), z = k >> (2 * (3 - scale));
                const float fx = (float) x, fy = (float) y, fz = (float) z;
                const F3 dl = f3((Dm[0] * fx + Dm[1] * fy) + Dm[2] * fz, (Dm[3] * fx + Dm[4] * fy) + Dm[5] * fz,
                                 (Dm[6] * fx + Dm[7] * fy) + Dm[8] * fz);
                p[u] = add(base_C, dl);
                float uu, vv;
                if (lidar ? lidar_project(S.L, p[u], uu, vv) : project(S.s, p[u], uu, vv))
                    pix[u] = (int) (uu + 0.5f) + (int) (vv + 0.5f) * S.w;
            }
        }
        float dv[kU], sg[kU];
        OccD d[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            dv[u] = 0.0f;
            sg[u] = 0.0f;
            d[u] = occ_default();
            if (pix[u] >= 0) {
                dv[u] = depth[pix[u]];
                sg[u] = sigma[pix[u]];
                d[u] = data[base + lane + 32 * u];
            }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            if (pix[u] < 0 || dv[u] < S.near_plane)
                continue;
            const int k = base + lane + 32 * u;
            const float three_sigma = 3.0f * sg[u];
            bool newly = false, count = true;
            if (low_var) {
                newly = !d[u].observed;
                occ_update(d[u], lom, m.cfg.max_weight);
                data[k] = d[u];
            }
            else {
                const float range = sqrtf(dot(p[u], p[u]));
                const float pm = lidar ? range : p[u].z;
                // for the LiDAR range / pm is range / range, exactly 1
                const float range_diff = lidar ? (pm - dv[u]) : (pm - dv[u]) * (range / pm);
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
                    newly = !d[u].observed;
                    occ_update(d[u], sample, m.cfg.max_weight);
                    data[k] = d[u];
                }
                if (dv[u] > S.far_plane)
                    count = false;
            }
            newly_lane += (newly && count) ? 1 : 0;
        }
    }
    unsigned long long newly_total = (unsigned long long) newly_lane;
    for (int o = 16; o > 0; o >>= 1)
        newly_total += __shfl_xor_sync(0xffffffffu, newly_total, o);
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

__device__ __forceinline__ int occ_recommended_scale(const OccLaunch& L, const OccDevice& m, int b,
                                                     const OccBlockState& st, F3 centre_C, bool free_min,
                                                     int& last_scale)
{
    last_scale = (st.min_scale == -1) ? 0 : st.current_scale;
    const int computed = L.sensor.lidar
        ? lidar_integration_scale(L.sensor.L, centre_C, m.res, last_scale, st.min_scale)
        : pinhole_integration_scale(L.sensor.s, centre_C.z, m.res, last_scale, st.min_scale);
    const OccD mx = blk_max(m, b, st.finest, kOccMaxScale)[0];
    const int min_integr = (free_min && (st.min_scale == -1 || (double) mx.occ < 0.95 * (double) m.cfg.log_odd_min))
        ? m.cfg.fs_integr_scale
        : max(0, last_scale - 1);
    const int max_integr = (st.min_scale == -1) ? kOccMaxScale : min(kOccMaxScale, last_scale + 1);
    return min(max(min_integr, computed), max_integr);
}

// Updater::updateBlock (free == false) / Updater::freeBlock (free == true), one warp per block
__device__ void occ_process_block(const OccLaunch& L, const OccJob& J, int b, bool low_var, bool inside, bool free,
                                  int lane)
{
    const OccDevice& m = J.m;
    const OccDyn& D = *J.dyn;
    OccBlockState st = m.block_state[b];
    const float off = 8.0f * 0.5f;
    const F3 centre_C = apply(D.T_SW, apply(m.T_WM, f3(((float) m.block_coord[3 * b] + off) * m.res,
                                                       ((float) m.block_coord[3 * b + 1] + off) * m.res,
                                                       ((float) m.block_coord[3 * b + 2] + off) * m.res)));
    int last_scale;
    const int rec = occ_recommended_scale(L, m, b, st, centre_C, free ? true : low_var, last_scale);
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
            occ_update_block_data(L, J, D, b, st, centre_C, rec, low_var, inside, true, lane);
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
            occ_update_block_data(L, J, D, b, st, centre_C, integration_scale, low_var, inside, false, lane);
        }
    }
    if (lane == 0)
        m.block_state[b] = st;
    __syncwarp();
}

// freeBlock on the freed blocks and updateBlock on the carver's blocks (disjoint: the carver
// does not descend below a free-space node), one warp per block, all maps.
__device__ void occ_blocks_stage(const OccLaunch& L, int bid, int nbid)
{
    __shared__ int pre[kOccMaxBatch + 1];
    const int total = batch_prefix(L, pre, [](const OccJob& J) {
        return clamp_count(J.m.counters[kOccFreedN], J.m.block_capacity)
            + clamp_count(J.m.counters[kOccBlockListN], J.m.block_capacity);
    });
    const int lane = threadIdx.x & 31;
    const int n_warps = (nbid * blockDim.x) >> 5;
    for (int idx = (bid * blockDim.x + threadIdx.x) >> 5; idx < total; idx += n_warps) {
        const int j = batch_find(pre, L.n, idx);
        const OccJob& J = L.job[j];
        const int n_freed = clamp_count(J.m.counters[kOccFreedN], J.m.block_capacity);
        const int i = idx - pre[j];
        if (i < n_freed)
            occ_process_block(L, J, J.freed[i], true, true, true, lane);
        else
            occ_process_block(L, J, J.block_list[i - n_freed], J.block_var[i - n_freed] == 0,
                              J.block_inside[i - n_freed] != 0, false, lane);
    }
}

__global__ void __launch_bounds__(256, 2) occ_blocks_kernel(const OccLaunch* __restrict__ Lp)
{
    occ_blocks_stage(*Lp, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------- propagation --

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

// Streaming forms of the two reductions: children in index order, the same comparisons and
// sums as occ_up_best / occ_up_mean.
struct UpBest {
    float best;
    OccD pick;
    int nv, no;
};
__device__ __forceinline__ void up_best_add(UpBest& a, const OccD& c, bool want_min)
{
    if (occ_valid(c)) {
        ++a.nv;
        a.no += c.observed ? 1 : 0;
        const float fv = occ_field(c);
        if (want_min ? (fv < a.best) : (fv > a.best)) {
            a.best = fv;
            a.pick = c;
        }
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
        const int np = 8 >> ps;
        OccD* pmin = blk_min(m, b, st.finest, ps);
        OccD* pmax = blk_max(m, b, st.finest, ps);
        OccD* pmean = blk_mean(m, b, ps);
        const OccD* cmean = blk_mean(m, b, cs);
        const OccD* cmin = blk_min(m, b, st.finest, cs);
        const OccD* cmax = blk_max(m, b, st.finest, cs);
        const bool first = ps == st.current_scale + 1;
        const bool do_mean = !(first && st.buffer_scale > st.current_scale);
        for (int k = lane; k < np * np * np; k += 32) {
            const int lp = 3 - ps; // np = 2^lp
            const int x = k & (np - 1), y = (k >> lp) & (np - 1), z = k >> (2 * lp);
            // ch[0] is visited first so that ties keep the lowest child index, as the array form
            UpBest lo{FLT_MAX, OccD{0.0f, 0.0f, 0}, 0, 0}, hi{-FLT_MAX, OccD{0.0f, 0.0f, 0}, 0, 0};
            float os = 0.0f, ws = 0.0f;
            int nmean = 0;
            bool lo_first = true, hi_first = true;
            for (int c = 0; c < 8; ++c) {
                const int ci = (2 * x + (c & 1)) + ((2 * y + ((c >> 1) & 1)) << (lp + 1))
                    + ((2 * z + (c >> 2)) << (2 * (lp + 1)));
                const OccD c0 = cmean[ci];
                const OccD c1 = first ? c0 : cmin[ci];
                const OccD c2 = first ? c0 : cmax[ci];
                if (occ_valid(c0)) {
                    ++nmean;
                    os += c0.occ;
                    ws += c0.weight;
                }
                // the array form starts from index 0 when no child beats the initial bound
                if (lo_first) {
                    lo.pick = c1;
                    lo_first = false;
                }
                if (hi_first) {
                    hi.pick = c2;
                    hi_first = false;
                }
                up_best_add(lo, c1, true);
                up_best_add(hi, c2, false);
            }
            if (do_mean && nmean > 0) {
                OccD& p = pmean[k];
                p.occ = os / (float) nmean;
                p.weight = ceilf(ws / (float) nmean);
                p.observed = 0;
            }
            if (lo.nv > 0) {
                OccD r = lo.pick;
                r.observed = (lo.no == 8) ? 1 : 0;
                pmin[k] = r;
            }
            if (hi.nv > 0) {
                OccD r = hi.pick;
                r.observed = (hi.no == 8) ? 1 : 0;
                pmax[k] = r;
            }
        }
        __syncwarp();
    }
}

// Block propagation on the freed and the carver's blocks (one warp per block); the carver's
// blocks also put their parents in the first propagation set (propagateToRoot's seeds).
__device__ void occ_propagate_blocks_stage(const OccLaunch& L, int bid, int nbid)
{
    __shared__ int pre[kOccMaxBatch + 1];
    const int total = batch_prefix(L, pre, [](const OccJob& J) {
        return clamp_count(J.m.counters[kOccFreedN], J.m.block_capacity)
            + clamp_count(J.m.counters[kOccBlockListN], J.m.block_capacity);
    });
    const int lane = threadIdx.x & 31;
    const int n_warps = (nbid * blockDim.x) >> 5;
    for (int idx = (bid * blockDim.x + threadIdx.x) >> 5; idx < total; idx += n_warps) {
        const int j = batch_find(pre, L.n, idx);
        const OccJob& J = L.job[j];
        const OccDevice& m = J.m;
        const int n_freed = clamp_count(m.counters[kOccFreedN], m.block_capacity);
        const int i = idx - pre[j];
        const int b = i < n_freed ? J.freed[i] : J.block_list[i - n_freed];
        occ_propagate_block(m, b, lane);
        if (i >= n_freed && lane == 0)
            occ_set_insert(m, J.sets, m.block_state[b].parent, J.dyn->frame_id);
    }
}

__global__ void __launch_bounds__(256) occ_propagate_blocks_kernel(const OccLaunch* __restrict__ Lp)
{
    occ_propagate_blocks_stage(*Lp, blockIdx.x, gridDim.x);
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

// One depth of propagateToRoot over every map's propagation set at that depth.
__device__ void occ_propagate_nodes_stage(const OccLaunch& L, int depth, int bid, int nbid)
{
    __shared__ int pre[kOccMaxBatch + 1];
    const int total = batch_prefix(
        L, pre, [depth](const OccJob& J) { return clamp_count(J.m.counters[kOccSetN + depth], J.m.node_capacity); });
    for (int idx = bid * blockDim.x + threadIdx.x; idx < total; idx += nbid * blockDim.x) {
        const int j = batch_find(pre, L.n, idx);
        const OccJob& J = L.job[j];
        const OccDevice& m = J.m;
        const OccDyn& D = *J.dyn;
        const int node = J.sets[(size_t) depth * m.node_capacity + (idx - pre[j])];
        if (m.node_ts[node] == D.timestamp)
            continue;
        if (m.node_parent[node] < 0)
            continue;
        const OccD nd = occ_propagate_node(m, node, D.timestamp);
        occ_set_insert(m, J.sets, m.node_parent[node], D.frame_id);
        if (nd.observed && (double) occ_field(nd) <= 0.95 * -100.0) {
            occ_delete_children(m, node);
            atomicAdd(&m.counters[kOccPruned], 1);
        }
    }
}

__global__ void occ_propagate_nodes_kernel(const OccLaunch* __restrict__ Lp, int depth)
{
    occ_propagate_nodes_stage(*Lp, depth, blockIdx.x, gridDim.x);
}

__global__ void occ_propagate_root_kernel(const OccLaunch* __restrict__ Lp)
{
    const OccLaunch& L = *Lp;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= L.n)
        return;
    const OccJob& J = L.job[j];
    occ_propagate_node(J.m, 0, J.dyn->timestamp);
}

// ------------------------------------------------------------- one persistent launch --

// A whole frame of every map of a batch in one cooperative launch: the stages above in order,
// each a grid-stride loop over the persistent grid, separated by grid barriers.

constexpr unsigned long long kOccBarrierNs = 1000000000ull; // 1 s per barrier wait

struct OccBarrier {
    unsigned count;
    int timeout;
};

__device__ __forceinline__ unsigned long long occ_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Every CTA adds itself with release semantics, then one thread per CTA polls with acquire
// semantics, so the CTA's loads after the barrier see every CTA's writes before it. A wait past
// kOccBarrierNs raises the timeout flag, and every CTA then leaves at its next check; false once
// the flag is up.
__device__ bool occ_grid_sync(OccBarrier* bar, unsigned& phase)
{
    ++phase;
    const unsigned target = phase * gridDim.x;
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&bar->count) : "memory");
        const unsigned long long t0 = occ_ns();
        unsigned spins = 0;
        for (;;) {
            unsigned v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(&bar->count) : "memory");
            if (v >= target)
                break;
            if ((++spins & 63u) == 0u && (*((volatile int*) &bar->timeout) != 0 || occ_ns() - t0 > kOccBarrierNs)) {
                atomicExch(&bar->timeout, 1);
                break;
            }
        }
    }
    __syncthreads();
    return *((volatile int*) &bar->timeout) == 0;
}

__global__ void __launch_bounds__(256, 2) occ_persistent_kernel(const OccLaunch* __restrict__ Lp,
                                                                const OccStep* __restrict__ step, OccBarrier* bar)
{
    const OccLaunch& L = *Lp;
    const int bid = blockIdx.x, nbid = gridDim.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const long long tid = (long long) bid * blockDim.x + threadIdx.x, nthreads = (long long) nbid * blockDim.x;
    const long long npx = (long long) L.sensor.w * L.sensor.h;
    unsigned phase = 0;
    for (int j = bid; j < L.n; j += nbid)
        occ_begin(L, *step, j);
    bool ok = occ_grid_sync(bar, phase);
    if (ok) {
        for (long long k = tid; k < L.n * npx; k += nthreads)
            occ_pixel(L, (int) (k / npx), (int) (k % npx));
        ok = occ_grid_sync(bar, phase);
    }
    for (int l = 1; ok && l < L.sensor.levels; ++l) {
        for (long long k = tid; k < 2 * L.n * npx; k += nthreads) {
            const int jj = (int) (k / npx);
            occ_pool_pixel(L, l, jj >> 1, jj & 1, (int) (k % npx));
        }
        ok = occ_grid_sync(bar, phase);
    }
    if (ok) {
        for (int j = bid * nwarps + warp; j < L.n; j += nbid * nwarps)
            occ_root(L, j, lane);
        ok = occ_grid_sync(bar, phase);
    }
    for (int d = 1; ok && d <= L.max_block_depth; ++d) {
        occ_carve_stage(L, d, bid, nbid);
        ok = occ_grid_sync(bar, phase);
    }
    if (ok) {
        occ_nodes_stage(L, bid, nbid);
        ok = occ_grid_sync(bar, phase);
    }
    for (int it = 0; ok && it <= L.max_block_depth; ++it) {
        occ_free_nodes_stage(L, it, bid, nbid);
        ok = occ_grid_sync(bar, phase);
    }
    if (ok) {
        occ_blocks_stage(L, bid, nbid);
        ok = occ_grid_sync(bar, phase);
    }
    if (ok) {
        occ_propagate_blocks_stage(L, bid, nbid);
        ok = occ_grid_sync(bar, phase);
    }
    for (int d = L.max_block_depth - 1; ok && d > 0; --d) {
        occ_propagate_nodes_stage(L, d, bid, nbid);
        ok = occ_grid_sync(bar, phase);
    }
    if (bid == 0 && threadIdx.x < L.n) {
        const OccJob& J = L.job[threadIdx.x];
        if (ok)
            occ_propagate_node(J.m, 0, J.dyn->timestamp);
        else
            atomicOr(&J.m.counters[kOccError], kOccErrTimeout);
    }
}

// ------------------------------------------------------------------------ host side --

Lidar make_lidar(const se_gpu_lidar& c)
{
    Lidar L;
    L.w = c.width;
    L.h = c.height;
    L.near_plane = c.near_plane;
    L.far_plane = c.far_plane;
    const float deg_to_rad = (float) M_PI / 180.0f;
    // beam elevations linear from the highest (row 0); OusterLidar's ctor (ouster_lidar.cpp:59-85)
    const float step = (c.elevation_max_deg - c.elevation_min_deg) / (float) (c.height - 1);
    float prev = c.elevation_max_deg, el_lo = prev, el_hi = prev, min_el = 0.0f;
    for (int i = 1; i < c.height; ++i) {
        const float e = c.elevation_max_deg - (float) i * step;
        const float d = std::fabs(prev - e);
        min_el = i == 1 ? d : std::min(min_el, d);
        el_lo = std::min(el_lo, e);
        el_hi = std::max(el_hi, e);
        prev = e;
    }
    const float az = 360.0f / (float) c.width;
    const float min_ray_angle = std::min(min_el, az);
    L.tan_half_min_angle = std::tan(min_ray_angle / 2.0f * deg_to_rad);
    L.el_min = el_lo * deg_to_rad;
    L.el_max = el_hi * deg_to_rad;
    L.u_scale = (float) c.width / (2.0f * 3.14159274f);
    L.v_scale = (float) (c.height - 1) / (L.el_max - L.el_min);
    return L;
}

static int pooling_levels(int w, int h)
{
    const int image_max_dim = w < h ? w : h;
    return (int) (std::log2((double) ((image_max_dim - 1) / 2)) + 2) - 1 + 1;
}

static OccSensor occ_sensor(const se_gpu_pinhole* pinhole, const se_gpu_lidar* lidar)
{
    OccSensor S;
    std::memset(&S, 0, sizeof(S));
    if (lidar) {
        S.lidar = 1;
        S.L = make_lidar(*lidar);
        S.w = lidar->width;
        S.h = lidar->height;
        S.near_plane = lidar->near_plane;
        S.far_plane = lidar->far_plane;
    }
    else {
        S.lidar = 0;
        S.s = make_pinhole(*pinhole);
        S.w = pinhole->width;
        S.h = pinhole->height;
        S.near_plane = pinhole->near_plane;
        S.far_plane = pinhole->far_plane;
    }
    S.levels = pooling_levels(S.w, S.h);
    return S;
}

static se_gpu_status occ_scratch_reserve(se_gpu_occ_map* om, int w, int h)
{
    OccScratch& s = om->scratch;
    OccDevice& m = om->dev;
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
        SE_CUDA_TRY(cudaMalloc(&s.dyn, sizeof(OccDyn)));
        SE_CUDA_TRY(cudaMemset(s.dyn, 0, sizeof(OccDyn)));
        SE_CUDA_TRY(cudaMalloc(&s.launch_dev, sizeof(OccLaunch)));
        s.launch_host = new OccLaunch();
        std::memset(s.launch_host, 0, sizeof(OccLaunch));
    }
    if (s.w == w && s.h == h && s.sigma)
        return SE_GPU_OK;
    cudaFree(s.sigma);
    cudaFree(s.pool_depth);
    cudaFree(s.pool_sigma);
    s.sigma = nullptr;
    s.pool_depth = s.pool_sigma = nullptr;
    const int levels = pooling_levels(w, h);
    const size_t npx = (size_t) w * h;
    SE_CUDA_TRY(cudaMalloc(&s.sigma, npx * sizeof(float)));
    SE_CUDA_TRY(cudaMalloc(&s.pool_depth, (size_t) levels * npx * sizeof(float4)));
    SE_CUDA_TRY(cudaMalloc(&s.pool_sigma, (size_t) levels * npx * sizeof(float4)));
    s.w = w;
    s.h = h;
    s.levels = levels;
    return SE_GPU_OK;
}

void occ_scratch_free(se_gpu_occ_map* om)
{
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
    cudaFree(s.dyn);
    cudaFree(s.launch_dev);
    delete s.launch_host;
    s = OccScratch();
}

static OccJob occ_job(const se_gpu_occ_map* om)
{
    const OccScratch& s = om->scratch;
    const OccDevice& m = om->dev;
    OccJob J;
    std::memset(&J, 0, sizeof(J));
    J.m = m;
    J.sigma = s.sigma;
    J.pool_depth = s.pool_depth;
    J.pool_sigma = s.pool_sigma;
    J.max_value = s.max_value;
    J.frontier[0] = s.frontier[0];
    J.frontier[1] = s.frontier[1];
    J.block_list = s.block_list;
    J.block_var = s.block_var;
    J.block_inside = s.block_inside;
    J.node_list = s.node_list;
    J.freed = s.freed;
    J.work[0] = s.work[0];
    J.work[1] = s.work[1];
    J.sets = s.sets;
    J.dyn = s.dyn;
    J.tau_min = m.cfg.tau_min_factor * m.res;
    J.tau_max = m.cfg.tau_max_factor * m.res;
    J.sigma_min = m.cfg.sigma_min_factor * m.res;
    J.sigma_max = m.cfg.sigma_max_factor * m.res;
    return J;
}

// Launch geometry of the grid-stride stages in CTAs per SM; the batch's autotuner picks one
// per stage kind.
enum { kTileCarve = 0, kTileList, kTileBlocks, kTileKinds };
struct OccTiles {
    int ctas[kTileKinds] = {8, 4, 8}; // carve (128 threads), lists (256), blocks (256, a warp per block)
};

// Events around the tunable launches of one frame, for the autotuner.
struct OccStageTimer {
    std::vector<cudaEvent_t> ev;
    std::vector<int> kind;
    int used = 0;
    se_gpu_status mark(int k, cudaStream_t stream)
    {
        if (used == (int) ev.size()) {
            cudaEvent_t e;
            SE_CUDA_TRY(cudaEventCreate(&e));
            ev.push_back(e);
            kind.push_back(0);
        }
        kind[used] = k;
        SE_CUDA_TRY(cudaEventRecord(ev[used++], stream));
        return SE_GPU_OK;
    }
    ~OccStageTimer()
    {
        for (cudaEvent_t e : ev)
            cudaEventDestroy(e);
    }
};

#define OCC_MARK(k)                                                                          \
    do {                                                                                     \
        if (timer) {                                                                         \
            const se_gpu_status _s = timer->mark((k), stream);                               \
            if (_s != SE_GPU_OK)                                                             \
                return _s;                                                                   \
        }                                                                                    \
    } while (0)

// Every launch of one frame of every map in L (device copy at Ld); no host synchronisation, so
// the sequence can be captured into a graph. The begin launch is the first. With a timer, an
// event is recorded before each tunable launch (kind) and after it (kind -1).
static se_gpu_status occ_enqueue(const OccLaunch& L, const OccLaunch* Ld, const OccStep& step, const OccStep* step_dev,
                                 const OccTiles& t, cudaStream_t stream, OccStageTimer* timer = nullptr)
{
    const int sms = device_sm_count();
    const int npx = L.sensor.w * L.sensor.h;
    const int n = L.n;
    const int carve = sms * t.ctas[kTileCarve], list = sms * t.ctas[kTileList], blocks = sms * t.ctas[kTileBlocks];
    if (step_dev)
        occ_begin_dev_kernel<<<n, 64, 0, stream>>>(Ld, step_dev);
    else
        occ_begin_kernel<<<n, 64, 0, stream>>>(Ld, step);
    occ_pixels_kernel<<<dim3((npx + 255) / 256, n), 256, 0, stream>>>(Ld);
    for (int l = 1; l < L.sensor.levels; ++l)
        occ_pool_level_kernel<<<dim3((npx + 255) / 256, 2 * n), 256, 0, stream>>>(Ld, l);
    occ_root_kernel<<<n, 32, 0, stream>>>(Ld);
    for (int d = 1; d <= L.max_block_depth; ++d) {
        OCC_MARK(kTileCarve);
        occ_carve_kernel<<<carve, 128, 0, stream>>>(Ld, d);
    }
    OCC_MARK(kTileList);
    occ_nodes_kernel<<<list, 256, 0, stream>>>(Ld);
    for (int it = 0; it <= L.max_block_depth; ++it) {
        OCC_MARK(kTileList);
        occ_free_nodes_kernel<<<list, 256, 0, stream>>>(Ld, it);
    }
    OCC_MARK(kTileBlocks);
    occ_blocks_kernel<<<blocks, 256, 0, stream>>>(Ld);
    OCC_MARK(kTileBlocks);
    occ_propagate_blocks_kernel<<<blocks, 256, 0, stream>>>(Ld);
    for (int d = L.max_block_depth - 1; d > 0; --d) {
        OCC_MARK(kTileList);
        occ_propagate_nodes_kernel<<<list, 256, 0, stream>>>(Ld, d);
    }
    OCC_MARK(-1);
    occ_propagate_root_kernel<<<1, 32, 0, stream>>>(Ld);
    SE_CUDA_TRY(cudaGetLastError());
    return SE_GPU_OK;
}

// The same frame as one cooperative launch of occ_persistent_kernel, ctas_per_sm CTAs per SM
// (capped at what fits on an SM), its barrier counter cleared on the stream first.
static se_gpu_status occ_enqueue_persistent(const OccLaunch* Ld, const OccStep* step_dev, OccBarrier* bar,
                                            int ctas_per_sm, cudaStream_t stream, OccStageTimer* timer = nullptr)
{
    static int fits = 0;
    if (fits == 0) {
        SE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fits, occ_persistent_kernel, 256, 0));
        if (fits < 1) {
            set_last_error("the persistent occupancy kernel does not fit on an SM");
            return SE_GPU_ERR_CUDA;
        }
    }
    const int grid = device_sm_count() * (ctas_per_sm < fits ? ctas_per_sm : fits);
    SE_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(OccBarrier), stream));
    OCC_MARK(kTileCarve);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SE_CUDA_TRY(cudaLaunchKernelEx(&cfg, occ_persistent_kernel, Ld, step_dev, bar));
    OCC_MARK(-1);
    return SE_GPU_OK;
}

// The autotuner of a batch: its first kSkip calls run the default geometry untimed (the maps
// grow from empty, so the first frames' work is not representative), then each of the next
// kCand * kRounds calls runs one candidate geometry (candidate c: carve 2 << c, lists 1 << c,
// blocks 2 << c CTAs per SM) with events around the tunable launches; afterwards each stage kind
// keeps the candidate with the least time in its best round (the minimum discards calls slowed
// by anything else). Results do not depend on the geometry: every stage is a grid-stride loop
// over the same work.
struct OccTuner {
    static constexpr int kSkip = 4, kCand = 4, kRounds = 3, kTuneFrames = kSkip + kCand * kRounds;
    int frames = 0;
    double ms[kTileKinds][kCand];
    OccStageTimer timer;
    OccTuner()
    {
        for (int k = 0; k < kTileKinds; ++k)
            for (int c = 0; c < kCand; ++c)
                ms[k][c] = 1e30;
    }
    static OccTiles candidate(int c)
    {
        OccTiles t;
        t.ctas[kTileCarve] = 2 << c;
        t.ctas[kTileList] = 1 << c;
        t.ctas[kTileBlocks] = 2 << c;
        return t;
    }
};

static void occ_fill_step(OccStep& step, int j, const float* T_WS16, const float* image, int timestamp)
{
    std::memcpy(step.T_WS[j], T_WS16, 16 * sizeof(float));
    step.depth[j] = image;
    step.timestamp[j] = timestamp;
}

// One map, one frame: the launch description goes to the map's device copy when it changed
// (stream-ordered; the host copy stays valid), then the frame's launches.
static se_gpu_status occ_integrate_one(se_gpu_occ_map* om, const float* image_dev, const OccSensor& S,
                                       const float* T16, int timestamp, cudaStream_t stream)
{
    se_gpu_status st = occ_scratch_reserve(om, S.w, S.h);
    if (st != SE_GPU_OK)
        return st;
    OccLaunch& L = *om->scratch.launch_host;
    OccLaunch next;
    std::memset(&next, 0, sizeof(next));
    next.n = 1;
    next.max_block_depth = om->dev.block_depth;
    next.sensor = S;
    next.job[0] = occ_job(om);
    if (std::memcmp(&next, &L, sizeof(OccLaunch)) != 0) {
        L = next;
        SE_CUDA_TRY(cudaMemcpyAsync(om->scratch.launch_dev, &L, sizeof(OccLaunch), cudaMemcpyHostToDevice, stream));
    }
    OccStep step;
    std::memset(&step, 0, sizeof(step));
    occ_fill_step(step, 0, T16, image_dev, timestamp);
    ProfScope ps(kProfUpdate, stream);
    return occ_enqueue(L, om->scratch.launch_dev, step, nullptr, OccTiles(), stream);
}

se_gpu_status occ_integrate(se_gpu_occ_map* om, const float* depth_dev, const se_gpu_pinhole& sensor,
                            const float* T_WC16, int timestamp, cudaStream_t stream)
{
    return occ_integrate_one(om, depth_dev, occ_sensor(&sensor, nullptr), T_WC16, timestamp, stream);
}

se_gpu_status occ_integrate_range(se_gpu_occ_map* om, const float* range_dev, const se_gpu_lidar& sensor,
                                  const float* T_WS16, int timestamp, cudaStream_t stream)
{
    return occ_integrate_one(om, range_dev, occ_sensor(nullptr, &sensor), T_WS16, timestamp, stream);
}

} // namespace se_gpu

using namespace se_gpu;

// --------------------------------------------------------------------------- batches --

struct se_gpu_occ_batch {
    std::vector<se_gpu_map*> maps;
    OccLaunch* launch_host = nullptr;
    OccLaunch* launch_dev = nullptr;
    OccTiles tiles;
    int use_graph = 0;
    int persistent = 0;          // SE_GPU_OCC_BATCH_PERSISTENT: one cooperative launch per call
    OccBarrier* bar = nullptr;   // its grid barrier
    OccTuner* tuner = nullptr; // while autotuning
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // the per-call parameters: a device copy that the launches read, filled on the stream from a
    // ring of pinned host copies (a slot is reused once its previous copy has completed)
    static constexpr int kStepRing = 4;
    OccStep* step_dev = nullptr;
    OccStep* step_pinned = nullptr;
    cudaEvent_t step_ev[kStepRing] = {};
    int ring = 0;
    int device = 0;
};

// The tuner's candidate c for this batch: in persistent mode 1 or 2 CTAs per SM of the one launch.
static OccTiles batch_candidate(const se_gpu_occ_batch* b, int c)
{
    if (!b->persistent)
        return OccTuner::candidate(c);
    OccTiles t;
    t.ctas[kTileCarve] = 1 + (c & 1);
    return t;
}

static se_gpu_status batch_enqueue(se_gpu_occ_batch* b, const OccStep& step, const OccTiles& t, cudaStream_t s,
                                   OccStageTimer* timer = nullptr)
{
    if (b->persistent)
        return occ_enqueue_persistent(b->launch_dev, b->step_dev, b->bar, t.ctas[kTileCarve], s, timer);
    return occ_enqueue(*b->launch_host, b->launch_dev, step, b->step_dev, t, s, timer);
}

static se_gpu_status bad(se_gpu_status st, const char* msg)
{
    set_last_error("%s", msg);
    return st;
}

static se_gpu_status lidar_check(const se_gpu_lidar* s)
{
    if (!s || s->width < 8 || s->height < 3 || !(s->elevation_max_deg > s->elevation_min_deg)
        || !(s->near_plane > 0.0f) || !(s->far_plane > s->near_plane))
        return bad(SE_GPU_ERR_BAD_ARG, "lidar: width >= 8, height >= 3, el_max > el_min, 0 < near < far");
    return SE_GPU_OK;
}

extern "C" {

se_gpu_status se_gpu_integrate_range(se_gpu_map* map, const float* range_dev, const se_gpu_lidar* sensor,
                                     const float T_WS[16], int timestamp, void* stream)
{
    if (!map || !range_dev || !T_WS)
        return bad(SE_GPU_ERR_BAD_ARG, "se_gpu_integrate_range: null argument");
    if (!map->occ)
        return bad(SE_GPU_ERR_NOT_SUPPORTED, "se_gpu_integrate_range: occupancy maps only");
    se_gpu_status st = lidar_check(sensor);
    if (st != SE_GPU_OK)
        return st;
    cudaStream_t s = (cudaStream_t) stream;
    map->last_stream = s;
    return occ_integrate_range(map->occ, range_dev, *sensor, T_WS, timestamp, s);
}

se_gpu_status se_gpu_occ_batch_create(se_gpu_map* const* maps, int n, const se_gpu_pinhole* pinhole,
                                      const se_gpu_lidar* lidar, int use_graph, se_gpu_occ_batch** out)
{
    if (!maps || !out || n < 1 || n > kOccMaxBatch || (!pinhole) == (!lidar))
        return bad(SE_GPU_ERR_BAD_ARG, "se_gpu_occ_batch_create: 1..16 maps and exactly one sensor");
    if (lidar) {
        const se_gpu_status st = lidar_check(lidar);
        if (st != SE_GPU_OK)
            return st;
    }
    for (int j = 0; j < n; ++j) {
        if (!maps[j] || !maps[j]->occ)
            return bad(SE_GPU_ERR_BAD_ARG, "se_gpu_occ_batch_create: occupancy maps only");
        if (maps[j]->device != maps[0]->device)
            return bad(SE_GPU_ERR_BAD_ARG, "se_gpu_occ_batch_create: maps on different devices");
        for (int k = 0; k < j; ++k)
            if (maps[k] == maps[j])
                return bad(SE_GPU_ERR_BAD_ARG, "se_gpu_occ_batch_create: a map appears twice");
    }
    const OccSensor S = occ_sensor(pinhole, lidar);
    se_gpu_occ_batch* b = new se_gpu_occ_batch();
    b->maps.assign(maps, maps + n);
    b->use_graph = use_graph & SE_GPU_OCC_BATCH_GRAPH;
    b->persistent = (use_graph & SE_GPU_OCC_BATCH_PERSISTENT) != 0;
    if (b->persistent)
        b->tiles.ctas[kTileCarve] = 2;
    if (use_graph & SE_GPU_OCC_BATCH_AUTOTUNE)
        b->tuner = new OccTuner();
    b->device = maps[0]->device;
    b->launch_host = new OccLaunch();
    std::memset(b->launch_host, 0, sizeof(OccLaunch));
    OccLaunch& L = *b->launch_host;
    L.n = n;
    L.sensor = S;
    L.max_block_depth = 0;
    for (int j = 0; j < n; ++j) {
        se_gpu_status st = occ_scratch_reserve(maps[j]->occ, S.w, S.h);
        if (st != SE_GPU_OK) {
            se_gpu_occ_batch_destroy(b);
            return st;
        }
        L.job[j] = occ_job(maps[j]->occ);
        L.max_block_depth = std::max(L.max_block_depth, maps[j]->occ->dev.block_depth);
    }
    cudaError_t e = cudaMalloc(&b->launch_dev, sizeof(OccLaunch));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->launch_dev, &L, sizeof(OccLaunch), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMalloc(&b->step_dev, sizeof(OccStep));
    if (e == cudaSuccess && b->persistent)
        e = cudaMalloc(&b->bar, sizeof(OccBarrier));
    if (e == cudaSuccess)
        e = cudaHostAlloc(&b->step_pinned, se_gpu_occ_batch::kStepRing * sizeof(OccStep), cudaHostAllocDefault);
    for (int r = 0; r < se_gpu_occ_batch::kStepRing && e == cudaSuccess; ++r)
        e = cudaEventCreateWithFlags(&b->step_ev[r], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        se_gpu_occ_batch_destroy(b);
        return cuda_status(e, "se_gpu_occ_batch_create");
    }
    *out = b;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_occ_batch_integrate(se_gpu_occ_batch* b, const float* const* images_dev, const float* T_WS,
                                         const int* timestamps, void* stream)
{
    if (!b || !images_dev || !T_WS || !timestamps)
        return bad(SE_GPU_ERR_BAD_ARG, "se_gpu_occ_batch_integrate: null argument");
    const int n = (int) b->maps.size();
    for (int j = 0; j < n; ++j)
        if (!images_dev[j])
            return bad(SE_GPU_ERR_BAD_ARG, "se_gpu_occ_batch_integrate: null image");
    cudaStream_t s = (cudaStream_t) stream;
    OccStep step;
    std::memset(&step, 0, sizeof(step));
    for (int j = 0; j < n; ++j) {
        occ_fill_step(step, j, T_WS + 16 * j, images_dev[j], timestamps[j]);
        b->maps[j]->last_stream = s;
    }
    // this call's parameters into the device copy, on the stream ahead of the launches
    {
        const int r = b->ring;
        b->ring = (r + 1) % se_gpu_occ_batch::kStepRing;
        SE_CUDA_TRY(cudaEventSynchronize(b->step_ev[r]));
        b->step_pinned[r] = step;
        SE_CUDA_TRY(cudaMemcpyAsync(b->step_dev, &b->step_pinned[r], sizeof(OccStep), cudaMemcpyHostToDevice, s));
        SE_CUDA_TRY(cudaEventRecord(b->step_ev[r], s));
    }
    if (b->tuner && b->tuner->frames < OccTuner::kSkip) {
        ++b->tuner->frames;
        return batch_enqueue(b, step, b->tiles, s);
    }
    if (b->tuner) {
        OccTuner& tu = *b->tuner;
        const int c = (tu.frames - OccTuner::kSkip) % OccTuner::kCand;
        tu.timer.used = 0;
        se_gpu_status st = batch_enqueue(b, step, batch_candidate(b, c), s, &tu.timer);
        if (st != SE_GPU_OK)
            return st;
        SE_CUDA_TRY(cudaEventSynchronize(tu.timer.ev[tu.timer.used - 1]));
        double round_ms[kTileKinds] = {};
        for (int i = 0; i + 1 < tu.timer.used; ++i) {
            float ms = 0.0f;
            SE_CUDA_TRY(cudaEventElapsedTime(&ms, tu.timer.ev[i], tu.timer.ev[i + 1]));
            if (tu.timer.kind[i] >= 0)
                round_ms[tu.timer.kind[i]] += ms;
        }
        for (int k = 0; k < kTileKinds; ++k)
            tu.ms[k][c] = round_ms[k] < tu.ms[k][c] ? round_ms[k] : tu.ms[k][c];
        if (++tu.frames == OccTuner::kTuneFrames) {
            for (int k = 0; k < kTileKinds; ++k) {
                int best = 0;
                for (int cc = 1; cc < OccTuner::kCand; ++cc)
                    if (tu.ms[k][cc] < tu.ms[k][best])
                        best = cc;
                b->tiles.ctas[k] = batch_candidate(b, best).ctas[k];
            }
            delete b->tuner;
            b->tuner = nullptr;
        }
        return SE_GPU_OK;
    }
    if (!b->use_graph)
        return batch_enqueue(b, step, b->tiles, s);
    if (!b->exec) {
        // captured once: the launches read this and every later call's parameters from step_dev
        cudaStream_t cs;
        SE_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        se_gpu_status st = SE_GPU_OK;
        if (e == cudaSuccess)
            st = batch_enqueue(b, step, b->tiles, cs);
        cudaGraph_t graph = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess || e2 != cudaSuccess || st != SE_GPU_OK) {
            if (graph)
                cudaGraphDestroy(graph);
            return st != SE_GPU_OK ? st : cuda_status(e != cudaSuccess ? e : e2, "occupancy batch capture");
        }
        b->graph = graph;
        SE_CUDA_TRY(cudaGraphInstantiate(&b->exec, graph, 0));
        SE_CUDA_TRY(cudaGraphUpload(b->exec, s)); // the graph's resources set up before its first launch
    }
    SE_CUDA_TRY(cudaGraphLaunch(b->exec, s));
    return SE_GPU_OK;
}

se_gpu_status se_gpu_occ_batch_stats_async(const se_gpu_occ_batch* b, int32_t* stats_host, void* stream)
{
    if (!b || !stats_host)
        return bad(SE_GPU_ERR_BAD_ARG, "se_gpu_occ_batch_stats_async: null argument");
    static_assert(kOccNodeListN == kOccBlockListN + 1 && kOccFreedN == kOccBlockListN + 2
                      && kOccPruned == kOccBlockListN + 3,
                  "the four per-frame counters are contiguous");
    for (size_t j = 0; j < b->maps.size(); ++j)
        SE_CUDA_TRY(cudaMemcpyAsync(stats_host + 4 * j, b->maps[j]->occ->dev.counters + kOccBlockListN,
                                    4 * sizeof(int32_t), cudaMemcpyDeviceToHost, (cudaStream_t) stream));
    return SE_GPU_OK;
}

se_gpu_status se_gpu_occ_batch_tiles(const se_gpu_occ_batch* b, int tiles[3], int* tuning)
{
    if (!b || !tiles)
        return bad(SE_GPU_ERR_BAD_ARG, "se_gpu_occ_batch_tiles: null argument");
    for (int k = 0; k < kTileKinds; ++k)
        tiles[k] = b->tiles.ctas[k];
    if (tuning)
        *tuning = b->tuner ? OccTuner::kTuneFrames - b->tuner->frames : 0;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_occ_batch_destroy(se_gpu_occ_batch* b)
{
    if (!b)
        return SE_GPU_OK;
    delete b->tuner;
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    if (b->graph)
        cudaGraphDestroy(b->graph);
    cudaFree(b->launch_dev);
    cudaFree(b->step_dev);
    cudaFree(b->bar);
    cudaFreeHost(b->step_pinned);
    for (int r = 0; r < se_gpu_occ_batch::kStepRing; ++r)
        if (b->step_ev[r])
            cudaEventDestroy(b->step_ev[r]);
    delete b->launch_host;
    delete b;
    return SE_GPU_OK;
}

} // extern "C"
