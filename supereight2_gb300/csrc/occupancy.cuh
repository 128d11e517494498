// occupancy.cuh — device state of a multi-resolution occupancy map (Map<Data<Occupancy>,
// Res::Multi, 8>): the reference's pointer octree as index-addressed node and block pools.
//
// Nodes hold 8 child slots (-1 empty, a node index >= 0, or a block index b as -2 - b) and
// min / max data (node.hpp:40-75). Blocks hold the BlockMultiRes<Occupancy> state
// (block.hpp:176-557): the mean pyramid from the finest allocated scale up, min / max pyramids
// that alias the mean data at the finest scale, the integration buffer (its own array when finer
// than the current scale, the mean data at its scale otherwise) and the four counters.
#pragma once

#include "se_gpu_internal.cuh"

namespace se_gpu {

struct OccD {
    float occ;
    float weight;
    int observed;
};

__host__ __device__ __forceinline__ OccD occ_default() { return OccD{0.0f, 0.0f, 0}; }
__device__ __forceinline__ bool occ_valid(const OccD& d) { return d.weight != 0.0f; }
__device__ __forceinline__ float occ_field(const OccD& d) { return d.occ * d.weight; }

struct OccFieldConfig {
    float k_sigma, sigma_min_factor, sigma_max_factor;
    float k_tau, tau_min_factor, tau_max_factor;
    float log_odd_min, log_odd_max;
    float max_weight;
    int fs_integr_scale;
};

struct OccBlockState {
    OccD init_data;
    int min_scale, current_scale, finest, buffer_scale;
    unsigned long long curr_integr, curr_obs, buf_integr, buf_obs;
    int parent;
    int live;
};

constexpr int kOccMaxScale = 3;

struct OccDevice {
    int size, log2_size, block_depth;
    float res, dim;
    Tf T_MW, T_WM;
    OccFieldConfig cfg;
    int node_capacity, block_capacity;
    // nodes
    int4* node_coord;      // x, y, z, size
    int* node_parent;
    int* node_child;       // 8 per node
    OccD* node_min;
    OccD* node_max;
    int* node_mark;        // frame stamp of the last propagation-set insertion
    int* node_ts;
    // blocks
    int* block_coord;      // 3 per block
    OccBlockState* block_state;
    OccD* block_mean;      // 585 per block
    OccD* block_min;       // 585 per block
    OccD* block_max;       // 585 per block
    OccD* block_buffer;    // 512 per block
    int* block_ts;         // Octant::timestamp of blocks (kept by the ray integrator)
    // map-wide
    int* aabb;             // min xyz, max xyz; aabb[6] = empty flag
    int* counters;         // see kOcc* below
};

// counters
constexpr int kOccMaxDepth = 24;
enum {
    kOccNodes = 0,
    kOccBlocks,
    kOccError,
    kOccBlockListN,
    kOccNodeListN,
    kOccFreedN,
    kOccPruned,
    kOccFrontierN,     // first of kOccMaxDepth + 1 per-depth carver frontier sizes
    kOccWorkN = kOccFrontierN + kOccMaxDepth + 1,  // per-level free-node work list sizes
    kOccSetN = kOccWorkN + kOccMaxDepth + 1,       // per-depth propagation-set sizes
    kOccCounters = kOccSetN + kOccMaxDepth
};
constexpr int kOccFirstFrameCounter = kOccBlockListN; // counters from here on restart every frame

constexpr int kOccErrNodePool = 1, kOccErrBlockPool = 2, kOccErrList = 4, kOccErrTimeout = 8;

// ------------------------------------------------------------------------ sensors --

// A spinning LiDAR (the reference's OusterLidar, whose projection model lives outside the
// reference): columns sweep 360 degrees of azimuth clockwise from +x, u = (pi - az) w / 2pi - 0.5
// wrapped into [-0.5, w - 0.5); rows are linear in elevation from el_max (row 0) down to el_min,
// v = (el_max - el) (h - 1) / (el_max - el_min), projection succeeds for v in [-0.5, h - 0.5).
struct Lidar {
    int w, h;
    float el_min, el_max; // radians
    float near_plane, far_plane;
    float u_scale, v_scale;
    float tan_half_min_angle; // tan(min_ray_angle / 2), min_ray_angle as in ouster_lidar.cpp:59-85
};

// atan on [0, 1] by the Abramowitz-Stegun 4.4.49 polynomial (|error| <= 1e-5 rad) and atan2 by
// octant reduction, in plain float operations so that the host and the device round alike.
__host__ __device__ __forceinline__ float atan01_as(float x)
{
    const float x2 = x * x;
    return x * (0.9998660f + x2 * (-0.3302995f + x2 * (0.1801410f + x2 * (-0.0851330f + x2 * 0.0208351f))));
}

__host__ __device__ __forceinline__ float atan2_as(float y, float x)
{
    const float ax = fabsf(x), ay = fabsf(y);
    if (ax == 0.0f && ay == 0.0f)
        return 0.0f;
    float a = ay <= ax ? atan01_as(ay / ax) : 1.57079637f - atan01_as(ax / ay);
    if (x < 0.0f)
        a = 3.14159274f - a;
    return y < 0.0f ? -a : a;
}

// Writes the pixel even when the projection fails (the carver uses it); false outside the rows.
__host__ __device__ __forceinline__ bool lidar_project(const Lidar& L, F3 p, float& u, float& v)
{
    const float rxy = sqrtf(p.x * p.x + p.y * p.y);
    if (rxy == 0.0f && p.z == 0.0f) {
        u = v = 0.0f;
        return false;
    }
    const float az = atan2_as(p.y, p.x);
    const float el = atan2_as(p.z, rxy);
    u = (3.14159274f - az) * L.u_scale - 0.5f;
    if (u < -0.5f)
        u += (float) L.w;
    if (u >= (float) L.w - 0.5f)
        u -= (float) L.w;
    v = (L.el_max - el) * L.v_scale;
    return v >= -0.5f && v < (float) L.h - 0.5f;
}

Lidar make_lidar(const se_gpu_lidar& c);

// The sensor of one integration launch: a pinhole camera or a LiDAR.
struct OccSensor {
    int lidar;
    Pinhole s;
    Lidar L;
    int w, h, levels;
    float near_plane, far_plane;
};

// ------------------------------------------------------------------ batched launches --

constexpr int kOccMaxBatch = 16;

// Per-frame state of one map in device memory, written by the first launch of each frame.
struct OccDyn {
    Tf T_WS, T_SW;
    const float* depth;
    int frame_id, timestamp;
};

// One map of a launch: the octree and its scratch (all device pointers).
struct OccJob {
    OccDevice m;
    float* sigma;
    float4* pool_depth; // levels * w * h of (min, max, crossing, known)
    float4* pool_sigma;
    float* max_value;   // [0] max pooled depth, [1] max_depth_value
    int* frontier[2];
    int* block_list;    // slot block index
    int* block_var;     // 0 Constant, 1 Gradient, 2 Undefined
    int* block_inside;
    int* node_list;
    int* freed;
    int2* work[2];      // (node, depth)
    int* sets;          // per depth, node_capacity entries each
    OccDyn* dyn;
    float tau_min, tau_max, sigma_min, sigma_max;
};

// Everything a launch needs except the per-frame inputs, passed by value (__grid_constant__).
struct OccLaunch {
    int n;
    int max_block_depth;
    OccSensor sensor;
    OccJob job[kOccMaxBatch];
};
static_assert(sizeof(OccLaunch) < 30000, "kernel parameter space");

// The per-frame inputs of every map of a launch.
struct OccStep {
    float T_WS[kOccMaxBatch][16];
    const float* depth[kOccMaxBatch];
    int timestamp[kOccMaxBatch];
};

// Scratch of one map, sized for the last sensor it integrated.
struct OccScratch {
    int w = 0, h = 0, levels = 0;
    float* sigma = nullptr;
    float4* pool_depth = nullptr;
    float4* pool_sigma = nullptr;
    float* max_value = nullptr;
    int* frontier[2] = {nullptr, nullptr};
    int* block_list = nullptr;
    int* block_var = nullptr;
    int* block_inside = nullptr;
    int* node_list = nullptr;
    int* freed = nullptr;
    int2* work[2] = {nullptr, nullptr};
    int* sets = nullptr;
    int set_depths = 0;
    OccDyn* dyn = nullptr;
    OccLaunch* launch_dev = nullptr; // the single-map launch description
    OccLaunch* launch_host = nullptr; // its last uploaded contents
};

__device__ __forceinline__ bool slot_is_block(int s) { return s <= -2; }
__device__ __forceinline__ int slot_block(int s) { return -2 - s; }

__host__ __device__ __forceinline__ int occ_scale_offset(int s)
{
    return s == 0 ? 0 : s == 1 ? 512 : s == 2 ? 576 : 584;
}

__device__ __forceinline__ OccD* blk_mean(const OccDevice& m, int b, int s)
{
    return m.block_mean + (size_t) b * 585 + occ_scale_offset(s);
}
__device__ __forceinline__ OccD* blk_min(const OccDevice& m, int b, int finest, int s)
{
    return s == finest ? blk_mean(m, b, s) : m.block_min + (size_t) b * 585 + occ_scale_offset(s);
}
__device__ __forceinline__ OccD* blk_max(const OccDevice& m, int b, int finest, int s)
{
    return s == finest ? blk_mean(m, b, s) : m.block_max + (size_t) b * 585 + occ_scale_offset(s);
}
__device__ __forceinline__ OccD* blk_buffer(const OccDevice& m, int b, const OccBlockState& st)
{
    return st.buffer_scale >= st.current_scale ? blk_mean(m, b, st.buffer_scale) : m.block_buffer + (size_t) b * 512;
}

__device__ __forceinline__ bool node_is_leaf(const OccDevice& m, int n)
{
    const int* c = m.node_child + 8 * (size_t) n;
    for (int i = 0; i < 8; ++i)
        if (c[i] != -1)
            return false;
    return true;
}

// NodeData<Occupancy>::data() (node.hpp:53-57)
__device__ __forceinline__ OccD node_data(const OccDevice& m, int n)
{
    const OccD mx = m.node_max[n];
    return (mx.observed && node_is_leaf(m, n)) ? mx : occ_default();
}

// fetcher::leaf: slot of the block holding the voxel, the deepest node on its path if that node
// has no children, or -1.
__device__ __forceinline__ int occ_leaf(const OccDevice& m, int x, int y, int z)
{
    int n = 0;
    for (int cs = m.size >> 1; cs >= 8; cs >>= 1) {
        const int idx = ((x & cs) > 0) + 2 * ((y & cs) > 0) + 4 * ((z & cs) > 0);
        const int ch = m.node_child[8 * (size_t) n + idx];
        if (ch == -1)
            return node_is_leaf(m, n) ? n : -1;
        if (slot_is_block(ch))
            return ch;
        n = ch;
    }
    return n;
}

__device__ __forceinline__ int occ_voxel_idx(int ox, int oy, int oz, int s)
{
    const int n = 8 >> s;
    return (ox >> s) + n * (oy >> s) + n * n * (oz >> s);
}

} // namespace se_gpu

namespace se_gpu {
struct RiScratch;
void ri_scratch_free(RiScratch* s);
} // namespace se_gpu

struct se_gpu_occ_map {
    se_gpu::OccDevice dev;
    se_gpu::OccScratch scratch;
    se_gpu::RiScratch* ri = nullptr; // ray-batch integration scratch, made on first use
};
