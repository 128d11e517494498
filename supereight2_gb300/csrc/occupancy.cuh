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
    // map-wide
    int* aabb;             // min xyz, max xyz; aabb[6] = empty flag
    int* counters;         // see kOcc* below
};

// counters
enum {
    kOccNodes = 0,
    kOccBlocks,
    kOccError,
    kOccFrontierN0,    // frontier sizes (two buffers)
    kOccFrontierN1,
    kOccBlockListN,
    kOccNodeListN,
    kOccFreedN,
    kOccWorkN0,        // free-node work lists
    kOccWorkN1,
    kOccPruned,
    kOccSetN,          // first of kOccMaxDepth per-depth propagation-set sizes
    kOccCounters = kOccSetN + 24
};

constexpr int kOccErrNodePool = 1, kOccErrBlockPool = 2, kOccErrList = 4;

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
