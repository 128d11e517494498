// map.cu — device map lifecycle: block hash + block pool + dense block index + occupancy
// pyramid, error latching, block download / upload and the allocated-block AABB.
#include <cmath>
#include <climits>
#include <cstring>
#include <vector>

#include "multires.cuh"
#include "pipeline.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

__global__ void upload_insert_kernel(MapDevice m, int n, const unsigned long long* __restrict__ keys)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint64_t code = keys[i] >> 5;
    const int x = (int) morton_compact(code), y = (int) morton_compact(code >> 1), z = (int) morton_compact(code >> 2);
    if (x >= m.size || y >= m.size || z >= m.size)
        return;
    if (block_at(m, x >> 3, y >> 3, z >> 3) < 0)
        insert_block(m, block_key(x, y, z), x >> 3, y >> 3, z >> 3);
}

template <int S>
__global__ void upload_voxels_kernel(MapDevice m, int n, const unsigned long long* __restrict__ keys,
                                     const float* __restrict__ tsdf, const float* __restrict__ weight)
{
    const int i = blockIdx.x;
    if (i >= n)
        return;
    const uint64_t code = keys[i] >> 5;
    const int x = (int) morton_compact(code), y = (int) morton_compact(code >> 1), z = (int) morton_compact(code >> 2);
    if (x >= m.size || y >= m.size || z >= m.size)
        return;
    const int blk = block_at(m, x >> 3, y >> 3, z >> 3);
    if (blk < 0)
        return;
    for (int v = threadIdx.x; v < kBlockVoxels; v += blockDim.x) {
        const float w = weight[(size_t) i * kBlockVoxels + v];
        store_voxel<S>(m, blk, v, tsdf[(size_t) i * kBlockVoxels + v],
                       S == SE_GPU_STORAGE_F32 ? w : rintf(fminf(fmaxf(w, 0.0f), 65535.0f)));
    }
}

template <int S>
__global__ void download_voxels_kernel(MapDevice m, int n, float* tsdf, float* weight)
{
    const size_t total = (size_t) n * kBlockVoxels;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total; i += (size_t) gridDim.x * blockDim.x) {
        float t, w;
        load_voxel<S>(m, (int) (i / kBlockVoxels), (int) (i % kBlockVoxels), t, w);
        if (tsdf)
            tsdf[i] = t;
        if (weight)
            weight[i] = w;
    }
}

// Multi-res blocks: the scale-0 level as tsdf / weight (se_gpu_map_download_blocks), or all
// 585 entries with past data and scales (se_gpu_map_download_multires).
template <int S>
__global__ void download_mr_kernel(MapDevice m, int n, int per_block, float* tsdf, float* weight, float* past_tsdf,
                                   float* past_weight)
{
    const size_t total = (size_t) n * per_block;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total; i += (size_t) gridDim.x * blockDim.x) {
        const MrVoxel v = mr_load<S>(m, (int) (i / per_block), (int) (i % per_block));
        if (tsdf)
            tsdf[i] = v.tsdf;
        if (weight)
            weight[i] = v.weight;
        if (past_tsdf)
            past_tsdf[i] = v.past_tsdf;
        if (past_weight)
            past_weight[i] = v.past_weight;
    }
}

__global__ void aabb_kernel(MapDevice m, int* out)
{
    int n = m.counters[kCntNumBlocks];
    n = n < m.capacity ? n : m.capacity;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (int a = 0; a < 3; ++a) {
            const int c = m.block_coord[3 * i + a];
            atomicMin(&out[a], c);
            atomicMax(&out[3 + a], c + kBlockSize - 1);
        }
    }
}

} // namespace se_gpu

using namespace se_gpu;

extern "C" {

se_gpu_status se_gpu_map_create(const se_gpu_map_config* cfg, se_gpu_map** out)
{
    if (!cfg || !out) {
        set_last_error("se_gpu_map_create: null argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    *out = nullptr;
    if (cfg->field == SE_GPU_FIELD_OCCUPANCY)
        return se_gpu_map_create_occupancy(cfg, nullptr, out);
    if (cfg->field != SE_GPU_FIELD_TSDF || (cfg->res_type != SE_GPU_RES_SINGLE && cfg->res_type != SE_GPU_RES_MULTI)) {
        set_last_error("se_gpu_map_create: only TSDF maps (single- or multi-resolution) are supported");
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    if (!(cfg->res > 0.0f) || cfg->max_blocks <= 0 || cfg->max_blocks > (1ll << 30) || !(cfg->max_weight >= 1.0f)
        || cfg->max_weight > 65535.0f || cfg->max_weight != std::floor(cfg->max_weight)
        || (cfg->storage != SE_GPU_STORAGE_F32 && cfg->storage != SE_GPU_STORAGE_F16)) {
        set_last_error("se_gpu_map_create: invalid configuration");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (cfg->storage == SE_GPU_STORAGE_F16 && cfg->max_weight > 255.0f) {
        set_last_error("se_gpu_map_create: FP16 storage keeps 8-bit weights (max_weight <= 255, got %g)",
                       (double) cfg->max_weight);
        return SE_GPU_ERR_BAD_ARG;
    }
    int dev = 0;
    SE_CUDA_TRY(cudaGetDevice(&dev));
    int major = 0, minor = 0;
    SE_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    SE_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10 || minor != 3) {
        set_last_error("se_gpu: device %d has compute capability %d.%d; this build targets sm_103a", dev, major,
                       minor);
        return SE_GPU_ERR_NO_DEVICE;
    }

    // Octree ctor (octree_impl.hpp:14-19): size = pow2ceil(max(ceil(max(dim)/res), 2 * block size))
    const float dmax = std::fmax(std::fmax(cfg->dim[0], cfg->dim[1]), cfg->dim[2]);
    const int requested = (int) std::ceil(dmax / cfg->res);
    int size = 1;
    while (size < (requested > 2 * kBlockSize ? requested : 2 * kBlockSize))
        size <<= 1;
    if (size > 8192) {
        set_last_error("se_gpu_map_create: octree side %d voxels exceeds the supported 8192", size);
        return SE_GPU_ERR_NOT_SUPPORTED;
    }

    se_gpu_map* map = new se_gpu_map();
    std::memset(&map->dev, 0, sizeof(map->dev));
    map->occ = nullptr;
    map->iparams = nullptr;
    map->rparams = nullptr;
    map->timestamp_dev = nullptr;
    map->config = *cfg;
    map->device = dev;
    map->last_stream = 0;
    MapDevice& m = map->dev;
    m.size = size;
    m.log2_size = 0;
    while ((1 << m.log2_size) < size)
        ++m.log2_size;
    m.bps = size / kBlockSize;
    m.log2_bps = m.log2_size - 3;
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
    m.inv_res = 1.0f / cfg->res;
    m.T_MW_translation = 1;
    for (int i = 0; i < 9; ++i)
        if (m.T_MW.R[i] != ((i % 4 == 0) ? 1.0f : 0.0f))
            m.T_MW_translation = 0;
    m.trunc = cfg->res * cfg->truncation_boundary_factor;
    m.max_weight = cfg->max_weight;
    m.storage = cfg->storage;
    m.capacity = (int) cfg->max_blocks;
    m.res_type = cfg->res_type;
    const bool mr = m.res_type == SE_GPU_RES_MULTI;

    uint64_t hslots = 1024;
    while (hslots < 2ull * (uint64_t) m.capacity)
        hslots <<= 1;
    m.hash_mask = (uint32_t) (hslots - 1);
    // single-res: 512 x {tsdf, weight}; multi-res: 585 x {data, past data} per block
    const size_t vox_bytes = mr ? (size_t) m.capacity * kMrVoxels * (m.storage == SE_GPU_STORAGE_F32 ? 16 : 8)
                                : (size_t) m.capacity * kBlockVoxels * (m.storage == SE_GPU_STORAGE_F32 ? 8 : 4);
    const size_t cells = (size_t) m.bps * m.bps * m.bps;

    auto fail = [&](cudaError_t e, const char* what) {
        se_gpu_status st = cuda_status(e, what);
        se_gpu_map_destroy(map);
        return st;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&m.hash, hslots * sizeof(ulonglong2))) != cudaSuccess) return fail(e, "cudaMalloc(hash)");
    if ((e = cudaMemset(m.hash, 0xff, hslots * sizeof(ulonglong2))) != cudaSuccess) return fail(e, "cudaMemset(hash)");
    if ((e = cudaMalloc(&m.block_coord, (size_t) m.capacity * 3 * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(coords)");
    if ((e = cudaMalloc(&m.block_keys, (size_t) m.capacity * sizeof(unsigned long long))) != cudaSuccess) return fail(e, "cudaMalloc(keys)");
    if ((e = cudaMalloc(&m.block_ts, (size_t) m.capacity * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(ts)");
    if ((e = cudaMalloc(&m.voxels, vox_bytes)) != cudaSuccess) return fail(e, "cudaMalloc(voxels)");
    if ((e = cudaMalloc(&m.update_list, (size_t) m.capacity * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(list)");
    if ((e = cudaMalloc(&m.counters, kNumCounters * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(counters)");
    if ((e = cudaMemset(m.counters, 0, kNumCounters * sizeof(int))) != cudaSuccess) return fail(e, "cudaMemset(counters)");
    if ((e = cudaMalloc(&map->iparams, sizeof(IntegrateParams))) != cudaSuccess) return fail(e, "cudaMalloc(params)");
    if ((e = cudaMalloc(&map->rparams, sizeof(RaycastParams))) != cudaSuccess) return fail(e, "cudaMalloc(params)");
    if ((e = cudaMalloc(&map->timestamp_dev, sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(timestamp)");
    if ((e = cudaMemset(map->timestamp_dev, 0, sizeof(int))) != cudaSuccess) return fail(e, "cudaMemset(timestamp)");
    if ((e = cudaMalloc(&m.aabb, 6 * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(aabb)");
    {
        const int init[6] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};
        if ((e = cudaMemcpy(m.aabb, init, sizeof(init), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "cudaMemcpy(aabb)");
    }
    if (mr) {
        if ((e = cudaMalloc(&m.block_scale, (size_t) m.capacity * 2)) != cudaSuccess) return fail(e, "cudaMalloc(scales)");
        if ((e = cudaMemset(m.block_scale, 0xff, (size_t) m.capacity * 2)) != cudaSuccess) return fail(e, "cudaMemset(scales)");
        if ((e = cudaMalloc(&m.block_nscale, (size_t) m.capacity)) != cudaSuccess) return fail(e, "cudaMalloc(scales)");
    }
    if ((e = cudaMalloc(&m.block_index, cells * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(block index)");
    if ((e = cudaMemset(m.block_index, 0xff, cells * sizeof(int))) != cudaSuccess) return fail(e, "cudaMemset(block index)");
    m.occ_levels = m.log2_bps + 1;
    for (int L = 0; L < m.occ_levels; ++L) {
        const uint64_t side = (uint64_t) m.bps >> L;
        const size_t words = (size_t) ((side * side * side + 31) / 32);
        if ((e = cudaMalloc(&m.occ[L], words * 4)) != cudaSuccess) return fail(e, "cudaMalloc(occupancy)");
        if ((e = cudaMemset(m.occ[L], 0, words * 4)) != cudaSuccess) return fail(e, "cudaMemset(occupancy)");
    }
    if ((e = cudaStreamCreateWithFlags(&map->side, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "cudaStreamCreate");
    if ((e = cudaEventCreateWithFlags(&map->fork_ev, cudaEventDisableTiming)) != cudaSuccess) return fail(e, "cudaEventCreate");
    if ((e = cudaEventCreateWithFlags(&map->join_ev, cudaEventDisableTiming)) != cudaSuccess) return fail(e, "cudaEventCreate");
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e, "cudaDeviceSynchronize");
    *out = map;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_create_occupancy(const se_gpu_map_config* cfg, const se_gpu_occupancy_config* occ,
                                          se_gpu_map** out)
{
    if (!cfg || !out) {
        set_last_error("se_gpu_map_create_occupancy: null argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    *out = nullptr;
    if (cfg->res_type != SE_GPU_RES_MULTI) {
        set_last_error("se_gpu_map_create_occupancy: occupancy maps are multi-resolution (res_type SE_GPU_RES_MULTI)");
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    if (!(cfg->res > 0.0f) || cfg->max_blocks <= 0 || cfg->max_blocks > (1ll << 26)) {
        set_last_error("se_gpu_map_create_occupancy: invalid configuration");
        return SE_GPU_ERR_BAD_ARG;
    }
    int dev = 0;
    SE_CUDA_TRY(cudaGetDevice(&dev));
    int major = 0, minor = 0;
    SE_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    SE_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10 || minor != 3) {
        set_last_error("se_gpu: device %d has compute capability %d.%d; this build targets sm_103a", dev, major,
                       minor);
        return SE_GPU_ERR_NO_DEVICE;
    }
    const float dmax = std::fmax(std::fmax(cfg->dim[0], cfg->dim[1]), cfg->dim[2]);
    const int requested = (int) std::ceil(dmax / cfg->res);
    int size = 1;
    while (size < (requested > 2 * kBlockSize ? requested : 2 * kBlockSize))
        size <<= 1;
    if (size > 8192) {
        set_last_error("se_gpu_map_create_occupancy: octree side %d voxels exceeds the supported 8192", size);
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    se_gpu_map* map = new se_gpu_map();
    std::memset(&map->dev, 0, sizeof(map->dev));
    map->config = *cfg;
    map->device = dev;
    map->last_stream = 0;
    map->iparams = nullptr;
    map->rparams = nullptr;
    map->timestamp_dev = nullptr;
    map->occ = nullptr;
    map->dev.size = size;
    map->dev.res = cfg->res;
    map->dev.inv_res = 1.0f / cfg->res;
    map->dev.dim = (float) size * cfg->res;
    map->dev.res_type = -1; // not a TSDF map
    const se_gpu_status st = occ_map_create(cfg, occ, size, &map->occ);
    if (st != SE_GPU_OK) {
        delete map;
        return st;
    }
    *out = map;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_destroy(se_gpu_map* map)
{
    if (!map)
        return SE_GPU_OK;
    if (map->occ) {
        occ_map_destroy(map->occ);
        delete map;
        return SE_GPU_OK;
    }
    MapDevice& m = map->dev;
    cudaFree(m.hash);
    cudaFree(m.block_coord);
    cudaFree(m.block_keys);
    cudaFree(m.block_ts);
    cudaFree(m.voxels);
    cudaFree(m.update_list);
    cudaFree(m.counters);
    cudaFree(m.block_index);
    cudaFree(m.aabb);
    cudaFree(m.block_scale);
    cudaFree(m.block_nscale);
    cudaFree(map->iparams);
    cudaFree(map->rparams);
    cudaFree(map->timestamp_dev);
    for (int L = 0; L < 11; ++L)
        cudaFree(m.occ[L]);
    if (map->side)
        cudaStreamDestroy(map->side);
    if (map->fork_ev)
        cudaEventDestroy(map->fork_ev);
    if (map->join_ev)
        cudaEventDestroy(map->join_ev);
    delete map;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_size(const se_gpu_map* map, int* size, float* dim_m)
{
    if (!map) {
        set_last_error("se_gpu_map_size: null map");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (size)
        *size = map->dev.size;
    if (dim_m)
        *dim_m = map->dev.dim;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_check(se_gpu_map* map)
{
    if (!map) {
        set_last_error("se_gpu_map_check: null map");
        return SE_GPU_ERR_BAD_ARG;
    }
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    if (map->occ)
        return occ_check(map->occ);
    int err = 0;
    SE_CUDA_TRY(cudaMemcpy(&err, map->dev.counters + kCntError, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        SE_CUDA_TRY(cudaMemset(map->dev.counters + kCntError, 0, sizeof(int)));
        if (err & kErrPoolFull) {
            set_last_error("block pool of %d blocks is full", map->dev.capacity);
            return SE_GPU_ERR_POOL_FULL;
        }
        set_last_error("block hash probe limit of %d reached", kMaxProbe);
        return SE_GPU_ERR_HASH_PROBE_LIMIT;
    }
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_integrate_stats(se_gpu_map* map, se_gpu_integrate_stats* st)
{
    if (!map || !st) {
        set_last_error("se_gpu_map_integrate_stats: null argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (map->occ) {
        set_last_error("se_gpu_map_integrate_stats: occupancy maps report se_gpu_map_occupancy_stats");
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    int c[kNumCounters];
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    SE_CUDA_TRY(cudaMemcpy(c, map->dev.counters, sizeof(c), cudaMemcpyDeviceToHost));
    const int nb = c[kCntNumBlocks] < map->dev.capacity ? c[kCntNumBlocks] : map->dev.capacity;
    st->n_new_blocks = nb - c[kCntNumOld];
    st->n_listed_blocks = c[kCntListed] + st->n_new_blocks;
    unsigned long long upd;
    std::memcpy(&upd, &c[kCntUpdated], sizeof(upd));
    st->n_updated_voxels = (int64_t) upd;
    st->n_valid_pixels = c[kCntValidPixels];
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_download_blocks(const se_gpu_map* map, int64_t capacity, uint64_t* keys, int32_t* coords,
                                         float* tsdf, float* weight, int32_t* timestamps, int64_t* count)
{
    if (!map || capacity < 0) {
        set_last_error("se_gpu_map_download_blocks: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (map->occ) {
        set_last_error("se_gpu_map_download_blocks: occupancy maps use se_gpu_map_download_occupancy");
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    const MapDevice& m = map->dev;
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    int nb = 0;
    SE_CUDA_TRY(cudaMemcpy(&nb, m.counters + kCntNumBlocks, sizeof(int), cudaMemcpyDeviceToHost));
    nb = nb < m.capacity ? nb : m.capacity;
    if (count)
        *count = nb;
    const int n = (int) (capacity < nb ? capacity : nb);
    if (n == 0)
        return SE_GPU_OK;
    if (keys)
        SE_CUDA_TRY(cudaMemcpy(keys, m.block_keys, (size_t) n * 8, cudaMemcpyDeviceToHost));
    if (coords)
        SE_CUDA_TRY(cudaMemcpy(coords, m.block_coord, (size_t) n * 12, cudaMemcpyDeviceToHost));
    if (timestamps)
        SE_CUDA_TRY(cudaMemcpy(timestamps, m.block_ts, (size_t) n * 4, cudaMemcpyDeviceToHost));
    if (tsdf || weight) {
        float *dt = nullptr, *dw = nullptr;
        const size_t bytes = (size_t) n * kBlockVoxels * sizeof(float);
        if (tsdf)
            SE_CUDA_TRY(cudaMalloc(&dt, bytes));
        if (weight)
            SE_CUDA_TRY(cudaMalloc(&dw, bytes));
        if (m.res_type == SE_GPU_RES_MULTI && m.storage == SE_GPU_STORAGE_F32)
            download_mr_kernel<SE_GPU_STORAGE_F32><<<device_sm_count() * 4, 256>>>(m, n, kBlockVoxels, dt, dw, nullptr,
                                                                                  nullptr);
        else if (m.res_type == SE_GPU_RES_MULTI)
            download_mr_kernel<SE_GPU_STORAGE_F16><<<device_sm_count() * 4, 256>>>(m, n, kBlockVoxels, dt, dw, nullptr,
                                                                                  nullptr);
        else if (m.storage == SE_GPU_STORAGE_F32)
            download_voxels_kernel<SE_GPU_STORAGE_F32><<<device_sm_count() * 4, 256>>>(m, n, dt, dw);
        else
            download_voxels_kernel<SE_GPU_STORAGE_F16><<<device_sm_count() * 4, 256>>>(m, n, dt, dw);
        cudaError_t e = cudaDeviceSynchronize();
        if (e == cudaSuccess && tsdf)
            e = cudaMemcpy(tsdf, dt, bytes, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && weight)
            e = cudaMemcpy(weight, dw, bytes, cudaMemcpyDeviceToHost);
        cudaFree(dt);
        cudaFree(dw);
        if (e != cudaSuccess)
            return cuda_status(e, "download voxels");
    }
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_upload_blocks(se_gpu_map* map, int64_t n, const uint64_t* keys, const float* tsdf,
                                       const float* weight)
{
    if (!map || n < 0 || n > (1ll << 30) || (n > 0 && (!keys || !tsdf || !weight))) {
        set_last_error("se_gpu_map_upload_blocks: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (map->occ || map->dev.res_type != SE_GPU_RES_SINGLE) {
        set_last_error("se_gpu_map_upload_blocks: single-resolution maps only");
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    if (n == 0)
        return SE_GPU_OK;
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    unsigned long long* dk = nullptr;
    float *dt = nullptr, *dw = nullptr;
    const size_t vb = (size_t) n * kBlockVoxels * sizeof(float);
    cudaError_t e = cudaMalloc(&dk, (size_t) n * 8);
    if (e == cudaSuccess)
        e = cudaMalloc(&dt, vb);
    if (e == cudaSuccess)
        e = cudaMalloc(&dw, vb);
    if (e == cudaSuccess)
        e = cudaMemcpy(dk, keys, (size_t) n * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(dt, tsdf, vb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(dw, weight, vb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        upload_insert_kernel<<<(unsigned) ((n + 255) / 256), 256>>>(map->dev, (int) n, dk);
        if (map->dev.storage == SE_GPU_STORAGE_F32)
            upload_voxels_kernel<SE_GPU_STORAGE_F32><<<(unsigned) n, 256>>>(map->dev, (int) n, dk, dt, dw);
        else
            upload_voxels_kernel<SE_GPU_STORAGE_F16><<<(unsigned) n, 256>>>(map->dev, (int) n, dk, dt, dw);
        e = cudaDeviceSynchronize();
    }
    cudaFree(dk);
    cudaFree(dt);
    cudaFree(dw);
    if (e != cudaSuccess)
        return cuda_status(e, "se_gpu_map_upload_blocks");
    map->last_stream = 0;
    return se_gpu_map_check(map);
}

se_gpu_status se_gpu_map_download_multires(const se_gpu_map* map, int64_t capacity, uint64_t* keys, int32_t* coords,
                                           float* tsdf, float* weight, float* past_tsdf, float* past_weight,
                                           int32_t* scales, int64_t* count)
{
    if (!map || capacity < 0) {
        set_last_error("se_gpu_map_download_multires: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    const MapDevice& m = map->dev;
    if (m.res_type != SE_GPU_RES_MULTI) {
        set_last_error("se_gpu_map_download_multires: not a multi-resolution map");
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    int nb = 0;
    SE_CUDA_TRY(cudaMemcpy(&nb, m.counters + kCntNumBlocks, sizeof(int), cudaMemcpyDeviceToHost));
    nb = nb < m.capacity ? nb : m.capacity;
    if (count)
        *count = nb;
    const int n = (int) (capacity < nb ? capacity : nb);
    if (n == 0)
        return SE_GPU_OK;
    if (keys)
        SE_CUDA_TRY(cudaMemcpy(keys, m.block_keys, (size_t) n * 8, cudaMemcpyDeviceToHost));
    if (coords)
        SE_CUDA_TRY(cudaMemcpy(coords, m.block_coord, (size_t) n * 12, cudaMemcpyDeviceToHost));
    if (scales) {
        std::vector<signed char> sc((size_t) n * 2);
        SE_CUDA_TRY(cudaMemcpy(sc.data(), m.block_scale, sc.size(), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < sc.size(); ++i)
            scales[i] = sc[i];
    }
    float* host[4] = {tsdf, weight, past_tsdf, past_weight};
    float* dev[4] = {nullptr, nullptr, nullptr, nullptr};
    const size_t bytes = (size_t) n * kMrVoxels * sizeof(float);
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 4 && e == cudaSuccess; ++k)
        if (host[k])
            e = cudaMalloc(&dev[k], bytes);
    if (e == cudaSuccess) {
        if (m.storage == SE_GPU_STORAGE_F32)
            download_mr_kernel<SE_GPU_STORAGE_F32><<<device_sm_count() * 4, 256>>>(m, n, kMrVoxels, dev[0], dev[1],
                                                                                  dev[2], dev[3]);
        else
            download_mr_kernel<SE_GPU_STORAGE_F16><<<device_sm_count() * 4, 256>>>(m, n, kMrVoxels, dev[0], dev[1],
                                                                                  dev[2], dev[3]);
        e = cudaDeviceSynchronize();
    }
    for (int k = 0; k < 4 && e == cudaSuccess; ++k)
        if (host[k])
            e = cudaMemcpy(host[k], dev[k], bytes, cudaMemcpyDeviceToHost);
    for (int k = 0; k < 4; ++k)
        cudaFree(dev[k]);
    if (e != cudaSuccess)
        return cuda_status(e, "se_gpu_map_download_multires");
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_aabb(const se_gpu_map* map, int32_t mn[3], int32_t mx[3], int* empty)
{
    if (map && map->occ && mn && mx && empty) {
        SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
        return occ_aabb(map->occ, mn, mx, empty);
    }
    if (!map || !mn || !mx || !empty) {
        set_last_error("se_gpu_map_aabb: null argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    int h[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, -1, -1, -1};
    int* d = nullptr;
    SE_CUDA_TRY(cudaMalloc(&d, sizeof(h)));
    cudaError_t e = cudaMemcpy(d, h, sizeof(h), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        aabb_kernel<<<device_sm_count() * 2, 256>>>(map->dev, d);
        e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    }
    cudaFree(d);
    if (e != cudaSuccess)
        return cuda_status(e, "se_gpu_map_aabb");
    *empty = h[3] < 0;
    for (int a = 0; a < 3; ++a) {
        mn[a] = h[a];
        mx[a] = h[3 + a];
    }
    return SE_GPU_OK;
}

} // extern "C"
