// map.cu — device map (block hash + block pool + occupancy pyramid) and TSDF integration.
//
// integrateDepth on the GPU is four stream-ordered launches:
//   begin_frame   snapshot the block count (blocks allocated before this frame)
//   carve         RaycastCarver: march every valid pixel's ray across the truncation band and
//                 insert the block key of every sample (raycast_carver_impl.hpp:74-111); keys
//                 are deduplicated within a warp with __match_any_sync before the hash insert
//   frustum       fetcher::frustum: old blocks whose bounding sphere, and the spheres of all
//                 their ancestor nodes below the root, pass sphereInFrustum
//                 (raycast_carver_impl.hpp:17-32, iterator.hpp:197-235)
//   update        single-res TSDF update (singleres_tsdf_updater_impl.hpp:44-129) over the
//                 listed old blocks and the new blocks; one CTA per block, 2 voxels per thread
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "profile.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

static thread_local char g_last_error[512] = "";

void set_last_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

se_gpu_status cuda_status(cudaError_t e, const char* what)
{
    set_last_error("%s: %s", what, cudaGetErrorString(e));
    return SE_GPU_ERR_CUDA;
}

/* se::math::plane_normal (include/se/common/impl/math_util_impl.hpp:88-101) */
static F3 plane_normal(F3 p1, F3 p2, F3 p3) { return normalized(cross(sub(p2, p1), sub(p3, p2))); }

Pinhole make_pinhole(int w, int h, float fx, float fy, float cx, float cy, float near_p, float far_p)
{
    Pinhole s;
    s.w = w;
    s.h = h;
    s.fx = fx;
    s.fy = fy;
    s.cx = cx;
    s.cy = cy;
    s.inv_fx = 1.0f / fx;
    s.inv_fy = 1.0f / fy;
    s.near_plane = near_p;
    s.far_plane = far_p;
    s.left_hand = (fx < 0.0f) ^ (fy < 0.0f);
    // computeFrustumVertices / computeFrustumNormals (src/sensor/pinhole_camera.cpp:246-310)
    const F3 tl = back_project(s, 0.0f, 0.0f);
    const F3 tr = back_project(s, (float) w, 0.0f);
    const F3 br = back_project(s, (float) w, (float) h);
    const F3 bl = back_project(s, 0.0f, (float) h);
    const F3 tl_n = mul(near_p, tl), tl_f = mul(far_p, tl), tr_n = mul(near_p, tr), tr_f = mul(far_p, tr);
    const F3 br_n = mul(near_p, br), br_f = mul(far_p, br), bl_n = mul(near_p, bl), bl_f = mul(far_p, bl);
    const F3 ns[4] = {plane_normal(tl_f, tl_n, bl_n), plane_normal(tr_n, tr_f, br_f),
                      plane_normal(bl_f, bl_n, br_n), plane_normal(tr_f, tr_n, tl_n)};
    float sign = fx * fy;
    sign = sign / fabsf(sign);
    for (int i = 0; i < 4; ++i) {
        s.planes[i][0] = ns[i].x * sign;
        s.planes[i][1] = ns[i].y * sign;
        s.planes[i][2] = ns[i].z * sign;
        s.planes[i][3] = 0.0f;
    }
    s.planes[4][0] = 0.0f;
    s.planes[4][1] = 0.0f;
    s.planes[4][2] = 1.0f;
    s.planes[4][3] = -near_p;
    s.planes[5][0] = 0.0f;
    s.planes[5][1] = 0.0f;
    s.planes[5][2] = -1.0f;
    s.planes[5][3] = far_p;
    return s;
}

Pinhole make_pinhole(const se_gpu_pinhole& p)
{
    return make_pinhole(p.width, p.height, p.fx, p.fy, p.cx, p.cy, p.near_plane, p.far_plane);
}

Pinhole downsampled(const Pinhole& s, float dsf)
{
    return make_pinhole((int) ((float) s.w / dsf), (int) ((float) s.h / dsf), s.fx / dsf, s.fy / dsf,
                        (s.cx + 0.5f) / dsf - 0.5f, (s.cy + 0.5f) / dsf - 0.5f, s.near_plane, s.far_plane);
}

// ------------------------------------------------------------------------------ kernels --

struct CarveParams {
    Tf T_WS;
    F3 t_WS;
    float band;
    float half_band;
    float far_limit; // far_plane + band * 0.5
    int num_steps;
};

struct FrustumParams {
    Tf T_SW;
    float radius[20]; // bounding-sphere radius per octant scale
};

struct UpdateParams {
    Tf T_CV; // T_CW * T_WM * Scaling(res) * Translation(0.5)
    int timestamp;
};

__global__ void begin_frame_kernel(int* counters, int capacity)
{
    const int nb = counters[kCntNumBlocks];
    counters[kCntNumOld] = nb < capacity ? nb : capacity;
    counters[kCntListed] = 0;
    counters[kCntValidPixels] = 0;
    reinterpret_cast<unsigned long long*>(counters)[kCntUpdated / 2] = 0ull;
}

// Insert a block key that the occupancy bitmap did not show; the thread whose CAS claims an
// empty slot allocates the pool entry.
__device__ void insert_block(const MapDevice& m, uint64_t key, int bx, int by, int bz)
{
    uint32_t slot = hash_slot(key, m.hash_mask);
    for (int p = 0; p < kMaxProbe; ++p) {
        unsigned long long* kp = &m.hash[slot].x;
        const unsigned long long k = *((volatile unsigned long long*) kp);
        if (k == key)
            return;
        if (k == kEmptyKey) {
            const unsigned long long prev = atomicCAS(kp, kEmptyKey, (unsigned long long) key);
            if (prev == key)
                return;
            if (prev == kEmptyKey) {
                const int idx = atomicAdd(&m.counters[kCntNumBlocks], 1);
                if (idx >= m.capacity) {
                    m.hash[slot].y = (unsigned long long) (long long) -1;
                    atomicOr(&m.counters[kCntError], kErrPoolFull);
                    return;
                }
                m.hash[slot].y = (unsigned long long) idx;
                m.block_coord[3 * idx + 0] = bx << 3;
                m.block_coord[3 * idx + 1] = by << 3;
                m.block_coord[3 * idx + 2] = bz << 3;
                m.block_keys[idx] = key;
                m.block_ts[idx] = -1;
                for (int L = 0; L < m.occ_levels; ++L) {
                    const int lg = m.log2_bps - L;
                    const uint32_t cx = (uint32_t) bx >> L, cy = (uint32_t) by >> L, cz = (uint32_t) bz >> L;
                    const uint32_t bit = (cz << (2 * lg)) | (cy << lg) | cx;
                    atomicOr(&m.occ[L][bit >> 5], 1u << (bit & 31));
                }
                return;
            }
        }
        slot = (slot + 1) & m.hash_mask;
    }
    atomicOr(&m.counters[kCntError], kErrProbeLimit);
}

// RaycastCarver::operator() hot loop (raycast_carver_impl.hpp:74-111). A CTA covers a 32 x 8
// pixel tile, one warp per image row segment.
__global__ void __launch_bounds__(256) carve_kernel(MapDevice m, Pinhole s, const float* __restrict__ depth,
                                                    CarveParams cp)
{
    const int lane = threadIdx.x & 31;
    const int x = blockIdx.x * 32 + lane;
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    bool valid = x < s.w && y < s.h;
    float dv = 0.0f;
    if (valid) {
        dv = __ldg(&depth[x + y * s.w]);
        valid = !(dv < s.near_plane || dv > cp.far_limit);
    }
    const unsigned vmask = __ballot_sync(0xffffffffu, valid);
    if (lane == 0 && vmask)
        atomicAdd(&m.counters[kCntValidPixels], __popc(vmask));
    if (!vmask)
        return;

    F3 pos = f3(0.0f, 0.0f, 0.0f), step = f3(0.0f, 0.0f, 0.0f);
    if (valid) {
        const F3 ray_C = back_project(s, (float) x, (float) y);
        const F3 point_W = apply(cp.T_WS, mul(dv, ray_C));
        const F3 rev = normalized(sub(cp.t_WS, point_W));
        pos = sub(point_W, mul(cp.half_band, rev));
        step = divs(mul(rev, cp.band), (float) cp.num_steps);
    }
    for (int i = 0; i < cp.num_steps; ++i) {
        uint64_t key = kEmptyKey;
        int vx = 0, vy = 0, vz = 0;
        if (valid) {
            if (point_to_voxel(m, pos, vx, vy, vz))
                key = block_key(vx, vy, vz);
            pos = add(pos, step);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, (unsigned long long) key);
        if (key != kEmptyKey && lane == __ffs(peers) - 1) {
            const int bx = vx >> 3, by = vy >> 3, bz = vz >> 3;
            // plain (coherent) load: bits are being set by this kernel; a stale 0 only costs a
            // probe of the hash, which is authoritative
            const uint32_t bit = ((uint32_t) bz << (2 * m.log2_bps)) | ((uint32_t) by << m.log2_bps) | (uint32_t) bx;
            if (!((m.occ[0][bit >> 5] >> (bit & 31)) & 1u))
                insert_block(m, key, bx, by, bz);
        }
    }
}

// fetcher::frustum over the blocks allocated before this frame: a block is listed when its
// bounding sphere and those of all its ancestors below the root pass sphereInFrustum.
__global__ void __launch_bounds__(256) frustum_kernel(MapDevice m, Pinhole s, FrustumParams fp)
{
    const int n_old = m.counters[kCntNumOld];
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * blockDim.x; base < n_old; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        bool pass = false;
        if (i < n_old) {
            const int c0 = m.block_coord[3 * i], c1 = m.block_coord[3 * i + 1], c2 = m.block_coord[3 * i + 2];
            pass = true;
            for (int scale = kMaxBlockScale; scale < m.log2_size; ++scale) {
                const int sz = 1 << scale;
                const int n0 = c0 & ~(sz - 1), n1 = c1 & ~(sz - 1), n2 = c2 & ~(sz - 1);
                const float off = (float) sz * 0.5f;
                const F3 p_M = f3(((float) n0 + off) * m.res, ((float) n1 + off) * m.res, ((float) n2 + off) * m.res);
                const F3 c_S = apply(fp.T_SW, apply(m.T_WM, p_M));
                if (!sphere_in_frustum(s, c_S, fp.radius[scale])) {
                    pass = false;
                    break;
                }
            }
        }
        const unsigned pm = __ballot_sync(0xffffffffu, pass);
        int slot0 = 0;
        if (lane == 0 && pm)
            slot0 = atomicAdd(&m.counters[kCntListed], __popc(pm));
        slot0 = __shfl_sync(0xffffffffu, slot0, 0);
        if (pass)
            m.update_list[slot0 + __popc(pm & ((1u << lane) - 1u))] = i;
    }
}

// Single-res TSDF Updater (singleres_tsdf_updater_impl.hpp:44-129) with FieldData<TSDF>::update
// (data_field_impl.hpp:39-54). Persistent CTAs walk the uneven per-frame list: entries
// [0, listed) are old blocks from the frustum pass, then the new blocks [n_old, n_blocks).
// Voxel memory is touched only when the update applies, except for new blocks, which are
// written in full (the update doubles as their initialisation to tsdf = 1, weight = 0).
__global__ void __launch_bounds__(256) update_kernel(MapDevice m, Pinhole s, const float* __restrict__ depth,
                                                     UpdateParams up)
{
    __shared__ int sh_blk[3 + 2];
    const int n_list = m.counters[kCntListed];
    const int n_old = m.counters[kCntNumOld];
    int n_new = m.counters[kCntNumBlocks];
    n_new = n_new < m.capacity ? n_new : m.capacity;
    const int total = n_list + (n_new - n_old);
    const float trunc = m.trunc;
    unsigned long long n_upd = 0;

    for (int item = blockIdx.x; item < total; item += gridDim.x) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const int blk = item < n_list ? m.update_list[item] : n_old + (item - n_list);
            sh_blk[0] = blk;
            sh_blk[1] = m.block_coord[3 * blk];
            sh_blk[2] = m.block_coord[3 * blk + 1];
            sh_blk[3] = m.block_coord[3 * blk + 2];
            m.block_ts[blk] = up.timestamp;
        }
        __syncthreads();
        const int blk = sh_blk[0];
        const int c0 = sh_blk[1], c1 = sh_blk[2], c2 = sh_blk[3];
        const bool is_new = item >= n_list;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int vi = threadIdx.x + 256 * k;
            const int x = vi & 7, y = (vi >> 3) & 7, z = vi >> 6;
            bool do_update = false;
            float upd = 0.0f;
            const F3 p_C = apply(up.T_CV, f3((float) (c0 + x), (float) (c1 + y), (float) (c2 + z)));
            const float sq = dot(p_C, p_C);
            const float pn = sqrtf(sq);
            // farDist(p) = far / p.normalized().z
            const float nz = sq > 0.0f ? p_C.z / pn : p_C.z;
            if (!(pn > s.far_plane / nz)) {
                float u, v;
                if (project(s, p_C, u, v)) {
                    const int px = (int) (u + 0.5f), py = (int) (v + 0.5f);
                    const float dv = __ldg(&depth[px + py * s.w]);
                    if (!(dv < s.near_plane)) {
                        const float mz = p_C.z;
                        const float sdf = (dv - mz) / mz * pn;
                        if (!(sdf < -trunc)) {
                            const float r = sdf / trunc;
                            upd = (1.0f < r) ? 1.0f : r;
                            do_update = true;
                        }
                    }
                }
            }
            if (do_update || is_new) {
                float tsdf = 1.0f, w = 0.0f;
                if (!is_new)
                    load_voxel(m, blk, vi, tsdf, w);
                if (do_update) {
                    if (w < m.max_weight)
                        w = w + 1.0f;
                    tsdf = (tsdf * (w - 1.0f) + upd) / w;
                    ++n_upd;
                }
                store_voxel(m, blk, vi, tsdf, w);
            }
        }
    }
    // one 64-bit atomic per warp
    for (int o = 16; o > 0; o >>= 1)
        n_upd += __shfl_down_sync(0xffffffffu, n_upd, o);
    if ((threadIdx.x & 31) == 0 && n_upd)
        atomicAdd(reinterpret_cast<unsigned long long*>(m.counters) + kCntUpdated / 2, n_upd);
}

__global__ void upload_insert_kernel(MapDevice m, int n, const unsigned long long* __restrict__ keys)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint64_t key = keys[i];
    const uint64_t code = key >> 5;
    const int x = (int) morton_compact(code), y = (int) morton_compact(code >> 1), z = (int) morton_compact(code >> 2);
    if (x >= m.size || y >= m.size || z >= m.size)
        return;
    const uint64_t k = block_key(x, y, z);
    if (hash_find(m, k) < 0)
        insert_block(m, k, x >> 3, y >> 3, z >> 3);
}

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
    const int blk = hash_find(m, block_key(x, y, z));
    if (blk < 0)
        return;
    for (int v = threadIdx.x; v < kBlockVoxels; v += blockDim.x) {
        const float w = weight[(size_t) i * kBlockVoxels + v];
        store_voxel(m, blk, v, tsdf[(size_t) i * kBlockVoxels + v],
                    m.storage == SE_GPU_STORAGE_F32 ? w : rintf(fminf(fmaxf(w, 0.0f), 65535.0f)));
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

__global__ void download_voxels_kernel(MapDevice m, int n, float* tsdf, float* weight)
{
    const size_t total = (size_t) n * kBlockVoxels;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total; i += (size_t) gridDim.x * blockDim.x) {
        float t, w;
        load_voxel(m, (int) (i / kBlockVoxels), (int) (i % kBlockVoxels), t, w);
        if (tsdf)
            tsdf[i] = t;
        if (weight)
            weight[i] = w;
    }
}

static int num_sms()
{
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0)
            n = 152;
    }
    return n;
}

int device_sm_count() { return num_sms(); }

} // namespace se_gpu

using namespace se_gpu;

// ==================================================================== C interface ==

extern "C" {

const char* se_gpu_last_error(void) { return se_gpu::g_last_error; }

const char* se_gpu_status_string(se_gpu_status s)
{
    switch (s) {
    case SE_GPU_OK: return "ok";
    case SE_GPU_ERR_BAD_ARG: return "bad argument";
    case SE_GPU_ERR_CUDA: return "CUDA error";
    case SE_GPU_ERR_POOL_FULL: return "block pool full";
    case SE_GPU_ERR_HASH_PROBE_LIMIT: return "block hash probe limit reached";
    case SE_GPU_ERR_NOT_SUPPORTED: return "not supported";
    case SE_GPU_ERR_NO_DEVICE: return "no compute capability 10.3 device";
    }
    return "unknown status";
}

int se_gpu_abi_version(void) { return 1; }

se_gpu_status se_gpu_map_create(const se_gpu_map_config* cfg, se_gpu_map** out)
{
    if (!cfg || !out) {
        set_last_error("se_gpu_map_create: null argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    *out = nullptr;
    if (cfg->field != SE_GPU_FIELD_TSDF || cfg->res_type != SE_GPU_RES_SINGLE) {
        set_last_error("se_gpu_map_create: only single-resolution TSDF maps are supported");
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    if (!(cfg->res > 0.0f) || cfg->max_blocks <= 0 || cfg->max_blocks > (1ll << 30)
        || !(cfg->max_weight >= 1.0f) || cfg->max_weight > 65535.0f
        || cfg->max_weight != std::floor(cfg->max_weight)
        || (cfg->storage != SE_GPU_STORAGE_F32 && cfg->storage != SE_GPU_STORAGE_F16)) {
        set_last_error("se_gpu_map_create: invalid configuration");
        return SE_GPU_ERR_BAD_ARG;
    }
    int dev = 0;
    SE_CUDA_TRY(cudaGetDevice(&dev));
    int major = 0, minor = 0;
    SE_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    SE_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10 || minor != 3) {
        set_last_error("se_gpu: device %d has compute capability %d.%d; this build targets sm_103a", dev, major, minor);
        return SE_GPU_ERR_NO_DEVICE;
    }

    // Octree ctor: size = pow2ceil(max(ceil(max(dim)/res), 2 * block size))
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
    m.trunc = cfg->res * cfg->truncation_boundary_factor;
    m.max_weight = cfg->max_weight;
    m.storage = cfg->storage;
    m.capacity = (int) cfg->max_blocks;

    uint64_t hslots = 1024;
    while (hslots < 2ull * (uint64_t) m.capacity)
        hslots <<= 1;
    m.hash_mask = (uint32_t) (hslots - 1);
    const size_t vox_bytes = (size_t) m.capacity * kBlockVoxels * (m.storage == SE_GPU_STORAGE_F32 ? 8 : 4);

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
    m.occ_levels = m.log2_bps + 1;
    for (int L = 0; L < m.occ_levels; ++L) {
        const uint64_t side = (uint64_t) m.bps >> L;
        const size_t words = (size_t) ((side * side * side + 31) / 32);
        if ((e = cudaMalloc(&m.occ[L], words * 4)) != cudaSuccess) return fail(e, "cudaMalloc(occupancy)");
        if ((e = cudaMemset(m.occ[L], 0, words * 4)) != cudaSuccess) return fail(e, "cudaMemset(occupancy)");
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e, "cudaDeviceSynchronize");
    *out = map;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_destroy(se_gpu_map* map)
{
    if (!map)
        return SE_GPU_OK;
    MapDevice& m = map->dev;
    cudaFree(m.hash);
    cudaFree(m.block_coord);
    cudaFree(m.block_keys);
    cudaFree(m.block_ts);
    cudaFree(m.voxels);
    cudaFree(m.update_list);
    cudaFree(m.counters);
    for (int L = 0; L < 11; ++L)
        cudaFree(m.occ[L]);
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

se_gpu_status se_gpu_integrate_depth(se_gpu_map* map, const float* depth_dev, const se_gpu_pinhole* sensor,
                                     const float T_WC[16], int timestamp, void* stream_p)
{
    if (!map || !depth_dev || !sensor || !T_WC || sensor->width <= 0 || sensor->height <= 0) {
        set_last_error("se_gpu_integrate_depth: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    cudaStream_t stream = (cudaStream_t) stream_p;
    map->last_stream = stream;
    MapDevice& m = map->dev;
    const Pinhole s = make_pinhole(*sensor);
    const Tf T_WS = tf_from16(T_WC);

    CarveParams cp;
    cp.T_WS = T_WS;
    cp.t_WS = f3(T_WS.t[0], T_WS.t[1], T_WS.t[2]);
    cp.band = 2.0f * m.res * map->config.truncation_boundary_factor;
    cp.half_band = cp.band * 0.5f;
    cp.far_limit = s.far_plane + cp.band * 0.5f;
    cp.num_steps = (int) std::ceil(cp.band / (2.0f * m.res));

    FrustumParams fp;
    fp.T_SW = inverse_iso(T_WS);
    for (int sc = 0; sc < 20; ++sc)
        fp.radius[sc] = std::sqrt(3.0f) / 2.0f * m.res * (float) (1 << (sc < 19 ? sc : 19));

    UpdateParams up;
    Tf T_CV = compose(inverse_iso(T_WS), m.T_WM);
    for (int i = 0; i < 9; ++i)
        T_CV.R[i] = T_CV.R[i] * m.res;
    for (int i = 0; i < 3; ++i)
        T_CV.t[i] = ((T_CV.R[3 * i] * 0.5f + T_CV.R[3 * i + 1] * 0.5f) + T_CV.R[3 * i + 2] * 0.5f) + T_CV.t[i];
    up.T_CV = T_CV;
    up.timestamp = timestamp;

    {
        ProfScope ps(kProfBeginFrame, stream);
        begin_frame_kernel<<<1, 1, 0, stream>>>(m.counters, m.capacity);
    }
    {
        ProfScope ps(kProfCarve, stream);
        dim3 cgrid((s.w + 31) / 32, (s.h + 7) / 8);
        carve_kernel<<<cgrid, 256, 0, stream>>>(m, s, depth_dev, cp);
    }
    {
        ProfScope ps(kProfFrustum, stream);
        frustum_kernel<<<num_sms() * 4, 256, 0, stream>>>(m, s, fp);
    }
    {
        ProfScope ps(kProfUpdate, stream);
        update_kernel<<<num_sms() * 8, 256, 0, stream>>>(m, s, depth_dev, up);
    }
    SE_CUDA_TRY(cudaGetLastError());
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_integrate_stats(se_gpu_map* map, se_gpu_integrate_stats* st)
{
    if (!map || !st) {
        set_last_error("se_gpu_map_integrate_stats: null argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    int c[kNumCounters];
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    SE_CUDA_TRY(cudaMemcpy(c, map->dev.counters, sizeof(c), cudaMemcpyDeviceToHost));
    int nb = c[kCntNumBlocks] < map->dev.capacity ? c[kCntNumBlocks] : map->dev.capacity;
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
        download_voxels_kernel<<<num_sms() * 4, 256>>>(m, n, dt, dw);
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
    if (!map || n < 0 || (n > 0 && (!keys || !tsdf || !weight))) {
        set_last_error("se_gpu_map_upload_blocks: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (n == 0)
        return SE_GPU_OK;
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    unsigned long long* dk = nullptr;
    float *dt = nullptr, *dw = nullptr;
    const size_t vb = (size_t) n * kBlockVoxels * sizeof(float);
    cudaError_t e = cudaMalloc(&dk, (size_t) n * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dt, vb);
    if (e == cudaSuccess) e = cudaMalloc(&dw, vb);
    if (e == cudaSuccess) e = cudaMemcpy(dk, keys, (size_t) n * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dt, tsdf, vb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dw, weight, vb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        upload_insert_kernel<<<(unsigned) ((n + 255) / 256), 256>>>(map->dev, (int) n, dk);
        upload_voxels_kernel<<<(unsigned) n, 256>>>(map->dev, (int) n, dk, dt, dw);
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

se_gpu_status se_gpu_map_aabb(const se_gpu_map* map, int32_t mn[3], int32_t mx[3], int* empty)
{
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
        aabb_kernel<<<num_sms() * 2, 256>>>(map->dev, d);
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
