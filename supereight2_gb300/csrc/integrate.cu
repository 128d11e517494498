// integrate.cu — se::MapIntegrator::integrateDepth for single-res TSDF maps.
//
// Four stream-ordered launches:
//   prep          per-frame parameters (from the caller's pose, or from a device pose for
//                 captured pipelines) and the per-frame counters; snapshot of the block count
//   carve         RaycastCarver: march every valid pixel's ray across the truncation band and
//                 insert the block of every sample (raycast_carver_impl.hpp:74-111); keys are
//                 deduplicated within a warp (__match_any_sync) before the dense-index check
//                 and the hash insert
//   frustum       fetcher::frustum: old blocks whose bounding sphere and the spheres of all
//                 their ancestor nodes below the root pass sphereInFrustum
//                 (raycast_carver_impl.hpp:17-32, iterator.hpp:197-235)
//   update        single-res TSDF update (singleres_tsdf_updater_impl.hpp:44-129): persistent
//                 warps walk the uneven list of listed old blocks then new blocks, one 8^3 block
//                 per warp and 16 voxels per lane, with no block-level barrier
#include <cmath>

#include "pipeline.cuh"
#include "profile.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

// Parameters for this frame, then the per-frame counters. With pose12 == nullptr the host's
// parameters are copied; otherwise they are derived from the device pose and the device frame
// counter, which is then advanced.
__global__ void integrate_prep_kernel(MapDevice m, float trunc_factor, Pinhole s, const float* pose12,
                                      IntegrateParams host_p, int* ts_counter, IntegrateParams* out)
{
    grid_dep_wait();
    if (pose12 == nullptr) {
        *out = host_p;
    }
    else {
        const int ts = *ts_counter;
        *out = make_integrate_params(m, trunc_factor, s, tf_from12(pose12), ts);
        *ts_counter = ts + 1;
    }
    int* counters = m.counters;
    const int nb = counters[kCntNumBlocks];
    counters[kCntNumOld] = nb < m.capacity ? nb : m.capacity;
    counters[kCntListed] = 0;
    counters[kCntValidPixels] = 0;
    reinterpret_cast<unsigned long long*>(counters)[kCntUpdated / 2] = 0ull;
}

// (int) (x / res) for 0 <= x (a coordinate inside the map), as point_to_voxel computes it, with
// the IEEE division only where it can matter: q = x (1/res) is within 2^-23 q of x / res (and so
// is the rounded quotient), so when q is more than q 2^-20 away from every integer both
// truncate to the same voxel; closer to an integer the division decides.
__device__ __forceinline__ int voxel_of(float x, float res, float inv_res)
{
    const float q = x * inv_res;
    const float f = q - truncf(q);
    const float tol = q * 0x1p-20f;
    if (f > tol && f < 1.0f - tol)
        return (int) q;
    return (int) (x / res);
}

// RaycastCarver::operator() hot loop. A CTA covers a 32 x 8 pixel tile, one warp per row
// segment, so the 8 samples of neighbouring rays fall in few distinct blocks. Lanes whose
// samples share a block are found by matching packed block coordinates; only the first of them
// forms the Morton key, and only when the block is not allocated yet.
__global__ void __launch_bounds__(256) carve_kernel(MapDevice m, Pinhole s, const float* __restrict__ depth,
                                                    const IntegrateParams* __restrict__ P)
{
    grid_dep_wait();
    const CarveParams cp = P->cp;
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
    const float inv_res = 1.0f / m.res;
    for (int i = 0; i < cp.num_steps; ++i) {
        unsigned long long packed = ~0ull; // no block
        int vx = 0, vy = 0, vz = 0;
        if (valid) {
            // point_to_voxel (se_gpu_internal.cuh) with the division shortcut of voxel_of
            const F3 p = apply(m.T_MW, pos);
            if (p.x >= 0.0f && p.x < m.dim && p.y >= 0.0f && p.y < m.dim && p.z >= 0.0f && p.z < m.dim) {
                // p < dim = size * res exactly, so v < size; the mask keeps the index in range
                // regardless (the reference's octree descent ignores bits >= size too)
                vx = voxel_of(p.x, m.res, inv_res) & (m.size - 1);
                vy = voxel_of(p.y, m.res, inv_res) & (m.size - 1);
                vz = voxel_of(p.z, m.res, inv_res) & (m.size - 1);
                packed = (unsigned long long) (vx >> 3) | ((unsigned long long) (vy >> 3) << 21)
                    | ((unsigned long long) (vz >> 3) << 42);
            }
            pos = add(pos, step);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, packed);
        if (packed != ~0ull && lane == __ffs(peers) - 1) {
            const int bx = vx >> 3, by = vy >> 3, bz = vz >> 3;
            // plain (coherent) load: entries are being published by this kernel; a stale -1
            // only costs a probe of the hash, which is the allocation arbiter
            const int idx = m.block_index[((size_t) bz << (2 * m.log2_bps)) | ((size_t) by << m.log2_bps) | (size_t) bx];
            if (idx < 0)
                insert_block(m, block_key(vx, vy, vz), bx, by, bz);
        }
    }
}

__global__ void __launch_bounds__(256) frustum_kernel(MapDevice m, Pinhole s, const IntegrateParams* __restrict__ P)
{
    grid_dep_wait();
    const Tf T_SW = P->fp.T_SW;
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
                const F3 c_S = apply(T_SW, apply(m.T_WM, p_M));
                if (!sphere_in_frustum(s, c_S, P->fp.radius[scale])) {
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

// FieldData<TSDF>::update (data_field_impl.hpp:39-54) preceded by the voxel's projection test
// (singleres_tsdf_updater_impl.hpp:57-78). Voxel memory is read only when the update applies;
// new blocks are written in full (the update doubles as their initialisation). Capped at 64
// registers (4 CTAs per SM): the extra warps hide more of the depth and voxel load latency than
// the cap costs.
template <int S, int KU>
__global__ void __launch_bounds__(256, 4) update_kernel(MapDevice m, Pinhole s, const float* __restrict__ depth,
                                                     const IntegrateParams* __restrict__ P)
{
    grid_dep_wait();
    const Tf T_CV = P->up.T_CV;
    const int timestamp = P->up.timestamp;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int n_warps = (gridDim.x * blockDim.x) >> 5;
    const int n_list = m.counters[kCntListed];
    const int n_old = m.counters[kCntNumOld];
    int n_new = m.counters[kCntNumBlocks];
    n_new = n_new < m.capacity ? n_new : m.capacity;
    const int total = n_list + (n_new - n_old);
    const float trunc = m.trunc;
    unsigned long long n_upd = 0;

    for (int item = warp; item < total; item += n_warps) {
        const bool is_new = item >= n_list;
        const int blk = is_new ? n_old + (item - n_list) : m.update_list[item];
        const int c0 = m.block_coord[3 * blk], c1 = m.block_coord[3 * blk + 1], c2 = m.block_coord[3 * blk + 2];
        if (lane == 0)
            m.block_ts[blk] = timestamp;
        // KU voxels per lane per round: their projections, then their depth loads in flight
        // together, then the voxel loads of those that update, then the updates (the per-voxel
        // arithmetic is that of one voxel at a time)
        constexpr int kU = KU;
        for (int k0 = 0; k0 < kBlockVoxels / 32; k0 += kU) {
            int pix[kU];
            float mz[kU], pn[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int vi = lane + 32 * (k0 + u);
                const int x = vi & 7, y = (vi >> 3) & 7, z = vi >> 6;
                const F3 p_C = apply(T_CV, f3((float) (c0 + x), (float) (c1 + y), (float) (c2 + z)));
                // A voxel with z <= 0 never updates: z < 0 fails the far test (far / nz < 0) and
                // z == 0 fails the projection; skipping it early changes no result.
                const float sq = p_C.z > 0.0f ? dot(p_C, p_C) : 0.0f;
                pn[u] = sqrtf(sq);
                mz[u] = p_C.z;
                pix[u] = -1;
                // farDist(p) = far / p.normalized().z; the test |p| > far / (z / |p|) is z > far in
                // exact arithmetic and the two rounded divisions move it by less than 2^-22
                // relative, so they only run within 2^-16 of the boundary
                bool beyond;
                if (p_C.z < s.far_plane * (1.0f - 0x1p-16f))
                    beyond = false;
                else if (p_C.z > s.far_plane * (1.0f + 0x1p-16f))
                    beyond = true;
                else
                    beyond = pn[u] > s.far_plane / (p_C.z / pn[u]);
                if (p_C.z > 0.0f && !beyond) {
                    float uu, vv;
                    if (project(s, p_C, uu, vv))
                        pix[u] = (int) (uu + 0.5f) + (int) (vv + 0.5f) * s.w;
                }
            }
            float dv[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u)
                dv[u] = pix[u] >= 0 ? __ldg(&depth[pix[u]]) : 0.0f;
            float upd[kU];
            bool du[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                du[u] = false;
                upd[u] = 0.0f;
                if (pix[u] >= 0 && !(dv[u] < s.near_plane)) {
                    const float sdf = (dv[u] - mz[u]) / mz[u] * pn[u];
                    if (!(sdf < -trunc)) {
                        const float r = sdf / trunc;
                        upd[u] = (1.0f < r) ? 1.0f : r;
                        du[u] = true;
                    }
                }
            }
            float tsdf[kU], w[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                tsdf[u] = 1.0f;
                w[u] = 0.0f;
                if (du[u] && !is_new)
                    load_voxel<S>(m, blk, lane + 32 * (k0 + u), tsdf[u], w[u]);
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                if (du[u] || is_new) {
                    if (du[u]) {
                        if (w[u] < m.max_weight)
                            w[u] = w[u] + 1.0f;
                        tsdf[u] = (tsdf[u] * (w[u] - 1.0f) + upd[u]) / w[u];
                        ++n_upd;
                    }
                    store_voxel<S>(m, blk, lane + 32 * (k0 + u), tsdf[u], w[u]);
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        n_upd += __shfl_down_sync(0xffffffffu, n_upd, o);
    if (lane == 0 && n_upd)
        atomicAdd(reinterpret_cast<unsigned long long*>(m.counters) + kCntUpdated / 2, n_upd);
}

se_gpu_status enqueue_integrate(se_gpu_map* map, const float* depth_dev, const se_gpu_pinhole& sensor,
                                const float* T_WC_host16, const float* pose12_dev, int timestamp,
                                cudaStream_t stream)
{
    MapDevice& m = map->dev;
    const Pinhole s = make_pinhole(sensor);
    IntegrateParams hp;
    if (T_WC_host16)
        hp = make_integrate_params(m, map->config.truncation_boundary_factor, s, tf_from16(T_WC_host16), timestamp);
    const int sms = device_sm_count();
    {
        ProfScope ps(kProfBeginFrame, stream);
        launch_chained(integrate_prep_kernel, 1, 1, stream, m, map->config.truncation_boundary_factor, s,
                       T_WC_host16 ? nullptr : pose12_dev, hp, map->timestamp_dev, map->iparams);
    }
    // the frustum test of the old blocks on the side stream, the carver on the caller's: the
    // carver only adds blocks past the old-block snapshot, and the frustum test only reads those
    // before it
    SE_CUDA_TRY(cudaEventRecord(map->fork_ev, stream));
    SE_CUDA_TRY(cudaStreamWaitEvent(map->side, map->fork_ev, 0));
    {
        ProfScope ps(kProfFrustum, map->side);
        frustum_kernel<<<sms * 4, 256, 0, map->side>>>(m, s, map->iparams);
        SE_CUDA_TRY(cudaGetLastError());
    }
    {
        ProfScope ps(kProfCarve, stream);
        dim3 cgrid((s.w + 31) / 32, (s.h + 7) / 8);
        launch_chained(carve_kernel, cgrid, 256, stream, m, s, depth_dev, map->iparams);
    }
    SE_CUDA_TRY(cudaEventRecord(map->join_ev, map->side));
    SE_CUDA_TRY(cudaStreamWaitEvent(stream, map->join_ev, 0));
    if (m.res_type == SE_GPU_RES_MULTI) {
        if (map->tune)
            SE_CUDA_TRY(cudaEventRecord(map->tune->ev[0], stream));
        enqueue_update_multires(m, s, depth_dev, map->iparams, stream);
        if (map->tune)
            SE_CUDA_TRY(cudaEventRecord(map->tune->ev[1], stream));
    }
    else {
        ProfScope ps(kProfUpdate, stream);
        const int grid = sms * map->tiles.update_ctas_per_sm;
        const bool r2 = map->tiles.update_round == 2;
        if (map->tune)
            SE_CUDA_TRY(cudaEventRecord(map->tune->ev[0], stream));
        if (m.storage == SE_GPU_STORAGE_F32 && r2)
            launch_chained(update_kernel<SE_GPU_STORAGE_F32, 2>, grid, 256, stream, m, s, depth_dev, map->iparams);
        else if (m.storage == SE_GPU_STORAGE_F32)
            launch_chained(update_kernel<SE_GPU_STORAGE_F32, 4>, grid, 256, stream, m, s, depth_dev, map->iparams);
        else if (r2)
            launch_chained(update_kernel<SE_GPU_STORAGE_F16, 2>, grid, 256, stream, m, s, depth_dev, map->iparams);
        else
            launch_chained(update_kernel<SE_GPU_STORAGE_F16, 4>, grid, 256, stream, m, s, depth_dev, map->iparams);
        if (map->tune)
            SE_CUDA_TRY(cudaEventRecord(map->tune->ev[1], stream));
    }
    SE_CUDA_TRY(cudaGetLastError());
    return SE_GPU_OK;
}

} // namespace se_gpu

using namespace se_gpu;

extern "C" se_gpu_status se_gpu_integrate_depth(se_gpu_map* map, const float* depth_dev,
                                                const se_gpu_pinhole* sensor, const float T_WC[16],
                                                int timestamp, void* stream_p)
{
    if (!map || !depth_dev || !sensor || !T_WC || sensor->width <= 0 || sensor->height <= 0) {
        set_last_error("se_gpu_integrate_depth: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    cudaStream_t stream = (cudaStream_t) stream_p;
    map->last_stream = stream;
    if (map->occ)
        return occ_integrate(map->occ, depth_dev, *sensor, T_WC, timestamp, stream);
    return enqueue_integrate(map, depth_dev, *sensor, T_WC, nullptr, timestamp, stream);
}
