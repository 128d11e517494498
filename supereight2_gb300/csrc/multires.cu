// multires.cu — the multi-resolution TSDF updater (se::Updater<Map<Data<TSDF>, Res::Multi>>,
// include/se/integrator/updater/impl/multires_tsdf_updater_impl.hpp:14-250).
//
// Allocation (carve, frustum) is shared with the single-res path. The per-block body of the
// reference's update loop runs as two launches over the frame's block list (listed old blocks,
// then new blocks), one warp per block:
//   mr_scale_down   integration scale with hysteresis (pinhole_camera.cpp:115-152), min scale,
//                   and, when the scale gets finer, delta down-propagation by one scale
//                   (propagator_impl.hpp:71-117, updater lines 70-146)
//   mr_update       strided voxel update at the block's scale (updater lines 148-230), then
//                   mean up-propagation to scale 3 (propagator_impl.hpp:17-67, data_impl.hpp:13-50)
// The reference's loop is one OpenMP region, so a block's down-propagation interpolates across
// neighbours that other threads may be updating concurrently. Splitting the body at that point
// fixes one of its schedules: every down-propagation reads the map as it was before the
// update. A down-propagation writes only scales finer than its block's previous scale and the
// interpolation reads each block at its previous scale or coarser, so the first launch has no
// races; the second touches only its own block.
#include "multires.cuh"
#include "pipeline.cuh"
#include "profile.cuh"

namespace se_gpu {

// PinholeCamera::computeIntegrationScaleImpl (pinhole_camera.cpp:115-152) with the default
// pixel_voxel_ratio_per_scale {1.5, 3, 6} (sensor.hpp:56) and scaled_pixel = 1 / fx.
__device__ int integration_scale(const Pinhole& s, float z, float res, int last_scale, int min_scale)
{
    for (int pass = 0; pass < 2; ++pass) {
        const float pixel_dim = z * s.inv_fx;
        const float pv_ratio = pixel_dim / res;
        int scale = 0;
        if (pv_ratio >= 1.5f) {
            scale = 1;
            if (pv_ratio >= 3.0f) {
                scale = 2;
                if (pv_ratio >= 6.0f)
                    scale = 3;
            }
        }
        // min(scale, max_block_scale = 3) holds by construction
        if (pass == 0 && min_scale != -1 && scale != last_scale) {
            // hysteresis: recompute once, 0.25 m closer when coarsening, farther when refining
            z = scale > last_scale ? z - 0.25f : z + 0.25f;
            continue;
        }
        return scale;
    }
    return 0; // unreachable
}

__device__ __forceinline__ int list_block(const MapDevice& m, int item, int n_list, int n_old)
{
    return item >= n_list ? n_old + (item - n_list) : m.update_list[item];
}

template <int S>
__global__ void __launch_bounds__(256) mr_scale_down_kernel(MapDevice m, Pinhole s,
                                                            const IntegrateParams* __restrict__ P)
{
    const Tf T_CW = P->fp.T_SW;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int n_warps = (gridDim.x * blockDim.x) >> 5;
    const int n_list = m.counters[kCntListed];
    const int n_old = m.counters[kCntNumOld];
    int n_new = m.counters[kCntNumBlocks];
    n_new = n_new < m.capacity ? n_new : m.capacity;
    const int total = n_list + (n_new - n_old);

    for (int item = warp; item < total; item += n_warps) {
        const int blk = list_block(m, item, n_list, n_old);
        const int c0 = m.block_coord[3 * blk], c1 = m.block_coord[3 * blk + 1], c2 = m.block_coord[3 * blk + 2];
        const int last = m.block_scale[2 * blk];
        int curr = 0;
        if (lane == 0) {
            // voxelToPoint(block_coord, block size): T_WM * ((coord + 8 * 0.5) * res)
            const float off = (float) kBlockSize * 0.5f;
            const F3 p_M = f3(((float) c0 + off) * m.res, ((float) c1 + off) * m.res, ((float) c2 + off) * m.res);
            const F3 centre_C = apply(T_CW, apply(m.T_WM, p_M));
            const int min_scale = m.block_scale[2 * blk + 1];
            const int sc = integration_scale(s, centre_C.z, m.res, last, min_scale);
            curr = sc > last - 1 ? sc : last - 1;
            m.block_scale[2 * blk + 1] = (signed char) (min_scale < 0 ? curr : (min_scale < curr ? min_scale : curr));
            m.block_nscale[blk] = (signed char) curr;
        }
        curr = __shfl_sync(0xffffffffu, curr, 0);
        if (curr >= last)
            continue;
        // propagateBlockDown from scale `last` to `last - 1`
        const int ps = last, cs = last - 1;
        const int cstride = 1 << cs;
        const int nc = kBlockSize >> cs; // children per axis
        const int n_children = nc * nc * nc;
        for (int k = lane; k < n_children; k += 32) {
            const int cx = (k % nc) * cstride, cy = ((k / nc) % nc) * cstride, cz = (k / (nc * nc)) * cstride;
            const int ci = mr_index(cx, cy, cz, cs);
            const int pi = mr_index(cx, cy, cz, ps);
            MrVoxel ch = mr_load<S>(m, blk, ci);
            const MrVoxel pa = mr_load<S>(m, blk, pi);
            if (ch.weight != 0.0f) {
                const float delta = pa.tsdf - pa.past_tsdf;
                const float t = ch.tsdf + delta;
                ch.tsdf = t < -1.0f ? -1.0f : t; // std::max(t, -1)
                ch.weight = fminf(ch.weight + pa.past_weight, m.max_weight);
                ch.past_weight = pa.past_weight;
                mr_store<S>(m, blk, ci, ch);
            }
            else {
                const float half = 0.5f * (float) cstride;
                const F3 cf = f3((float) (c0 + cx) + half, (float) (c1 + cy) + half, (float) (c2 + cz) + half);
                float iv;
                if (mr_interp<S>(m, cf, cs, iv, nullptr)) {
                    ch.tsdf = iv;
                    ch.weight = pa.weight;
                    ch.past_tsdf = iv;
                    ch.past_weight = 0.0f;
                    mr_store<S>(m, blk, ci, ch);
                }
            }
        }
        __syncwarp();
        // parent function: reset the parent delta once all its children have taken it
        const int np = kBlockSize >> ps;
        for (int k = lane; k < np * np * np; k += 32) {
            const int pi = mr_scale_offset(ps) + k;
            MrVoxel pa = mr_load<S>(m, blk, pi);
            pa.past_tsdf = pa.tsdf;
            pa.past_weight = 0.0f;
            mr_store<S>(m, blk, pi, pa);
        }
        __syncwarp();
    }
}

template <int S>
__global__ void __launch_bounds__(256) mr_update_kernel(MapDevice m, Pinhole s, const float* __restrict__ depth,
                                                        const IntegrateParams* __restrict__ P)
{
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
        const int blk = list_block(m, item, n_list, n_old);
        const int c0 = m.block_coord[3 * blk], c1 = m.block_coord[3 * blk + 1], c2 = m.block_coord[3 * blk + 2];
        const int curr = m.block_nscale[blk];
        if (is_new) {
            // BlockMultiRes ctor: data and past data default (tsdf 1, weight 0)
            const MrVoxel def{1.0f, 0.0f, 1.0f, 0.0f};
            for (int i = lane; i < kMrVoxels; i += 32)
                mr_store<S>(m, blk, i, def);
            __syncwarp();
        }
        if (lane == 0) {
            m.block_ts[blk] = timestamp;
            m.block_scale[2 * blk] = (signed char) curr;
        }
        const int stride = 1 << curr;
        const int n = kBlockSize >> curr;
        for (int k = lane; k < n * n * n; k += 32) {
            const int x = (k % n) * stride, y = ((k / n) % n) * stride, z = (k / (n * n)) * stride;
            const F3 p_C = apply(T_CV, f3((float) (c0 + x), (float) (c1 + y), (float) (c2 + z)));
            // z <= 0 never passes: z < 0 fails the far test (far / nz < 0), z == 0 the projection
            const float sq = p_C.z > 0.0f ? dot(p_C, p_C) : 0.0f;
            const float pn = sqrtf(sq);
            if (!(p_C.z > 0.0f))
                continue;
            // the far test |p| > far / (z / |p|): z > far up to 2^-22 relative (see update_kernel)
            if (p_C.z > s.far_plane * (1.0f + 0x1p-16f)
                || (!(p_C.z < s.far_plane * (1.0f - 0x1p-16f)) && pn > s.far_plane / (p_C.z / pn)))
                continue;
            float u, v;
            if (!project(s, p_C, u, v))
                continue;
            const int px = (int) (u + 0.5f), py = (int) (v + 0.5f);
            const float dv = __ldg(&depth[px + py * s.w]);
            if (dv < s.near_plane)
                continue;
            const float mz = p_C.z;
            const float sdf = (dv - mz) / mz * pn;
            const int idx = mr_index(x, y, z, curr);
            MrVoxel vx = mr_load<S>(m, blk, idx);
            if (!(sdf < -trunc)) {
                const float r = sdf / trunc;
                const float upd = (1.0f < r) ? 1.0f : r;
                if (vx.weight < m.max_weight)
                    vx.weight = vx.weight + 1.0f;
                vx.tsdf = (vx.tsdf * (vx.weight - 1.0f) + upd) / vx.weight;
                ++n_upd;
            }
            vx.past_weight = vx.past_weight + 1.0f;
            mr_store<S>(m, blk, idx, vx);
        }
        __syncwarp();
        // propagateBlockUp with up_prop_mean, one scale at a time
        for (int cs = curr; cs < kMaxBlockScale; ++cs) {
            const int ps = cs + 1;
            const int np = kBlockSize >> ps;
            const int cstride = 1 << cs, pstride = 1 << ps;
            for (int k = lane; k < np * np * np; k += 32) {
                const int px = (k % np) * pstride, py = ((k / np) % np) * pstride, pz = (k / (np * np)) * pstride;
                float tsdf_sum = 0.0f, weight_sum = 0.0f;
                int n_valid = 0;
                for (int c = 0; c < 8; ++c) {
                    float t, w;
                    mr_load_data<S>(m, blk,
                                    mr_index(px + (c & 1) * cstride, py + ((c >> 1) & 1) * cstride,
                                             pz + (c >> 2) * cstride, cs),
                                    t, w);
                    if (w != 0.0f) {
                        ++n_valid;
                        tsdf_sum += t;
                        weight_sum += w;
                    }
                }
                const int pi = mr_index(px, py, pz, ps);
                MrVoxel pa = mr_load<S>(m, blk, pi);
                if (n_valid > 0) {
                    pa.tsdf = tsdf_sum / (float) n_valid;
                    pa.weight = ceilf(weight_sum / (float) n_valid);
                    pa.past_tsdf = pa.tsdf;
                    pa.past_weight = 0.0f;
                }
                else {
                    pa.past_tsdf = 1.0f;
                    pa.past_weight = 0.0f;
                }
                mr_store<S>(m, blk, pi, pa);
            }
            __syncwarp();
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        n_upd += __shfl_down_sync(0xffffffffu, n_upd, o);
    if (lane == 0 && n_upd)
        atomicAdd(reinterpret_cast<unsigned long long*>(m.counters) + kCntUpdated / 2, n_upd);
}

void enqueue_update_multires(const MapDevice& m, const Pinhole& s, const float* depth_dev,
                             const IntegrateParams* params, cudaStream_t stream)
{
    const int sms = device_sm_count();
    ProfScope ps(kProfUpdate, stream);
    if (m.storage == SE_GPU_STORAGE_F32) {
        mr_scale_down_kernel<SE_GPU_STORAGE_F32><<<sms * 8, 256, 0, stream>>>(m, s, params);
        mr_update_kernel<SE_GPU_STORAGE_F32><<<sms * 8, 256, 0, stream>>>(m, s, depth_dev, params);
    }
    else {
        mr_scale_down_kernel<SE_GPU_STORAGE_F16><<<sms * 8, 256, 0, stream>>>(m, s, params);
        mr_update_kernel<SE_GPU_STORAGE_F16><<<sms * 8, 256, 0, stream>>>(m, s, depth_dev, params);
    }
}

} // namespace se_gpu
