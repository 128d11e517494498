// raycast.cu — se::raycaster::raycast_volume for single-res TSDF maps, and the batched
// Map::getFieldInterp / Map::getFieldGrad queries.
//
// One thread per pixel (an 8 x 4 pixel tile per warp for coherent block lookups):
//   1. first allocated block on the ray (VoxelBlockRayIterator,
//      voxel_block_ray_iterator_impl.hpp:19-249): a level DDA over the occupancy pyramid from
//      cells of 4^3 blocks down to blocks, with the reference traversal's plane parameters and
//      child choices (first_block in raycast_core.cuh);
//   2. the TSDF march of raycast<TSDF> (raycaster_impl.hpp:456-533): voxel fetches through the
//      dense block index with a one-block cache, trilinear interpolation near the surface
//      (visitor_impl.hpp:976-1024) and the linear zero-crossing estimate;
//   3. the surface normal from the 32-sample central-difference gradient
//      (visitor_impl.hpp:1094-1251, map_impl.hpp:236-262), its 32 loads issued together.
// The gradient's block table lives in shared memory; the register cap of 9 CTAs per SM (a few
// spilled words) is faster than the 5 CTAs that 92 registers allow.
// Sample loops are deliberately not unrolled: one copy of the fetch path keeps the kernel
// inside the instruction cache.
#include <cmath>

#include "pipeline.cuh"
#include "profile.cuh"
#include "raycast_core.cuh"

namespace se_gpu {

__global__ void raycast_prep_kernel(const float* pose12, RaycastParams host_p, RaycastParams* out)
{
    grid_dep_wait();
    RaycastParams p = host_p;
    if (pose12 != nullptr)
        p.T_WS = tf_from12(pose12);
    *out = p;
}

// TILE 0: each warp takes 8 x 4 pixels (a CTA 16 x 8); TILE 1: 16 x 2 (a CTA 32 x 4).
template <int S, bool MR, int TILE>
__global__ void __launch_bounds__(128, 9) raycast_kernel(MapDevice m, Pinhole s, const RaycastParams* __restrict__ P,
                                                      float* __restrict__ pts, float* __restrict__ nrm,
                                                      int8_t* __restrict__ scale)
{
    grid_dep_wait();
    // per-thread scratch in shared memory (column threadIdx.x): the gradient's block table
    __shared__ int sh_bt[8 * 128];
    const RaycastParams rp = *P;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kWx = TILE == 0 ? 8 : 16, kWy = 32 / kWx; // warp tile
    const int x = blockIdx.x * (2 * kWx) + (warp & 1) * kWx + (lane % kWx);
    const int y = blockIdx.y * (2 * kWy) + (warp >> 1) * kWy + (lane / kWx);
    if (x >= s.w || y >= s.h)
        return;
    const size_t idx = (size_t) x + (size_t) y * s.w;
    const F3 ray_S = back_project(s, (float) x, (float) y);
    const F3 nS = normalized(ray_S);
    const F3 dir_W = rot(rp.T_WS, nS);
    const F3 origin = f3(rp.T_WS.t[0], rp.T_WS.t[1], rp.T_WS.t[2]);
    const float t_near = s.near_plane / nS.z;
    const float t_far = s.far_plane / nS.z;
    BlockCache c{-1, -1, -1, -1};
    F3 hit;
    F3 n = f3(0.0f, 0.0f, 0.0f);
    F3 p = f3(0.0f, 0.0f, 0.0f);
    int hit_scale = 0;
    if (raycast_tsdf<S, MR>(m, rp, c, origin, dir_W, t_near, t_far, hit, hit_scale)) {
        p = hit;
        F3 g;
        bool ok;
        if constexpr (MR)
            ok = mr_field_grad<S>(m, hit, g);
        else
            ok = field_grad_batched<S>(m, c, hit, g, sh_bt + threadIdx.x, 128);
        if (ok)
            n = normalized(g);
    }
    pts[3 * idx + 0] = p.x;
    pts[3 * idx + 1] = p.y;
    pts[3 * idx + 2] = p.z;
    nrm[3 * idx + 0] = n.x;
    nrm[3 * idx + 1] = n.y;
    nrm[3 * idx + 2] = n.z;
    if (scale)
        scale[idx] = (int8_t) hit_scale;
}

template <int S, bool MR>
__global__ void field_query_kernel(MapDevice m, int n, const float* __restrict__ pts, float* __restrict__ out,
                                   int* __restrict__ valid, int grad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const F3 p = f3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    BlockCache c{-1, -1, -1, -1};
    bool ok;
    if (grad) {
        F3 g = f3(0.0f, 0.0f, 0.0f);
        if constexpr (MR)
            ok = mr_field_grad<S>(m, p, g);
        else
            ok = field_grad<S>(m, c, p, g);
        out[3 * i] = ok ? g.x : 0.0f;
        out[3 * i + 1] = ok ? g.y : 0.0f;
        out[3 * i + 2] = ok ? g.z : 0.0f;
    }
    else {
        float v = 0.0f;
        if constexpr (MR)
            ok = mr_field_interp<S>(m, p, v, nullptr);
        else
            ok = field_interp<S>(m, c, p, v);
        out[i] = ok ? v : 0.0f;
    }
    if (valid)
        valid[i] = ok ? 1 : 0;
}

} // namespace se_gpu

using namespace se_gpu;

namespace se_gpu {

se_gpu_status enqueue_raycast(const se_gpu_map* map, const se_gpu_pinhole& sensor, const float* T_WS_host16,
                              const float* pose12_dev, float* pts_dev, float* nrm_dev, int8_t* scale_dev,
                              cudaStream_t stream)
{
    const MapDevice& m = map->dev;
    const Pinhole s = make_pinhole(sensor);
    RaycastParams rp;
    for (int i = 0; i < 9; ++i)
        rp.T_WS.R[i] = (i % 4 == 0) ? 1.0f : 0.0f;
    rp.T_WS.t[0] = rp.T_WS.t[1] = rp.T_WS.t[2] = 0.0f;
    if (T_WS_host16)
        rp.T_WS = tf_from16(T_WS_host16);
    rp.scaling = (float) m.size * m.res;
    rp.eps = std::exp2((float) (-std::log2((double) m.size)));
    rp.min_scale = 23 - m.log2_bps;
    launch_chained(raycast_prep_kernel, 1, 1, stream, T_WS_host16 ? nullptr : pose12_dev, rp, map->rparams);
    const int tile = map->tiles.raycast_tile;
    const dim3 grid = tile == 0 ? dim3((s.w + 15) / 16, (s.h + 7) / 8) : dim3((s.w + 31) / 32, (s.h + 3) / 4);
    ProfScope ps(kProfRaycast, stream);
    const bool mr = m.res_type == SE_GPU_RES_MULTI;
    if (map->tune)
        SE_CUDA_TRY(cudaEventRecord(map->tune->ev[2], stream));
#define SE_RAYCAST_LAUNCH(S_, MR_)                                                                                  \
    do {                                                                                                            \
        if (tile == 0)                                                                                              \
            launch_chained(raycast_kernel<S_, MR_, 0>, grid, 128, stream, m, s, map->rparams, pts_dev, nrm_dev,     \
                           scale_dev);                                                                              \
        else                                                                                                        \
            launch_chained(raycast_kernel<S_, MR_, 1>, grid, 128, stream, m, s, map->rparams, pts_dev, nrm_dev,     \
                           scale_dev);                                                                              \
    } while (0)
    if (m.storage == SE_GPU_STORAGE_F32 && !mr)
        SE_RAYCAST_LAUNCH(SE_GPU_STORAGE_F32, false);
    else if (!mr)
        SE_RAYCAST_LAUNCH(SE_GPU_STORAGE_F16, false);
    else if (m.storage == SE_GPU_STORAGE_F32)
        SE_RAYCAST_LAUNCH(SE_GPU_STORAGE_F32, true);
    else
        SE_RAYCAST_LAUNCH(SE_GPU_STORAGE_F16, true);
#undef SE_RAYCAST_LAUNCH
    if (map->tune)
        SE_CUDA_TRY(cudaEventRecord(map->tune->ev[3], stream));
    SE_CUDA_TRY(cudaGetLastError());
    return SE_GPU_OK;
}

} // namespace se_gpu

extern "C" se_gpu_status se_gpu_raycast(const se_gpu_map* map, const se_gpu_pinhole* sensor, const float T_WS[16],
                                        float* pts_dev, float* nrm_dev, int8_t* scale_dev, void* stream_p)
{
    if (!map || !sensor || !T_WS || !pts_dev || !nrm_dev || sensor->width <= 0 || sensor->height <= 0) {
        set_last_error("se_gpu_raycast: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    cudaStream_t stream = (cudaStream_t) stream_p;
    const_cast<se_gpu_map*>(map)->last_stream = stream;
    if (map->occ)
        return occ_raycast_volume(map->occ, *sensor, T_WS, pts_dev, nrm_dev, scale_dev, stream);
    return enqueue_raycast(map, *sensor, T_WS, nullptr, pts_dev, nrm_dev, scale_dev, stream);
}

static se_gpu_status field_query(const se_gpu_map* map, int64_t n, const float* pts, float* out, int* valid,
                                 void* stream_p, int grad)
{
    if (!map || n < 0 || n > (1ll << 31) - 1 || (n > 0 && (!pts || !out))) {
        set_last_error("se_gpu_map_field_%s: invalid argument", grad ? "grad" : "interp");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (map->occ) {
        set_last_error("se_gpu_map_field_%s: TSDF maps only", grad ? "grad" : "interp");
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    if (n == 0)
        return SE_GPU_OK;
    cudaStream_t stream = (cudaStream_t) stream_p;
    const unsigned blocks = (unsigned) ((n + 127) / 128);
    const bool mr = map->dev.res_type == SE_GPU_RES_MULTI;
    if (map->dev.storage == SE_GPU_STORAGE_F32 && !mr)
        field_query_kernel<SE_GPU_STORAGE_F32, false><<<blocks, 128, 0, stream>>>(map->dev, (int) n, pts, out, valid, grad);
    else if (!mr)
        field_query_kernel<SE_GPU_STORAGE_F16, false><<<blocks, 128, 0, stream>>>(map->dev, (int) n, pts, out, valid, grad);
    else if (map->dev.storage == SE_GPU_STORAGE_F32)
        field_query_kernel<SE_GPU_STORAGE_F32, true><<<blocks, 128, 0, stream>>>(map->dev, (int) n, pts, out, valid, grad);
    else
        field_query_kernel<SE_GPU_STORAGE_F16, true><<<blocks, 128, 0, stream>>>(map->dev, (int) n, pts, out, valid, grad);
    SE_CUDA_TRY(cudaGetLastError());
    return SE_GPU_OK;
}

extern "C" se_gpu_status se_gpu_map_field_interp(const se_gpu_map* map, int64_t n, const float* pts, float* values,
                                                 int* valid, void* stream)
{
    return field_query(map, n, pts, values, valid, stream, 0);
}

extern "C" se_gpu_status se_gpu_map_field_grad(const se_gpu_map* map, int64_t n, const float* pts, float* grads,
                                               int* valid, void* stream)
{
    return field_query(map, n, pts, grads, valid, stream, 1);
}
