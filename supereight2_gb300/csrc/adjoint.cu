// adjoint.cu — a differentiable depth render of a single-res TSDF map and its adjoint with
// respect to the camera pose and the TSDF voxel values. No counterpart in the reference.
//
// Forward (se_gpu_render_depth), one thread per pixel:
//   1. the march of raycast<TSDF> (raycaster_impl.hpp:456-533) up to the first sample below the
//      surface, which brackets the zero crossing between the last two samples;
//   2. regula falsi (Illinois) on the trilinear field g(t) = F(o + t d) inside the bracket until
//      |g| < 1e-6 (truncation units): the rendered depth is z = t* n_z, with t* the root and
//      n_z the z component of the unit ray in the camera frame.
// A pixel renders 0 where the march finds no crossing or the trilinear interpolation is
// undefined at the bracket ends (an unallocated or unobserved voxel).
//
// Adjoint (se_gpu_raycast_adjoint): the march is recomputed per ray (nothing is stored between
// the passes), and the implicit function theorem at the root gives, with grad F taken in world
// coordinates (the analytic gradient of the trilinear interpolant) and the pose perturbed on
// the left, T = exp(xi) T_WS, xi = [rho; omega]:
//   dt*/dxi  = -[grad F, p* x grad F] / (grad F . d)
//   dt*/df_k = -w_k / (grad F . d)            (w_k the trilinear weight of corner voxel k)
// and dz/d. = n_z dt*/d. . The twist row [grad F, p* x grad F] is the point-to-plane ICP
// Jacobian row of icp_impl.hpp:92-99 with the plane normal grad F.
#include <cmath>

#include "pipeline.cuh"
#include "profile.cuh"
#include "raycast_core.cuh"

namespace se_gpu {

// The 8 corners of a trilinear sample, with what the adjoint needs.
struct Tri {
    int blk[8];
    short vi[8];
    float f[8];
    F3 t; // fractional position in the cell
};

template <int S>
__device__ bool tri_sample(const MapDevice& m, BlockCache& c, F3 p_W, Tri& q, float& value)
{
    F3 vf;
    if (!point_to_voxel_f(m, p_W, vf))
        return false;
    const F3 bf = f3(vf.x - 0.5f, vf.y - 0.5f, vf.z - 0.5f);
    const int b0 = (int) bf.x, b1 = (int) bf.y, b2 = (int) bf.z;
    if (b0 < 0 || b1 < 0 || b2 < 0 || b0 + 1 >= m.size || b1 + 1 >= m.size || b2 + 1 >= m.size)
        return false;
#pragma unroll 1
    for (int n = 0; n < 8; ++n) {
        const int vx = b0 + (n & 1), vy = b1 + ((n >> 1) & 1), vz = b2 + (n >> 2);
        const int blk = lookup_block(m, c, vx, vy, vz);
        if (blk < 0)
            return false;
        const int vi = (vx & 7) + 8 * (vy & 7) + 64 * (vz & 7);
        float w;
        load_voxel<S>(m, blk, vi, q.f[n], w);
        if (!(w != 0.0f))
            return false;
        q.blk[n] = blk;
        q.vi[n] = (short) vi;
    }
    q.t = f3(bf.x - floorf(bf.x), bf.y - floorf(bf.y), bf.z - floorf(bf.z));
    const F3 t = q.t;
    const F3 tc = f3(1.0f - t.x, 1.0f - t.y, 1.0f - t.z);
    const float* f = q.f;
    value = ((f[0] * tc.x + f[1] * t.x) * tc.y + (f[2] * tc.x + f[3] * t.x) * t.y) * tc.z
        + ((f[4] * tc.x + f[5] * t.x) * tc.y + (f[6] * tc.x + f[7] * t.x) * t.y) * t.z;
    return true;
}

// Root of the trilinear field on the ray: false when there is none to differentiate.
template <int S>
__device__ bool diff_hit(const MapDevice& m, const RaycastParams& rp, BlockCache& c, F3 o, F3 d, float t_near,
                         float t_far, float& t_star, Tri& q)
{
    float t_min, t_max;
    first_block(m, rp, o, d, t_near, t_far, t_min, t_max);
    if (t_min <= 0.0f || !(t_near < t_max))
        return false;
    const float step = m.res;
    const float largestep = (float) kBlockSize * step;
    float t = t_min;
    float stepsize = largestep;
    F3 p = add(o, mul(d, t));
    float f_t, w_t;
    map_get_data<S>(m, c, p, f_t, w_t);
    float f_tt = 0.0f;
    if (!(f_t >= 0.0f))
        return false;
    for (; t < t_far; t += stepsize) {
        float f, w;
        map_get_data<S>(m, c, p, f, w);
        if (!(w != 0.0f)) {
            stepsize = largestep;
            p = add(p, mul(stepsize, d));
            continue;
        }
        f_tt = f;
        if (f_tt < 0.1f && f_tt >= -0.5f) {
            float fi;
            if (field_interp<S>(m, c, p, fi))
                f_tt = fi;
        }
        if (f_tt < 0.0f)
            break;
        stepsize = fmax_std(f_tt * m.trunc, step);
        p = add(p, mul(stepsize, d));
    }
    if (!(f_tt < 0.0f))
        return false;
    // bracket [t - stepsize, t] on the trilinear field
    float ta = t - stepsize, tb = t, fa, fb;
    if (!tri_sample<S>(m, c, add(o, mul(d, ta)), q, fa) || !tri_sample<S>(m, c, add(o, mul(d, tb)), q, fb))
        return false;
    if (!(fa >= 0.0f && fb < 0.0f))
        return false;
    float tm = tb;
    int side = 0;
#pragma unroll 1
    for (int it = 0; it < 40; ++it) {
        tm = (ta * fb - tb * fa) / (fb - fa);
        float fm;
        if (!tri_sample<S>(m, c, add(o, mul(d, tm)), q, fm))
            return false;
        if (fabsf(fm) < 1.0e-6f)
            break;
        if (fm < 0.0f) {
            tb = tm;
            fb = fm;
            if (side == -1)
                fa *= 0.5f;
            side = -1;
        }
        else {
            ta = tm;
            fa = fm;
            if (side == 1)
                fb *= 0.5f;
            side = 1;
        }
        if (!(tb - ta > 1.0e-7f * tb))
            break;
    }
    // q holds the cell of the last sample, at tm
    t_star = tm;
    return true;
}

// grad F in world coordinates at the sample q: R_MW^T (grad_v F) / res
__device__ __forceinline__ F3 tri_grad_W(const MapDevice& m, const Tri& q)
{
    const float* f = q.f;
    const F3 t = q.t;
    const F3 tc = f3(1.0f - t.x, 1.0f - t.y, 1.0f - t.z);
    const float gx = ((f[1] - f[0]) * tc.y + (f[3] - f[2]) * t.y) * tc.z + ((f[5] - f[4]) * tc.y + (f[7] - f[6]) * t.y) * t.z;
    const float gy = ((f[2] - f[0]) * tc.x + (f[3] - f[1]) * t.x) * tc.z + ((f[6] - f[4]) * tc.x + (f[7] - f[5]) * t.x) * t.z;
    const float gz = ((f[4] - f[0]) * tc.x + (f[5] - f[1]) * t.x) * tc.y + ((f[6] - f[2]) * tc.x + (f[7] - f[3]) * t.x) * t.y;
    const float* R = m.T_MW.R;
    return f3((R[0] * gx + R[3] * gy + R[6] * gz) / m.res, (R[1] * gx + R[4] * gy + R[7] * gz) / m.res,
              (R[2] * gx + R[5] * gy + R[8] * gz) / m.res);
}

struct RayGeom {
    F3 o, d;
    float nz, t_near, t_far;
};

__device__ __forceinline__ RayGeom ray_geom(const Pinhole& s, const RaycastParams& rp, int x, int y)
{
    RayGeom g;
    const F3 ray_S = back_project(s, (float) x, (float) y);
    const F3 nS = normalized(ray_S);
    g.d = rot(rp.T_WS, nS);
    g.o = f3(rp.T_WS.t[0], rp.T_WS.t[1], rp.T_WS.t[2]);
    g.nz = nS.z;
    g.t_near = s.near_plane / nS.z;
    g.t_far = s.far_plane / nS.z;
    return g;
}

template <int S>
__global__ void __launch_bounds__(128) render_depth_kernel(MapDevice m, Pinhole s, RaycastParams rp,
                                                           float* __restrict__ depth)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
    if (x >= s.w || y >= s.h)
        return;
    const RayGeom g = ray_geom(s, rp, x, y);
    BlockCache c{-1, -1, -1, -1};
    Tri q;
    float t_star;
    depth[(size_t) x + (size_t) y * s.w] = diff_hit<S>(m, rp, c, g.o, g.d, g.t_near, g.t_far, t_star, q) ? t_star * g.nz : 0.0f;
}

// Per pixel: dL/dz = grad_depth[i]. Accumulates dL/dxi into twist_acc (6 doubles) and dL/df
// into voxel_grad (pool block * 512 + voxel); jac receives dz/dxi per pixel (0 if no root).
template <int S>
__global__ void __launch_bounds__(128) adjoint_kernel(MapDevice m, Pinhole s, RaycastParams rp,
                                                      const float* __restrict__ grad_depth, double* __restrict__ twist_acc,
                                                      float* __restrict__ voxel_grad, float* __restrict__ jac)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
    float acc[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (x < s.w && y < s.h) {
        const size_t i = (size_t) x + (size_t) y * s.w;
        const float gd = grad_depth ? grad_depth[i] : 0.0f;
        float row[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        if (gd != 0.0f || jac) {
            const RayGeom g = ray_geom(s, rp, x, y);
            BlockCache c{-1, -1, -1, -1};
            Tri q;
            float t_star;
            if (diff_hit<S>(m, rp, c, g.o, g.d, g.t_near, g.t_far, t_star, q)) {
                const F3 gF = tri_grad_W(m, q);
                const float den = dot(gF, g.d);
                if (fabsf(den) > 1.0e-12f) {
                    const F3 p = add(g.o, mul(g.d, t_star));
                    const F3 pxg = cross(p, gF);
                    const float k = -g.nz / den; // dz/dF at fixed geometry
                    row[0] = k * gF.x;
                    row[1] = k * gF.y;
                    row[2] = k * gF.z;
                    row[3] = k * pxg.x;
                    row[4] = k * pxg.y;
                    row[5] = k * pxg.z;
                    if (gd != 0.0f) {
                        for (int j = 0; j < 6; ++j)
                            acc[j] = gd * row[j];
                        if (voxel_grad) {
                            const F3 t = q.t;
                            const F3 tc = f3(1.0f - t.x, 1.0f - t.y, 1.0f - t.z);
                            const float c0 = gd * k;
#pragma unroll 1
                            for (int n = 0; n < 8; ++n) {
                                const float w = ((n & 1) ? t.x : tc.x) * (((n >> 1) & 1) ? t.y : tc.y) * ((n >> 2) ? t.z : tc.z);
                                atomicAdd(&voxel_grad[(size_t) q.blk[n] * kBlockVoxels + q.vi[n]], c0 * w);
                            }
                        }
                    }
                }
            }
            if (jac)
                for (int j = 0; j < 6; ++j)
                    jac[6 * i + j] = row[j];
        }
    }
    // warp sums, then one double atomic per warp and component
    for (int j = 0; j < 6; ++j) {
        float v = acc[j];
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0 && v != 0.0f)
            atomicAdd(&twist_acc[j], (double) v);
    }
}

static RaycastParams host_raycast_params(const MapDevice& m, const float* T_WS)
{
    RaycastParams rp;
    rp.T_WS = tf_from16(T_WS);
    rp.scaling = (float) m.size * m.res;
    rp.eps = std::exp2((float) (-std::log2((double) m.size)));
    rp.min_scale = 23 - m.log2_bps;
    return rp;
}

} // namespace se_gpu

using namespace se_gpu;

static se_gpu_status adjoint_args(const se_gpu_map* map, const se_gpu_pinhole* sensor, const float* T, const char* fn)
{
    if (!map || !sensor || !T || sensor->width <= 0 || sensor->height <= 0) {
        set_last_error("%s: invalid argument", fn);
        return SE_GPU_ERR_BAD_ARG;
    }
    if (map->dev.res_type != SE_GPU_RES_SINGLE) {
        set_last_error("%s: single-resolution maps only", fn);
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    return SE_GPU_OK;
}

extern "C" se_gpu_status se_gpu_render_depth(const se_gpu_map* map, const se_gpu_pinhole* sensor, const float T_WS[16],
                                             float* depth_dev, void* stream_p)
{
    se_gpu_status st = adjoint_args(map, sensor, T_WS, "se_gpu_render_depth");
    if (st != SE_GPU_OK)
        return st;
    if (!depth_dev) {
        set_last_error("se_gpu_render_depth: null depth");
        return SE_GPU_ERR_BAD_ARG;
    }
    cudaStream_t stream = (cudaStream_t) stream_p;
    const MapDevice& m = map->dev;
    const Pinhole s = make_pinhole(*sensor);
    const RaycastParams rp = host_raycast_params(m, T_WS);
    dim3 grid((s.w + 15) / 16, (s.h + 7) / 8);
    if (m.storage == SE_GPU_STORAGE_F32)
        render_depth_kernel<SE_GPU_STORAGE_F32><<<grid, 128, 0, stream>>>(m, s, rp, depth_dev);
    else
        render_depth_kernel<SE_GPU_STORAGE_F16><<<grid, 128, 0, stream>>>(m, s, rp, depth_dev);
    SE_CUDA_TRY(cudaGetLastError());
    const_cast<se_gpu_map*>(map)->last_stream = stream;
    return SE_GPU_OK;
}

extern "C" se_gpu_status se_gpu_raycast_adjoint(const se_gpu_map* map, const se_gpu_pinhole* sensor,
                                                const float T_WS[16], const float* grad_depth_dev,
                                                double* twist_grad_dev, float* voxel_grad_dev, float* jac_dev,
                                                void* stream_p)
{
    se_gpu_status st = adjoint_args(map, sensor, T_WS, "se_gpu_raycast_adjoint");
    if (st != SE_GPU_OK)
        return st;
    if (!twist_grad_dev || (!grad_depth_dev && !jac_dev)) {
        set_last_error("se_gpu_raycast_adjoint: twist_grad_dev and one of grad_depth_dev / jac_dev are required");
        return SE_GPU_ERR_BAD_ARG;
    }
    cudaStream_t stream = (cudaStream_t) stream_p;
    const MapDevice& m = map->dev;
    const Pinhole s = make_pinhole(*sensor);
    const RaycastParams rp = host_raycast_params(m, T_WS);
    dim3 grid((s.w + 15) / 16, (s.h + 7) / 8);
    if (m.storage == SE_GPU_STORAGE_F32)
        adjoint_kernel<SE_GPU_STORAGE_F32><<<grid, 128, 0, stream>>>(m, s, rp, grad_depth_dev, twist_grad_dev,
                                                                     voxel_grad_dev, jac_dev);
    else
        adjoint_kernel<SE_GPU_STORAGE_F16><<<grid, 128, 0, stream>>>(m, s, rp, grad_depth_dev, twist_grad_dev,
                                                                     voxel_grad_dev, jac_dev);
    SE_CUDA_TRY(cudaGetLastError());
    const_cast<se_gpu_map*>(map)->last_stream = stream;
    return SE_GPU_OK;
}
