// raycast.cu — se::raycaster::raycast_volume for single-res TSDF maps, and the batched
// Map::getFieldInterp / Map::getFieldGrad queries.
//
// One thread per pixel (an 8 x 4 pixel tile per warp for coherent block lookups):
//   1. first allocated block on the ray: the sparse-voxel-octree traversal of
//      VoxelBlockRayIterator (voxel_block_ray_iterator_impl.hpp:19-249, Laine & Karras 2010)
//      with the same float expressions; node existence is a bit test in the occupancy pyramid
//      instead of a child-pointer chase, and the traversal stack keeps only t_max;
//   2. the TSDF march of raycast<TSDF> (raycaster_impl.hpp:456-533): voxel fetches through the
//      dense block index with a one-block cache, trilinear interpolation near the surface
//      (visitor_impl.hpp:976-1024) and the linear zero-crossing estimate;
//   3. the surface normal from the 32-sample central-difference gradient
//      (visitor_impl.hpp:1094-1251, map_impl.hpp:236-262).
// Sample loops are deliberately not unrolled: one copy of the fetch path keeps the kernel
// inside the instruction cache.
#include <cmath>

#include "pipeline.cuh"
#include "profile.cuh"
#include "multires.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

__device__ __forceinline__ float fmax_std(float a, float b) { return (a < b) ? b : a; } // std::max
__device__ __forceinline__ float fmin_std(float a, float b) { return (b < a) ? b : a; } // std::min

// The state of VoxelBlockRayIterator after its first next(): found, tcmin(), tmax().
__device__ bool first_block(const MapDevice& m, const RaycastParams& rp, F3 o_W, F3 d_W, float near_p,
                            float far_p, float& tcmin, float& tmax)
{
    constexpr int kStackDepth = 23;
    float d[3] = {d_W.x, d_W.y, d_W.z};
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (fabsf(d[a]) < rp.eps)
            d[a] = copysignf(rp.eps, d[a]);
    const F3 o_M = apply(m.T_MW, o_W);
    const float ov[3] = {o_M.x / m.res, o_M.y / m.res, o_M.z / m.res};
    float t_coef[3], t_bias[3];
    int mirror_mask = 7;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float o = ov[a] / (float) m.size + 1.0f;
        t_coef[a] = -1.0f * (1.0f / fabsf(d[a]));
        t_bias[a] = t_coef[a] * o;
        if (d[a] > 0.0f) {
            mirror_mask ^= (1 << a);
            t_bias[a] = 3.0f * t_coef[a] - t_bias[a];
        }
    }
    float t_min = fmax_std(fmax_std(2.0f * t_coef[0] - t_bias[0], 2.0f * t_coef[1] - t_bias[1]),
                           2.0f * t_coef[2] - t_bias[2]);
    float t_max = fmin_std(fmin_std(t_coef[0] - t_bias[0], t_coef[1] - t_bias[1]), t_coef[2] - t_bias[2]);
    float h = t_max;
    t_min = fmax_std(t_min, near_p / rp.scaling);
    t_max = fmin_std(t_max, far_p / rp.scaling);
    tmax = t_max * rp.scaling;

    int idx = 0;
    float pos[3] = {1.0f, 1.0f, 1.0f};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (1.5f * t_coef[a] - t_bias[a] > t_min) {
            idx ^= (1 << a);
            pos[a] = 1.5f;
        }
    }
    int scale = kStackDepth - 1;
    float scale_exp2 = 0.5f;
    float stack_tmax[kStackDepth];
#pragma unroll
    for (int i = 0; i < kStackDepth; ++i)
        stack_tmax[i] = 0.0f;

    // Bounded: every iteration descends (at most 23 times between advances) or advances the
    // ray past a cell boundary; the cap only guards against a malformed map.
    for (int iter = 0; iter < (1 << 20) && scale < kStackDepth; ++iter) {
        float tc[3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
            tc[a] = pos[a] * t_coef[a] - t_bias[a];
        const float tc_max = fmin_std(fmin_std(tc[0], tc[1]), tc[2]);

        // The child at (pos, scale). Its index in the mirrored frame comes from the float bits
        // of pos (pos is in [1, 2), cells of side 2^(scale - 23)); mirrored axes flip back to
        // the real index, which is the cell idx ^ mirror_mask ^ 7 of the reference.
        const int L = scale - rp.min_scale;
        bool child = false;
        if (L >= 0) {
            const int lg = 23 - scale;
            const uint32_t n = 1u << lg;
            uint32_t c[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const uint32_t k = (uint32_t) (__float_as_int(pos[a]) - 0x3f800000) >> scale;
                c[a] = (mirror_mask & (1 << a)) ? k : (n - 1u - k);
            }
            child = occ_test(m, L, c[0], c[1], c[2]);
        }
        if (scale == rp.min_scale && child) {
            tcmin = t_min * rp.scaling;
            return true;
        }
        if (child && t_min <= t_max) {
            const float tv_max = fmin_std(t_max, tc_max);
            const float half = scale_exp2 * 0.5f;
            float t_centre[3];
#pragma unroll
            for (int a = 0; a < 3; ++a)
                t_centre[a] = half * t_coef[a] + tc[a];
            if (tc_max < h)
                stack_tmax[scale] = t_max;
            h = tc_max;
            idx = 0;
            --scale;
            scale_exp2 = half;
#pragma unroll
            for (int a = 0; a < 3; ++a)
                if (t_centre[a] > t_min)
                    idx ^= (1 << a);
#pragma unroll
            for (int a = 0; a < 3; ++a)
                if (idx & (1 << a))
                    pos[a] += scale_exp2;
            t_max = tv_max;
            continue;
        }
        int step_mask = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
            if (tc[a] <= tc_max)
                step_mask |= (1 << a);
#pragma unroll
        for (int a = 0; a < 3; ++a)
            if (step_mask & (1 << a))
                pos[a] -= scale_exp2;
        t_min = tc_max;
        idx ^= step_mask;
        if ((idx & step_mask) != 0) {
            uint32_t differing = 0;
#pragma unroll
            for (int a = 0; a < 3; ++a)
                if (step_mask & (1 << a))
                    differing |= (uint32_t) (__float_as_int(pos[a]) ^ __float_as_int(pos[a] + scale_exp2));
            scale = (__float_as_int((float) differing) >> 23) - 127;
            if (scale >= kStackDepth)
                break;
            scale_exp2 = __int_as_float((scale - kStackDepth + 127) << 23);
            t_max = stack_tmax[scale];
            int sh[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                sh[a] = __float_as_int(pos[a]) >> scale;
                pos[a] = __int_as_float(sh[a] << scale);
            }
            idx = (sh[0] & 1) | ((sh[1] & 1) << 1) | ((sh[2] & 1) << 2);
            h = 0.0f;
        }
    }
    tcmin = t_min * rp.scaling;
    return false;
}

// One-entry cache of the last block touched by this thread.
struct BlockCache {
    int bx, by, bz;
    int idx; // pool index or -1
};

__device__ __forceinline__ int lookup_block(const MapDevice& m, BlockCache& c, int vx, int vy, int vz)
{
    const int bx = vx >> 3, by = vy >> 3, bz = vz >> 3;
    if (bx != c.bx || by != c.by || bz != c.bz) {
        c.bx = bx;
        c.by = by;
        c.bz = bz;
        c.idx = __ldg(&m.block_index[((size_t) bz << (2 * m.log2_bps)) | ((size_t) by << m.log2_bps) | (size_t) bx]);
    }
    return c.idx;
}

// visitor::getData single-res: block voxel or the default data (tsdf 1, weight 0).
template <int S>
__device__ __forceinline__ bool fetch_voxel(const MapDevice& m, BlockCache& c, int vx, int vy, int vz, float& t,
                                            float& w)
{
    const int b = lookup_block(m, c, vx, vy, vz);
    if (b < 0) {
        t = 1.0f;
        w = 0.0f;
        return false;
    }
    load_voxel<S>(m, b, (vx & 7) + 8 * (vy & 7) + 64 * (vz & 7), t, w);
    return true;
}

template <int S>
__device__ __forceinline__ void map_get_data(const MapDevice& m, BlockCache& c, F3 p, float& t, float& w)
{
    int vx, vy, vz;
    if (!point_to_voxel(m, p, vx, vy, vz)) {
        t = 1.0f;
        w = 0.0f;
        return;
    }
    fetch_voxel<S>(m, c, vx, vy, vz, t, w);
}

// visitor::getInterp single-res: any unallocated block or invalid voxel gives nullopt.
template <int S>
__device__ bool field_interp(const MapDevice& m, BlockCache& c, F3 p_W, float& out)
{
    F3 vf;
    if (!point_to_voxel_f(m, p_W, vf))
        return false;
    const F3 bf = f3(vf.x - 0.5f, vf.y - 0.5f, vf.z - 0.5f);
    const int b0 = (int) bf.x, b1 = (int) bf.y, b2 = (int) bf.z;
    if (b0 < 0 || b1 < 0 || b2 < 0 || b0 + 1 >= m.size || b1 + 1 >= m.size || b2 + 1 >= m.size)
        return false;
    float f[8];
    if ((b0 & 7) != 7 && (b1 & 7) != 7 && (b2 & 7) != 7) {
        // the 8 neighbours share one block
        const int blk = lookup_block(m, c, b0, b1, b2);
        if (blk < 0)
            return false;
        const int base = (b0 & 7) + 8 * (b1 & 7) + 64 * (b2 & 7);
        bool ok = true;
#pragma unroll
        for (int n = 0; n < 8; ++n) {
            float w;
            load_voxel<S>(m, blk, base + (n & 1) + 8 * ((n >> 1) & 1) + 64 * (n >> 2), f[n], w);
            ok = ok && (w != 0.0f);
        }
        if (!ok)
            return false;
    }
    else {
        bool ok = true;
#pragma unroll 1
        for (int n = 0; n < 8; ++n) {
            float w;
            if (!fetch_voxel<S>(m, c, b0 + (n & 1), b1 + ((n >> 1) & 1), b2 + ((n >> 2) & 1), f[n], w))
                return false; // an unallocated block fails before any validity test
            ok = ok && (w != 0.0f);
        }
        if (!ok)
            return false;
    }
    const F3 t = f3(bf.x - floorf(bf.x), bf.y - floorf(bf.y), bf.z - floorf(bf.z));
    const F3 tc = f3(1.0f - t.x, 1.0f - t.y, 1.0f - t.z);
    out = ((f[0] * tc.x + f[1] * t.x) * tc.y + (f[2] * tc.x + f[3] * t.x) * t.y) * tc.z
        + ((f[4] * tc.x + f[5] * t.x) * tc.y + (f[6] * tc.x + f[7] * t.x) * t.y) * t.z;
    return true;
}

// The 32 gradient samples: per axis a selector of {base-1, base, base+1, base+2} (clamped to
// the map), in the reference's order. Packed 2 bits per axis: x | y << 2 | z << 4.
__constant__ unsigned char kGradSel[32] = {
    0x14, 0x18, 0x24, 0x28, 0x11, 0x21, 0x05, 0x15, 0x25, 0x35, 0x09, 0x19, 0x29, 0x39, 0x1d, 0x2d,
    0x12, 0x22, 0x06, 0x16, 0x26, 0x36, 0x0a, 0x1a, 0x2a, 0x3a, 0x1e, 0x2e, 0x17, 0x1b, 0x27, 0x2b};

// visitor::getFieldGrad single-res with Map::getFieldGrad's division by the resolution.
template <int S>
__device__ bool field_grad(const MapDevice& m, BlockCache& c, F3 p_W, F3& g)
{
    F3 vf;
    if (!point_to_voxel_f(m, p_W, vf))
        return false;
    const F3 s = f3(vf.x - 0.5f, vf.y - 0.5f, vf.z - 0.5f);
    const F3 fac = f3(s.x - floorf(s.x), s.y - floorf(s.y), s.z - floorf(s.z));
    const int base[3] = {(int) s.x, (int) s.y, (int) s.z};
    const int top = m.size - 1;
    int sel[3][4];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        sel[i][0] = max(base[i] - 1, 0);
        sel[i][1] = max(base[i], 0);
        sel[i][2] = min(base[i] + 1, top);
        sel[i][3] = min(base[i] + 2, top);
    }
    if (lookup_block(m, c, base[0], base[1], base[2]) < 0)
        return false;
    float v[32];
#pragma unroll 1
    for (int i = 0; i < 32; ++i) {
        const int code = kGradSel[i];
        float t, w;
        fetch_voxel<S>(m, c, sel[0][code & 3], sel[1][(code >> 2) & 3], sel[2][(code >> 4) & 3], t, w);
        if (!(w != 0.0f))
            return false;
        v[i] = t;
    }
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
    g = f3((0.5f * gx) / m.res, (0.5f * gy) / m.res, (0.5f * gz) / m.res);
    return true;
}

// Map::getData<Safe::On> on a multi-res map: the data at the block's current scale.
template <int S>
__device__ __forceinline__ void mr_map_get_data(const MapDevice& m, F3 p, float& t, float& w)
{
    int vx, vy, vz;
    if (!point_to_voxel(m, p, vx, vy, vz)) {
        t = 1.0f;
        w = 0.0f;
        return;
    }
    mr_get_data<S>(m, vx, vy, vz, t, w);
}

// Map::getFieldInterp(point, returned_scale) on a multi-res map (map_impl.hpp:176-196).
template <int S>
__device__ __forceinline__ bool mr_field_interp(const MapDevice& m, F3 p_W, float& out, int* returned_scale)
{
    F3 vf;
    if (!point_to_voxel_f(m, p_W, vf))
        return false;
    return mr_interp<S>(m, vf, 0, out, returned_scale);
}

// Map::getFieldGrad on a multi-res map (map_impl.hpp:236-262).
template <int S>
__device__ __forceinline__ bool mr_field_grad(const MapDevice& m, F3 p_W, F3& g)
{
    F3 vf;
    if (!point_to_voxel_f(m, p_W, vf))
        return false;
    F3 gv;
    if (!mr_grad<S>(m, vf, gv))
        return false;
    g = f3(gv.x / m.res, gv.y / m.res, gv.z / m.res);
    return true;
}

// raycast<TSDF> (raycaster_impl.hpp:456-533). MR selects the multi-res data access; the
// returned scale is the one of the last successful interpolation (0 for single-res maps).
template <int S, bool MR>
__device__ bool raycast_tsdf(const MapDevice& m, const RaycastParams& rp, BlockCache& c, F3 o, F3 d, float t_near,
                             float t_far, F3& hit, int& scale_out)
{
    int scale_tt = 0;
    float t_min, t_max;
    first_block(m, rp, o, d, t_near, t_far, t_min, t_max);
    if (t_min <= 0.0f)
        return false;
    const float step = m.res;
    const float largestep = (float) kBlockSize * step;
    float t = t_min;
    if (!(t_near < t_max))
        return false;
    float stepsize = largestep;
    F3 p = add(o, mul(d, t));
    float f_t, w_t;
    if constexpr (MR)
        mr_map_get_data<S>(m, p, f_t, w_t);
    else
        map_get_data<S>(m, c, p, f_t, w_t);
    float f_tt = 0.0f;
    if (!(f_t >= 0.0f))
        return false;
    // every step is at least res > 0, so the march ends at t_far (NaN poses end it at once)
    for (; t < t_far; t += stepsize) {
        float f, w;
        if constexpr (MR)
            mr_map_get_data<S>(m, p, f, w);
        else
            map_get_data<S>(m, c, p, f, w);
        if (!(w != 0.0f)) {
            stepsize = largestep;
            p = add(p, mul(stepsize, d));
            continue;
        }
        f_tt = f;
        // The reference compares with the double literal 0.1; no float lies in (0.1, 0.1f), so
        // (double) f <= 0.1 is exactly f < 0.1f, with no FP64 instruction.
        if (f_tt < 0.1f && f_tt >= -0.5f) {
            float fi;
            bool ok;
            if constexpr (MR)
                ok = mr_field_interp<S>(m, p, fi, &scale_tt);
            else
                ok = field_interp<S>(m, c, p, fi);
            if (ok)
                f_tt = fi;
        }
        if (f_tt < 0.0f)
            break;
        stepsize = fmax_std(f_tt * m.trunc, step);
        p = add(p, mul(stepsize, d));
        f_t = f_tt;
    }
    if (f_tt < 0.0f) {
        t = t - stepsize * (f_tt - 0.0f) / (f_tt - f_t);
        hit = add(o, mul(d, t));
        scale_out = scale_tt;
        return true;
    }
    return false;
}

__global__ void raycast_prep_kernel(const float* pose12, RaycastParams host_p, RaycastParams* out)
{
    RaycastParams p = host_p;
    if (pose12 != nullptr)
        p.T_WS = tf_from12(pose12);
    *out = p;
}

template <int S, bool MR>
__global__ void __launch_bounds__(128) raycast_kernel(MapDevice m, Pinhole s, const RaycastParams* __restrict__ P,
                                                      float* __restrict__ pts, float* __restrict__ nrm,
                                                      int8_t* __restrict__ scale)
{
    const RaycastParams rp = *P;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
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
            ok = field_grad<S>(m, c, hit, g);
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
    raycast_prep_kernel<<<1, 1, 0, stream>>>(T_WS_host16 ? nullptr : pose12_dev, rp, map->rparams);
    dim3 grid((s.w + 15) / 16, (s.h + 7) / 8);
    ProfScope ps(kProfRaycast, stream);
    const bool mr = m.res_type == SE_GPU_RES_MULTI;
    if (m.storage == SE_GPU_STORAGE_F32 && !mr)
        raycast_kernel<SE_GPU_STORAGE_F32, false><<<grid, 128, 0, stream>>>(m, s, map->rparams, pts_dev, nrm_dev, scale_dev);
    else if (!mr)
        raycast_kernel<SE_GPU_STORAGE_F16, false><<<grid, 128, 0, stream>>>(m, s, map->rparams, pts_dev, nrm_dev, scale_dev);
    else if (m.storage == SE_GPU_STORAGE_F32)
        raycast_kernel<SE_GPU_STORAGE_F32, true><<<grid, 128, 0, stream>>>(m, s, map->rparams, pts_dev, nrm_dev, scale_dev);
    else
        raycast_kernel<SE_GPU_STORAGE_F16, true><<<grid, 128, 0, stream>>>(m, s, map->rparams, pts_dev, nrm_dev, scale_dev);
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
    return enqueue_raycast(map, *sensor, T_WS, nullptr, pts_dev, nrm_dev, scale_dev, stream);
}

static se_gpu_status field_query(const se_gpu_map* map, int64_t n, const float* pts, float* out, int* valid,
                                 void* stream_p, int grad)
{
    if (!map || n < 0 || n > (1ll << 31) - 1 || (n > 0 && (!pts || !out))) {
        set_last_error("se_gpu_map_field_%s: invalid argument", grad ? "grad" : "interp");
        return SE_GPU_ERR_BAD_ARG;
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
