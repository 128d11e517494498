// raycast_core.cuh — device functions of the single-res TSDF raycast shared by the raycast,
// field-query and raycast-adjoint kernels: the first allocated block on a ray (the
// VoxelBlockRayIterator traversal, voxel_block_ray_iterator_impl.hpp:19-249), voxel fetches
// through the dense block index with a one-block cache, trilinear interpolation
// (visitor_impl.hpp:976-1024), the 32-sample gradient (visitor_impl.hpp:1094-1251) and the
// march of raycast<TSDF> (raycaster_impl.hpp:456-533).
#pragma once

#include "multires.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

__device__ __forceinline__ float fmax_std(float a, float b) { return (a < b) ? b : a; } // std::max
__device__ __forceinline__ float fmin_std(float a, float b) { return (b < a) ? b : a; } // std::min

constexpr int kEsvoStackDepth = 23;

// The state of VoxelBlockRayIterator after its first next(): found, tcmin(), tmax(). The
// traversal stack (t_max per scale) is stack[scale * stride]: a caller with many threads per SM
// passes this thread's column of a shared-memory array; with stack == nullptr it lives in the
// thread's local memory.
static __device__ bool first_block(const MapDevice& m, const RaycastParams& rp, F3 o_W, F3 d_W, float near_p,
                                   float far_p, float& tcmin, float& tmax, float* stack = nullptr, int stride = 1)
{
    constexpr int kStackDepth = kEsvoStackDepth;
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
    float local_stack[kStackDepth];
    float* stack_tmax = stack;
    if (stack_tmax == nullptr) {
        stack_tmax = local_stack;
        stride = 1;
    }
    for (int i = 0; i < kStackDepth; ++i)
        stack_tmax[i * stride] = 0.0f;

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
                stack_tmax[scale * stride] = t_max;
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
            t_max = stack_tmax[scale * stride];
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
__device__ bool field_interp_vf(const MapDevice& m, BlockCache& c, F3 vf, float& out);

template <int S>
__device__ bool field_interp(const MapDevice& m, BlockCache& c, F3 p_W, float& out)
{
    F3 vf;
    if (!point_to_voxel_f(m, p_W, vf))
        return false;
    return field_interp_vf<S>(m, c, vf, out);
}

// field_interp from the point's voxel coordinates (point_to_voxel_f, inside the map).
template <int S>
__device__ bool field_interp_vf(const MapDevice& m, BlockCache& c, F3 vf, float& out)
{
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
static __constant__ unsigned char kGradSel[32] = {
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
    g = f3(div_res(m, 0.5f * gx), div_res(m, 0.5f * gy), div_res(m, 0.5f * gz));
    return true;
}

// kGradSel as a compile-time function, for the unrolled loads below.
__host__ __device__ constexpr int grad_sel(int i)
{
    constexpr unsigned char t[32] = {0x14, 0x18, 0x24, 0x28, 0x11, 0x21, 0x05, 0x15, 0x25, 0x35, 0x09,
                                     0x19, 0x29, 0x39, 0x1d, 0x2d, 0x12, 0x22, 0x06, 0x16, 0x26, 0x36,
                                     0x0a, 0x1a, 0x2a, 0x3a, 0x1e, 0x2e, 0x17, 0x1b, 0x27, 0x2b};
    return t[i];
}

// field_grad with the 32 samples loaded together: the blocks of the sample neighbourhood
// [base - 1, base + 2]^3 (at most 2 per axis) are looked up once into bt (this thread's 8
// entries, bt[k * bs] for k = x | y << 1 | z << 2 block offsets), then the 32 voxel loads are
// independent of one another. A failed sample fails the query as it does in field_grad, so the
// result and its arithmetic are field_grad's.
template <int S>
__device__ bool field_grad_batched(const MapDevice& m, BlockCache& c, F3 p_W, F3& g, int* bt, int bs)
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
    int lo[3], two[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = sel[a][0] >> 3;
        two[a] = (sel[a][3] >> 3) != lo[a];
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int ox = k & 1, oy = (k >> 1) & 1, oz = k >> 2;
        int b = -1;
        if ((!ox || two[0]) && (!oy || two[1]) && (!oz || two[2]))
            b = __ldg(&m.block_index[((size_t) (lo[2] + oz) << (2 * m.log2_bps)) | ((size_t) (lo[1] + oy) << m.log2_bps)
                                     | (size_t) (lo[0] + ox)]);
        bt[k * bs] = b;
    }
    float v[32];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 32; ++i) {
        const int code = grad_sel(i);
        const int x = sel[0][code & 3], y = sel[1][(code >> 2) & 3], z = sel[2][(code >> 4) & 3];
        const int b = bt[(((x >> 3) - lo[0]) | (((y >> 3) - lo[1]) << 1) | (((z >> 3) - lo[2]) << 2)) * bs];
        float t = 1.0f, w = 0.0f;
        if (b >= 0)
            load_voxel<S>(m, b, (x & 7) + 8 * (y & 7) + 64 * (z & 7), t, w);
        ok = ok && (w != 0.0f);
        v[i] = t;
    }
    if (!ok)
        return false;
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
    g = f3(div_res(m, 0.5f * gx), div_res(m, 0.5f * gy), div_res(m, 0.5f * gz));
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
    g = f3(div_res(m, gv.x), div_res(m, gv.y), div_res(m, gv.z));
    return true;
}

// raycast<TSDF> (raycaster_impl.hpp:456-533). MR selects the multi-res data access; the
// returned scale is the one of the last successful interpolation (0 for single-res maps).
template <int S, bool MR>
__device__ bool raycast_tsdf(const MapDevice& m, const RaycastParams& rp, BlockCache& c, F3 o, F3 d, float t_near,
                             float t_far, F3& hit, int& scale_out, float* stack = nullptr, int stride = 1)
{
    int scale_tt = 0;
    float t_min, t_max;
    first_block(m, rp, o, d, t_near, t_far, t_min, t_max, stack, stride);
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
        // single-res: the sample's voxel coordinates serve both the data lookup (their integer
        // part, point_to_voxel) and the interpolation below
        F3 vf;
        bool in_map = false;
        if constexpr (MR) {
            mr_map_get_data<S>(m, p, f, w);
        }
        else {
            in_map = point_to_voxel_f(m, p, vf);
            f = 1.0f;
            w = 0.0f;
            if (in_map)
                fetch_voxel<S>(m, c, (int) vf.x, (int) vf.y, (int) vf.z, f, w);
        }
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
                ok = in_map && field_interp_vf<S>(m, c, vf, fi);
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

} // namespace se_gpu
