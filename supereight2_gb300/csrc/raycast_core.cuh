// raycast_core.cuh — device functions of the single-res TSDF raycast shared by the raycast,
// field-query and raycast-adjoint kernels: the first allocated block on a ray (the result of
// VoxelBlockRayIterator, voxel_block_ray_iterator_impl.hpp:19-249, found by a level DDA over the
// occupancy pyramid), voxel fetches
// through the dense block index with a one-block cache, trilinear interpolation
// (visitor_impl.hpp:976-1024), the 32-sample gradient (visitor_impl.hpp:1094-1251) and the
// march of raycast<TSDF> (raycaster_impl.hpp:456-533).
#pragma once

#include "multires.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

__device__ __forceinline__ float fmax_std(float a, float b) { return (a < b) ? b : a; } // std::max
__device__ __forceinline__ float fmin_std(float a, float b) { return (b < a) ? b : a; } // std::min

// The first level of the pyramid that the first-block search steps through: cells of 4^3
// blocks. Starting lower (fewer levels, more cells) or higher (more descents) measured slower.
constexpr int kDdaTopLevel = 2;

// The state of VoxelBlockRayIterator after its first next() (found, tcmin(), tmax()): the first
// allocated block along the ray and the ray parameter where it enters it.
//
// The reference walks its pointer octree from the root with the sparse-voxel-octree traversal
// (voxel_block_ray_iterator_impl.hpp:19-249, Laine & Karras 2010) in the mirrored unit cube
// [1, 2)^3, where the ray runs towards smaller coordinates on every axis and a cell's exit plane
// q on axis a is crossed at t = q * t_coef[a] - t_bias[a]. Here the same cells are visited by a
// level DDA over the occupancy pyramid with integer cell indices:
//   - the descent from the root to level kDdaTopLevel is replayed in arithmetic (the child that
//     holds the ray at t_min, chosen by the reference's centre test half * t_coef + t_cell > t_min);
//   - at each level the ray steps through cells along the axes whose exit plane comes first
//     (all tied axes at once, as the reference's step mask), enters an occupied cell by the same
//     centre test, and climbs back up by the highest bit in which a stepped index changed (the
//     reference's pop), never above kDdaTopLevel;
//   - every plane parameter is the reference's expression q * t_coef - t_bias of the plane's
//     exact coordinate, so a block found through the same face has the same tcmin float.
// An occupied cell is entered only while t_min <= t_max (far plane, root exit), except that a
// block is returned whenever it is reached inside a level-1 cell that was entered, as in the
// reference. A ray that finds no block returns the root's exit parameter, which is where the
// reference's traversal ends. The two walks can differ only where a ray passes within rounding of
// a cell edge, where the reference decides a tie at a coarser level than this walk: 0 of 921,600
// rays of three 640x480 frames of the 1 cm benchmark map (and 1-2 per frame when starting at
// levels 0 or 1).
static __device__ bool first_block(const MapDevice& m, const RaycastParams& rp, F3 o_W, F3 d_W, float near_p,
                                   float far_p, float& tcmin, float& tmax)
{
    float d[3] = {d_W.x, d_W.y, d_W.z};
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (fabsf(d[a]) < rp.eps)
            d[a] = copysignf(rp.eps, d[a]);
    const F3 o_M = apply(m.T_MW, o_W);
    const float ov[3] = {o_M.x / m.res, o_M.y / m.res, o_M.z / m.res};
    float t_coef[3], t_bias[3];
    bool flip[3]; // the axes the unit cube mirrors (the ray runs towards larger coordinates)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float o = ov[a] / (float) m.size + 1.0f;
        t_coef[a] = -1.0f * (1.0f / fabsf(d[a]));
        t_bias[a] = t_coef[a] * o;
        flip[a] = d[a] > 0.0f;
        if (flip[a])
            t_bias[a] = 3.0f * t_coef[a] - t_bias[a];
    }
    float t_min = fmax_std(fmax_std(2.0f * t_coef[0] - t_bias[0], 2.0f * t_coef[1] - t_bias[1]),
                           2.0f * t_coef[2] - t_bias[2]);
    float t_max = fmin_std(fmin_std(t_coef[0] - t_bias[0], t_coef[1] - t_bias[1]), t_coef[2] - t_bias[2]);
    const float root_exit = t_max;
    t_min = fmax_std(t_min, near_p / rp.scaling);
    t_max = fmin_std(t_max, far_p / rp.scaling);
    tmax = t_max * rp.scaling;

    // the root's children hold 2^(log2_bps - 1) blocks per axis: level log2_bps - 1
    const int top = m.log2_bps - 1;
    const int Lc = top < kDdaTopLevel ? top : kDdaTopLevel;
    float pos[3]; // lower corner of the current cell in the mirrored cube
#pragma unroll
    for (int a = 0; a < 3; ++a)
        pos[a] = (1.5f * t_coef[a] - t_bias[a] > t_min) ? 1.5f : 1.0f;
    float cell = 0.5f;
    for (int L = top; L > Lc; --L) {
        const float half = cell * 0.5f;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float tc = pos[a] * t_coef[a] - t_bias[a];
            if (half * t_coef[a] + tc > t_min)
                pos[a] += half;
        }
        cell = half;
    }

    // Level L has 2^mL cells per axis; k is the mirrored cell index, the plane of index k is the
    // float 1 + k * 2^-mL (exact), tcs its crossing parameter, bit the real cell's bit at level L.
    int L = Lc;
    int mL = m.log2_bps - Lc;
    int k[3];
    float tcs[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        k[a] = (__float_as_int(pos[a]) - 0x3f800000) >> (23 - mL);
        tcs[a] = pos[a] * t_coef[a] - t_bias[a];
    }
    const uint32_t* occ_l = m.occ[L];
    uint32_t bit;
    int step_bit[3]; // change of bit when k[a] decreases by one
    auto level_index = [&]() {
        const int nm1 = (1 << mL) - 1;
        bit = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            bit |= (uint32_t) (flip[a] ? nm1 - k[a] : k[a]) << (a * mL);
            step_bit[a] = flip[a] ? (1 << (a * mL)) : -(1 << (a * mL));
        }
    };
    level_index();
    // Bounded: each step moves one cell along the ray and each descent goes one level down; the
    // cap only guards against NaN parameters.
    for (int it = 0; it < (1 << 16); ++it) {
        if (L >= 1 && t_min > t_max)
            break;
        if ((__ldg(&occ_l[bit >> 5]) >> (bit & 31)) & 1u) {
            if (L == 0) {
                tcmin = t_min * rp.scaling;
                return true;
            }
            const float half = __int_as_float((126 - mL) << 23); // 2^-(mL + 1)
            --L;
            ++mL;
            occ_l = m.occ[L];
            const int sh = 23 - mL;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const bool upper = half * t_coef[a] + tcs[a] > t_min;
                k[a] = 2 * k[a] + (upper ? 1 : 0);
                if (upper)
                    tcs[a] = __int_as_float(0x3f800000 + (k[a] << sh)) * t_coef[a] - t_bias[a];
            }
            level_index();
            continue;
        }
        const float tc_max = fmin_std(fmin_std(tcs[0], tcs[1]), tcs[2]);
        uint32_t changed = 0;
        int k_low = 0;
        const int sh = 23 - mL;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (tcs[a] <= tc_max) {
                const int kn = k[a] - 1;
                changed |= (uint32_t) (k[a] ^ kn);
                k[a] = kn;
                k_low = kn < k_low ? kn : k_low;
                bit += step_bit[a];
                tcs[a] = __int_as_float(0x3f800000 + (kn << sh)) * t_coef[a] - t_bias[a];
            }
        }
        t_min = tc_max;
        if (k_low < 0) // left the root
            break;
        if (t_min > t_max && (L >= 1 || (changed >> 1) != 0))
            break;
        int up = 31 - __clz((int) changed);
        if (up > Lc - L)
            up = Lc - L;
        if (up > 0) {
            L += up;
            mL -= up;
            occ_l = m.occ[L];
            const int sh2 = 23 - mL;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                k[a] >>= up;
                tcs[a] = __int_as_float(0x3f800000 + (k[a] << sh2)) * t_coef[a] - t_bias[a];
            }
            level_index();
        }
    }
    tcmin = root_exit * rp.scaling;
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
