// multires.cuh — voxel access for multi-resolution TSDF maps (Map<Data<TSDF>, Res::Multi, 8>).
//
// Each block keeps the reference's voxel pyramid (BlockMultiRes, block.hpp:66-166): scale 0
// holds 8^3 voxels at offset 0, scale 1 4^3 at 512, scale 2 2^3 at 576, scale 3 one at 584,
// each x + n*y + n^2*z. Every entry stores the data and the past data used by delta
// down-propagation, side by side so that one 16-byte (FP32) or 8-byte (FP16) access moves both:
//   SE_GPU_STORAGE_F32: float4 {tsdf, weight, past tsdf, past weight}
//   SE_GPU_STORAGE_F16: uint2  {f16x_pack(tsdf, weight), f16x_pack(past tsdf, past weight)}
// A block's current scale is the one it integrates at; reads "at the block's data" use it.
#pragma once

#include "se_gpu_internal.cuh"

namespace se_gpu {

__host__ __device__ __forceinline__ int mr_scale_offset(int scale)
{
    return scale == 0 ? 0 : scale == 1 ? 512 : scale == 2 ? 576 : 584;
}

// BlockMultiRes::getVoxelIdx (block_impl.hpp:80-91) from offsets within the block.
__device__ __forceinline__ int mr_index(int ox, int oy, int oz, int scale)
{
    const int n = kBlockSize >> scale;
    return mr_scale_offset(scale) + (ox >> scale) + n * (oy >> scale) + n * n * (oz >> scale);
}

struct MrVoxel {
    float tsdf, weight, past_tsdf, past_weight;
};

template <int S>
__device__ __forceinline__ MrVoxel mr_load(const MapDevice& m, int blk, int i)
{
    MrVoxel v;
    if (S == SE_GPU_STORAGE_F32) {
        const float4 d = reinterpret_cast<const float4*>(m.voxels)[(size_t) blk * kMrVoxels + i];
        v.tsdf = d.x;
        v.weight = d.y;
        v.past_tsdf = d.z;
        v.past_weight = d.w;
    }
    else {
        const uint2 d = reinterpret_cast<const uint2*>(m.voxels)[(size_t) blk * kMrVoxels + i];
        f16x_unpack(d.x, v.tsdf, v.weight);
        f16x_unpack(d.y, v.past_tsdf, v.past_weight);
    }
    return v;
}

// Data half only (tsdf, weight).
template <int S>
__device__ __forceinline__ void mr_load_data(const MapDevice& m, int blk, int i, float& t, float& w)
{
    if (S == SE_GPU_STORAGE_F32) {
        const float2 d = reinterpret_cast<const float2*>(m.voxels)[2 * ((size_t) blk * kMrVoxels + i)];
        t = d.x;
        w = d.y;
    }
    else {
        f16x_unpack(reinterpret_cast<const uint32_t*>(m.voxels)[2 * ((size_t) blk * kMrVoxels + i)], t, w);
    }
}

template <int S>
__device__ __forceinline__ void mr_store(const MapDevice& m, int blk, int i, const MrVoxel& v)
{
    if (S == SE_GPU_STORAGE_F32) {
        reinterpret_cast<float4*>(m.voxels)[(size_t) blk * kMrVoxels + i] =
            make_float4(v.tsdf, v.weight, v.past_tsdf, v.past_weight);
    }
    else {
        reinterpret_cast<uint2*>(m.voxels)[(size_t) blk * kMrVoxels + i] =
            make_uint2(f16x_pack(v.tsdf, v.weight), f16x_pack(v.past_tsdf, v.past_weight));
    }
}

__device__ __forceinline__ int mr_block_of(const MapDevice& m, int vx, int vy, int vz)
{
    return __ldg(&m.block_index[((size_t) (vz >> 3) << (2 * m.log2_bps)) | ((size_t) (vy >> 3) << m.log2_bps)
                                | (size_t) (vx >> 3)]);
}

// visitor::getData multi-res (visitor_impl.hpp:704-717): the data at the block's current scale,
// or the default data (tsdf 1, weight 0) where no block is allocated. A block that has never
// been integrated holds the default data.
template <int S>
__device__ __forceinline__ void mr_get_data(const MapDevice& m, int vx, int vy, int vz, float& t, float& w)
{
    const int b = mr_block_of(m, vx, vy, vz);
    int cur = b < 0 ? -1 : (int) m.block_scale[2 * b];
    if (cur < 0) {
        t = 1.0f;
        w = 0.0f;
        return;
    }
    mr_load_data<S>(m, b, mr_index(vx & 7, vy & 7, vz & 7, cur), t, w);
}

// visitor::getInterp multi-res (visitor_impl.hpp:906-972) with detail::get_neighbours
// (:398-697). From max(current scale of the query's block, desired scale) upwards, a scale is
// skipped when a block its neighbourhood touches is unallocated or integrates at a coarser
// scale; a base outside the AABB or an invalid neighbour ends the query.
template <int S>
__device__ bool mr_interp(const MapDevice& m, F3 vf, int desired_scale, float& out, int* returned_scale)
{
    const int q = mr_block_of(m, (int) vf.x, (int) vf.y, (int) vf.z);
    if (q < 0)
        return false;
    const int qcur = (int) m.block_scale[2 * q];
    const int init = qcur > desired_scale ? qcur : desired_scale;
#pragma unroll 1
    for (int scale = init; scale <= kMaxBlockScale; ++scale) {
        const int stride = 1 << scale;
        const float inv = 1.0f / (float) stride;
        const F3 bf = f3(inv * vf.x - 0.5f, inv * vf.y - 0.5f, inv * vf.z - 0.5f);
        const int b0 = stride * (int) bf.x, b1 = stride * (int) bf.y, b2 = stride * (int) bf.z;
        if (b0 < m.aabb[0] || b1 < m.aabb[1] || b2 < m.aabb[2] || b0 > m.aabb[3] || b1 > m.aabb[4] || b2 > m.aabb[5])
            return false;
        if (b0 < 0 || b1 < 0 || b2 < 0 || b0 + stride >= m.size || b1 + stride >= m.size || b2 + stride >= m.size)
            continue;
        float f[8], w[8];
        bool ok = true;
#pragma unroll 1
        for (int n = 0; n < 8 && ok; ++n) {
            const int cx = b0 + stride * (n & 1), cy = b1 + stride * ((n >> 1) & 1), cz = b2 + stride * (n >> 2);
            const int b = mr_block_of(m, cx, cy, cz);
            if (b < 0 || (int) m.block_scale[2 * b] > scale) {
                ok = false;
                break;
            }
            // a block never integrated (current scale -1) holds the default data
            if ((int) m.block_scale[2 * b] < 0) {
                f[n] = 1.0f;
                w[n] = 0.0f;
            }
            else {
                mr_load_data<S>(m, b, mr_index(cx & 7, cy & 7, cz & 7, scale), f[n], w[n]);
            }
        }
        if (!ok)
            continue;
        for (int n = 0; n < 8; ++n)
            if (!(w[n] != 0.0f))
                return false;
        if (returned_scale)
            *returned_scale = scale;
        const F3 t = f3(bf.x - floorf(bf.x), bf.y - floorf(bf.y), bf.z - floorf(bf.z));
        const F3 tc = f3(1.0f - t.x, 1.0f - t.y, 1.0f - t.z);
        out = ((f[0] * tc.x + f[1] * t.x) * tc.y + (f[2] * tc.x + f[3] * t.x) * t.y) * tc.z
            + ((f[4] * tc.x + f[5] * t.x) * tc.y + (f[6] * tc.x + f[7] * t.x) * t.y) * t.z;
        return true;
    }
    return false;
}

// The 32 gradient samples (visitor_impl.hpp:1332-1412): per axis a selector of
// {base-1, base, base+1, base+2} strides (clamped to the map), packed x | y << 2 | z << 4.
static __constant__ unsigned char kMrGradSel[32] = {
    0x14, 0x18, 0x24, 0x28, 0x11, 0x21, 0x05, 0x15, 0x25, 0x35, 0x09, 0x19, 0x29, 0x39, 0x1d, 0x2d,
    0x12, 0x22, 0x06, 0x16, 0x26, 0x36, 0x0a, 0x1a, 0x2a, 0x3a, 0x1e, 0x2e, 0x17, 0x1b, 0x27, 0x2b};

// visitor::getFieldGrad multi-res with desired scale 0 (visitor_impl.hpp:1257-1497): the
// central-difference gradient at the first scale, from the block's current one up, whose 32
// samples are all valid and stored at exactly that scale; in voxel units (the caller divides
// by the resolution).
template <int S>
__device__ bool mr_grad(const MapDevice& m, F3 vf, F3& g)
{
    const int q = mr_block_of(m, (int) vf.x, (int) vf.y, (int) vf.z);
    if (q < 0)
        return false;
    const int qcur = (int) m.block_scale[2 * q];
    const int init = qcur > 0 ? qcur : 0;
    const int top = m.size - 1;
#pragma unroll 1
    for (int scale = init; scale <= kMaxBlockScale; ++scale) {
        const int stride = 1 << scale;
        const float inv = 1.0f / (float) stride;
        const F3 sv = f3(inv * vf.x - 0.5f, inv * vf.y - 0.5f, inv * vf.z - 0.5f);
        const F3 fac = f3(sv.x - floorf(sv.x), sv.y - floorf(sv.y), sv.z - floorf(sv.z));
        const int base[3] = {stride * (int) sv.x, stride * (int) sv.y, stride * (int) sv.z};
        int sel[3][4];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            sel[i][0] = max(base[i] - stride, 0);
            sel[i][1] = max(base[i], 0);
            sel[i][2] = min(base[i] + stride, top);
            sel[i][3] = min(base[i] + 2 * stride, top);
        }
        // finest_octant(base, scale): a TSDF node holds no data, so only a block goes on
        const int hint = mr_block_of(m, base[0], base[1], base[2]);
        if (hint < 0)
            continue;
        float v[32];
        bool ok = true;
#pragma unroll 1
        for (int i = 0; i < 32; ++i) {
            const unsigned code = kMrGradSel[i];
            const int cx = sel[0][code & 3], cy = sel[1][(code >> 2) & 3], cz = sel[2][(code >> 4) & 3];
            const int b = mr_block_of(m, cx, cy, cz);
            if (b < 0) {
                ok = false;
                break;
            }
            const int cur = (int) m.block_scale[2 * b];
            const int rs = cur > scale ? cur : scale;
            if (rs != scale) {
                ok = false;
                break;
            }
            float t, w;
            if (cur < 0) {
                t = 1.0f;
                w = 0.0f;
            }
            else {
                mr_load_data<S>(m, b, mr_index(cx & 7, cy & 7, cz & 7, scale), t, w);
            }
            if (!(w != 0.0f)) {
                ok = false;
                break;
            }
            v[i] = t;
        }
        if (!ok)
            continue;
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
        const float sf = (float) stride;
        g = f3((0.5f * gx) / sf, (0.5f * gy) / sf, (0.5f * gz) / sf);
        return true;
    }
    return false;
}

} // namespace se_gpu
