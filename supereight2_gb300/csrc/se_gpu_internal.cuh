// se_gpu_internal.cuh — device data structures and helpers shared by the kernels.
//
// Float arithmetic follows one fixed operation order (the CPU oracle uses the same):
//   dot3 = (a0*b0 + a1*b1) + a2*b2;   (T*p)_i = ((R_i0 p0 + R_i1 p1) + R_i2 p2) + t_i
//   norm = sqrtf(dot3(v, v));         normalized(v) = v / norm (component-wise division)
// The library is compiled with --fmad=false and IEEE division / square root, so every
// operation rounds separately and the allocation key set and integer weights are bit-exact
// against the oracle.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/se_gpu.h"

namespace se_gpu {

constexpr int kBlockSize = 8;
constexpr int kBlockVoxels = 512;
constexpr int kMaxBlockScale = 3;
constexpr int kMrVoxels = 585; // 8^3 + 4^3 + 2^3 + 1 (BlockMultiRes, block.hpp:126-157)
constexpr unsigned long long kEmptyKey = 0xffffffffffffffffULL;
constexpr int kMaxProbe = 256;

// error bits latched in MapDevice::counters[kCntError]
constexpr int kErrPoolFull = 1;
constexpr int kErrProbeLimit = 2;

// device counters
enum {
    kCntNumBlocks = 0,   // allocated blocks (may exceed capacity on overflow: clamp on read)
    kCntError = 1,
    kCntListed = 2,      // update list length of the current frame
    kCntNumOld = 3,      // blocks allocated before the current frame
    kCntValidPixels = 4,
    kCntUpdated = 6,     // 64-bit (slots 6, 7)
    kNumCounters = 16
};

struct F3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__host__ __device__ __forceinline__ F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ F3 mul(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ F3 mul(float s, F3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ __forceinline__ F3 divs(F3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__host__ __device__ __forceinline__ float dot(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__host__ __device__ __forceinline__ float norm(F3 a) { return sqrtf(dot(a, a)); }
__host__ __device__ __forceinline__ F3 normalized(F3 a)
{
    const float sq = dot(a, a);
    if (sq > 0.0f) {
        const float n = sqrtf(sq);
        return f3(a.x / n, a.y / n, a.z / n);
    }
    return a;
}
__host__ __device__ __forceinline__ F3 cross(F3 a, F3 b)
{
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Rigid / affine transform with a row-major 3x3 part.
struct Tf {
    float R[9];
    float t[3];
};
__host__ __device__ __forceinline__ F3 rot(const Tf& T, F3 v)
{
    return f3((T.R[0] * v.x + T.R[1] * v.y) + T.R[2] * v.z,
              (T.R[3] * v.x + T.R[4] * v.y) + T.R[5] * v.z,
              (T.R[6] * v.x + T.R[7] * v.y) + T.R[8] * v.z);
}
__host__ __device__ __forceinline__ F3 apply(const Tf& T, F3 v)
{
    const F3 r = rot(T, v);
    return f3(r.x + T.t[0], r.y + T.t[1], r.z + T.t[2]);
}
__host__ __device__ inline Tf compose(const Tf& A, const Tf& B)
{
    Tf C;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            C.R[3 * i + j] = (A.R[3 * i] * B.R[j] + A.R[3 * i + 1] * B.R[3 + j]) + A.R[3 * i + 2] * B.R[6 + j];
        C.t[i] = ((A.R[3 * i] * B.t[0] + A.R[3 * i + 1] * B.t[1]) + A.R[3 * i + 2] * B.t[2]) + A.t[i];
    }
    return C;
}
__host__ __device__ inline Tf inverse_iso(const Tf& A)
{
    Tf B;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            B.R[3 * i + j] = A.R[3 * j + i];
    for (int i = 0; i < 3; ++i)
        B.t[i] = -((B.R[3 * i] * A.t[0] + B.R[3 * i + 1] * A.t[1]) + B.R[3 * i + 2] * A.t[2]);
    return B;
}
__host__ __device__ inline Tf tf_from16(const float* m)
{
    Tf T;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            T.R[3 * i + j] = m[4 * i + j];
        T.t[i] = m[4 * i + 3];
    }
    return T;
}
__host__ __device__ inline void tf_to16(const Tf& T, float* m)
{
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            m[4 * i + j] = T.R[3 * i + j];
        m[4 * i + 3] = T.t[i];
    }
    m[12] = m[13] = m[14] = 0.0f;
    m[15] = 1.0f;
}

// ---------------------------------------------------------------------- Morton keys --
// include/se/map/utils/impl/key_util_impl.hpp:44-101: 19 bits per axis, x at bit 0.
__host__ __device__ __forceinline__ uint64_t morton_expand(uint64_t v)
{
    uint64_t x = v & 0x7ffff;
    x = (x | x << 32) & 0x1f00000000ffffULL;
    x = (x | x << 16) & 0x1f0000ff0000ffULL;
    x = (x | x << 8) & 0x100f00f00f00f00fULL;
    x = (x | x << 4) & 0x10c30c30c30c30c3ULL;
    x = (x | x << 2) & 0x1249249249249249ULL;
    return x;
}
__host__ __device__ __forceinline__ uint64_t morton_compact(uint64_t v)
{
    uint64_t x = v & 0x49249249249249ULL;
    x = (x | x >> 2) & 0x10c30c30c30c30c3ULL;
    x = (x | x >> 4) & 0x100f00f00f00f00fULL;
    x = (x | x >> 8) & 0x1f0000ff0000ffULL;
    x = (x | x >> 16) & 0x1f00000000ffffULL;
    x = (x | x >> 32) & 0x1fffffULL;
    return x;
}
// Key of the 8^3 block containing voxel (x, y, z): code masked at scale 3, << 5 | 3.
__host__ __device__ __forceinline__ uint64_t block_key(int x, int y, int z)
{
    const uint64_t code = morton_expand((uint64_t) (x & ~7)) | (morton_expand((uint64_t) (y & ~7)) << 1)
        | (morton_expand((uint64_t) (z & ~7)) << 2);
    return (code << 5) | (uint64_t) kMaxBlockScale;
}
__host__ __device__ __forceinline__ uint32_t hash_slot(uint64_t key, uint32_t mask)
{
    // the low 9 code bits and the 5 scale bits of a block key are constant
    const uint64_t h = (key >> 14) * 0x9E3779B97F4A7C15ULL;
    return (uint32_t) (h >> 32) & mask;
}

// ------------------------------------------------------------------------ map state --
struct MapDevice {
    // geometry
    int size;            // voxels per side
    int log2_size;
    int bps;             // blocks per side = size / 8
    int log2_bps;
    float res;
    float inv_res;       // RN(1 / res), for div_res
    float dim;           // size * res
    Tf T_MW;
    Tf T_WM;
    int T_MW_translation; // T_MW's rotation is exactly the identity (the reference's default)
    float trunc;         // res * truncation_boundary_factor
    float max_weight;
    int storage;         // se_gpu_storage
    int capacity;        // block pool capacity
    // block hash: Morton block key -> pool index (open addressing, linear probing). One
    // 16-byte slot per entry: x = key (kEmptyKey when free), y = pool index (or -1).
    ulonglong2* hash;
    uint32_t hash_mask;
    // block pool
    int* block_coord;             // 3 ints per block
    unsigned long long* block_keys;
    int* block_ts;
    void* voxels;                 // F32: float2 {tsdf, weight}; F16: f16x_pack words
    // Occupancy pyramid for the raycast's first-block search: level 0 has one bit per block (bps^3 bits, x fastest), level L one bit
    // per (2^L)^3 blocks. A bit is set iff an allocated block lies inside the cell, which is
    // exactly when the reference's pointer octree holds the node.
    uint32_t* occ[11];
    int occ_levels;               // log2(bps) + 1
    // Dense block index, bps^3 int32 (x fastest), -1 where no block is allocated: one load
    // per lookup on the read paths (at most 1024^3 entries = 4 GiB for an 8192^3 map). The
    // hash above stays the allocation arbiter and the Morton-key index.
    int* block_index;
    // scratch / counters
    int* counters;                // kNumCounters ints
    int* update_list;             // capacity ints
    // Allocated-block AABB in voxels (min xyz, max xyz, inclusive), extended on every insert
    // like Octree::aabbExtend; INT_MAX / INT_MIN while the map is empty.
    int* aabb;
    // Multi-resolution TSDF (res_type SE_GPU_RES_MULTI): `voxels` holds kMrVoxels entries per
    // block, each {data, past data}; block_scale holds (current_scale, min_scale) per block
    // (-1 before the first update) and block_nscale this frame's integration scale.
    int res_type;
    signed char* block_scale;
    signed char* block_nscale;
};

__device__ __forceinline__ int hash_find(const MapDevice& m, uint64_t key)
{
    uint32_t slot = hash_slot(key, m.hash_mask);
    for (int p = 0; p < kMaxProbe; ++p) {
        const ulonglong2 e = m.hash[slot];
        if (e.x == key)
            return (int) (long long) e.y;
        if (e.x == kEmptyKey)
            return -1;
        slot = (slot + 1) & m.hash_mask;
    }
    return -1;
}

// Occupancy bit of the cell (cx, cy, cz) at pyramid level L.
__device__ __forceinline__ bool occ_test(const MapDevice& m, int L, uint32_t cx, uint32_t cy, uint32_t cz)
{
    const int lg = m.log2_bps - L;
    const uint32_t bit = (cz << (2 * lg)) | (cy << lg) | cx;
    return (__ldg(&m.occ[L][bit >> 5]) >> (bit & 31)) & 1u;
}

// Pool index of the block containing voxel block coordinates (bx, by, bz), or -1.
__device__ __forceinline__ int block_at(const MapDevice& m, int bx, int by, int bz)
{
    return m.block_index[((size_t) bz << (2 * m.log2_bps)) | ((size_t) by << m.log2_bps) | (size_t) bx];
}

// FP16 storage word (SE_GPU_STORAGE_F16, 4 bytes per voxel):
//   bits 31..8  the tsdf as an FP16 number carrying 8 more significand bits: FP16's sign and
//               5-bit exponent (bias 15) with an 18-bit significand. Bits 31..16 alone are the
//               binary16 value truncated toward zero; the low 8 bits of the field are the
//               running mean's rounding guard.
//   bits 7..0   the integer weight (max_weight <= 255).
// Rounding is to nearest (ties to even) on the 18-bit significand: |error| <= 2^-19 for
// |tsdf| <= 1. A running mean over weights up to W then stays within W * 2^-19 of the FP32
// layout's (each update shrinks the carried error by (w - 1) / w and adds at most 2^-19):
// 1.9e-4 truncation units at the reference's max_weight = 100. Plain binary16 storage would
// carry W * 2^-11 (0.049) in the worst case.
// Both directions work on the float's bits scaled by 2^-112, which puts FP16's exponent range
// (bias 15) at the bottom of FP32's (bias 127): a tsdf of at least 2^-14 keeps its significand
// and loses 112 from its exponent, a smaller one becomes an FP32 subnormal in units of 2^-149
// (the scaling rounds it to nearest even there), and dropping the 5 low bits of those bits with
// rounding to nearest even gives the 23-bit field in either case. Unpacking shifts the field
// back into an FP32 pattern and scales by 2^112, exact for normal and subnormal fields alike.
// The weight moves through the low bits of 2^23 + w. No branches, no conversion instructions.
__device__ __forceinline__ uint32_t f16x_pack(float t, float w)
{
    const uint32_t b = __float_as_uint(fabsf(t) * 0x1p-112f);
    uint32_t em = (b + 0xfu + ((b >> 5) & 1u)) >> 5; // exponent and significand, 23 bits
    em = em < 0x7fffffu ? em : 0x7fffffu;            // beyond the format's range (not reached: |tsdf| <= 1)
    const float wc = w < 255.0f ? w : 255.0f;
    return (__float_as_uint(t) & 0x80000000u) | (em << 8) | (__float_as_uint(wc + 8388608.0f) & 0xffu);
}
__device__ __forceinline__ void f16x_unpack(uint32_t d, float& t, float& w)
{
    const float mag = __uint_as_float((d >> 3) & 0x0fffffe0u) * 0x1p112f;
    t = __uint_as_float(__float_as_uint(mag) | (d & 0x80000000u));
    w = __uint_as_float(0x4b000000u | (d & 0xffu)) - 8388608.0f;
}

// Voxel data access; S is the se_gpu_storage layout (F32: float2 {tsdf, weight};
// F16: the uint32 word of f16x_pack).
template <int S>
__device__ __forceinline__ void load_voxel(const MapDevice& m, int blk, int vi, float& tsdf, float& w)
{
    if (S == SE_GPU_STORAGE_F32) {
        const float2 d = reinterpret_cast<const float2*>(m.voxels)[(size_t) blk * kBlockVoxels + vi];
        tsdf = d.x;
        w = d.y;
    }
    else {
        f16x_unpack(reinterpret_cast<const uint32_t*>(m.voxels)[(size_t) blk * kBlockVoxels + vi], tsdf, w);
    }
}
template <int S>
__device__ __forceinline__ void store_voxel(const MapDevice& m, int blk, int vi, float tsdf, float w)
{
    if (S == SE_GPU_STORAGE_F32) {
        reinterpret_cast<float2*>(m.voxels)[(size_t) blk * kBlockVoxels + vi] = make_float2(tsdf, w);
    }
    else {
        reinterpret_cast<uint32_t*>(m.voxels)[(size_t) blk * kBlockVoxels + vi] = f16x_pack(tsdf, w);
    }
}

// x / res, correctly rounded, without a division: q = RN(x r) with r = RN(1 / res), the
// residual x - q res is exact as one fused multiply-add, and RN(q + (x - q res) r) is RN(x / res)
// (Markstein's theorem on the correction step of Newton-Raphson division: r within half an ulp
// of 1 / res and q within one ulp of the quotient give the correctly rounded quotient, barring
// underflow and overflow). Tiny and non-finite x take the IEEE division. The identity is checked
// exhaustively for every float x in [2^-72, 2^14) and ten resolutions (tests/test_exact_division.py).
__host__ __device__ __forceinline__ float div_res(const MapDevice& m, float x)
{
    if (!(fabsf(x) >= 0x1p-100f && fabsf(x) < 0x1p100f))
        return x / m.res;
    const float q = x * m.inv_res;
    return fmaf(fmaf(-q, m.res, x), m.inv_res, q);
}

// T_MW p: with an identity rotation the three products by 1 and the six by 0 change nothing
// but the sign of a zero, so p + t gives the same voxel coordinates.
__host__ __device__ __forceinline__ F3 to_map(const MapDevice& m, F3 p_W)
{
    if (m.T_MW_translation)
        return f3(p_W.x + m.T_MW.t[0], p_W.y + m.T_MW.t[1], p_W.z + m.T_MW.t[2]);
    return apply(m.T_MW, p_W);
}

// Map::contains + pointToVoxel<Safe::On> (include/se/map/impl/map_impl.hpp:58-64,538-550).
__host__ __device__ __forceinline__ bool point_to_voxel(const MapDevice& m, F3 p_W, int& vx, int& vy, int& vz)
{
    const F3 p = to_map(m, p_W);
    if (!(p.x >= 0.0f && p.x < m.dim && p.y >= 0.0f && p.y < m.dim && p.z >= 0.0f && p.z < m.dim))
        return false;
    vx = (int) div_res(m, p.x);
    vy = (int) div_res(m, p.y);
    vz = (int) div_res(m, p.z);
    return true;
}
__host__ __device__ __forceinline__ bool point_to_voxel_f(const MapDevice& m, F3 p_W, F3& v)
{
    const F3 p = to_map(m, p_W);
    if (!(p.x >= 0.0f && p.x < m.dim && p.y >= 0.0f && p.y < m.dim && p.z >= 0.0f && p.z < m.dim))
        return false;
    v = f3(div_res(m, p.x), div_res(m, p.y), div_res(m, p.z));
    return true;
}

// ---------------------------------------------------------------------------- sensor --
struct Pinhole {
    int w, h;
    float fx, fy, cx, cy;
    float inv_fx, inv_fy;
    float near_plane, far_plane;
    int left_hand;
    float planes[6][4]; // left, right, bottom, top, near, far
};

__host__ __device__ __forceinline__ F3 back_project(const Pinhole& s, float u, float v)
{
    return f3((u - s.cx) * s.inv_fx, (v - s.cy) * s.inv_fy, 1.0f);
}
__host__ __device__ __forceinline__ bool project(const Pinhole& s, F3 p, float& u, float& v)
{
    if (fabsf(p.z) < 1.0e-12f)
        return false;
    const float rz = 1.0f / p.z;
    u = s.fx * (p.x * rz) + s.cx;
    v = s.fy * (p.y * rz) + s.cy;
    if (!(u >= -0.5f && u < (float) s.w - 0.5f && v >= -0.5f && v < (float) s.h - 0.5f))
        return false;
    return p.z > 0.0f;
}
__host__ __device__ __forceinline__ bool sphere_in_frustum(const Pinhole& s, F3 c, float radius)
{
    for (int i = 0; i < 6; ++i) {
        const float d = ((c.x * s.planes[i][0] + c.y * s.planes[i][1]) + c.z * s.planes[i][2]) + s.planes[i][3];
        if (d < -radius)
            return false;
    }
    return true;
}

// PinholeCamera ctor / downsampling ctor (src/sensor/pinhole_camera.cpp:63-111,246-310).
Pinhole make_pinhole(int w, int h, float fx, float fy, float cx, float cy, float near_p, float far_p);
Pinhole make_pinhole(const se_gpu_pinhole& p);
Pinhole downsampled(const Pinhole& s, float dsf);

// host-side error reporting
void set_last_error(const char* fmt, ...);
se_gpu_status cuda_status(cudaError_t e, const char* what);

} // namespace se_gpu

#define SE_CUDA_TRY(call)                                                                    \
    do {                                                                                     \
        cudaError_t _e = (call);                                                             \
        if (_e != cudaSuccess)                                                               \
            return ::se_gpu::cuda_status(_e, #call);                                         \
    } while (0)

namespace se_gpu {

// ------------------------------------------------------------- per-call parameters --
// Every per-frame quantity the kernels need is derived from one pose by the functions below,
// which run on the host (pose given by the caller) or in a one-thread prep kernel (pose
// produced on the device, e.g. by the tracker inside a captured CUDA graph). Both compile to
// the same IEEE operations, so either route gives bit-identical parameters.

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

struct IntegrateParams {
    CarveParams cp;
    FrustumParams fp;
    UpdateParams up;
};

struct RaycastParams {
    Tf T_WS;
    float scaling; // octree size * res
    float eps;     // 2^-log2(size)
    int min_scale; // 23 - log2(size / 8)
};

// RaycastCarver ctor / operator() (raycast_carver_impl.hpp:39-67), fetcher::frustum and the
// updater's T_CV (singleres_tsdf_updater_impl.hpp:37-42).
__host__ __device__ inline IntegrateParams make_integrate_params(const MapDevice& m, float trunc_factor,
                                                                 const Pinhole& s, const Tf& T_WS, int timestamp)
{
    IntegrateParams p;
    p.cp.T_WS = T_WS;
    p.cp.t_WS = f3(T_WS.t[0], T_WS.t[1], T_WS.t[2]);
    p.cp.band = 2.0f * m.res * trunc_factor;
    p.cp.half_band = p.cp.band * 0.5f;
    p.cp.far_limit = s.far_plane + p.cp.band * 0.5f;
    p.cp.num_steps = (int) ceilf(p.cp.band / (2.0f * m.res));
    p.fp.T_SW = inverse_iso(T_WS);
    for (int sc = 0; sc < 20; ++sc)
        p.fp.radius[sc] = sqrtf(3.0f) / 2.0f * m.res * (float) (1 << (sc < 19 ? sc : 19));
    Tf T_CV = compose(inverse_iso(T_WS), m.T_WM);
    for (int i = 0; i < 9; ++i)
        T_CV.R[i] = T_CV.R[i] * m.res;
    for (int i = 0; i < 3; ++i)
        T_CV.t[i] = ((T_CV.R[3 * i] * 0.5f + T_CV.R[3 * i + 1] * 0.5f) + T_CV.R[3 * i + 2] * 0.5f) + T_CV.t[i];
    p.up.T_CV = T_CV;
    p.up.timestamp = timestamp;
    return p;
}

__host__ __device__ inline Tf tf_from12(const float* m)
{
    Tf T;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            T.R[3 * i + j] = m[4 * i + j];
        T.t[i] = m[4 * i + 3];
    }
    return T;
}

} // namespace se_gpu

struct se_gpu_occ_map;

namespace se_gpu {
// Launch geometry of the frame path's two largest kernels, chosen by the frame pipeline's
// autotuner (se_gpu_frame_autotune); results do not depend on it.
struct FrameTiles {
    int update_ctas_per_sm = 8; // update_kernel grid: SMs x this (a grid-stride loop over the listed blocks)
    int update_round = 4;       // voxels a lane projects together per round (2 or 4)
    int raycast_tile = 0;       // raycast warp tile: 0 = 8 x 4 pixels, 1 = 16 x 2
};
// Events around the update and raycast launches while the autotuner times a frame.
struct FrameTuneEvents {
    cudaEvent_t ev[4];          // update start / end, raycast start / end
};
} // namespace se_gpu

struct se_gpu_map {
    se_gpu::MapDevice dev;
    se_gpu_occ_map* occ;              // occupancy maps only (dev holds the geometry)
    se_gpu_map_config config;
    int device;
    cudaStream_t last_stream;
    se_gpu::IntegrateParams* iparams; // device copy of the current integrate's parameters
    se_gpu::RaycastParams* rparams;   // device copy of the current raycast's parameters
    int* timestamp_dev;               // device frame counter used by captured pipelines
    se_gpu::FrameTiles tiles;         // launch geometry of the update and raycast kernels
    se_gpu::FrameTuneEvents* tune;    // non-null while the frame autotuner times a run
    // the frustum test runs beside the carver (neither reads what the other writes): a second
    // stream forked from and joined back into the caller's stream around them
    cudaStream_t side;
    cudaEvent_t fork_ev, join_ev;
};

namespace se_gpu {

// Insert a block key that the caller did not find; the thread whose CAS claims an empty hash
// slot allocates the pool entry and publishes it in the dense index and the occupancy pyramid.
// Probing is bounded: on exhaustion the map latches kErrProbeLimit.
__device__ __forceinline__ void insert_block(const MapDevice& m, uint64_t key, int bx, int by, int bz)
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
                if (m.block_scale) {
                    m.block_scale[2 * idx] = -1;
                    m.block_scale[2 * idx + 1] = -1;
                }
                atomicMin(&m.aabb[0], bx << 3);
                atomicMin(&m.aabb[1], by << 3);
                atomicMin(&m.aabb[2], bz << 3);
                atomicMax(&m.aabb[3], (bx << 3) + kBlockSize - 1);
                atomicMax(&m.aabb[4], (by << 3) + kBlockSize - 1);
                atomicMax(&m.aabb[5], (bz << 3) + kBlockSize - 1);
                m.block_index[((size_t) bz << (2 * m.log2_bps)) | ((size_t) by << m.log2_bps) | (size_t) bx] = idx;
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

int device_sm_count();

// Kernels on the per-frame path are launched with programmatic stream serialisation: a kernel's
// CTAs may be scheduled while the previous kernel on the stream drains, and each of these kernels
// begins with grid_dep_wait(), which returns once that kernel has completed and its writes are
// visible. Nothing runs earlier than before; only the launch latency between the kernels is
// hidden. Each such kernel then lets the next one be scheduled at once (launch_dependents): the
// next kernel's CTAs take free slots in this one's tail and wait there. (Without the launch
// attribute, griddepcontrol.wait returns at once.)
__device__ __forceinline__ void grid_dep_wait()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Rule: a cooperative kernel, or any kernel whose CTAs wait for one another (a grid barrier,
// like the persistent ICP's), is never launched with this attribute. Early-scheduled CTAs hold
// SM slots while they wait for their predecessor, and a grid barrier assumes that all of its
// CTAs are resident at once. Such kernels get an ordinary (or cooperative) launch, which starts
// only after the previous kernel has finished.
template <typename... KArgs, typename... Args>
inline void launch_chained(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t stream, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

} // namespace se_gpu
