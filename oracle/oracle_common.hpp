// oracle_common.hpp — shared pieces of the CPU oracle (test infrastructure only): the float
// algebra with the fixed operation order, Morton keys, the pointer octree of the TSDF maps and
// the pinhole camera. Included by the oracle's translation units; nothing here is exported.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "se_oracle.h"

/* The type of IEEE binary32 bit manipulations; the FP64 build of the oracle (se_oracle_f64.cpp)
 * turns every other float into a double. */
#ifndef SO_BITS_FLOAT
#define SO_BITS_FLOAT float
#endif

namespace {

/* ---------------------------------------------------------------- small float algebra -- */

struct V3 {
    float x, y, z;
};
static inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
static inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
static inline V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline float norm(V3 a) { return std::sqrt(dot(a, a)); }
static inline V3 normalized(V3 a)
{
    const float sq = dot(a, a);
    if (sq > 0.0f) {
        const float n = std::sqrt(sq);
        return v3(a.x / n, a.y / n, a.z / n);
    }
    return a;
}
static inline V3 cross(V3 a, V3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline bool is_zero(V3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }

/* Rigid or affine transform, R row-major. */
struct Tf {
    float R[3][3];
    float t[3];
};

static inline V3 rot(const Tf& T, V3 v)
{
    return v3((T.R[0][0] * v.x + T.R[0][1] * v.y) + T.R[0][2] * v.z,
              (T.R[1][0] * v.x + T.R[1][1] * v.y) + T.R[1][2] * v.z,
              (T.R[2][0] * v.x + T.R[2][1] * v.y) + T.R[2][2] * v.z);
}
static inline V3 apply(const Tf& T, V3 v)
{
    const V3 r = rot(T, v);
    return v3(r.x + T.t[0], r.y + T.t[1], r.z + T.t[2]);
}
static inline Tf compose(const Tf& A, const Tf& B)
{
    Tf C;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) {
            C.R[i][j] = (A.R[i][0] * B.R[0][j] + A.R[i][1] * B.R[1][j]) + A.R[i][2] * B.R[2][j];
        }
        C.t[i] = ((A.R[i][0] * B.t[0] + A.R[i][1] * B.t[1]) + A.R[i][2] * B.t[2]) + A.t[i];
    }
    return C;
}
/* Isometry inverse: (R^T, -(R^T t)). */
static inline Tf inverse_iso(const Tf& A)
{
    Tf B;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            B.R[i][j] = A.R[j][i];
    for (int i = 0; i < 3; ++i) {
        B.t[i] = -((B.R[i][0] * A.t[0] + B.R[i][1] * A.t[1]) + B.R[i][2] * A.t[2]);
    }
    return B;
}
static inline Tf tf_from16(const float* m)
{
    Tf T;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            T.R[i][j] = m[4 * i + j];
        T.t[i] = m[4 * i + 3];
    }
    return T;
}
static inline void tf_to16(const Tf& T, float* m)
{
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            m[4 * i + j] = T.R[i][j];
        m[4 * i + 3] = T.t[i];
    }
    m[12] = m[13] = m[14] = 0.0f;
    m[15] = 1.0f;
}
static inline Tf tf_identity()
{
    Tf T;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            T.R[i][j] = (i == j) ? 1.0f : 0.0f;
        T.t[i] = 0.0f;
    }
    return T;
}

/* ------------------------------------------------------------------------ Morton keys -- */
/* include/se/map/utils/key_util.hpp:19-58, impl/key_util_impl.hpp:44-436 */

constexpr uint64_t kCodeMask[] = {
    0x1ffffffffffffffULL, 0x1fffffffffffff8ULL, 0x1ffffffffffffc0ULL, 0x1fffffffffffe00ULL,
    0x1fffffffffff000ULL, 0x1ffffffffff8000ULL, 0x1fffffffffc0000ULL, 0x1ffffffffe00000ULL,
    0x1ffffffff000000ULL, 0x1fffffff8000000ULL, 0x1ffffffc0000000ULL, 0x1fffffe00000000ULL,
    0x1fffff000000000ULL, 0x1ffff8000000000ULL, 0x1fffc0000000000ULL, 0x1ffe00000000000ULL,
    0x1ff000000000000ULL, 0x1f8000000000000ULL, 0x1c0000000000000ULL};
constexpr uint64_t kScaleMask = 0x1f;
constexpr int kScaleOffset = 5;

/* Spread the low 19 bits of value so that bit i lands on bit 3i. */
static inline uint64_t morton_expand(uint64_t v)
{
    uint64_t x = v & 0x7ffff;
    x = (x | x << 32) & 0x1f00000000ffffULL;
    x = (x | x << 16) & 0x1f0000ff0000ffULL;
    x = (x | x << 8) & 0x100f00f00f00f00fULL;
    x = (x | x << 4) & 0x10c30c30c30c30c3ULL;
    x = (x | x << 2) & 0x1249249249249249ULL;
    return x;
}
/* Inverse of morton_expand. */
static inline uint64_t morton_compact(uint64_t v)
{
    uint64_t x = v & 0x49249249249249ULL;
    x = (x | x >> 2) & 0x10c30c30c30c30c3ULL;
    x = (x | x >> 4) & 0x100f00f00f00f00fULL;
    x = (x | x >> 8) & 0x1f0000ff0000ffULL;
    x = (x | x >> 16) & 0x1f00000000ffffULL;
    x = (x | x >> 32) & 0x1fffffULL;
    return x;
}
static inline uint64_t encode_code(int x, int y, int z)
{
    return morton_expand((uint64_t) x) | (morton_expand((uint64_t) y) << 1)
        | (morton_expand((uint64_t) z) << 2);
}
static inline uint64_t encode_key(int x, int y, int z, uint64_t scale)
{
    return ((encode_code(x, y, z) & kCodeMask[scale]) << kScaleOffset) | scale;
}
static inline uint64_t key_to_code(uint64_t key) { return key >> kScaleOffset; }
static inline uint64_t key_to_scale(uint64_t key) { return key & kScaleMask; }
static inline void decode_code(uint64_t code, int c[3])
{
    c[0] = (int) morton_compact(code);
    c[1] = (int) morton_compact(code >> 1);
    c[2] = (int) morton_compact(code >> 2);
}
static inline bool key_at_scale(uint64_t key, uint64_t scale, uint64_t& out)
{
    out = (key & (kCodeMask[scale] << kScaleOffset)) | scale;
    return key_to_scale(key) <= scale;
}
static inline uint64_t block_key_of(uint64_t key, uint64_t max_block_scale)
{
    return key & ((kCodeMask[max_block_scale] << kScaleOffset) | kScaleMask);
}
static inline bool is_child_key(uint64_t parent, uint64_t child)
{
    const uint64_t ps = key_to_scale(parent), cs = key_to_scale(child);
    if (cs >= ps)
        return false;
    return (key_to_code(parent) ^ (key_to_code(child) & kCodeMask[ps])) == 0;
}

/* ------------------------------------------------------------------------- the octree -- */
/* Pointer octree like include/se/map/octree/octree.hpp: nodes own 8 child slots, blocks are
 * 8^3 leaves with std::array<Data, 512>. Octants live in index-addressed vectors. */

constexpr int kBlockSize = 8;
constexpr int kBlockVoxels = 512;
constexpr int kMaxBlockScale = 3;

struct Octant {
    int32_t child[8];
    int32_t coord[3];
    int32_t size;
    int32_t block; /* index into blocks, -1 for nodes */
    int32_t timestamp;
};

struct BlockData {
    float tsdf[kBlockVoxels];
    float weight[kBlockVoxels];
};

/* BlockMultiRes<Data<TSDF>> (block.hpp:66-166, block_impl.hpp:80-202): the 8^3 + 4^3 + 2^3 + 1
 * voxel pyramid of data and of past data (delta down-propagation), the current integration
 * scale and the finest scale ever integrated (-1 before the first update). */
constexpr int kMrVoxels = 585;
constexpr int kMrScaleOffset[4] = {0, 512, 576, 584};
struct MRBlock {
    float tsdf[kMrVoxels];
    float weight[kMrVoxels];
    float past_tsdf[kMrVoxels];
    float past_weight[kMrVoxels];
    int current_scale;
    int min_scale;
};

struct Octree {
    int size = 0;
    std::vector<Octant> octants; /* octants[0] is the root */
    std::vector<BlockData> blocks;
    bool multires = false;
    std::vector<MRBlock> mr; /* multi-res blocks (Octant::block indexes this when multires) */
    std::vector<int32_t> block_octant;
    bool aabb_empty = true;
    int32_t aabb_min[3] = {0, 0, 0};
    int32_t aabb_max[3] = {0, 0, 0};

    void init(int sz)
    {
        size = sz;
        octants.clear();
        blocks.clear();
        mr.clear();
        block_octant.clear();
        Octant root{};
        std::fill(root.child, root.child + 8, -1);
        root.size = sz;
        root.block = -1;
        root.timestamp = -1;
        octants.push_back(root);
        aabb_empty = true;
    }

    void aabb_extend(const int32_t c[3], int sz)
    {
        for (int i = 0; i < 3; ++i) {
            const int lo = c[i], hi = c[i] + sz - 1;
            if (aabb_empty) {
                aabb_min[i] = lo;
                aabb_max[i] = hi;
            }
            else {
                aabb_min[i] = std::min(aabb_min[i], lo);
                aabb_max[i] = std::max(aabb_max[i], hi);
            }
        }
        aabb_empty = false;
    }

    /* Octree::allocate, octree_impl.hpp:171-199 (new octants take the parent's default data). */
    bool allocate(int parent, int child_idx, int& child)
    {
        child = octants[parent].child[child_idx];
        if (child >= 0)
            return false;
        Octant o{};
        std::fill(o.child, o.child + 8, -1);
        const int psize = octants[parent].size;
        const int csize = psize / 2;
        for (int i = 0; i < 3; ++i)
            o.coord[i] = octants[parent].coord[i] + csize * ((child_idx >> i) & 1);
        o.size = csize;
        o.timestamp = -1;
        o.block = -1;
        if (psize == 2 * kBlockSize && multires) {
            o.block = (int32_t) mr.size();
            mr.emplace_back();
            MRBlock& b = mr.back();
            std::fill(b.tsdf, b.tsdf + kMrVoxels, 1.0f);
            std::fill(b.weight, b.weight + kMrVoxels, 0.0f);
            std::fill(b.past_tsdf, b.past_tsdf + kMrVoxels, 1.0f);
            std::fill(b.past_weight, b.past_weight + kMrVoxels, 0.0f);
            b.current_scale = -1;
            b.min_scale = -1;
        }
        else if (psize == 2 * kBlockSize) {
            o.block = (int32_t) blocks.size();
            blocks.emplace_back();
            BlockData& b = blocks.back();
            std::fill(b.tsdf, b.tsdf + kBlockVoxels, 1.0f);
            std::fill(b.weight, b.weight + kBlockVoxels, 0.0f);
        }
        child = (int) octants.size();
        octants.push_back(o);
        if (o.block >= 0) {
            block_octant.push_back(child);
            aabb_extend(o.coord, csize);
        }
        octants[parent].child[child_idx] = child;
        return true;
    }

    /* allocator::detail::allocate_key, allocator_impl.hpp:124-147 */
    bool allocate_key(uint64_t key, int& out)
    {
        int parent = 0;
        int child = -1;
        int child_scale = (int) std::log2(octants[0].size) - 1;
        const uint64_t code = key_to_code(key);
        const int min_scale = std::max((int) key_to_scale(key), kMaxBlockScale);
        bool did = false;
        for (; child_scale >= min_scale; --child_scale) {
            const int idx = (int) ((code >> (child_scale * 3)) & 7);
            did = allocate(parent, idx, child);
            parent = child;
        }
        out = child;
        return did;
    }

    /* fetcher::block, fetcher_impl.hpp:107-126 */
    int block_at(const int32_t c[3]) const
    {
        int parent = 0;
        int child = -1;
        for (int cs = size >> 1; cs >= kBlockSize; cs >>= 1) {
            const int idx = ((c[0] & cs) > 0) + 2 * ((c[1] & cs) > 0) + 4 * ((c[2] & cs) > 0);
            child = octants[parent].child[idx];
            if (child < 0)
                return -1;
            parent = child;
        }
        return child;
    }
};

/* ------------------------------------------------------------------------------ sensor -- */

struct Pinhole {
    int w, h;
    float fx, fy, cx, cy;
    float inv_fx, inv_fy;
    float near_plane, far_plane;
    bool left_hand;
    float normals[6][4]; /* frustum planes: left, right, bottom, top, near, far */
};

static inline V3 back_project(const Pinhole& s, float u, float v)
{
    return v3((u - s.cx) * s.inv_fx, (v - s.cy) * s.inv_fy, 1.0f);
}

static inline bool project(const Pinhole& s, V3 p, float& u, float& v)
{
    if (std::fabs(p.z) < 1.0e-12f)
        return false;
    const float rz = 1.0f / p.z;
    u = s.fx * (p.x * rz) + s.cx;
    v = s.fy * (p.y * rz) + s.cy;
    if (!(u >= -0.5f && u < (float) s.w - 0.5f && v >= -0.5f && v < (float) s.h - 0.5f))
        return false;
    return p.z > 0.0f;
}

/* se::math::plane_normal, math_util_impl.hpp:88-101 */
static inline V3 plane_normal(V3 p1, V3 p2, V3 p3)
{
    return normalized(cross(p2 - p1, p3 - p2));
}

/* PinholeCamera ctor + computeFrustumVertices/Normals, pinhole_camera.cpp:63-84,246-310 */
static Pinhole make_pinhole(int w, int h, float fx, float fy, float cx, float cy, float near_p,
                            float far_p)
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
    const V3 tl = back_project(s, 0.0f, 0.0f);
    const V3 tr = back_project(s, (float) w, 0.0f);
    const V3 br = back_project(s, (float) w, (float) h);
    const V3 bl = back_project(s, 0.0f, (float) h);
    const V3 tl_n = near_p * tl, tl_f = far_p * tl, tr_n = near_p * tr, tr_f = far_p * tr;
    const V3 br_n = near_p * br, br_f = far_p * br, bl_n = near_p * bl, bl_f = far_p * bl;
    const V3 n_left = plane_normal(tl_f, tl_n, bl_n);
    const V3 n_right = plane_normal(tr_n, tr_f, br_f);
    const V3 n_bottom = plane_normal(bl_f, bl_n, br_n);
    const V3 n_top = plane_normal(tr_f, tr_n, tl_n);
    const V3 ns[4] = {n_left, n_right, n_bottom, n_top};
    float sign = fx * fy;
    sign = sign / std::fabs(sign);
    for (int i = 0; i < 4; ++i) {
        s.normals[i][0] = ns[i].x * sign;
        s.normals[i][1] = ns[i].y * sign;
        s.normals[i][2] = ns[i].z * sign;
        s.normals[i][3] = 0.0f;
    }
    s.normals[4][0] = 0.0f;
    s.normals[4][1] = 0.0f;
    s.normals[4][2] = 1.0f;
    s.normals[4][3] = -near_p;
    s.normals[5][0] = 0.0f;
    s.normals[5][1] = 0.0f;
    s.normals[5][2] = -1.0f;
    s.normals[5][3] = far_p;
    return s;
}

static Pinhole make_pinhole(const so_pinhole* p)
{
    return make_pinhole(
        p->width, p->height, p->fx, p->fy, p->cx, p->cy, p->near_plane, p->far_plane);
}

/* PinholeCamera(const PinholeCamera&, dsf), pinhole_camera.cpp:95-111 */
static Pinhole downsampled(const Pinhole& s, float dsf)
{
    return make_pinhole((int) ((float) s.w / dsf),
                        (int) ((float) s.h / dsf),
                        s.fx / dsf,
                        s.fy / dsf,
                        (s.cx + 0.5f) / dsf - 0.5f,
                        (s.cy + 0.5f) / dsf - 0.5f,
                        s.near_plane,
                        s.far_plane);
}

/* sphereInFrustumImpl, pinhole_camera.cpp:189-204: distance = ((x*nx + y*ny) + z*nz) + nw */
static inline bool sphere_in_frustum(const Pinhole& s, V3 c, float radius)
{
    for (int i = 0; i < 6; ++i) {
        const float d =
            ((c.x * s.normals[i][0] + c.y * s.normals[i][1]) + c.z * s.normals[i][2])
            + s.normals[i][3];
        if (d < -radius)
            return false;
    }
    return true;
}

/* nearDistImpl / farDistImpl, pinhole_camera_impl.hpp:15-25 */
static inline float near_dist(const Pinhole& s, V3 ray) { return s.near_plane / normalized(ray).z; }
static inline float far_dist(const Pinhole& s, V3 ray) { return s.far_plane / normalized(ray).z; }

static inline void round_pixel(float u, float v, int& x, int& y)
{
    x = (int) (u + 0.5f);
    y = (int) (v + 0.5f);
}

/* e^x for x <= 0 in float operations only: Cody & Waite (1980) argument reduction
 * x = n ln2 + r with ln2 split into a 12-bit-short head and a tail, the degree-7 Taylor
 * polynomial of e^r (|r| <= ln2/2, relative error < 3e-8) by Horner's rule in fused
 * multiply-adds, then 2^n exactly. The GPU build evaluates the same operations (IEEE fused
 * multiply-add is exactly specified), so both round identically. */
static inline float exp_cw(float x)
{
    if (x < -87.0f)
        return 0.0f;
    const float n = std::rint(x * 1.44269504f);
    const float r = std::fmaf(-n, 1.42860677e-06f, std::fmaf(-n, 0.693145751953125f, x));
    float p = 0.000198412701f;
    p = std::fmaf(p, r, 0.00138888892f);
    p = std::fmaf(p, r, 0.00833333377f);
    p = std::fmaf(p, r, 0.0416666679f);
    p = std::fmaf(p, r, 0.166666672f);
    p = std::fmaf(p, r, 0.5f);
    p = std::fmaf(p, r, 1.0f);
    p = std::fmaf(p, r, 1.0f);
    return std::ldexp(p, (int) n);
}

/* The project-defined bilateral pre-filter of the tracking input (the reference has none):
 * invalid (<= 0 or NaN) centres stay 0; valid taps of the (2r+1)^2 window inside the image are
 * weighted by ws[dy][dx] (spatial Gaussian, host-computed) times exp_cw(-(d - c)^2 k) with
 * k = 1 / (2 sigma_r^2); the sums run dy outer, dx inner, the numerator by fused multiply-adds. */
static inline float bilateral_pixel(const float* in, int w, int h, int x, int y, int radius, const float* ws, float k)
{
    const float c = in[x + y * w];
    if (!(c > 0.0f))
        return 0.0f;
    float num = 0.0f, den = 0.0f;
    const int n = 2 * radius + 1;
    for (int dy = -radius; dy <= radius; ++dy) {
        const int yy = y + dy;
        if (yy < 0 || yy >= h)
            continue;
        for (int dx = -radius; dx <= radius; ++dx) {
            const int xx = x + dx;
            if (xx < 0 || xx >= w)
                continue;
            const float d = in[xx + yy * w];
            if (!(d > 0.0f))
                continue;
            const float diff = d - c;
            const float wgt = ws[(dy + radius) * n + (dx + radius)] * exp_cw(-(diff * diff) * k);
            num = std::fmaf(wgt, d, num);
            den = den + wgt;
        }
    }
    return num / den;
}

} // namespace
