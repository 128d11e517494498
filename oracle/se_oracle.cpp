/*
 * se_oracle.cpp — CPU oracle for the supereight2 dense-mapping hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker the GPU product is compared against and the timed CPU
 * baseline. It is never linked into or called by the product library.
 *
 * It restates the reference algorithms (cited per function, paths relative to the supereight2
 * source tree) with the same loop structure and the same float arithmetic. Where the reference's
 * float operation order is decided by Eigen expression templates (unavailable here), this file
 * fixes one order and the GPU kernels use the same one:
 *   dot3(a, b)      = (a0*b0 + a1*b1) + a2*b2
 *   (M*v)_i         = (M_i0*v0 + M_i1*v1) + M_i2*v2
 *   (T*p)_i         = ((R_i0*p0 + R_i1*p1) + R_i2*p2) + t_i
 *   norm(v)         = sqrtf(dot3(v, v));  normalized(v) = v / norm(v) component-wise
 *   compose(A, B)   = (R_A*R_B, R_A*t_B + t_A)
 * Build with -ffp-contract=off so that no multiply-add is fused.
 *
 * Pinhole projection lives in the un-vendored srl_projection module. The convention used here
 * (and in the GPU kernels) is the okvis-style pinhole model: rz = 1/z, u = fx*(x*rz) + cx,
 * v = fy*(y*rz) + cy, Successful iff z > 0 and (u, v) in [-0.5, w-0.5) x [-0.5, h-0.5), so that
 * round_pixel() always lands inside the image. backProject(u, v) = ((u-cx)*(1/fx),
 * (v-cy)*(1/fy), 1).
 */
#include "se_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <set>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_common.hpp"
#include "oracle_dual_mc.hpp"


/* --------------------------------------------------------------------------------- map -- */

struct so_map {
    Octree octree;
    float res;
    float dim; /* octree size * res */
    Tf T_MW;
    Tf T_WM;
    float trunc_factor;
    float max_weight;

    /* Map::contains + pointToVoxel<Safe::On>, map_impl.hpp:58-64,538-550 */
    bool point_to_voxel(V3 p_W, int32_t v[3]) const
    {
        const V3 p_M = apply(T_MW, p_W);
        if (!(p_M.x >= 0.0f && p_M.x < dim && p_M.y >= 0.0f && p_M.y < dim && p_M.z >= 0.0f
              && p_M.z < dim)) {
            v[0] = v[1] = v[2] = -1;
            return false;
        }
        v[0] = (int) (p_M.x / res);
        v[1] = (int) (p_M.y / res);
        v[2] = (int) (p_M.z / res);
        return true;
    }
    bool point_to_voxel_f(V3 p_W, V3& v) const
    {
        const V3 p_M = apply(T_MW, p_W);
        if (!(p_M.x >= 0.0f && p_M.x < dim && p_M.y >= 0.0f && p_M.y < dim && p_M.z >= 0.0f
              && p_M.z < dim)) {
            v = v3(-1.0f, -1.0f, -1.0f);
            return false;
        }
        v = p_M / res;
        return true;
    }
    /* voxelToPoint(coord, stride), map_impl.hpp:503-509 */
    V3 voxel_to_point(const int32_t c[3], int stride) const
    {
        const float off = (float) stride * 0.5f;
        const V3 p_M =
            v3(((float) c[0] + off) * res, ((float) c[1] + off) * res, ((float) c[2] + off) * res);
        return apply(T_WM, p_M);
    }
};

namespace {

/* Measurement hook: when set (per thread), every single-res voxel read below appends the voxel's
 * linear index, so that so_raycast_touched can count the distinct voxels a raycast reads. */
static thread_local std::vector<uint64_t>* g_touched = nullptr;

static inline void touch_voxel(const so_map& m, const int32_t c[3])
{
    if (g_touched) {
        const uint64_t n = (uint64_t) m.octree.size;
        g_touched->push_back((uint64_t) c[0] + n * ((uint64_t) c[1] + n * (uint64_t) c[2]));
    }
}

/* visitor::getData (single-res), visitor_impl.hpp:704-717: block voxel or the default data. */
static inline bool get_voxel(const so_map& m, const int32_t c[3], float& tsdf, float& weight)
{
    touch_voxel(m, c);
    const int o = m.octree.block_at(c);
    if (o < 0) {
        tsdf = 1.0f;
        weight = 0.0f;
        return false;
    }
    const Octant& oc = m.octree.octants[o];
    const BlockData& b = m.octree.blocks[oc.block];
    const int idx = (c[0] - oc.coord[0]) + 8 * (c[1] - oc.coord[1]) + 64 * (c[2] - oc.coord[2]);
    tsdf = b.tsdf[idx];
    weight = b.weight[idx];
    return true;
}

/* visitor::getData(octree, block_ptr, coord), visitor_impl.hpp:718-735 */
static inline void get_voxel_hint(const so_map& m, int hint_octant, const int32_t c[3],
                                  float& tsdf, float& weight)
{
    const Octant& oc = m.octree.octants[hint_octant];
    if (c[0] >= oc.coord[0] && c[0] <= oc.coord[0] + 7 && c[1] >= oc.coord[1]
        && c[1] <= oc.coord[1] + 7 && c[2] >= oc.coord[2] && c[2] <= oc.coord[2] + 7) {
        const BlockData& b = m.octree.blocks[oc.block];
        const int idx =
            (c[0] - oc.coord[0]) + 8 * (c[1] - oc.coord[1]) + 64 * (c[2] - oc.coord[2]);
        touch_voxel(m, c);
        tsdf = b.tsdf[idx];
        weight = b.weight[idx];
        return;
    }
    get_voxel(m, c, tsdf, weight);
}

/* visitor::getInterp single-res, visitor_impl.hpp:976-1024 (with get_neighbours :67-302: the
 * neighbour gather fails if any of the up to 8 blocks touched is unallocated). */
static bool field_interp_voxel(const so_map& m, V3 vf, float& out)
{
    const V3 bf = v3(vf.x - 0.5f, vf.y - 0.5f, vf.z - 0.5f);
    const int32_t base[3] = {(int) bf.x, (int) bf.y, (int) bf.z};
    const Octree& o = m.octree;
    if (o.aabb_empty)
        return false;
    for (int i = 0; i < 3; ++i)
        if (base[i] < o.aabb_min[i] || base[i] > o.aabb_max[i])
            return false;
    for (int i = 0; i < 3; ++i)
        if (base[i] + 1 >= o.size || base[i] < 0)
            return false;
    /* every crossmask case of get_neighbours fetches the block of base first, then the other
     * blocks touched; any unallocated block, then any invalid voxel, gives nullopt */
    float f[8], wt[8];
    for (int n = 0; n < 8; ++n) {
        const int32_t c[3] = {base[0] + (n & 1), base[1] + ((n >> 1) & 1), base[2] + ((n >> 2) & 1)};
        if (!get_voxel(m, c, f[n], wt[n]))
            return false;
    }
    for (int n = 0; n < 8; ++n)
        if (!(wt[n] != 0.0f))
            return false;
    const V3 t = v3(bf.x - std::floor(bf.x), bf.y - std::floor(bf.y), bf.z - std::floor(bf.z));
    const V3 tc = v3(1.0f - t.x, 1.0f - t.y, 1.0f - t.z);
    out = ((f[0] * tc.x + f[1] * t.x) * tc.y + (f[2] * tc.x + f[3] * t.x) * t.y) * tc.z
        + ((f[4] * tc.x + f[5] * t.x) * tc.y + (f[6] * tc.x + f[7] * t.x) * t.y) * t.z;
    return true;
}

/* visitor::getFieldGrad single-res, visitor_impl.hpp:1094-1251 */
static bool field_grad_voxel(const so_map& m, V3 vf, V3& g)
{
    const V3 s = v3(vf.x - 0.5f, vf.y - 0.5f, vf.z - 0.5f);
    const V3 fac = v3(s.x - std::floor(s.x), s.y - std::floor(s.y), s.z - std::floor(s.z));
    const int32_t base[3] = {(int) s.x, (int) s.y, (int) s.z};
    const int top = m.octree.size - 1;
    int32_t ll[3], lu[3], ul[3], uu[3];
    for (int i = 0; i < 3; ++i) {
        ll[i] = std::max(base[i] - 1, 0);
        lu[i] = std::max(base[i], 0);
        ul[i] = std::min(base[i] + 1, top);
        uu[i] = std::min(base[i] + 2, top);
    }
    const int hint = m.octree.block_at(base);
    if (hint < 0)
        return false;
    /* the 32 sample coordinates, in the reference's order */
    const int32_t* X[32] = {ll, ll, ll, ll, lu, lu, lu, lu, lu, lu, lu, lu, lu, lu, lu, lu,
                            ul, ul, ul, ul, ul, ul, ul, ul, ul, ul, ul, ul, uu, uu, uu, uu};
    const int32_t* Y[32] = {lu, ul, lu, ul, ll, ll, lu, lu, lu, lu, ul, ul, ul, ul, uu, uu,
                            ll, ll, lu, lu, lu, lu, ul, ul, ul, ul, uu, uu, lu, ul, lu, ul};
    const int32_t* Z[32] = {lu, lu, ul, ul, lu, ul, ll, lu, ul, uu, ll, lu, ul, uu, lu, ul,
                            lu, ul, ll, lu, ul, uu, ll, lu, ul, uu, lu, ul, lu, lu, ul, ul};
    float v[32];
    for (int i = 0; i < 32; ++i) {
        const int32_t c[3] = {X[i][0], Y[i][1], Z[i][2]};
        float t, w;
        get_voxel_hint(m, hint, c, t, w);
        if (!(w != 0.0f))
            return false;
        v[i] = t;
    }
    const float rx = 1.0f - fac.x, ry = 1.0f - fac.y, rz = 1.0f - fac.z;
    const float gx = (((v[19] - v[0]) * rx + (v[28] - v[7]) * fac.x) * ry
                      + ((v[23] - v[1]) * rx + (v[29] - v[11]) * fac.x) * fac.y)
            * rz
        + (((v[20] - v[2]) * rx + (v[30] - v[8]) * fac.x) * ry
           + ((v[24] - v[3]) * rx + (v[31] - v[12]) * fac.x) * fac.y)
            * fac.z;
    const float gy = (((v[11] - v[4]) * rx + (v[23] - v[16]) * fac.x) * ry
                      + ((v[14] - v[7]) * rx + (v[26] - v[19]) * fac.x) * fac.y)
            * rz
        + (((v[12] - v[5]) * rx + (v[24] - v[17]) * fac.x) * ry
           + ((v[15] - v[8]) * rx + (v[27] - v[20]) * fac.x) * fac.y)
            * fac.z;
    const float gz = (((v[8] - v[6]) * rx + (v[20] - v[18]) * fac.x) * ry
                      + ((v[12] - v[10]) * rx + (v[24] - v[22]) * fac.x) * fac.y)
            * rz
        + (((v[9] - v[7]) * rx + (v[21] - v[19]) * fac.x) * ry
           + ((v[13] - v[11]) * rx + (v[25] - v[23]) * fac.x) * fac.y)
            * fac.z;
    g = v3(0.5f * gx, 0.5f * gy, 0.5f * gz);
    return true;
}

static bool map_field_interp(const so_map& m, V3 p_W, float& out)
{
    V3 vf;
    if (!m.point_to_voxel_f(p_W, vf))
        return false;
    return field_interp_voxel(m, vf, out);
}

/* Map::getFieldGrad, map_impl.hpp:236-262 */
static bool map_field_grad(const so_map& m, V3 p_W, V3& g)
{
    V3 vf;
    if (!m.point_to_voxel_f(p_W, vf))
        return false;
    if (!field_grad_voxel(m, vf, g))
        return false;
    g = g / m.res;
    return true;
}

/* Map::getData<Safe::On>, map_impl.hpp:68-86 */
static inline void map_get_data(const so_map& m, V3 p_W, float& tsdf, float& weight)
{
    int32_t c[3];
    if (!m.point_to_voxel(p_W, c)) {
        tsdf = 1.0f;
        weight = 0.0f;
        return;
    }
    get_voxel(m, c, tsdf, weight);
}

/* ---------------------------------------------------------- multi-res TSDF access -- */

/* BlockMultiRes::getVoxelIdx, block_impl.hpp:80-91 */
static inline int mr_index(const Octant& oc, const int32_t c[3], int scale)
{
    const int n = kBlockSize >> scale;
    return kMrScaleOffset[scale] + ((c[0] - oc.coord[0]) >> scale) + n * ((c[1] - oc.coord[1]) >> scale)
        + n * n * ((c[2] - oc.coord[2]) >> scale);
}

/* The current scale of a block as a data index. A block is updated in the frame that allocates
 * it, so -1 (never integrated) is only seen by queries between allocation and update, for
 * which the reference's index is undefined; scale 0 is used. */
static inline int mr_cur(const MRBlock& b) { return b.current_scale < 0 ? 0 : b.current_scale; }

static inline V3 fracf(V3 v) { return v3(v.x - std::floor(v.x), v.y - std::floor(v.y), v.z - std::floor(v.z)); }

/* visitor::getData multi-res: the block's data at its current scale (visitor_impl.hpp:704-717,
 * block_impl.hpp:117-133). */
static inline bool mr_get_voxel(const so_map& m, const int32_t c[3], float& tsdf, float& weight)
{
    const int o = m.octree.block_at(c);
    if (o < 0) {
        tsdf = 1.0f;
        weight = 0.0f;
        return false;
    }
    const Octant& oc = m.octree.octants[o];
    const MRBlock& b = m.octree.mr[oc.block];
    const int i = mr_index(oc, c, mr_cur(b));
    tsdf = b.tsdf[i];
    weight = b.weight[i];
    return true;
}

/* visitor::getData(octree, block_ptr, coord, scale_desired, scale_returned) multi-res
 * (visitor_impl.hpp:740-790): data at max(scale_desired, current_scale) of the block holding
 * the voxel (the hint block first); returns false when no block holds it. */
static inline bool mr_get_voxel_at(const so_map& m, int hint_octant, const int32_t c[3], int scale_desired,
                                   float& tsdf, float& weight, int& scale_returned)
{
    int o = hint_octant;
    const Octant* oc = &m.octree.octants[o];
    if (!(c[0] >= oc->coord[0] && c[0] <= oc->coord[0] + 7 && c[1] >= oc->coord[1] && c[1] <= oc->coord[1] + 7
          && c[2] >= oc->coord[2] && c[2] <= oc->coord[2] + 7)) {
        o = m.octree.block_at(c);
        if (o < 0) {
            tsdf = 1.0f;
            weight = 0.0f;
            return false;
        }
        oc = &m.octree.octants[o];
    }
    const MRBlock& b = m.octree.mr[oc->block];
    scale_returned = std::max(scale_desired, b.current_scale);
    const int i = mr_index(*oc, c, scale_returned < 0 ? 0 : scale_returned);
    tsdf = b.tsdf[i];
    weight = b.weight[i];
    return true;
}

/* visitor::getInterp multi-res (visitor_impl.hpp:906-972) with detail::get_neighbours
 * (:398-697). Starting at max(current scale of the query's block, desired scale), a scale is
 * skipped when one of the up to 8 blocks its neighbourhood touches is unallocated or integrates
 * at a coarser scale; an invalid neighbour ends the query. */
static bool mr_interp_voxel(const so_map& m, V3 vf, int desired_scale, float& out, int* returned_scale)
{
    const Octree& o = m.octree;
    const int32_t c0[3] = {(int) vf.x, (int) vf.y, (int) vf.z};
    const int oq = o.block_at(c0);
    if (oq < 0)
        return false;
    const int init = std::max(o.mr[o.octants[oq].block].current_scale, desired_scale);
    for (int scale = init; scale <= kMaxBlockScale; ++scale) {
        const int stride = 1 << scale;
        const float inv = 1.0f / (float) stride;
        const V3 bf = v3(inv * vf.x - 0.5f, inv * vf.y - 0.5f, inv * vf.z - 0.5f);
        const int32_t base[3] = {stride * (int) bf.x, stride * (int) bf.y, stride * (int) bf.z};
        if (o.aabb_empty)
            return false;
        for (int i = 0; i < 3; ++i)
            if (base[i] < o.aabb_min[i] || base[i] > o.aabb_max[i])
                return false;
        bool ok = true;
        for (int i = 0; i < 3; ++i)
            if (base[i] + stride >= o.size || base[i] < 0)
                ok = false;
        float f[8], w[8];
        for (int n = 0; ok && n < 8; ++n) {
            const int32_t c[3] = {base[0] + stride * (n & 1), base[1] + stride * ((n >> 1) & 1),
                                  base[2] + stride * ((n >> 2) & 1)};
            const int ob = o.block_at(c);
            if (ob < 0) {
                ok = false;
                break;
            }
            const Octant& oc = o.octants[ob];
            const MRBlock& b = o.mr[oc.block];
            if (b.current_scale > scale) {
                ok = false;
                break;
            }
            const int i = mr_index(oc, c, scale);
            f[n] = b.tsdf[i];
            w[n] = b.weight[i];
        }
        if (!ok)
            continue;
        for (int n = 0; n < 8; ++n)
            if (!(w[n] != 0.0f))
                return false;
        if (returned_scale)
            *returned_scale = scale;
        const V3 t = fracf(bf);
        const V3 tc = v3(1.0f - t.x, 1.0f - t.y, 1.0f - t.z);
        out = ((f[0] * tc.x + f[1] * t.x) * tc.y + (f[2] * tc.x + f[3] * t.x) * t.y) * tc.z
            + ((f[4] * tc.x + f[5] * t.x) * tc.y + (f[6] * tc.x + f[7] * t.x) * t.y) * t.z;
        return true;
    }
    return false;
}

/* visitor::getFieldGrad multi-res (visitor_impl.hpp:1257-1497), desired scale 0: the 32-sample
 * central-difference gradient at the first scale (from the block's current one up) whose 32
 * samples are all valid and stored at exactly that scale. */
static bool mr_grad_voxel(const so_map& m, V3 vf, V3& g, int& scale_returned)
{
    const Octree& o = m.octree;
    const int32_t c0[3] = {(int) vf.x, (int) vf.y, (int) vf.z};
    const int oq = o.block_at(c0);
    if (oq < 0)
        return false;
    const int init = std::max(0, o.mr[o.octants[oq].block].current_scale);
    const int top = o.size - 1;
    for (int scale = init; scale <= kMaxBlockScale; ++scale) {
        scale_returned = scale;
        const int stride = 1 << scale;
        const float inv = 1.0f / (float) stride;
        const V3 sv = v3(inv * vf.x - 0.5f, inv * vf.y - 0.5f, inv * vf.z - 0.5f);
        const V3 fac = fracf(sv);
        const int32_t base[3] = {stride * (int) sv.x, stride * (int) sv.y, stride * (int) sv.z};
        int32_t ll[3], lu[3], ul[3], uu[3];
        for (int i = 0; i < 3; ++i) {
            ll[i] = std::max(base[i] - stride, 0);
            lu[i] = std::max(base[i], 0);
            ul[i] = std::min(base[i] + stride, top);
            uu[i] = std::min(base[i] + 2 * stride, top);
        }
        /* finest_octant(base, scale): a TSDF node holds no data, so only a block continues */
        const int hint = o.block_at(base);
        if (hint < 0)
            continue;
        const int32_t* X[32] = {ll, ll, ll, ll, lu, lu, lu, lu, lu, lu, lu, lu, lu, lu, lu, lu,
                                ul, ul, ul, ul, ul, ul, ul, ul, ul, ul, ul, ul, uu, uu, uu, uu};
        const int32_t* Y[32] = {lu, ul, lu, ul, ll, ll, lu, lu, lu, lu, ul, ul, ul, ul, uu, uu,
                                ll, ll, lu, lu, lu, lu, ul, ul, ul, ul, uu, uu, lu, ul, lu, ul};
        const int32_t* Z[32] = {lu, lu, ul, ul, lu, ul, ll, lu, ul, uu, ll, lu, ul, uu, lu, ul,
                                lu, ul, ll, lu, ul, uu, ll, lu, ul, uu, lu, ul, lu, lu, ul, ul};
        float v[32];
        bool ok = true;
        for (int i = 0; i < 32 && ok; ++i) {
            const int32_t c[3] = {X[i][0], Y[i][1], Z[i][2]};
            float t, w;
            int rs = -1;
            if (!mr_get_voxel_at(m, hint, c, scale, t, w, rs) || !(w != 0.0f) || rs != scale)
                ok = false;
            v[i] = t;
        }
        if (!ok)
            continue;
        const float rx = 1.0f - fac.x, ry = 1.0f - fac.y, rz = 1.0f - fac.z;
        const float gx = (((v[19] - v[0]) * rx + (v[28] - v[7]) * fac.x) * ry
                          + ((v[23] - v[1]) * rx + (v[29] - v[11]) * fac.x) * fac.y)
                * rz
            + (((v[20] - v[2]) * rx + (v[30] - v[8]) * fac.x) * ry
               + ((v[24] - v[3]) * rx + (v[31] - v[12]) * fac.x) * fac.y)
                * fac.z;
        const float gy = (((v[11] - v[4]) * rx + (v[23] - v[16]) * fac.x) * ry
                          + ((v[14] - v[7]) * rx + (v[26] - v[19]) * fac.x) * fac.y)
                * rz
            + (((v[12] - v[5]) * rx + (v[24] - v[17]) * fac.x) * ry
               + ((v[15] - v[8]) * rx + (v[27] - v[20]) * fac.x) * fac.y)
                * fac.z;
        const float gz = (((v[8] - v[6]) * rx + (v[20] - v[18]) * fac.x) * ry
                          + ((v[12] - v[10]) * rx + (v[24] - v[22]) * fac.x) * fac.y)
                * rz
            + (((v[9] - v[7]) * rx + (v[21] - v[19]) * fac.x) * ry
               + ((v[13] - v[11]) * rx + (v[25] - v[23]) * fac.x) * fac.y)
                * fac.z;
        const float sf = (float) stride;
        g = v3((0.5f * gx) / sf, (0.5f * gy) / sf, (0.5f * gz) / sf);
        return true;
    }
    return false;
}

static bool map_field_interp_mr(const so_map& m, V3 p_W, float& out, int* returned_scale)
{
    V3 vf;
    if (!m.point_to_voxel_f(p_W, vf))
        return false;
    return mr_interp_voxel(m, vf, 0, out, returned_scale);
}

static bool map_field_grad_mr(const so_map& m, V3 p_W, V3& g)
{
    V3 vf;
    if (!m.point_to_voxel_f(p_W, vf))
        return false;
    int sr;
    if (!mr_grad_voxel(m, vf, g, sr))
        return false;
    g = g / m.res;
    return true;
}

static inline void map_get_data_mr(const so_map& m, V3 p_W, float& tsdf, float& weight)
{
    int32_t c[3];
    if (!m.point_to_voxel(p_W, c)) {
        tsdf = 1.0f;
        weight = 0.0f;
        return;
    }
    mr_get_voxel(m, c, tsdf, weight);
}

/* ------------------------------------------------------- VoxelBlockRayIterator (ESVO) -- */
/* voxel_block_ray_iterator_impl.hpp:19-249: Laine & Karras sparse-voxel-octree traversal in the
 * [1, 2]^3 scaled frame, mirrored so that every direction component is negative. Returns the
 * state after the first next(): whether a block was found, tcmin() and tmax(). */

/* The traversal's bit manipulations act on IEEE binary32 values (SO_BITS_FLOAT is float in
 * every build, also the FP64 one). */
static inline int32_t f_as_i(float f)
{
    const SO_BITS_FLOAT g = (SO_BITS_FLOAT) f;
    int32_t i;
    std::memcpy(&i, &g, 4);
    return i;
}
static inline float i_as_f(int32_t i)
{
    SO_BITS_FLOAT g;
    std::memcpy(&g, &i, 4);
    return (float) g;
}

struct RayBlockHit {
    bool found;
    float tcmin; /* metres */
    float tmax;  /* metres */
};

static RayBlockHit first_block_on_ray(const so_map& m, V3 origin_W, V3 dir_W, float near_p,
                                      float far_p)
{
    constexpr int kStackDepth = 23;
    const Octree& oct = m.octree;
    const float scaling = (float) oct.size * m.res;
    const int min_scale = kStackDepth - (int) std::log2((double) (oct.size / kBlockSize));
    const float eps = std::exp2((float) (-std::log2((double) oct.size)));

    float d[3] = {dir_W.x, dir_W.y, dir_W.z};
    for (int a = 0; a < 3; ++a)
        if (std::fabs(d[a]) < eps)
            d[a] = std::copysign(eps, d[a]);

    /* pointToVoxel<Safe::Off> (float), then scale into [1, 2] */
    const V3 o_M = apply(m.T_MW, origin_W);
    const float o_v[3] = {o_M.x / m.res, o_M.y / m.res, o_M.z / m.res};
    float o[3];
    for (int a = 0; a < 3; ++a)
        o[a] = o_v[a] / (float) oct.size + 1.0f;

    float t_coef[3], t_bias[3];
    for (int a = 0; a < 3; ++a) {
        t_coef[a] = -1.0f * (1.0f / std::fabs(d[a]));
        t_bias[a] = t_coef[a] * o[a];
    }
    int mirror_mask = 7;
    for (int a = 0; a < 3; ++a) {
        if (d[a] > 0.0f) {
            mirror_mask ^= (1 << a);
            t_bias[a] = 3.0f * t_coef[a] - t_bias[a];
        }
    }
    float t_min = std::max(std::max(2.0f * t_coef[0] - t_bias[0], 2.0f * t_coef[1] - t_bias[1]),
                           2.0f * t_coef[2] - t_bias[2]);
    float t_max = std::min(std::min(t_coef[0] - t_bias[0], t_coef[1] - t_bias[1]),
                           t_coef[2] - t_bias[2]);
    float h = t_max;
    t_min = std::max(t_min, near_p / scaling);
    t_max = std::min(t_max, far_p / scaling);
    const float t_max_init = t_max;

    int idx = 0;
    float pos[3] = {1.0f, 1.0f, 1.0f};
    for (int a = 0; a < 3; ++a) {
        if (1.5f * t_coef[a] - t_bias[a] > t_min) {
            idx ^= (1 << a);
            pos[a] = 1.5f;
        }
    }
    int parent = 0;
    int scale = kStackDepth - 1;
    float scale_exp2 = 0.5f;
    struct Entry {
        int parent;
        float t_max;
    } stack[kStackDepth];
    for (int i = 0; i < kStackDepth; ++i)
        stack[i] = Entry{-1, 0.0f};

    while (scale < kStackDepth) {
        float tc[3];
        for (int a = 0; a < 3; ++a)
            tc[a] = pos[a] * t_coef[a] - t_bias[a];
        const float tc_max = std::min(std::min(tc[0], tc[1]), tc[2]);
        const int child = (parent >= 0) ? oct.octants[parent].child[idx ^ mirror_mask ^ 7] : -1;

        if (scale == min_scale && child >= 0) {
            return RayBlockHit{true, t_min * scaling, t_max_init * scaling};
        }
        if (child >= 0 && t_min <= t_max) {
            /* descend */
            const float tv_max = std::min(t_max, tc_max);
            const float half = scale_exp2 * 0.5f;
            float t_centre[3];
            for (int a = 0; a < 3; ++a)
                t_centre[a] = half * t_coef[a] + tc[a];
            if (tc_max < h)
                stack[scale] = Entry{parent, t_max};
            h = tc_max;
            parent = child;
            idx = 0;
            --scale;
            scale_exp2 = half;
            for (int a = 0; a < 3; ++a)
                if (t_centre[a] > t_min)
                    idx ^= (1 << a);
            for (int a = 0; a < 3; ++a)
                if (idx & (1 << a))
                    pos[a] += scale_exp2;
            t_max = tv_max;
            continue;
        }
        /* advance */
        int step_mask = 0;
        for (int a = 0; a < 3; ++a)
            if (tc[a] <= tc_max)
                step_mask |= (1 << a);
        for (int a = 0; a < 3; ++a)
            if (step_mask & (1 << a))
                pos[a] -= scale_exp2;
        t_min = tc_max;
        idx ^= step_mask;
        if ((idx & step_mask) != 0) {
            /* pop to the level where the position bits first differ */
            uint32_t differing = 0;
            for (int a = 0; a < 3; ++a)
                if (step_mask & (1 << a))
                    differing |= (uint32_t) (f_as_i(pos[a]) ^ f_as_i(pos[a] + scale_exp2));
            scale = (f_as_i((float) differing) >> 23) - 127;
            if (scale >= kStackDepth)
                break;
            scale_exp2 = i_as_f((scale - kStackDepth + 127) << 23);
            parent = stack[scale].parent;
            t_max = stack[scale].t_max;
            int sh[3];
            for (int a = 0; a < 3; ++a) {
                sh[a] = f_as_i(pos[a]) >> scale;
                pos[a] = i_as_f(sh[a] << scale);
            }
            idx = (sh[0] & 1) | ((sh[1] & 1) << 1) | ((sh[2] & 1) << 2);
            h = 0.0f;
        }
    }
    return RayBlockHit{false, t_min * scaling, t_max_init * scaling};
}

/* raycast<TSDF>, raycaster_impl.hpp:456-533. Returns true on a hit with point_W and scale. */
static bool raycast_tsdf(const so_map& m, V3 origin_W, V3 dir_W, float t_near, float t_far,
                         V3& hit_W, int& scale_out)
{
    const bool mres = m.octree.multires;
    int scale_tt = 0;
    const RayBlockHit rb = first_block_on_ray(m, origin_W, dir_W, t_near, t_far);
    const float step = m.res;
    const float largestep = (float) kBlockSize * step;
    const float t_min = rb.tcmin;
    if (t_min <= 0.0f)
        return false;
    const float t_max = rb.tmax;
    float t = t_min;
    const float trunc = m.res * m.trunc_factor;
    if (!(t_near < t_max))
        return false;
    float stepsize = largestep;
    V3 p = origin_W + dir_W * t;
    float f_t, w_t;
    if (mres)
        map_get_data_mr(m, p, f_t, w_t);
    else
        map_get_data(m, p, f_t, w_t);
    float f_tt = 0.0f;
    if (!(f_t >= 0.0f))
        return false;
    for (; t < t_far; t += stepsize) {
        float f, w;
        if (mres)
            map_get_data_mr(m, p, f, w);
        else
            map_get_data(m, p, f, w);
        if (!(w != 0.0f)) {
            stepsize = largestep;
            p = p + stepsize * dir_W;
            continue;
        }
        f_tt = f;
        /* the reference compares against the double literal 0.1 */
        if ((double) f_tt <= 0.1 && f_tt >= -0.5f) {
            float fi;
            if (mres ? map_field_interp_mr(m, p, fi, &scale_tt) : map_field_interp(m, p, fi))
                f_tt = fi;
        }
        if (f_tt < 0.0f)
            break;
        stepsize = std::max(f_tt * trunc, step);
        p = p + stepsize * dir_W;
        f_t = f_tt;
    }
    if (f_tt < 0.0f) {
        t = t - stepsize * (f_tt - 0.0f) / (f_tt - f_t);
        hit_W = origin_W + dir_W * t;
        scale_out = scale_tt;
        return true;
    }
    return false;
}

/* ------------------------------------- differentiable depth render, FP64 (no reference) -- */
/* The CPU check of the GPU's differentiable render and its adjoint: the same algorithm (march
 * of raycast<TSDF> to the first sample below the surface, then regula falsi on the trilinear
 * field inside the last step) evaluated in double precision on the map's float voxels, with
 * the root found to 1e-13. The gradients follow from the implicit function theorem at the
 * root with the pose perturbed on the left, T = exp(xi) T_WS, xi = [rho; omega]. */

struct D3 {
    double x, y, z;
};
static inline D3 d3(double x, double y, double z) { return D3{x, y, z}; }
static inline D3 dadd(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline D3 dmul(D3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
static inline double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline D3 dcross(D3 a, D3 b) { return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }

struct TriD {
    int oct[8];
    int vi[8];
    double f[8];
    D3 t;
};

static inline D3 to_map_voxels(const so_map& m, D3 p)
{
    const Tf& T = m.T_MW;
    const D3 q = d3((double) T.R[0][0] * p.x + (double) T.R[0][1] * p.y + (double) T.R[0][2] * p.z + (double) T.t[0],
                    (double) T.R[1][0] * p.x + (double) T.R[1][1] * p.y + (double) T.R[1][2] * p.z + (double) T.t[1],
                    (double) T.R[2][0] * p.x + (double) T.R[2][1] * p.y + (double) T.R[2][2] * p.z + (double) T.t[2]);
    return q;
}

static inline bool in_map(const so_map& m, D3 q)
{
    const double dim = (double) m.dim;
    return q.x >= 0.0 && q.x < dim && q.y >= 0.0 && q.y < dim && q.z >= 0.0 && q.z < dim;
}

static bool tri_sample_d(const so_map& m, D3 p, TriD& q, double& value)
{
    const D3 pm = to_map_voxels(m, p);
    if (!in_map(m, pm))
        return false;
    const double r = (double) m.res;
    const D3 bf = d3(pm.x / r - 0.5, pm.y / r - 0.5, pm.z / r - 0.5);
    const int b[3] = {(int) bf.x, (int) bf.y, (int) bf.z};
    for (int i = 0; i < 3; ++i)
        if (b[i] < 0 || b[i] + 1 >= m.octree.size)
            return false;
    for (int n = 0; n < 8; ++n) {
        const int32_t c[3] = {b[0] + (n & 1), b[1] + ((n >> 1) & 1), b[2] + (n >> 2)};
        const int o = m.octree.block_at(c);
        if (o < 0)
            return false;
        const Octant& oc = m.octree.octants[o];
        const BlockData& bd = m.octree.blocks[oc.block];
        const int vi = (c[0] - oc.coord[0]) + 8 * (c[1] - oc.coord[1]) + 64 * (c[2] - oc.coord[2]);
        if (!(bd.weight[vi] != 0.0f))
            return false;
        q.f[n] = (double) bd.tsdf[vi];
        q.oct[n] = o;
        q.vi[n] = vi;
    }
    q.t = d3(bf.x - std::floor(bf.x), bf.y - std::floor(bf.y), bf.z - std::floor(bf.z));
    const D3 t = q.t, tc = d3(1.0 - t.x, 1.0 - t.y, 1.0 - t.z);
    const double* f = q.f;
    value = ((f[0] * tc.x + f[1] * t.x) * tc.y + (f[2] * tc.x + f[3] * t.x) * t.y) * tc.z
        + ((f[4] * tc.x + f[5] * t.x) * tc.y + (f[6] * tc.x + f[7] * t.x) * t.y) * t.z;
    return true;
}

static inline void get_data_d(const so_map& m, D3 p, double& f, double& w)
{
    const D3 pm = to_map_voxels(m, p);
    f = 1.0;
    w = 0.0;
    if (!in_map(m, pm))
        return;
    const double r = (double) m.res;
    const int32_t c[3] = {(int) (pm.x / r), (int) (pm.y / r), (int) (pm.z / r)};
    float tf, wf;
    if (get_voxel(m, c, tf, wf)) {
        f = tf;
        w = wf;
    }
}

static bool diff_hit_d(const so_map& m, D3 o, D3 d, double t_near, double t_far, double& t_star, TriD& q)
{
    const RayBlockHit rb = first_block_on_ray(m, v3((float) o.x, (float) o.y, (float) o.z),
                                              v3((float) d.x, (float) d.y, (float) d.z), (float) t_near,
                                              (float) t_far);
    const double t_min = rb.tcmin, t_max = rb.tmax;
    if (t_min <= 0.0 || !(t_near < t_max))
        return false;
    const double step = m.res, largestep = kBlockSize * step, trunc = (double) m.res * m.trunc_factor;
    double t = t_min, stepsize = largestep, f_t, w_t, f_tt = 0.0;
    get_data_d(m, dadd(o, dmul(d, t)), f_t, w_t);
    if (!(f_t >= 0.0))
        return false;
    for (; t < t_far; t += stepsize) {
        double f, w;
        get_data_d(m, dadd(o, dmul(d, t)), f, w);
        if (!(w != 0.0)) {
            stepsize = largestep;
            continue;
        }
        f_tt = f;
        if (f_tt < 0.1 && f_tt >= -0.5) {
            double fi;
            TriD tq;
            if (tri_sample_d(m, dadd(o, dmul(d, t)), tq, fi))
                f_tt = fi;
        }
        if (f_tt < 0.0)
            break;
        stepsize = std::max(f_tt * trunc, step);
    }
    if (!(f_tt < 0.0))
        return false;
    double ta = t - stepsize, tb = t, fa, fb;
    if (!tri_sample_d(m, dadd(o, dmul(d, ta)), q, fa) || !tri_sample_d(m, dadd(o, dmul(d, tb)), q, fb))
        return false;
    if (!(fa >= 0.0 && fb < 0.0))
        return false;
    double tm = tb;
    int side = 0;
    for (int it = 0; it < 200; ++it) {
        tm = (ta * fb - tb * fa) / (fb - fa);
        double fm;
        if (!tri_sample_d(m, dadd(o, dmul(d, tm)), q, fm))
            return false;
        if (std::fabs(fm) < 1.0e-13)
            break;
        if (fm < 0.0) {
            tb = tm;
            fb = fm;
            if (side == -1)
                fa *= 0.5;
            side = -1;
        }
        else {
            ta = tm;
            fa = fm;
            if (side == 1)
                fb *= 0.5;
            side = 1;
        }
        if (!(tb - ta > 1.0e-15 * tb))
            break;
    }
    t_star = tm;
    return true;
}

struct RayD {
    D3 o, d;
    double nz, t_near, t_far;
};

static RayD ray_d(const so_pinhole& sp, const double T[16], int x, int y)
{
    const double rx = (x - (double) sp.cx) / (double) sp.fx, ry = (y - (double) sp.cy) / (double) sp.fy;
    const double nrm = std::sqrt(rx * rx + ry * ry + 1.0);
    const D3 n = d3(rx / nrm, ry / nrm, 1.0 / nrm);
    RayD r;
    r.d = d3(T[0] * n.x + T[1] * n.y + T[2] * n.z, T[4] * n.x + T[5] * n.y + T[6] * n.z,
             T[8] * n.x + T[9] * n.y + T[10] * n.z);
    r.o = d3(T[3], T[7], T[11]);
    r.nz = n.z;
    r.t_near = sp.near_plane / n.z;
    r.t_far = sp.far_plane / n.z;
    return r;
}

static D3 tri_grad_world_d(const so_map& m, const TriD& q)
{
    const double* f = q.f;
    const D3 t = q.t, tc = d3(1.0 - t.x, 1.0 - t.y, 1.0 - t.z);
    const double gx = ((f[1] - f[0]) * tc.y + (f[3] - f[2]) * t.y) * tc.z + ((f[5] - f[4]) * tc.y + (f[7] - f[6]) * t.y) * t.z;
    const double gy = ((f[2] - f[0]) * tc.x + (f[3] - f[1]) * t.x) * tc.z + ((f[6] - f[4]) * tc.x + (f[7] - f[5]) * t.x) * t.z;
    const double gz = ((f[4] - f[0]) * tc.x + (f[5] - f[1]) * t.x) * tc.y + ((f[6] - f[2]) * tc.x + (f[7] - f[3]) * t.x) * t.y;
    const Tf& T = m.T_MW;
    const double r = m.res;
    return d3((T.R[0][0] * gx + T.R[1][0] * gy + T.R[2][0] * gz) / r, (T.R[0][1] * gx + T.R[1][1] * gy + T.R[2][1] * gz) / r,
              (T.R[0][2] * gx + T.R[1][2] * gy + T.R[2][2] * gz) / r);
}

/* ----------------------------------------------------------------- ICP helpers (float) -- */

/* Eigen-style unblocked Cholesky (LLT) on the lower triangle, then forward/back substitution.
 * Returns false on a non-positive pivot (icp.cpp:33-41 returns zero in that case). */
static bool llt_solve6(const float C_in[6][6], const float b[6], float x[6])
{
    float L[6][6];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j)
            L[i][j] = C_in[i][j];
    for (int k = 0; k < 6; ++k) {
        float sq = 0.0f;
        for (int j = 0; j < k; ++j)
            sq += L[k][j] * L[k][j];
        float xk = L[k][k] - sq;
        if (xk <= 0.0f)
            return false;
        xk = std::sqrt(xk);
        L[k][k] = xk;
        for (int i = k + 1; i < 6; ++i) {
            float s = 0.0f;
            for (int j = 0; j < k; ++j)
                s += L[i][j] * L[k][j];
            L[i][k] = (L[i][k] - s) / xk;
        }
    }
    float y[6];
    for (int i = 0; i < 6; ++i) {
        float s = b[i];
        for (int j = 0; j < i; ++j)
            s -= L[i][j] * y[j];
        y[i] = s / L[i][i];
    }
    for (int i = 5; i >= 0; --i) {
        float s = y[i];
        for (int j = i + 1; j < 6; ++j)
            s -= L[j][i] * x[j];
        x[i] = s / L[i][i];
    }
    return true;
}

/* math::exp_and_theta + math::exp, math_util_impl.hpp:117-174 */
static Tf se3_exp(const float a[6])
{
    const V3 w = v3(a[3], a[4], a[5]);
    const float theta_sq = dot(w, w);
    const float theta = std::sqrt(theta_sq);
    const float half_theta = 0.5f * theta;
    float imag, real;
    if ((double) theta < 1e-10) {
        const float theta_po4 = theta_sq * theta_sq;
        imag = 0.5f - 1.0f / 48.0f * theta_sq + 1.0f / 3840.0f * theta_po4;
        real = 1.0f - 0.5f * theta_sq + 1.0f / 384.0f * theta_po4;
    }
    else {
        imag = std::sin(half_theta) / theta;
        real = std::cos(half_theta);
    }
    float qw = real, qx = imag * w.x, qy = imag * w.y, qz = imag * w.z;
    /* Eigen stores (x, y, z, w); the norm sums in that order */
    const float qn = std::sqrt(((qx * qx + qy * qy) + qz * qz) + qw * qw);
    qw /= qn;
    qx /= qn;
    qy /= qn;
    qz /= qn;
    const float tx = 2.0f * qx, ty = 2.0f * qy, tz = 2.0f * qz;
    const float twx = tx * qw, twy = ty * qw, twz = tz * qw;
    const float txx = tx * qx, txy = ty * qx, txz = tz * qx;
    const float tyy = ty * qy, tyz = tz * qy, tzz = tz * qz;
    float R[3][3] = {{1.0f - (tyy + tzz), txy - twz, txz + twy},
                     {txy + twz, 1.0f - (txx + tzz), tyz - twx},
                     {txz - twy, tyz + twx, 1.0f - (txx + tyy)}};
    const float O[3][3] = {{0.0f, -w.z, w.y}, {w.z, 0.0f, -w.x}, {-w.y, w.x, 0.0f}};
    float O2[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            O2[i][j] = (O[i][0] * O[0][j] + O[i][1] * O[1][j]) + O[i][2] * O[2][j];
    float V[3][3];
    if ((double) theta < 1e-10) {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                V[i][j] = R[i][j];
    }
    else {
        const float tsq = theta * theta;
        const float c1 = (1.0f - std::cos(theta)) / tsq;
        const float c2 = (theta - std::sin(theta)) / (tsq * theta);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                V[i][j] = ((i == j ? 1.0f : 0.0f) + c1 * O[i][j]) + c2 * O2[i][j];
    }
    Tf T;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            T.R[i][j] = R[i][j];
        T.t[i] = (V[i][0] * a[0] + V[i][1] * a[1]) + V[i][2] * a[2];
    }
    return T;
}

/* half_sample_robust_image, preprocessor.cpp:156-195 */
static void half_sample_robust(const float* in, int in_w, int in_h, float e_d, int radius,
                               float* out)
{
    const int ow = in_w / 2, oh = in_h / 2;
#pragma omp parallel for
    for (int y = 0; y < oh; y++) {
        for (int x = 0; x < ow; x++) {
            const int px = 2 * x, py = 2 * y;
            float count = 0.0f, sum = 0.0f;
            const float centre = in[px + py * in_w];
            for (int i = -radius + 1; i <= radius; ++i) {
                for (int j = -radius + 1; j <= radius; ++j) {
                    int qx = px + j, qy = py + i;
                    qx = std::min(std::max(qx, 0), 2 * ow - 1);
                    qy = std::min(std::max(qy, 0), 2 * oh - 1);
                    const float v = in[qx + qy * in_w];
                    if (std::fabs(v - centre) < e_d) {
                        count += 1.0f;
                        sum += v;
                    }
                }
            }
            out[x + y * ow] = sum / count;
        }
    }
}

/* depth_to_point_cloud, preprocessor_impl.hpp:18-40 */
static void depth_to_points(const float* depth, const Pinhole& s, V3* pts)
{
#pragma omp parallel for
    for (int y = 0; y < s.h; y++) {
        for (int x = 0; x < s.w; x++) {
            const float d = depth[x + y * s.w];
            if (d > 0.0f) {
                pts[x + y * s.w] = d * back_project(s, (float) x, (float) y);
            }
            else {
                pts[x + y * s.w] = v3(0.0f, 0.0f, 0.0f);
            }
        }
    }
}

/* point_cloud_to_normal<NegY>, preprocessor.cpp:109-152 */
static void points_to_normals(const V3* pts, int w, int h, bool neg_y, V3* nrm)
{
#pragma omp parallel for
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            const V3 p = pts[x + w * y];
            if (p.z == 0.0f) {
                nrm[x + y * w] = v3(0.0f, 0.0f, 0.0f);
                continue;
            }
            const int lx = std::max(x - 1, 0), rx = std::min(x + 1, w - 1);
            int uy, dy;
            if (neg_y) {
                uy = std::max(y - 1, 0);
                dy = std::min(y + 1, h - 1);
            }
            else {
                dy = std::max(y - 1, 0);
                uy = std::min(y + 1, h - 1);
            }
            const V3 left = pts[lx + w * y], right = pts[rx + w * y];
            const V3 up = pts[x + w * uy], down = pts[x + w * dy];
            if (left.z == 0.0f || right.z == 0.0f || up.z == 0.0f || down.z == 0.0f) {
                nrm[x + y * w] = v3(0.0f, 0.0f, 0.0f);
                continue;
            }
            nrm[x + y * w] = normalized(cross(right - left, up - down));
        }
    }
}

enum { kSuccess = 1, kInvalidInputNormal = -1, kProjOutside = -2, kInvalidRefNormal = -3,
       kDistThreshold = -4, kNormalThreshold = -5 };

/* --------------------------------------------------------- multi-res TSDF updater -- */

/* PinholeCamera::computeIntegrationScaleImpl, pinhole_camera.cpp:115-152, with the default
 * pixel_voxel_ratio_per_scale {1.5, 3, 6} (sensor.hpp:56) and scaled_pixel = 1/fx. */
static int integration_scale(const Pinhole& s, V3 c_S, float res, int last_scale, int min_scale, int max_scale)
{
    static const float kRatio[3] = {1.5f, 3.0f, 6.0f};
    const float dist = c_S.z;
    const float pixel_dim = dist * s.inv_fx;
    const float pv_ratio = pixel_dim / res;
    int scale = 0;
    for (float r : kRatio) {
        if (pv_ratio < r)
            break;
        scale++;
    }
    scale = std::min(scale, max_scale);
    if (scale > last_scale && min_scale != -1) {
        c_S.z -= 0.25f;
        return integration_scale(s, c_S, res, last_scale, -1, max_scale);
    }
    if (scale < last_scale && min_scale != -1) {
        c_S.z += 0.25f;
        return integration_scale(s, c_S, res, last_scale, -1, max_scale);
    }
    return scale;
}

/* propagator::propagateBlockDown (propagator_impl.hpp:71-117) by one scale, with the multi-res
 * TSDF updater's child / parent functions (multires_tsdf_updater_impl.hpp:70-146): observed
 * children take the parent's change since its last down-propagation, unobserved children are
 * initialised by interpolation at their scale. */
static void mr_propagate_down(const so_map& m, const Octant& oc, MRBlock& b, int parent_scale)
{
    const int ps = parent_scale, cs = ps - 1;
    const int pstride = 1 << ps, cstride = pstride >> 1;
    for (int z = 0; z < kBlockSize; z += pstride) {
        for (int y = 0; y < kBlockSize; y += pstride) {
            for (int x = 0; x < kBlockSize; x += pstride) {
                const int32_t pc[3] = {oc.coord[0] + x, oc.coord[1] + y, oc.coord[2] + z};
                const int pi = mr_index(oc, pc, ps);
                for (int k = 0; k < pstride; k += cstride) {
                    for (int j = 0; j < pstride; j += cstride) {
                        for (int i = 0; i < pstride; i += cstride) {
                            const int32_t cc[3] = {pc[0] + i, pc[1] + j, pc[2] + k};
                            const int ci = mr_index(oc, cc, cs);
                            if (b.weight[ci] != 0.0f) {
                                const float delta = b.tsdf[pi] - b.past_tsdf[pi];
                                b.tsdf[ci] = std::max(b.tsdf[ci] + delta, (float) -1.0f);
                                b.weight[ci] = std::fmin(b.weight[ci] + b.past_weight[pi], m.max_weight);
                                b.past_weight[ci] = b.past_weight[pi];
                            }
                            else {
                                const float half = 0.5f * (float) cstride;
                                const V3 cf = v3((float) cc[0] + half, (float) cc[1] + half, (float) cc[2] + half);
                                float iv;
                                if (mr_interp_voxel(m, cf, cs, iv, nullptr)) {
                                    b.tsdf[ci] = iv;
                                    b.weight[ci] = b.weight[pi];
                                    b.past_tsdf[ci] = iv;
                                    b.past_weight[ci] = 0.0f;
                                }
                            }
                        }
                    }
                }
                b.past_tsdf[pi] = b.tsdf[pi];
                b.past_weight[pi] = 0.0f;
            }
        }
    }
}

/* propagator::propagateBlockUp (propagator_impl.hpp:17-67) with data::up_prop_mean
 * (data_impl.hpp:13-50) and the updater's aggregate function (multires_tsdf_updater_impl.hpp:
 * 234-246). */
static void mr_propagate_up(const Octant& oc, MRBlock& b, int init_scale)
{
    for (int cs = init_scale; cs < kMaxBlockScale; ++cs) {
        const int cstride = 1 << cs, pstride = cstride << 1;
        for (int z = 0; z < kBlockSize; z += pstride) {
            for (int y = 0; y < kBlockSize; y += pstride) {
                for (int x = 0; x < kBlockSize; x += pstride) {
                    const int32_t pc[3] = {oc.coord[0] + x, oc.coord[1] + y, oc.coord[2] + z};
                    float tsdf_sum = 0.0f, weight_sum = 0.0f;
                    int n_valid = 0;
                    for (int k = 0; k < pstride; k += cstride) {
                        for (int j = 0; j < pstride; j += cstride) {
                            for (int i = 0; i < pstride; i += cstride) {
                                const int32_t cc[3] = {pc[0] + i, pc[1] + j, pc[2] + k};
                                const int ci = mr_index(oc, cc, cs);
                                if (b.weight[ci] != 0.0f) {
                                    ++n_valid;
                                    tsdf_sum += b.tsdf[ci];
                                    weight_sum += b.weight[ci];
                                }
                            }
                        }
                    }
                    const int pi = mr_index(oc, pc, cs + 1);
                    if (n_valid > 0) {
                        b.tsdf[pi] = tsdf_sum / (float) n_valid;
                        b.weight[pi] = std::ceil(weight_sum / (float) n_valid);
                        b.past_tsdf[pi] = b.tsdf[pi];
                        b.past_weight[pi] = 0.0f;
                    }
                    else {
                        b.past_tsdf[pi] = 1.0f;
                        b.past_weight[pi] = 0.0f;
                    }
                }
            }
        }
    }
}

/* Multi-res TSDF Updater, multires_tsdf_updater_impl.hpp:14-250.
 *
 * The reference runs the per-block body in one OpenMP loop, so a block's down-propagation
 * (which interpolates across neighbouring blocks) reads neighbours that other threads may be
 * updating at the same time. This restatement fixes one schedule of that loop: every block's
 * scale selection and down-propagation first (reading the map as it was before the update),
 * then every block's voxel update and up-propagation. A block's down-propagation writes only
 * scales finer than its previous scale, and the interpolation reads each block only at its
 * previous scale or coarser, so the first phase is free of races. */
static long long mr_update(so_map& m, const Pinhole& s, const Tf& T_WS, const float* depth,
                           const std::vector<int>& list, int timestamp)
{
    Octree& oct = m.octree;
    const float trunc = m.res * m.trunc_factor;
    const Tf T_CW = inverse_iso(T_WS);
    Tf T_CV = compose(T_CW, m.T_WM);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            T_CV.R[i][j] = T_CV.R[i][j] * m.res;
    for (int i = 0; i < 3; ++i)
        T_CV.t[i] = ((T_CV.R[i][0] * 0.5f + T_CV.R[i][1] * 0.5f) + T_CV.R[i][2] * 0.5f) + T_CV.t[i];
    const long long n = (long long) list.size();
    std::vector<int> new_scale((size_t) n);
#pragma omp parallel for
    for (long long i = 0; i < n; i++) {
        const Octant& oc = oct.octants[list[i]];
        MRBlock& b = oct.mr[oc.block];
        const V3 centre_C = apply(T_CW, m.voxel_to_point(oc.coord, kBlockSize));
        const int last = b.current_scale;
        const int curr = std::max(integration_scale(s, centre_C, m.res, last, b.min_scale, kMaxBlockScale), last - 1);
        b.min_scale = b.min_scale < 0 ? curr : std::min(b.min_scale, curr);
        new_scale[(size_t) i] = curr;
        if (curr < last)
            mr_propagate_down(m, oc, b, last);
    }
    long long n_upd = 0;
#pragma omp parallel for reduction(+ : n_upd)
    for (long long i = 0; i < n; i++) {
        Octant& oc = oct.octants[list[i]];
        MRBlock& b = oct.mr[oc.block];
        oc.timestamp = timestamp;
        const int curr = new_scale[(size_t) i];
        b.current_scale = curr;
        const int stride = 1 << curr;
        for (int x = 0; x < kBlockSize; x += stride) {
            for (int y = 0; y < kBlockSize; y += stride) {
                for (int z = 0; z < kBlockSize; z += stride) {
                    const int32_t c[3] = {oc.coord[0] + x, oc.coord[1] + y, oc.coord[2] + z};
                    const V3 vc = v3((float) c[0], (float) c[1], (float) c[2]);
                    const V3 p_C = apply(T_CV, vc);
                    const float pn = norm(p_C);
                    if (pn > far_dist(s, p_C))
                        continue;
                    float u, v;
                    if (!project(s, p_C, u, v))
                        continue;
                    int px, py;
                    round_pixel(u, v, px, py);
                    const float dv = depth[px + py * s.w];
                    if (dv < s.near_plane)
                        continue;
                    const float mz = p_C.z;
                    const float sdf = (dv - mz) / mz * pn;
                    const int idx = mr_index(oc, c, curr);
                    if (!(sdf < -trunc)) {
                        const float upd = std::min(sdf / trunc, (float) 1.0f);
                        float w = b.weight[idx];
                        if (w < m.max_weight)
                            w = w + 1.0f;
                        b.tsdf[idx] = (b.tsdf[idx] * (w - 1.0f) + upd) / w;
                        b.weight[idx] = w;
                        ++n_upd;
                    }
                    b.past_weight[idx] = b.past_weight[idx] + 1.0f;
                }
            }
        }
        mr_propagate_up(oc, b, curr);
    }
    return n_upd;
}

struct IcpRow {
    int result;
    float error;
    float J[6];
};

} // namespace

/* ===================================================================== C interface === */

extern "C" {

void so_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0)
        omp_set_num_threads(n);
#else
    (void) n;
#endif
}

int so_get_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Map ctor, map_impl.hpp:37-55; Octree ctor, octree_impl.hpp:14-19 */
so_map* so_map_create(const float dim[3], float res, float truncation_boundary_factor,
                      float max_weight, const float* T_MW)
{
    so_map* m = new so_map();
    const float dmax = std::max(std::max(dim[0], dim[1]), dim[2]);
    const int requested = (int) std::ceil(dmax / res);
    int sz = 1;
    while (sz < std::max(requested, 2 * kBlockSize))
        sz <<= 1;
    m->octree.init(sz);
    m->res = res;
    m->dim = (float) sz * res;
    if (T_MW) {
        m->T_MW = tf_from16(T_MW);
    }
    else {
        m->T_MW = tf_identity();
        m->T_MW.t[0] = dim[0] / 2.0f;
        m->T_MW.t[1] = dim[1] / 2.0f;
        m->T_MW.t[2] = dim[2] / 2.0f;
    }
    m->T_WM = inverse_iso(m->T_MW);
    m->trunc_factor = truncation_boundary_factor;
    m->max_weight = max_weight;
    return m;
}

so_map* so_map_create_multires(const float dim[3], float res, float truncation_boundary_factor,
                               float max_weight, const float* T_MW)
{
    so_map* m = so_map_create(dim, res, truncation_boundary_factor, max_weight, T_MW);
    m->octree.multires = true;
    return m;
}

int so_map_is_multires(const so_map* map) { return map->octree.multires ? 1 : 0; }

void so_map_mr_blocks(const so_map* map, uint64_t* keys, int32_t* coords, float* tsdf, float* weight,
                      float* past_tsdf, float* past_weight, int32_t* scales)
{
    const Octree& o = map->octree;
    if (!o.multires)
        return;
    for (size_t i = 0; i < o.block_octant.size(); ++i) {
        const Octant& oc = o.octants[o.block_octant[i]];
        const MRBlock& b = o.mr[oc.block];
        if (keys)
            keys[i] = encode_key(oc.coord[0], oc.coord[1], oc.coord[2], kMaxBlockScale);
        if (coords)
            for (int k = 0; k < 3; ++k)
                coords[3 * i + k] = oc.coord[k];
        if (tsdf)
            std::memcpy(tsdf + i * kMrVoxels, b.tsdf, sizeof(b.tsdf));
        if (weight)
            std::memcpy(weight + i * kMrVoxels, b.weight, sizeof(b.weight));
        if (past_tsdf)
            std::memcpy(past_tsdf + i * kMrVoxels, b.past_tsdf, sizeof(b.past_tsdf));
        if (past_weight)
            std::memcpy(past_weight + i * kMrVoxels, b.past_weight, sizeof(b.past_weight));
        if (scales) {
            scales[2 * i] = b.current_scale;
            scales[2 * i + 1] = b.min_scale;
        }
    }
}

void so_map_destroy(so_map* map) { delete map; }
int so_map_size(const so_map* map) { return map->octree.size; }
float so_map_dim(const so_map* map) { return map->dim; }

void so_integrate_depth(so_map* map, const float* depth, const so_pinhole* sensor_c,
                        const float T_WC_m[16], int timestamp, so_integrate_stats* stats)
{
    so_map& m = *map;
    Octree& oct = m.octree;
    const Pinhole s = make_pinhole(sensor_c);
    const Tf T_WS = tf_from16(T_WC_m);
    const float band = 2.0f * m.res * m.trunc_factor;

    /* fetcher::frustum (raycast_carver_impl.hpp:17-32): FrustumIterator DFS over the octree; an
     * octant whose bounding sphere misses the frustum is skipped with its subtree. The root is
     * never tested (iterator_impl.hpp:88-118 pushes its children before testing it). */
    const Tf T_SW = inverse_iso(T_WS);
    std::vector<int> frustum_blocks;
    {
        std::vector<int> stack;
        for (int c = 0; c < 8; ++c)
            if (oct.octants[0].child[c] >= 0)
                stack.push_back(oct.octants[0].child[c]);
        while (!stack.empty()) {
            const int o = stack.back();
            stack.pop_back();
            const Octant& oc = oct.octants[o];
            const V3 centre_W = m.voxel_to_point(oc.coord, oc.size);
            const V3 centre_S = apply(T_SW, centre_W);
            const float radius = std::sqrt(3.0f) / 2.0f * m.res * (float) oc.size;
            if (!sphere_in_frustum(s, centre_S, radius))
                continue;
            if (oc.block >= 0) {
                frustum_blocks.push_back(o);
                continue;
            }
            for (int c = 0; c < 8; ++c)
                if (oc.child[c] >= 0)
                    stack.push_back(oc.child[c]);
        }
    }

    /* RaycastCarver::operator(), raycast_carver_impl.hpp:56-128 */
    const int num_steps = (int) std::ceil(band / (2.0f * m.res));
    const V3 t_WS = v3(T_WS.t[0], T_WS.t[1], T_WS.t[2]);
    long long n_valid = 0;
#pragma omp declare reduction(merge : std::set<uint64_t> : omp_out.insert(omp_in.begin(), omp_in.end()))
    std::set<uint64_t> key_set;
#pragma omp parallel for reduction(merge : key_set) reduction(+ : n_valid)
    for (int x = 0; x < s.w; ++x) {
        for (int y = 0; y < s.h; ++y) {
            const float dv = depth[x + y * s.w];
            if (dv < s.near_plane || dv > (s.far_plane + band * 0.5f))
                continue;
            ++n_valid;
            const V3 ray_C = back_project(s, (float) x, (float) y);
            const V3 point_W = apply(T_WS, dv * ray_C);
            const V3 rev = normalized(t_WS - point_W);
            const V3 origin = point_W - (band * 0.5f) * rev;
            const V3 step = (rev * band) / (float) num_steps;
            V3 pos = origin;
            for (int i = 0; i < num_steps; i++) {
                int32_t vc[3];
                if (m.point_to_voxel(pos, vc)) {
                    if (oct.block_at(vc) < 0) {
                        key_set.insert(encode_key(vc[0], vc[1], vc[2], kMaxBlockScale));
                    }
                }
                pos = pos + step;
            }
        }
    }
    const std::vector<uint64_t> keys(key_set.begin(), key_set.end());

    /* allocator::blocks(keys, only_allocated = true), allocator_impl.hpp:68-116 (serial here:
     * allocation order does not change the resulting tree) */
    std::vector<int> list;
    for (uint64_t k : keys) {
        int o;
        if (oct.allocate_key(k, o))
            list.push_back(o);
    }
    const long long n_new = (long long) list.size();
    list.insert(list.end(), frustum_blocks.begin(), frustum_blocks.end());

    if (oct.multires) {
        const long long n_upd = mr_update(m, s, T_WS, depth, list, timestamp);
        if (stats) {
            stats->n_valid_pixels = n_valid;
            stats->n_new_blocks = n_new;
            stats->n_frustum_blocks = (long long) frustum_blocks.size();
            stats->n_updated_voxels = n_upd;
        }
        return;
    }

    /* single-res TSDF Updater, singleres_tsdf_updater_impl.hpp:14-132 */
    const float trunc = m.res * m.trunc_factor;
    const Tf T_CW = inverse_iso(T_WS);
    Tf T_CV = compose(T_CW, m.T_WM);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            T_CV.R[i][j] = T_CV.R[i][j] * m.res;
    for (int i = 0; i < 3; ++i)
        T_CV.t[i] = ((T_CV.R[i][0] * 0.5f + T_CV.R[i][1] * 0.5f) + T_CV.R[i][2] * 0.5f) + T_CV.t[i];
    long long n_upd = 0;
#pragma omp parallel for reduction(+ : n_upd)
    for (long long i = 0; i < (long long) list.size(); i++) {
        Octant& oc = oct.octants[list[i]];
        oc.timestamp = timestamp;
        BlockData& b = oct.blocks[oc.block];
        for (int x = 0; x < kBlockSize; ++x) {
            for (int y = 0; y < kBlockSize; ++y) {
                for (int z = 0; z < kBlockSize; ++z) {
                    const V3 vc = v3((float) (oc.coord[0] + x), (float) (oc.coord[1] + y),
                                     (float) (oc.coord[2] + z));
                    const V3 p_C = apply(T_CV, vc);
                    const float pn = norm(p_C);
                    if (pn > far_dist(s, p_C))
                        continue;
                    float u, v;
                    if (!project(s, p_C, u, v))
                        continue;
                    int px, py;
                    round_pixel(u, v, px, py);
                    const float dv = depth[px + py * s.w];
                    if (dv < s.near_plane)
                        continue;
                    const float mz = p_C.z;
                    const float sdf = (dv - mz) / mz * pn;
                    /* FieldData<TSDF>::update, data_field_impl.hpp:39-54 */
                    if (sdf < -trunc)
                        continue;
                    const float upd = std::min(sdf / trunc, (float) 1.0f);
                    const int idx = x + 8 * y + 64 * z;
                    float w = b.weight[idx];
                    if (w < m.max_weight)
                        w = w + 1.0f;
                    b.tsdf[idx] = (b.tsdf[idx] * (w - 1.0f) + upd) / w;
                    b.weight[idx] = w;
                    ++n_upd;
                }
            }
        }
    }
    if (stats) {
        stats->n_valid_pixels = n_valid;
        stats->n_new_blocks = n_new;
        stats->n_frustum_blocks = (long long) frustum_blocks.size();
        stats->n_updated_voxels = n_upd;
    }
}

/* raycaster::raycast_volume, raycaster_impl.hpp:537-627 */
void so_raycast_volume(const so_map* map, const so_pinhole* sensor_c, const float T_WS_m[16],
                       float* pts_W, float* nrm_W, int8_t* scale)
{
    const so_map& m = *map;
    const Pinhole s = make_pinhole(sensor_c);
    const Tf T_WS = tf_from16(T_WS_m);
    const V3 origin = v3(T_WS.t[0], T_WS.t[1], T_WS.t[2]);
#pragma omp parallel for
    for (int y = 0; y < s.h; y++) {
        for (int x = 0; x < s.w; x++) {
            const size_t idx = (size_t) x + (size_t) y * (size_t) s.w;
            const V3 ray_S = back_project(s, (float) x, (float) y);
            const V3 dir_W = rot(T_WS, normalized(ray_S));
            V3 hit;
            int hit_scale = 0;
            if (raycast_tsdf(m, origin, dir_W, near_dist(s, ray_S), far_dist(s, ray_S), hit, hit_scale)) {
                scale[idx] = (int8_t) hit_scale;
                pts_W[3 * idx + 0] = hit.x;
                pts_W[3 * idx + 1] = hit.y;
                pts_W[3 * idx + 2] = hit.z;
                V3 g;
                if (m.octree.multires ? map_field_grad_mr(m, hit, g) : map_field_grad(m, hit, g)) {
                    const V3 n = normalized(g);
                    nrm_W[3 * idx + 0] = n.x;
                    nrm_W[3 * idx + 1] = n.y;
                    nrm_W[3 * idx + 2] = n.z;
                }
                else {
                    nrm_W[3 * idx + 0] = nrm_W[3 * idx + 1] = nrm_W[3 * idx + 2] = 0.0f;
                }
            }
            else {
                /* raycast_volume leaves the scale image untouched on a miss; it is set to 0 here */
                scale[idx] = 0;
                pts_W[3 * idx + 0] = pts_W[3 * idx + 1] = pts_W[3 * idx + 2] = 0.0f;
                nrm_W[3 * idx + 0] = nrm_W[3 * idx + 1] = nrm_W[3 * idx + 2] = 0.0f;
            }
        }
    }
}

/* The number of distinct voxels so_raycast_volume reads on a single-res map at T_WS (the
 * algorithmic voxel traffic of the raycast; a measurement aid, not part of the restatement). */
long long so_raycast_touched(const so_map* map, const so_pinhole* sensor, const float T_WS[16])
{
    const Pinhole s = make_pinhole(sensor);
    const int nt = omp_get_max_threads();
    std::vector<std::vector<uint64_t>> per((size_t) nt);
    std::vector<float> pts((size_t) s.w * s.h * 3), nrm(pts.size());
    std::vector<int8_t> sc((size_t) s.w * s.h);
    // the raycast's parallel loop runs on the same pool threads that set their hook here
    omp_set_dynamic(0);
#pragma omp parallel num_threads(nt)
    g_touched = &per[(size_t) omp_get_thread_num()];
    so_raycast_volume(map, sensor, T_WS, pts.data(), nrm.data(), sc.data());
#pragma omp parallel num_threads(nt)
    g_touched = nullptr;
    std::vector<uint64_t> all;
    for (auto& v : per)
        all.insert(all.end(), v.begin(), v.end());
    std::sort(all.begin(), all.end());
    return (long long) (std::unique(all.begin(), all.end()) - all.begin());
}

/* Tracker::track(depth, T_WS, pts, nrm), tracker_impl.hpp:30-116 */
int so_track(const so_pinhole* sensor_c, const so_tracker_config* cfg, const float* depth,
             float T_WS_m[16], const float* ref_pts_W, const float* ref_nrm_W,
             so_track_stats* stats)
{
    const Pinhole s = make_pinhole(sensor_c);
    Tf T_WS = tf_from16(T_WS_m);
    const Tf T_WS_ref = T_WS;
    const int W = s.w, H = s.h;
    const int L = std::min(std::max(cfg->num_levels, 1), 3);
    std::vector<std::vector<float>> dimg(L);
    std::vector<std::vector<V3>> pts(L), nrm(L);
    std::vector<int> lw(L), lh(L);
    for (int i = 0; i < L; ++i) {
        lw[i] = W / (1 << i);
        lh[i] = H / (1 << i);
        dimg[i].assign((size_t) lw[i] * lh[i], 0.0f);
        pts[i].assign((size_t) lw[i] * lh[i], v3(0, 0, 0));
        nrm[i].assign((size_t) lw[i] * lh[i], v3(0, 0, 0));
    }
    std::memcpy(dimg[0].data(), depth, sizeof(float) * (size_t) W * H);
    for (int i = 1; i < L; ++i)
        half_sample_robust(dimg[i - 1].data(), lw[i - 1], lh[i - 1], 0.1f * 3.0f, 1, dimg[i].data());
    for (int i = 0; i < L; ++i) {
        const Pinhole si = downsampled(s, (float) (1 << i));
        depth_to_points(dimg[i].data(), si, pts[i].data());
        points_to_normals(pts[i].data(), si.w, si.h, s.left_hand, nrm[i].data());
    }

    std::vector<IcpRow> rows((size_t) W * H, IcpRow{0, 0.0f, {0, 0, 0, 0, 0, 0}});
    float red[8][32];
    std::memset(red, 0, sizeof(red));
    const V3* rp = reinterpret_cast<const V3*>(ref_pts_W);
    const V3* rn = reinterpret_cast<const V3*>(ref_nrm_W);
    int iters_run[3] = {0, 0, 0};

    for (int level = L - 1; level >= 0; --level) {
        const int w = lw[level], h = lh[level];
        for (int it = 0; it < cfg->iterations[level]; ++it) {
            ++iters_run[level];
            /* icp::trackKernel, icp_impl.hpp:16-102 */
            const Tf T_ref_inv = inverse_iso(T_WS_ref);
#pragma omp parallel for
            for (int y = 0; y < h; y++) {
                for (int x = 0; x < w; x++) {
                    IcpRow& row = rows[(size_t) x + (size_t) y * W];
                    const V3 n_in = nrm[level][x + y * w];
                    if (is_zero(n_in)) {
                        row.result = kInvalidInputNormal;
                        continue;
                    }
                    const V3 p_W = apply(T_WS, pts[level][x + y * w]);
                    const V3 p_ref = apply(T_ref_inv, p_W);
                    float u, v;
                    if (!project(s, p_ref, u, v)) {
                        row.result = kProjOutside;
                        continue;
                    }
                    int px, py;
                    round_pixel(u, v, px, py);
                    const size_t ri = (size_t) px + (size_t) py * W;
                    const V3 n_ref = v3(-rn[ri].x, -rn[ri].y, -rn[ri].z);
                    if (is_zero(n_ref)) {
                        row.result = kInvalidRefNormal;
                        continue;
                    }
                    const V3 diff = rp[ri] - p_W;
                    const V3 n_W = rot(T_WS, n_in);
                    if (norm(diff) > cfg->dist_threshold) {
                        row.result = kDistThreshold;
                        continue;
                    }
                    if (dot(n_W, n_ref) < cfg->normal_threshold) {
                        row.result = kNormalThreshold;
                        continue;
                    }
                    row.result = kSuccess;
                    row.error = dot(n_ref, diff);
                    row.J[0] = n_ref.x;
                    row.J[1] = n_ref.y;
                    row.J[2] = n_ref.z;
                    const V3 c = cross(p_W, n_ref);
                    row.J[3] = c.x;
                    row.J[4] = c.y;
                    row.J[5] = c.z;
                }
            }
            /* icp::reduceKernel / newReduce, icp.cpp:45-204: 8 row-interleaved partials */
            for (int b = 0; b < 8; ++b) {
                float s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0, s5 = 0, s6 = 0, s7 = 0, s8 = 0,
                      s9 = 0, s10 = 0, s11 = 0, s12 = 0, s13 = 0, s14 = 0, s15 = 0, s16 = 0,
                      s17 = 0, s18 = 0, s19 = 0, s20 = 0, s21 = 0, s22 = 0, s23 = 0, s24 = 0,
                      s25 = 0, s26 = 0, s27 = 0, s28 = 0, s29 = 0, s30 = 0, s31 = 0;
#pragma omp parallel for reduction(+ : s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, s10, s11, s12, s13, s14, s15, s16, s17, s18, s19, s20, s21, s22, s23, s24, s25, s26, s27, s28, s29, s30, s31)
                for (int y = b; y < h; y += 8) {
                    for (int x = 0; x < w; x++) {
                        const IcpRow& r = rows[(size_t) x + (size_t) y * W];
                        if (r.result < kSuccess) {
                            s29 += r.result == kDistThreshold ? 1 : 0;
                            s30 += r.result == kNormalThreshold ? 1 : 0;
                            s31 += r.result > kDistThreshold ? 1 : 0;
                            continue;
                        }
                        const float e = r.error;
                        const float* J = r.J;
                        s0 += e * e;
                        s1 += e * J[0];
                        s2 += e * J[1];
                        s3 += e * J[2];
                        s4 += e * J[3];
                        s5 += e * J[4];
                        s6 += e * J[5];
                        s7 += J[0] * J[0];
                        s8 += J[0] * J[1];
                        s9 += J[0] * J[2];
                        s10 += J[0] * J[3];
                        s11 += J[0] * J[4];
                        s12 += J[0] * J[5];
                        s13 += J[1] * J[1];
                        s14 += J[1] * J[2];
                        s15 += J[1] * J[3];
                        s16 += J[1] * J[4];
                        s17 += J[1] * J[5];
                        s18 += J[2] * J[2];
                        s19 += J[2] * J[3];
                        s20 += J[2] * J[4];
                        s21 += J[2] * J[5];
                        s22 += J[3] * J[3];
                        s23 += J[3] * J[4];
                        s24 += J[3] * J[5];
                        s25 += J[4] * J[4];
                        s26 += J[4] * J[5];
                        s27 += J[5] * J[5];
                        s28 += 1;
                    }
                }
                const float vals[32] = {s0,  s1,  s2,  s3,  s4,  s5,  s6,  s7,  s8,  s9,  s10,
                                        s11, s12, s13, s14, s15, s16, s17, s18, s19, s20, s21,
                                        s22, s23, s24, s25, s26, s27, s28, s29, s30, s31};
                for (int k = 0; k < 32; ++k)
                    red[b][k] = vals[k];
            }
            for (int j = 1; j < 8; ++j)
                for (int k = 0; k < 32; ++k)
                    red[0][k] += red[j][k];

            /* icp::updatePoseKernel + solve/makeJTJ, icp.cpp:15-41,208-223 */
            const float* v = &red[0][1];
            float b6[6] = {v[0], v[1], v[2], v[3], v[4], v[5]};
            float C[6][6];
            int k = 6;
            for (int r = 0; r < 6; ++r)
                for (int c = r; c < 6; ++c)
                    C[r][c] = v[k++];
            for (int r = 1; r < 6; ++r)
                for (int c = 0; c < r; ++c)
                    C[r][c] = C[c][r];
            float x6[6] = {0, 0, 0, 0, 0, 0};
            if (!llt_solve6(C, b6, x6))
                for (int q = 0; q < 6; ++q)
                    x6[q] = 0.0f;
            const Tf delta = se3_exp(x6);
            T_WS = compose(delta, T_WS);
            float xn2 = 0.0f;
            for (int q = 0; q < 6; ++q)
                xn2 += x6[q] * x6[q];
            if (std::sqrt(xn2) < cfg->icp_threshold)
                break;
        }
    }
    /* icp::checkPoseKernel, icp.cpp:227-246 */
    int accepted = 1;
    if (((double) std::sqrt(red[0][0] / red[0][28]) > 2e-2)
        || (red[0][28] / (float) (W * H) < cfg->track_threshold)) {
        T_WS = T_WS_ref;
        accepted = 0;
    }
    tf_to16(T_WS, T_WS_m);
    if (stats) {
        for (int l = 0; l < 3; ++l)
            stats->converged_iterations[l] = iters_run[l];
        stats->accepted = accepted;
        for (int q = 0; q < 32; ++q)
            stats->reduction[q] = red[0][q];
    }
    return accepted;
}

long long so_map_num_blocks(const so_map* map) { return (long long) map->octree.block_octant.size(); }

void so_map_blocks(const so_map* map, uint64_t* keys, int32_t* coords, float* tsdf,
                   float* weight, int32_t* timestamps)
{
    const Octree& oct = map->octree;
    for (size_t i = 0; i < oct.block_octant.size(); ++i) {
        const Octant& oc = oct.octants[oct.block_octant[i]];
        if (keys)
            keys[i] = encode_key(oc.coord[0], oc.coord[1], oc.coord[2], kMaxBlockScale);
        if (coords) {
            coords[3 * i + 0] = oc.coord[0];
            coords[3 * i + 1] = oc.coord[1];
            coords[3 * i + 2] = oc.coord[2];
        }
        /* multi-res maps report their finest (scale 0) level here */
        const float* bt = oct.multires ? oct.mr[oc.block].tsdf : oct.blocks[oc.block].tsdf;
        const float* bw = oct.multires ? oct.mr[oc.block].weight : oct.blocks[oc.block].weight;
        if (tsdf)
            std::memcpy(tsdf + i * kBlockVoxels, bt, sizeof(float) * kBlockVoxels);
        if (weight)
            std::memcpy(weight + i * kBlockVoxels, bw, sizeof(float) * kBlockVoxels);
        if (timestamps)
            timestamps[i] = oc.timestamp;
    }
}

/* ------------------------------------------------------------------ marching cubes -- */
/* The case table is the reference's (include/se/map/algorithms/edge_tables.hpp, triTable), in the
 * encoding of mc_case_table.inc (generated from the reference's sources; the GPU library reads
 * the same file): per case the face count and the cube edges of the faces in triTable's order.
 * Corners in the order of meshing::gather_data: c0 (0,0,0), c1 (1,0,0), c2 (1,0,1), c3 (0,0,1),
 * c4 (0,1,0), c5 (1,1,0), c6 (1,1,1), c7 (0,1,1); edges as edge_to_corners
 * (marching_cube_impl.hpp:96-127); case index bit i = corner i inside. */
#include "../supereight2_gb300/csrc/mc_case_table.inc"

namespace {

constexpr int kMcCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1},
                                 {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}};
constexpr int kMcEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {0, 3}, {4, 5}, {5, 6},
                                {6, 7}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
constexpr int kMcMaxTri = 8;

struct McTable {
    int ntri[256];
    signed char tri[256][3 * kMcMaxTri];
};

static McTable build_mc_table()
{
    McTable T;
    std::memset(&T, 0, sizeof(T));
    for (int cfg = 0; cfg < 256; ++cfg) {
        const unsigned long long w = kMcCaseWords[cfg];
        T.ntri[cfg] = (int) (w >> 60);
        for (int k = 0; k < 3 * T.ntri[cfg]; ++k)
            T.tri[cfg][k] = (signed char) ((w >> (4 * k)) & 0xf);
    }
    return T;
}

static const McTable& mc_table()
{
    static const McTable t = build_mc_table();
    return t;
}

/* meshing::compute_intersection (marching_cube_impl.hpp:82-93): corner values by getData */
static V3 mc_vertex(const so_map& m, int x, int y, int z, int e)
{
    const int* a = kMcCorner[kMcEdge[e][0]];
    const int* b = kMcCorner[kMcEdge[e][1]];
    const int32_t c0[3] = {x + a[0], y + a[1], z + a[2]}, c1[3] = {x + b[0], y + b[1], z + b[2]};
    float v0, w0, v1, w1;
    get_voxel(m, c0, v0, w0);
    get_voxel(m, c1, v1, w1);
    const V3 p0 = v3((float) c0[0] + 0.5f, (float) c0[1] + 0.5f, (float) c0[2] + 0.5f);
    const V3 p1 = v3((float) c1[0] + 0.5f, (float) c1[1] + 0.5f, (float) c1[2] + 0.5f);
    const float sfac = (0.0f - v0) / (v1 - v0);
    return v3(p0.x + sfac * (p1.x - p0.x), p0.y + sfac * (p1.y - p0.y), p0.z + sfac * (p1.z - p0.z));
}

} // namespace

/* The case table (for the tests): ntri[256], tri[256][24] edge indices. */
void so_mc_table(int32_t* ntri, int32_t* tri)
{
    const McTable& t = mc_table();
    for (int c = 0; c < 256; ++c) {
        ntri[c] = t.ntri[c];
        for (int k = 0; k < 3 * kMcMaxTri; ++k)
            tri[c * 3 * kMcMaxTri + k] = k < 3 * t.ntri[c] ? t.tri[c][k] : -1;
    }
}

/* algorithms::marching_cube single-res (marching_cube_impl.hpp:830-890, 1175-1201) with the
 * isosurface::occupied index: per allocated block the cubes [coord, min(coord + 8, size - 1))
 * per axis; a cube with an unobserved corner (weight 0) has no faces; a face with a vertex
 * coordinate <= 0 or > size (checkVertex) is dropped. faces: 9 floats each (three vertices in
 * voxel units, the map frame divided by the resolution); returns the face count (faces may be
 * NULL to count). */
long long so_marching_cubes(const so_map* mp, float* faces, long long capacity)
{
    const so_map& m = *mp;
    const Octree& oct = m.octree;
    const McTable& T = mc_table();
    const int size = oct.size;
    std::vector<std::vector<float>> per_block(oct.block_octant.size());
#pragma omp parallel for schedule(dynamic, 16)
    for (long long i = 0; i < (long long) oct.block_octant.size(); ++i) {
        const Octant& oc = oct.octants[oct.block_octant[(size_t) i]];
        std::vector<float>& out = per_block[(size_t) i];
        const int lx = std::min(oc.coord[0] + kBlockSize, size - 1), ly = std::min(oc.coord[1] + kBlockSize, size - 1),
                  lz = std::min(oc.coord[2] + kBlockSize, size - 1);
        for (int x = oc.coord[0]; x < lx; ++x)
            for (int y = oc.coord[1]; y < ly; ++y)
                for (int z = oc.coord[2]; z < lz; ++z) {
                    int cfg = 0;
                    bool valid = true;
                    for (int k = 0; k < 8 && valid; ++k) {
                        const int32_t c[3] = {x + kMcCorner[k][0], y + kMcCorner[k][1], z + kMcCorner[k][2]};
                        float t, w;
                        get_voxel(m, c, t, w);
                        if (w == 0.0f)
                            valid = false;
                        else if (t < 0.0f)
                            cfg |= 1 << k;
                    }
                    if (!valid || T.ntri[cfg] == 0)
                        continue;
                    for (int f = 0; f < T.ntri[cfg]; ++f) {
                        V3 v[3];
                        bool keep = true;
                        for (int j = 0; j < 3; ++j) {
                            v[j] = mc_vertex(m, x, y, z, T.tri[cfg][3 * f + j]);
                            if (v[j].x <= 0.0f || v[j].y <= 0.0f || v[j].z <= 0.0f || v[j].x > (float) size
                                || v[j].y > (float) size || v[j].z > (float) size)
                                keep = false;
                        }
                        if (!keep)
                            continue;
                        for (int j = 0; j < 3; ++j) {
                            out.push_back(v[j].x);
                            out.push_back(v[j].y);
                            out.push_back(v[j].z);
                        }
                    }
                }
    }
    long long n = 0;
    for (const auto& b : per_block) {
        const long long k = (long long) b.size() / 9;
        if (faces)
            for (long long j = 0; j < k && n + j < capacity; ++j)
                std::memcpy(faces + 9 * (n + j), b.data() + 9 * j, 9 * sizeof(float));
        n += k;
    }
    return n;
}

namespace {

/* A multi-res TSDF map seen by the dual marching cubes: BlockMultiRes<TSDF>::data(voxel, scale)
 * (block_impl.hpp:164-170) reads the pyramid at any scale; get_field = tsdf (data.hpp:117-121),
 * is_valid = weight != 0 (data_field_impl.hpp:32-35), is_inside = tsdf < 0 (data.hpp:133-137). */
struct MrTsdfView {
    const Octree& o;
    int size() const { return o.size; }
    int num_blocks() const { return (int) o.mr.size(); }
    bool live(int) const { return true; }
    const int32_t* coord(int b) const { return o.octants[(size_t) o.block_octant[(size_t) b]].coord; }
    int current_scale(int b) const { return o.mr[(size_t) b].current_scale; }
    int block_at(const int32_t c[3]) const
    {
        const int oc = o.block_at(c);
        return oc < 0 ? -1 : o.octants[(size_t) oc].block;
    }
    bool data(int b, const int32_t c[3], int scale, float& field) const
    {
        const MRBlock& B = o.mr[(size_t) b];
        const int32_t* bc = coord(b);
        const int n = kBlockSize >> scale;
        const int i = kMrScaleOffset[scale] + (c[0] - bc[0]) / (1 << scale) + n * ((c[1] - bc[1]) / (1 << scale))
            + n * n * ((c[2] - bc[2]) / (1 << scale));
        field = B.tsdf[i];
        return B.weight[i] != 0.0f;
    }
    bool inside(float field) const { return field < 0.0f; }
};

} // namespace

/* Dual marching cubes of a multi-res TSDF map (algorithms::marching_cube for Res::Multi,
 * marching_cube_impl.hpp:895-975, 1175-1201): faces (9 floats each, voxel units) and the
 * integration scale of each face; returns the face count (faces and scales may be NULL). */
long long so_dual_marching_cubes(const so_map* map, int min_desired_scale, float* faces, int8_t* scales,
                                 long long capacity)
{
    if (!map->octree.multires)
        return -1;
    std::vector<int32_t> ntri(256), tri(256 * 3 * kMcMaxTri);
    so_mc_table(ntri.data(), tri.data());
    return dual_mc::dual_marching_cubes(MrTsdfView{map->octree}, min_desired_scale, ntri.data(), tri.data(),
                                        3 * kMcMaxTri, faces, scales, capacity);
}

/* The dual-corner partition of a primal corner at block-relative coordinate rel (each in
 * [0, 8]): group_of[i] (0 = inside the block), above[g] (1 above, 0 below, -1 inside group). */
void so_dual_groups(const int32_t rel[3], int32_t group_of[8], int32_t above[8], int32_t* n_groups)
{
    const int r[3] = {rel[0], rel[1], rel[2]};
    const dual_mc::Groups g = dual_mc::dual_groups(r, kBlockSize);
    for (int i = 0; i < 8; ++i) {
        group_of[i] = g.group_of[i];
        above[i] = i < g.n_groups ? g.above[i] : -1;
    }
    *n_groups = g.n_groups;
}

int so_map_aabb(const so_map* map, int32_t mn[3], int32_t mx[3])
{
    const Octree& oct = map->octree;
    if (oct.aabb_empty)
        return 0;
    for (int i = 0; i < 3; ++i) {
        mn[i] = oct.aabb_min[i];
        mx[i] = oct.aabb_max[i];
    }
    return 1;
}

void so_map_set_block(so_map* map, const int32_t c[3], const float* tsdf512, const float* weight512)
{
    if (map->octree.multires)
        return;
    int o;
    map->octree.allocate_key(encode_key(c[0], c[1], c[2], 0), o);
    BlockData& b = map->octree.blocks[map->octree.octants[o].block];
    if (tsdf512)
        std::memcpy(b.tsdf, tsdf512, sizeof(float) * kBlockVoxels);
    if (weight512)
        std::memcpy(b.weight, weight512, sizeof(float) * kBlockVoxels);
}

/* Test set-up of a multi-res map: allocates the block holding voxel c and sets its data
 * pyramid (585 entries each, NULL keeps the default), its past data to the same values, and its
 * current and minimum scales. */
void so_map_set_mr_block(so_map* map, const int32_t c[3], const float* tsdf585, const float* weight585,
                         int current_scale, int min_scale)
{
    if (!map->octree.multires)
        return;
    int o;
    map->octree.allocate_key(encode_key(c[0], c[1], c[2], 0), o);
    MRBlock& b = map->octree.mr[(size_t) map->octree.octants[(size_t) o].block];
    if (tsdf585) {
        std::memcpy(b.tsdf, tsdf585, sizeof(float) * kMrVoxels);
        std::memcpy(b.past_tsdf, tsdf585, sizeof(float) * kMrVoxels);
    }
    if (weight585) {
        std::memcpy(b.weight, weight585, sizeof(float) * kMrVoxels);
        std::memcpy(b.past_weight, weight585, sizeof(float) * kMrVoxels);
    }
    b.current_scale = current_scale;
    b.min_scale = min_scale;
}

int so_map_get_data(const so_map* map, const float p[3], float* tsdf, float* weight)
{
    float t, w;
    if (map->octree.multires)
        map_get_data_mr(*map, v3(p[0], p[1], p[2]), t, w);
    else
        map_get_data(*map, v3(p[0], p[1], p[2]), t, w);
    *tsdf = t;
    *weight = w;
    return w != 0.0f;
}

int so_map_get_field_interp(const so_map* map, const float p[3], float* value)
{
    float v;
    const V3 q = v3(p[0], p[1], p[2]);
    if (!(map->octree.multires ? map_field_interp_mr(*map, q, v, nullptr) : map_field_interp(*map, q, v)))
        return 0;
    *value = v;
    return 1;
}

int so_map_get_field_grad(const so_map* map, const float p[3], float grad[3])
{
    V3 g;
    const V3 q = v3(p[0], p[1], p[2]);
    if (!(map->octree.multires ? map_field_grad_mr(*map, q, g) : map_field_grad(*map, q, g)))
        return 0;
    grad[0] = g.x;
    grad[1] = g.y;
    grad[2] = g.z;
    return 1;
}

int so_first_block_tmin(const so_map* map, const float o[3], const float d[3], float t_near,
                        float t_far, float* tcmin)
{
    const RayBlockHit r =
        first_block_on_ray(*map, v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2]), t_near, t_far);
    *tcmin = r.tcmin;
    return r.found ? 1 : 0;
}

void so_render_depth_f64(const so_map* map, const so_pinhole* sensor, const double T_WS[16], double* depth)
{
    const int W = sensor->width, H = sensor->height;
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            const RayD r = ray_d(*sensor, T_WS, x, y);
            double t;
            TriD q;
            depth[(size_t) x + (size_t) y * W] =
                diff_hit_d(*map, r.o, r.d, r.t_near, r.t_far, t, q) ? t * r.nz : 0.0;
        }
    }
}

void so_raycast_adjoint_f64(const so_map* map, const so_pinhole* sensor, const double T_WS[16],
                            const double* grad_depth, double twist_grad[6], double* voxel_grad, double* jac)
{
    const so_map& m = *map;
    const int W = sensor->width, H = sensor->height;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    std::vector<int> block_of_octant;
    if (voxel_grad) {
        block_of_octant.assign(m.octree.octants.size(), -1);
        for (size_t i = 0; i < m.octree.block_octant.size(); ++i)
            block_of_octant[m.octree.block_octant[i]] = (int) i;
    }
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            const size_t i = (size_t) x + (size_t) y * W;
            double row[6] = {0, 0, 0, 0, 0, 0};
            const double gd = grad_depth ? grad_depth[i] : 0.0;
            if (gd != 0.0 || jac) {
                const RayD r = ray_d(*sensor, T_WS, x, y);
                double t;
                TriD q;
                if (diff_hit_d(m, r.o, r.d, r.t_near, r.t_far, t, q)) {
                    const D3 g = tri_grad_world_d(m, q);
                    const double den = ddot(g, r.d);
                    if (std::fabs(den) > 1e-12) {
                        const D3 p = dadd(r.o, dmul(r.d, t));
                        const D3 pg = dcross(p, g);
                        const double k = -r.nz / den;
                        row[0] = k * g.x;
                        row[1] = k * g.y;
                        row[2] = k * g.z;
                        row[3] = k * pg.x;
                        row[4] = k * pg.y;
                        row[5] = k * pg.z;
                        for (int j = 0; j < 6; ++j)
                            acc[j] += gd * row[j];
                        if (voxel_grad && gd != 0.0) {
                            const D3 tt = q.t, tc = d3(1.0 - tt.x, 1.0 - tt.y, 1.0 - tt.z);
                            for (int n = 0; n < 8; ++n) {
                                const double w = ((n & 1) ? tt.x : tc.x) * (((n >> 1) & 1) ? tt.y : tc.y)
                                    * ((n >> 2) ? tt.z : tc.z);
                                voxel_grad[(size_t) block_of_octant[q.oct[n]] * kBlockVoxels + q.vi[n]] += gd * k * w;
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
    for (int j = 0; j < 6; ++j)
        twist_grad[j] = acc[j];
}

void so_map_set_voxel(so_map* map, const int32_t c[3], float tsdf, float weight)
{
    const int o = map->octree.block_at(c);
    if (o < 0 || map->octree.multires)
        return;
    const Octant& oc = map->octree.octants[o];
    BlockData& b = map->octree.blocks[oc.block];
    const int vi = (c[0] - oc.coord[0]) + 8 * (c[1] - oc.coord[1]) + 64 * (c[2] - oc.coord[2]);
    b.tsdf[vi] = tsdf;
    b.weight[vi] = weight;
}

uint64_t so_expand(uint64_t value) { return morton_expand(value); }
uint64_t so_compact(uint64_t value) { return morton_compact(value); }
uint64_t so_encode_code(int32_t x, int32_t y, int32_t z) { return encode_code(x, y, z); }
void so_decode_code(uint64_t code, int32_t coord[3])
{
    int c[3];
    decode_code(code, c);
    coord[0] = c[0];
    coord[1] = c[1];
    coord[2] = c[2];
}
int so_encode_key(int32_t x, int32_t y, int32_t z, uint64_t scale, uint64_t* key)
{
    const uint64_t detailed = encode_code(x, y, z);
    const uint64_t code = detailed & kCodeMask[scale];
    *key = (code << kScaleOffset) | scale;
    return detailed == code;
}
void so_decode_key(uint64_t key, int32_t coord[3], uint64_t* scale)
{
    *scale = key_to_scale(key);
    so_decode_code(key_to_code(key), coord);
}
uint64_t so_code_to_child_idx(uint64_t code, uint64_t child_scale)
{
    return (code >> (child_scale * 3)) & 7;
}
uint64_t so_parent_key(uint64_t key)
{
    const uint64_t ps = key_to_scale(key) + 1;
    return (key & (kCodeMask[ps] << kScaleOffset)) | ps;
}
int so_key_at_scale(uint64_t key, uint64_t scale, uint64_t* out)
{
    return key_at_scale(key, scale, *out) ? 1 : 0;
}
int so_code_at_scale(uint64_t key, uint64_t scale, uint64_t* out)
{
    *out = key_to_code(key) & kCodeMask[scale];
    return key_to_scale(key) <= scale;
}
uint64_t so_block_key(uint64_t key, uint64_t max_block_scale)
{
    return block_key_of(key, max_block_scale);
}
uint64_t so_block_code(uint64_t key, uint64_t max_block_scale)
{
    return key_to_code(key) & kCodeMask[max_block_scale];
}
int so_is_child(uint64_t parent_key, uint64_t child_key)
{
    return is_child_key(parent_key, child_key) ? 1 : 0;
}
int so_is_siblings(uint64_t a, uint64_t b)
{
    const uint64_t sa = key_to_scale(a), sb = key_to_scale(b);
    if (sa != sb)
        return 0;
    const uint64_t ps = sa + 1;
    return ((key_to_code(a) & kCodeMask[ps]) ^ (key_to_code(b) & kCodeMask[ps])) == 0;
}
long long so_unique_keys(uint64_t* keys, long long n, uint64_t* out)
{
    if (n == 0)
        return 0;
    std::sort(keys, keys + n);
    long long m = 0;
    out[m++] = keys[0];
    for (long long i = 0; i < n; ++i)
        if (out[m - 1] != keys[i])
            out[m++] = keys[i];
    return m;
}
long long so_unique_codes(uint64_t* keys, long long n, uint64_t* out)
{
    if (n == 0)
        return 0;
    std::sort(keys, keys + n);
    long long m = 0;
    out[m++] = keys[0];
    for (long long i = 0; i < n; ++i) {
        if (key_to_code(out[m - 1]) != key_to_code(keys[i]))
            out[m++] = keys[i];
        else if (key_to_scale(out[m - 1]) > key_to_scale(keys[i]))
            out[m - 1] = keys[i];
    }
    return m;
}
long long so_unique_allocation(uint64_t* keys, long long n, uint64_t max_block_scale, uint64_t* out)
{
    if (n == 0)
        return 0;
    std::sort(keys, keys + n);
    long long m = 0;
    out[m++] = block_key_of(keys[0], max_block_scale);
    for (long long i = 0; i < n; ++i) {
        const uint64_t bk = block_key_of(keys[i], max_block_scale);
        if (is_child_key(out[m - 1], bk))
            out[m - 1] = bk;
        else if (out[m - 1] != bk)
            out[m++] = bk;
    }
    return m;
}
long long so_unique_at_scale(uint64_t* keys, long long n, uint64_t scale, uint64_t* out)
{
    if (n == 0)
        return 0;
    std::sort(keys, keys + n);
    long long m = 0;
    long long restart = 1;
    uint64_t k;
    for (long long i = 0; i < n; ++i) {
        if (key_at_scale(keys[i], scale, k)) {
            out[m++] = k;
            break;
        }
        ++restart;
    }
    for (long long i = restart; i < n; ++i) {
        if (key_at_scale(keys[i], scale, k) && out[m - 1] != k)
            out[m++] = k;
    }
    return m;
}

void so_se3_exp(const float twist[6], float T[16]) { tf_to16(se3_exp(twist), T); }

/* spatial weights of the bilateral window, (2r+1)^2 floats: exp(-(dx^2 + dy^2) / (2 s^2)) in
 * double, rounded to float */
void so_bilateral_weights(int radius, float sigma_space, float* ws)
{
    const int n = 2 * radius + 1;
    for (int dy = -radius; dy <= radius; ++dy)
        for (int dx = -radius; dx <= radius; ++dx)
            ws[(dy + radius) * n + (dx + radius)] =
                (float) std::exp(-(double) (dx * dx + dy * dy) / (2.0 * (double) sigma_space * (double) sigma_space));
}

void so_bilateral_filter(const float* in, int w, int h, int radius, float sigma_space, float sigma_range, float* out)
{
    std::vector<float> ws((size_t) (2 * radius + 1) * (2 * radius + 1));
    so_bilateral_weights(radius, sigma_space, ws.data());
    const float k = 1.0f / (2.0f * sigma_range * sigma_range);
#pragma omp parallel for
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
            out[x + y * w] = bilateral_pixel(in, w, h, x, y, radius, ws.data(), k);
}

float so_exp_cw(float x) { return exp_cw(x); }

/* preprocessor::downsample_depth (src/map/preprocessor.cpp:19-84): per output pixel the median
 * (the upper middle element for an even count) of the region's depths >= 1e-5, or 0 with the
 * region's first pixel when none is valid; map = the chosen input pixel x + y * w_in. The
 * reference sorts with std::sort, which leaves the order of equal depths unspecified; here they
 * keep their region scan order (stable sort), the order the GPU uses too. */
void so_downsample_depth(const float* in, int w_in, int h_in, float* out, int w_out, int h_out, int64_t* map)
{
    const int ratio = w_in / w_out;
    (void) h_in;
#pragma omp parallel for
    for (int y_out = 0; y_out < h_out; ++y_out) {
        std::vector<std::pair<float, int64_t>> region;
        region.reserve((size_t) ratio * ratio);
        for (int x_out = 0; x_out < w_out; ++x_out) {
            const int xb = x_out * ratio, yb = y_out * ratio;
            region.clear();
            for (int yr = 0; yr < ratio; ++yr)
                for (int xr = 0; xr < ratio; ++xr) {
                    const int x = xb + xr, y = yb + yr;
                    const float d = in[x + (size_t) y * w_in];
                    if (d >= 1e-5f)
                        region.push_back({d, (int64_t) x + (int64_t) y * w_in});
                }
            const size_t o = (size_t) x_out + (size_t) y_out * w_out;
            if (region.empty()) {
                out[o] = 0.0f;
                if (map)
                    map[o] = (int64_t) xb + (int64_t) yb * w_in;
                continue;
            }
            std::stable_sort(region.begin(), region.end(),
                             [](const std::pair<float, int64_t>& a, const std::pair<float, int64_t>& b) {
                                 return a.first < b.first;
                             });
            const auto& v = region[region.size() / 2];
            out[o] = v.first;
            if (map)
                map[o] = v.second;
        }
    }
}

void so_half_sample_robust(const float* in, int w, int h, float e_d, int radius, float* out)
{
    half_sample_robust(in, w, h, e_d, radius, out);
}
void so_depth_to_point_cloud(const float* depth, const so_pinhole* sensor, float* pts)
{
    depth_to_points(depth, make_pinhole(sensor), reinterpret_cast<V3*>(pts));
}
void so_point_cloud_to_normal(const float* pts, int w, int h, int neg_y, float* nrm)
{
    points_to_normals(reinterpret_cast<const V3*>(pts), w, h, neg_y != 0, reinterpret_cast<V3*>(nrm));
}

/* The tracker's input pyramid exactly as so_track forms it (tracker_impl.hpp:30-60): level l
 * (l < levels) is (W >> l) x (H >> l); depth_out, pts_out and nrm_out hold the levels one after
 * another (level 0's depth is the input itself). */
void so_tracker_pyramid(const so_pinhole* sensor_c, const float* depth, int levels, float* depth_out,
                        float* pts_out, float* nrm_out)
{
    const Pinhole s = make_pinhole(sensor_c);
    const int L = std::min(std::max(levels, 1), 3);
    size_t off = 0;
    std::memcpy(depth_out, depth, sizeof(float) * (size_t) s.w * s.h);
    for (int i = 0; i < L; ++i) {
        const int w = s.w / (1 << i), h = s.h / (1 << i);
        if (i > 0) {
            const int pw = s.w / (1 << (i - 1)), ph = s.h / (1 << (i - 1));
            half_sample_robust(depth_out + off - (size_t) pw * ph, pw, ph, 0.1f * 3.0f, 1, depth_out + off);
        }
        const Pinhole si = downsampled(s, (float) (1 << i));
        depth_to_points(depth_out + off, si, reinterpret_cast<V3*>(pts_out + 3 * off));
        points_to_normals(reinterpret_cast<const V3*>(pts_out + 3 * off), si.w, si.h, s.left_hand,
                          reinterpret_cast<V3*>(nrm_out + 3 * off));
        off += (size_t) w * h;
    }
}

} /* extern "C" */
