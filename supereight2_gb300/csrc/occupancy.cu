// occupancy.cu — multi-resolution occupancy maps (Map<Data<Occupancy>, Res::Multi, 8>): the
// map's pools (creation, destruction, checks, downloads) and the raycast over the octree
// (raycaster_impl.hpp:32-452). Integration lives in occ_integrate.cu.
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "occupancy.cuh"
#include "pipeline.cuh"
#include "profile.cuh"

namespace se_gpu {

// ----------------------------------------------------------------- queries / raycast --

// fetcher::finest_octant (fetcher_impl.hpp:69-94) as a slot: the octant of size max(2^scale, 8)
// on the voxel's path, the deepest node when it has no children, or -1.
__device__ int occ_finest_octant(const OccDevice& m, int x, int y, int z, int scale_desired)
{
    const int size_desired = max(1 << scale_desired, 8);
    int n = 0, child = -1;
    for (int cs = m.size >> 1; cs >= size_desired; cs >>= 1) {
        const int idx = ((x & cs) > 0) + 2 * ((y & cs) > 0) + 4 * ((z & cs) > 0);
        child = m.node_child[8 * (size_t) n + idx];
        if (child == -1)
            return node_is_leaf(m, n) ? n : -1;
        if (slot_is_block(child))
            return child;
        n = child;
    }
    return child;
}

__device__ __forceinline__ int blk_voxel_idx(const OccDevice& m, int b, int x, int y, int z, int s)
{
    return occ_voxel_idx(x - m.block_coord[3 * b], y - m.block_coord[3 * b + 1], z - m.block_coord[3 * b + 2], s);
}

// visitor::getMaxData (visitor_impl.hpp:815-835)
__device__ OccD occ_max_data(const OccDevice& m, int x, int y, int z, int scale_desired)
{
    const int slot = occ_finest_octant(m, x, y, z, scale_desired);
    if (slot == -1)
        return occ_default();
    if (slot_is_block(slot)) {
        const int b = slot_block(slot);
        const OccBlockState& st = m.block_state[b];
        const int so = max(scale_desired, st.current_scale);
        return blk_max(m, b, st.finest, so)[blk_voxel_idx(m, b, x, y, z, so)];
    }
    return m.node_max[slot];
}

// visitor::getData(octree, voxel): a block's data at its current scale, a leaf node's data
__device__ OccD occ_get_data_voxel(const OccDevice& m, int x, int y, int z)
{
    const int slot = occ_leaf(m, x, y, z);
    if (slot == -1)
        return occ_default();
    if (slot_is_block(slot)) {
        const int b = slot_block(slot);
        const OccBlockState& st = m.block_state[b];
        return blk_mean(m, b, st.current_scale)[blk_voxel_idx(m, b, x, y, z, st.current_scale)];
    }
    return node_data(m, slot);
}

__device__ __forceinline__ F3 occ_to_voxel_f(const OccDevice& m, F3 p_W)
{
    const F3 p = apply(m.T_MW, p_W);
    return f3(p.x / m.res, p.y / m.res, p.z / m.res);
}

// Map::getData (Safe::Off)
__device__ __forceinline__ OccD occ_get_data(const OccDevice& m, F3 p_W)
{
    const F3 v = occ_to_voxel_f(m, p_W);
    return occ_get_data_voxel(m, (int) v.x, (int) v.y, (int) v.z);
}

__device__ __forceinline__ OccD occ_block_data_at(const OccDevice& m, int b, int x, int y, int z, int s)
{
    const OccBlockState& st = m.block_state[b];
    if (s < st.finest)
        return st.init_data;
    return blk_mean(m, b, s)[blk_voxel_idx(m, b, x, y, z, s)];
}

// visitor::getInterp multi-res with get_neighbours on an occupancy octree (leaf nodes take part)
__device__ bool occ_interp(const OccDevice& m, F3 vf, int desired_scale, float& out, int* returned_scale)
{
    const int q = occ_leaf(m, (int) vf.x, (int) vf.y, (int) vf.z);
    if (q == -1)
        return false;
    const bool q_block = slot_is_block(q);
    const int init = q_block ? max(m.block_state[slot_block(q)].current_scale, desired_scale) : 0;
#pragma unroll 1
    for (int scale = init; scale <= kOccMaxScale; ++scale) {
        const int stride = 1 << scale;
        const float inv = 1.0f / (float) stride;
        const F3 bf = f3(inv * vf.x - 0.5f, inv * vf.y - 0.5f, inv * vf.z - 0.5f);
        const int b0 = stride * (int) bf.x, b1 = stride * (int) bf.y, b2 = stride * (int) bf.z;
        if (m.aabb[6])
            return false;
        if (b0 < m.aabb[0] || b1 < m.aabb[1] || b2 < m.aabb[2] || b0 > m.aabb[3] || b1 > m.aabb[4] || b2 > m.aabb[5])
            return false;
        if (b0 + stride >= m.size || b1 + stride >= m.size || b2 + stride >= m.size || b0 < 0 || b1 < 0 || b2 < 0)
            continue;
        float f[8];
        bool ok = true, valid = true;
#pragma unroll 1
        for (int n = 0; n < 8; ++n) {
            const int cx = b0 + stride * (n & 1), cy = b1 + stride * ((n >> 1) & 1), cz = b2 + stride * (n >> 2);
            const int slot = occ_leaf(m, cx, cy, cz);
            if (slot == -1) {
                ok = false;
                break;
            }
            OccD d;
            if (slot_is_block(slot)) {
                const int b = slot_block(slot);
                if (m.block_state[b].current_scale > scale) {
                    ok = false;
                    break;
                }
                d = occ_block_data_at(m, b, cx, cy, cz, scale);
            }
            else {
                d = node_data(m, slot);
            }
            valid = valid && occ_valid(d);
            f[n] = occ_field(d);
        }
        if (!ok)
            continue;
        if (!valid)
            return false;
        if (returned_scale)
            *returned_scale = q_block ? scale : (31 - __clz(m.node_coord[q].w));
        const F3 t = f3(bf.x - floorf(bf.x), bf.y - floorf(bf.y), bf.z - floorf(bf.z));
        const F3 tc = f3(1.0f - t.x, 1.0f - t.y, 1.0f - t.z);
        out = ((f[0] * tc.x + f[1] * t.x) * tc.y + (f[2] * tc.x + f[3] * t.x) * t.y) * tc.z
            + ((f[4] * tc.x + f[5] * t.x) * tc.y + (f[6] * tc.x + f[7] * t.x) * t.y) * t.z;
        return true;
    }
    return false;
}

static __constant__ unsigned char kOccGradSel[32] = {
    0x14, 0x18, 0x24, 0x28, 0x11, 0x21, 0x05, 0x15, 0x25, 0x35, 0x09, 0x19, 0x29, 0x39, 0x1d, 0x2d,
    0x12, 0x22, 0x06, 0x16, 0x26, 0x36, 0x0a, 0x1a, 0x2a, 0x3a, 0x1e, 0x2e, 0x17, 0x1b, 0x27, 0x2b};

// visitor::getFieldGrad multi-res, desired scale 0 (visitor_impl.hpp:1257-1497), occupancy
__device__ bool occ_grad(const OccDevice& m, F3 vf, F3& g)
{
    const int q = occ_finest_octant(m, (int) vf.x, (int) vf.y, (int) vf.z, 0);
    if (q == -1)
        return false;
    if (!slot_is_block(q)) {
        if (occ_valid(node_data(m, q))) {
            g = f3(0.0f, 0.0f, 0.0f);
            return true;
        }
        return false;
    }
    const int qc = m.block_state[slot_block(q)].current_scale;
    const int init = qc > 0 ? qc : 0;
    const int top = m.size - 1;
#pragma unroll 1
    for (int scale = init; scale <= kOccMaxScale; ++scale) {
        const int stride = 1 << scale;
        const float inv = 1.0f / (float) stride;
        const F3 sv = f3(inv * vf.x - 0.5f, inv * vf.y - 0.5f, inv * vf.z - 0.5f);
        const F3 fac = f3(sv.x - floorf(sv.x), sv.y - floorf(sv.y), sv.z - floorf(sv.z));
        const int base[3] = {stride * (int) sv.x, stride * (int) sv.y, stride * (int) sv.z};
        int sel[3][4];
        for (int i = 0; i < 3; ++i) {
            sel[i][0] = max(base[i] - stride, 0);
            sel[i][1] = max(base[i], 0);
            sel[i][2] = min(base[i] + stride, top);
            sel[i][3] = min(base[i] + 2 * stride, top);
        }
        const int oct = occ_finest_octant(m, base[0], base[1], base[2], scale);
        if (oct == -1)
            continue;
        if (!slot_is_block(oct)) {
            if (node_is_leaf(m, oct) && occ_valid(node_data(m, oct))) {
                g = f3(0.0f, 0.0f, 0.0f);
                return true;
            }
            continue;
        }
        const int hb = slot_block(oct);
        const int hx = m.block_coord[3 * hb], hy = m.block_coord[3 * hb + 1], hz = m.block_coord[3 * hb + 2];
        float v[32];
        bool ok = true;
#pragma unroll 1
        for (int i = 0; i < 32; ++i) {
            const unsigned code = kOccGradSel[i];
            const int cx = sel[0][code & 3], cy = sel[1][(code >> 2) & 3], cz = sel[2][(code >> 4) & 3];
            int slot = oct;
            if (!(cx >= hx && cx <= hx + 7 && cy >= hy && cy <= hy + 7 && cz >= hz && cz <= hz + 7))
                slot = occ_leaf(m, cx, cy, cz);
            if (slot == -1) {
                ok = false;
                break;
            }
            OccD d;
            int rs;
            if (slot_is_block(slot)) {
                const int b = slot_block(slot);
                const OccBlockState& st = m.block_state[b];
                rs = max(scale, st.current_scale);
                d = blk_mean(m, b, rs)[blk_voxel_idx(m, b, cx, cy, cz, rs)];
            }
            else {
                rs = scale;
                d = node_data(m, slot);
            }
            if (!occ_valid(d) || rs != scale) {
                ok = false;
                break;
            }
            v[i] = occ_field(d);
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

__device__ __forceinline__ bool occ_contains(const OccDevice& m, F3 p_W)
{
    const F3 p = apply(m.T_MW, p_W);
    return p.x >= 0.0f && p.x < m.dim && p.y >= 0.0f && p.y < m.dim && p.z >= 0.0f && p.z < m.dim;
}

// find_valid_point (raycaster_impl.hpp:32-70)
__device__ bool occ_find_valid_point(const OccDevice& m, F3 o, F3 d, float step, float t_max, float& t, F3& point_W,
                                     float& value)
{
    bool has = false;
    F3 p = add(o, mul(t, d));
    if (occ_contains(m, p) && occ_valid(occ_get_data(m, p)))
        has = occ_interp(m, occ_to_voxel_f(m, p), 0, value, nullptr);
#pragma unroll 1
    while (!has) {
        t += step;
        if (t > t_max)
            return false;
        p = add(o, mul(t, d));
        if (occ_contains(m, p) && occ_valid(occ_get_data(m, p)))
            has = occ_interp(m, occ_to_voxel_f(m, p), 0, value, nullptr);
    }
    point_W = p;
    return true;
}

// compute_map_intersection (raycaster_impl.hpp:85-173)
__device__ float occ_map_intersection(const OccDevice& m, F3 pos_W, F3 dir_W, float t_far, bool& valid)
{
    const F3 p = apply(m.T_MW, pos_W), dr = rot(m.T_MW, dir_W);
    const float pm[3] = {p.x, p.y, p.z}, dm[3] = {dr.x, dr.y, dr.z};
    const float mx = m.dim;
    bool inside = true;
    int quadrant[3];
    float cand[3] = {0.0f, 0.0f, 0.0f}, maxT[3];
    for (int i = 0; i < 3; ++i) {
        if (pm[i] < 0.0f) {
            quadrant[i] = 1;
            cand[i] = 0.0f;
            inside = false;
        }
        else if (pm[i] > mx) {
            quadrant[i] = 0;
            cand[i] = mx;
            inside = false;
        }
        else {
            quadrant[i] = 2;
        }
    }
    if (inside)
        return 0.0f;
    for (int i = 0; i < 3; ++i)
        maxT[i] = (quadrant[i] != 2 && dm[i] != 0.0f) ? (cand[i] - pm[i]) / dm[i] : -1.0f;
    int which = 0;
    for (int i = 1; i < 3; ++i)
        if (maxT[which] < maxT[i])
            which = i;
    if (maxT[which] < 0.0f) {
        valid = false;
        return 0.0f;
    }
    float hit[3];
    for (int i = 0; i < 3; ++i) {
        if (which != i) {
            hit[i] = pm[i] + maxT[which] * dm[i];
            if (hit[i] < 0.0f || hit[i] > mx) {
                valid = false;
                return 0.0f;
            }
        }
        else {
            hit[i] = cand[i];
        }
    }
    const F3 dh = f3(hit[0] - pm[0], hit[1] - pm[1], hit[2] - pm[2]);
    const float t = sqrtf(dot(dh, dh));
    if (t_far < t) {
        valid = false;
        return 0.0f;
    }
    return t;
}

__device__ __forceinline__ float occ_max_field(const OccDevice& m, F3 c, int s)
{
    return occ_field(occ_max_data(m, (int) c.x, (int) c.y, (int) c.z, s));
}

// advance_ray (raycaster_impl.hpp:189-338)
__device__ void occ_advance_ray(const OccDevice& m, F3 o, F3 d, float& t, float& t_far, int max_scale, bool& valid)
{
    const float voxel_dim = m.res;
    int scale = max_scale;
    float v_add = 0.0f;
    const float v = 1.0f / voxel_dim * t;
    float v_far = 1.0f / voxel_dim * t_far;
    F3 oc = f3(-1.0f, -1.0f, -1.0f);
    if (occ_contains(m, o))
        oc = occ_to_voxel_f(m, o);
    const float sz = (float) m.size;
    const float dv[3] = {d.x, d.y, d.z};
    const float ocv[3] = {oc.x, oc.y, oc.z};
    float vmap[3];
    for (int i = 0; i < 3; ++i) {
        const float dvm = sz / fabsf(dv[i]);
        const float frac = ocv[i] / sz;
        vmap[i] = dv[i] < 0 ? frac * dvm : (1 - frac) * dvm;
    }
    v_far = fminf(fminf(fminf(vmap[0], vmap[1]), vmap[2]) + v, v_far);
    t_far = voxel_dim * v_far;
    float f = occ_max_field(m, oc, scale);
    while (f > -0.2f && scale > 2) {
        scale -= 1;
        f = occ_max_field(m, oc, scale);
    }
    F3 rc = oc;
#pragma unroll 1
    for (int guard = 0; (v + v_add) < v_far && guard < (1 << 22); ++guard) {
        if (scale <= 2) {
            t = voxel_dim * (v + v_add - 4);
            return;
        }
        const int node_size = 1 << scale;
        const float rcv[3] = {rc.x, rc.y, rc.z};
        float Vmax[3];
        for (int i = 0; i < 3; ++i) {
            const int curr = node_size * (int) (floorf(rcv[i]) / (float) node_size);
            const float frac = (rcv[i] - (float) curr) / (float) node_size;
            const float dV = (float) node_size / fabsf(dv[i]);
            Vmax[i] = dv[i] < 0 ? frac * dV : (1 - frac) * dV;
            if (fabsf(dv[i]) < 1.0e-6f)
                Vmax[i] = __int_as_float(0x7f800000);
        }
        const float Vmin = fminf(fminf(Vmax[0], Vmax[1]), Vmax[2]);
        v_add = (float) ((double) v_add + ((double) Vmin + 0.01));
        rc = add(mul(v + v_add, d), oc);
        f = occ_max_field(m, rc, scale);
        if (f > -0.2f) {
            while (f > -0.2f && scale > 2) {
                scale -= 1;
                f = occ_max_field(m, rc, scale);
            }
        }
        else {
            for (int s = scale + 1; s <= max_scale; s++) {
                f = occ_max_field(m, rc, s);
                if (f > -0.2f)
                    break;
                scale += 1;
            }
        }
    }
    valid = false;
}

// raycast<Occupancy> (raycaster_impl.hpp:352-452)
__device__ bool occ_raycast(const OccDevice& m, F3 o, F3 d, float t_far, F3& hit, int& scale_out)
{
    bool valid = true;
    float t = occ_map_intersection(m, o, d, t_far, valid);
    if (!valid)
        return false;
    const int max_scale = min(7, m.log2_size - 1);
    occ_advance_ray(m, o, d, t, t_far, max_scale, valid);
    if (!valid)
        return false;
    const float step = m.res / 2;
    float value_t = 0.0f, value_tt = 0.0f;
    bool has_tt = false;
    F3 pt = f3(0.0f, 0.0f, 0.0f), ptt = f3(0.0f, 0.0f, 0.0f);
    int scale_tt = 0;
    if (!occ_find_valid_point(m, o, d, step, t_far, t, pt, value_t))
        return false;
    t += step;
    if (value_t <= 0.0f) {
#pragma unroll 1
        for (; t < t_far; t += step) {
            const F3 p = add(o, mul(d, t));
            const OccD data = occ_get_data(m, p);
            if (!occ_valid(data)) {
                t += step;
                if (!occ_find_valid_point(m, o, d, step, t_far, t, pt, value_t)) {
                    hit = f3(0.0f, 0.0f, 0.0f);
                    scale_out = 0;
                    return true;
                }
                if (value_t > 0.0f)
                    break;
                continue;
            }
            value_tt = occ_field(data);
            has_tt = true;
            ptt = p;
            if (value_tt > -0.2f) {
                float vi;
                int sc = scale_tt;
                if (occ_interp(m, occ_to_voxel_f(m, p), 0, vi, &sc)) {
                    value_tt = vi;
                    scale_tt = sc;
                }
                else {
                    has_tt = false;
                    t += step;
                    if (!occ_find_valid_point(m, o, d, step, t_far, t, pt, value_t))
                        return false;
                    if (value_t > 0.0f)
                        break;
                    continue;
                }
            }
            if (value_tt > 0.0f)
                break;
            value_t = value_tt;
            pt = ptt;
        }
        if (has_tt && value_tt > 0.0f && value_t < 0.0f) {
            const F3 dd = sub(ptt, pt);
            t = t - sqrtf(dot(dd, dd)) * (value_tt - 0.0f) / (value_tt - value_t);
            hit = add(o, mul(d, t));
            scale_out = scale_tt;
            return true;
        }
    }
    return false;
}

// raycaster::raycast_volume for occupancy maps: normals are -normalize(grad F)
__global__ void __launch_bounds__(128) occ_raycast_kernel(OccDevice m, Pinhole s, Tf T_WS, float* __restrict__ pts,
                                                          float* __restrict__ nrm, int8_t* __restrict__ scale)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
    if (x >= s.w || y >= s.h)
        return;
    const size_t idx = (size_t) x + (size_t) y * s.w;
    const F3 ray_S = back_project(s, (float) x, (float) y);
    const F3 nS = normalized(ray_S);
    const F3 dir_W = rot(T_WS, nS);
    const F3 origin = f3(T_WS.t[0], T_WS.t[1], T_WS.t[2]);
    F3 hit, p = f3(0.0f, 0.0f, 0.0f), n = f3(0.0f, 0.0f, 0.0f);
    int sc = 0;
    if (occ_raycast(m, origin, dir_W, s.far_plane / nS.z, hit, sc)) {
        p = hit;
        F3 g;
        if (occ_grad(m, occ_to_voxel_f(m, hit), g)) {
            g = f3(g.x / m.res, g.y / m.res, g.z / m.res);
            const float nn = sqrtf(dot(g, g));
            n = nn > 0.0f ? f3(-(g.x / nn), -(g.y / nn), -(g.z / nn)) : f3(-g.x, -g.y, -g.z);
        }
    }
    else {
        sc = 0;
    }
    pts[3 * idx + 0] = p.x;
    pts[3 * idx + 1] = p.y;
    pts[3 * idx + 2] = p.z;
    nrm[3 * idx + 0] = n.x;
    nrm[3 * idx + 1] = n.y;
    nrm[3 * idx + 2] = n.z;
    if (scale)
        scale[idx] = (int8_t) sc;
}

se_gpu_status occ_raycast_volume(const se_gpu_occ_map* om, const se_gpu_pinhole& sensor, const float* T_WS16,
                                 float* pts, float* nrm, int8_t* scale, cudaStream_t stream)
{
    const Pinhole s = make_pinhole(sensor);
    dim3 grid((s.w + 15) / 16, (s.h + 7) / 8);
    ProfScope ps(kProfRaycast, stream);
    occ_raycast_kernel<<<grid, 128, 0, stream>>>(om->dev, s, tf_from16(T_WS16), pts, nrm, scale);
    SE_CUDA_TRY(cudaGetLastError());
    return SE_GPU_OK;
}

} // namespace se_gpu

using namespace se_gpu;

namespace se_gpu {

se_gpu_status occ_map_create(const se_gpu_map_config* cfg, const se_gpu_occupancy_config* occ, int size,
                             se_gpu_occ_map** out)
{
    se_gpu_occ_map* om = new se_gpu_occ_map();
    std::memset(&om->dev, 0, sizeof(om->dev));
    om->scratch = OccScratch();
    OccDevice& m = om->dev;
    m.size = size;
    m.log2_size = 0;
    while ((1 << m.log2_size) < size)
        ++m.log2_size;
    m.block_depth = m.log2_size - 3;
    m.res = cfg->res;
    m.dim = (float) size * cfg->res;
    if (cfg->has_T_MW) {
        m.T_MW = tf_from16(cfg->T_MW);
    }
    else {
        for (int i = 0; i < 9; ++i)
            m.T_MW.R[i] = (i % 4 == 0) ? 1.0f : 0.0f;
        m.T_MW.t[0] = cfg->dim[0] / 2.0f;
        m.T_MW.t[1] = cfg->dim[1] / 2.0f;
        m.T_MW.t[2] = cfg->dim[2] / 2.0f;
    }
    m.T_WM = inverse_iso(m.T_MW);
    se_gpu_occupancy_config c;
    if (occ) {
        c = *occ;
    }
    else {
        c.k_sigma = 0.052f;
        c.sigma_min_factor = 1.5f;
        c.sigma_max_factor = 6.0f;
        c.k_tau = 0.026f;
        c.tau_min_factor = 6.0f;
        c.tau_max_factor = 16.0f;
        c.log_odd_min = (float) -5.015;
        c.log_odd_max = (float) 5.015;
        c.fs_integr_scale = 1;
    }
    m.cfg.k_sigma = c.k_sigma;
    m.cfg.sigma_min_factor = c.sigma_min_factor;
    m.cfg.sigma_max_factor = c.sigma_max_factor;
    m.cfg.k_tau = c.k_tau;
    m.cfg.tau_min_factor = c.tau_min_factor;
    m.cfg.tau_max_factor = c.tau_max_factor;
    m.cfg.log_odd_min = c.log_odd_min;
    m.cfg.log_odd_max = c.log_odd_max;
    m.cfg.fs_integr_scale = c.fs_integr_scale;
    // FieldData<Occupancy>::Config::max_weight keeps its default (data_field.hpp:67): the YAML
    // reader does not recompute it from a configured log_odd_min
    m.cfg.max_weight = std::floor(std::fabs(-100.0f / (0.97f * (float) -5.015)));
    m.block_capacity = (int) cfg->max_blocks;
    // nodes per block stay below 0.3 in the tests' scenes; half the block capacity leaves margin
    m.node_capacity = (int) (cfg->max_blocks / 2 + 4096);
    auto fail = [&](cudaError_t e, const char* what) {
        se_gpu_status st = cuda_status(e, what);
        occ_map_destroy(om);
        return st;
    };
    cudaError_t e;
    const size_t nc = (size_t) m.node_capacity, bc = (size_t) m.block_capacity;
    if ((e = cudaMalloc(&m.node_coord, nc * sizeof(int4))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_parent, nc * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_child, nc * 8 * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_min, nc * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_max, nc * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_mark, nc * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.node_ts, nc * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(nodes)");
    if ((e = cudaMalloc(&m.block_coord, bc * 3 * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.block_state, bc * sizeof(OccBlockState))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.block_mean, bc * 585 * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.block_min, bc * 585 * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.block_max, bc * 585 * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.block_buffer, bc * 512 * sizeof(OccD))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.block_ts, bc * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(blocks)");
    if ((e = cudaMalloc(&m.aabb, 8 * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(aabb)");
    if ((e = cudaMalloc(&m.counters, kOccCounters * sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc(counters)");
    {
        const int aabb[8] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN, 1, 0};
        if ((e = cudaMemcpy(m.aabb, aabb, sizeof(aabb), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "aabb");
        if ((e = cudaMemset(m.counters, 0, kOccCounters * sizeof(int))) != cudaSuccess) return fail(e, "counters");
        // the root: node 0
        const int one = 1;
        if ((e = cudaMemcpy(m.counters + kOccNodes, &one, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(e, "counters");
        const int4 rc = make_int4(0, 0, 0, size);
        const int minus1[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
        const int rp = -1;
        const OccD def = occ_default();
        if ((e = cudaMemcpy(m.node_coord, &rc, sizeof(rc), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_parent, &rp, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_child, minus1, sizeof(minus1), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_min, &def, sizeof(def), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_max, &def, sizeof(def), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_mark, &rp, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
        if ((e = cudaMemcpy(m.node_ts, &rp, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "root");
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e, "cudaDeviceSynchronize");
    *out = om;
    return SE_GPU_OK;
}

void occ_map_destroy(se_gpu_occ_map* om)
{
    if (!om)
        return;
    OccDevice& m = om->dev;
    cudaFree(m.node_coord);
    cudaFree(m.node_parent);
    cudaFree(m.node_child);
    cudaFree(m.node_min);
    cudaFree(m.node_max);
    cudaFree(m.node_mark);
    cudaFree(m.node_ts);
    cudaFree(m.block_coord);
    cudaFree(m.block_state);
    cudaFree(m.block_mean);
    cudaFree(m.block_min);
    cudaFree(m.block_max);
    cudaFree(m.block_buffer);
    cudaFree(m.block_ts);
    cudaFree(m.aabb);
    cudaFree(m.counters);
    occ_scratch_free(om);
    ri_scratch_free(om->ri);
    delete om;
}

} // namespace se_gpu

namespace se_gpu {

se_gpu_status occ_check(se_gpu_occ_map* om)
{
    int err = 0;
    SE_CUDA_TRY(cudaMemcpy(&err, om->dev.counters + kOccError, sizeof(int), cudaMemcpyDeviceToHost));
    if (!err)
        return SE_GPU_OK;
    SE_CUDA_TRY(cudaMemset(om->dev.counters + kOccError, 0, sizeof(int)));
    if (err & kOccErrBlockPool) {
        set_last_error("occupancy block pool of %d blocks is full", om->dev.block_capacity);
        return SE_GPU_ERR_POOL_FULL;
    }
    if (err & kOccErrNodePool) {
        set_last_error("occupancy node pool of %d nodes is full", om->dev.node_capacity);
        return SE_GPU_ERR_POOL_FULL;
    }
    if (err & kOccErrTimeout) {
        set_last_error("a grid barrier of the persistent batch launch waited past its limit; the frame is incomplete");
        return SE_GPU_ERR_CUDA;
    }
    set_last_error("an occupancy work list overflowed");
    return SE_GPU_ERR_POOL_FULL;
}

se_gpu_status occ_aabb(const se_gpu_occ_map* om, int32_t mn[3], int32_t mx[3], int* empty)
{
    int a[8];
    SE_CUDA_TRY(cudaMemcpy(a, om->dev.aabb, sizeof(a), cudaMemcpyDeviceToHost));
    *empty = a[6];
    for (int i = 0; i < 3; ++i) {
        mn[i] = a[6] ? 0 : a[i];
        mx[i] = a[6] ? 0 : a[3 + i];
    }
    return SE_GPU_OK;
}

} // namespace se_gpu

static se_gpu_status occ_args(const se_gpu_map* map, const char* fn)
{
    if (!map) {
        set_last_error("%s: null map", fn);
        return SE_GPU_ERR_BAD_ARG;
    }
    if (!map->occ) {
        set_last_error("%s: not an occupancy map", fn);
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    return SE_GPU_OK;
}

extern "C" {

se_gpu_status se_gpu_map_occupancy_stats(se_gpu_map* map, int64_t stats[4])
{
    se_gpu_status st = occ_args(map, "se_gpu_map_occupancy_stats");
    if (st != SE_GPU_OK)
        return st;
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    int c[kOccCounters];
    SE_CUDA_TRY(cudaMemcpy(c, map->occ->dev.counters, sizeof(c), cudaMemcpyDeviceToHost));
    stats[0] = c[kOccBlockListN];
    stats[1] = c[kOccNodeListN];
    stats[2] = c[kOccFreedN];
    stats[3] = c[kOccPruned];
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_download_occupancy(const se_gpu_map* map, int64_t capacity, int32_t* coords, int32_t* scales,
                                            int64_t* counts, float* mean, float* min_data, float* max_data,
                                            int64_t* count)
{
    se_gpu_status st = occ_args(map, "se_gpu_map_download_occupancy");
    if (st != SE_GPU_OK)
        return st;
    if (capacity < 0) {
        set_last_error("se_gpu_map_download_occupancy: negative capacity");
        return SE_GPU_ERR_BAD_ARG;
    }
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    const OccDevice& m = map->occ->dev;
    int nb = 0;
    SE_CUDA_TRY(cudaMemcpy(&nb, m.counters + kOccBlocks, sizeof(int), cudaMemcpyDeviceToHost));
    nb = nb < m.block_capacity ? nb : m.block_capacity;
    std::vector<OccBlockState> states((size_t) nb);
    std::vector<int> bc((size_t) nb * 3);
    if (nb) {
        SE_CUDA_TRY(cudaMemcpy(states.data(), m.block_state, (size_t) nb * sizeof(OccBlockState), cudaMemcpyDeviceToHost));
        SE_CUDA_TRY(cudaMemcpy(bc.data(), m.block_coord, (size_t) nb * 3 * sizeof(int), cudaMemcpyDeviceToHost));
    }
    int64_t live = 0;
    for (int b = 0; b < nb; ++b)
        live += states[(size_t) b].live ? 1 : 0;
    if (count)
        *count = live;
    const bool want_data = mean || min_data || max_data;
    std::vector<OccD> hm, hn, hx;
    if (want_data && nb) {
        hm.resize((size_t) nb * 585);
        hn.resize((size_t) nb * 585);
        hx.resize((size_t) nb * 585);
        SE_CUDA_TRY(cudaMemcpy(hm.data(), m.block_mean, hm.size() * sizeof(OccD), cudaMemcpyDeviceToHost));
        SE_CUDA_TRY(cudaMemcpy(hn.data(), m.block_min, hn.size() * sizeof(OccD), cudaMemcpyDeviceToHost));
        SE_CUDA_TRY(cudaMemcpy(hx.data(), m.block_max, hx.size() * sizeof(OccD), cudaMemcpyDeviceToHost));
    }
    int64_t k = 0;
    for (int b = 0; b < nb && k < capacity; ++b) {
        const OccBlockState& s = states[(size_t) b];
        if (!s.live)
            continue;
        if (coords)
            for (int a = 0; a < 3; ++a)
                coords[3 * k + a] = bc[(size_t) b * 3 + a];
        if (scales) {
            scales[3 * k] = s.current_scale;
            scales[3 * k + 1] = s.min_scale;
            scales[3 * k + 2] = s.buffer_scale;
        }
        if (counts) {
            counts[4 * k] = (int64_t) s.curr_integr;
            counts[4 * k + 1] = (int64_t) s.curr_obs;
            counts[4 * k + 2] = (int64_t) s.buf_integr;
            counts[4 * k + 3] = (int64_t) s.buf_obs;
        }
        if (want_data) {
            for (int sc = 0; sc <= kOccMaxScale; ++sc) {
                const int nv = (8 >> sc) * (8 >> sc) * (8 >> sc);
                for (int v = 0; v < nv; ++v) {
                    const size_t src = (size_t) b * 585 + occ_scale_offset(sc) + v;
                    const size_t o = ((size_t) k * 585 + occ_scale_offset(sc) + v) * 3;
                    const OccD e = sc < s.finest ? s.init_data : hm[src];
                    const OccD mn = sc < s.finest ? s.init_data : (sc == s.finest ? hm[src] : hn[src]);
                    const OccD mx = sc < s.finest ? s.init_data : (sc == s.finest ? hm[src] : hx[src]);
                    const OccD* ds[3] = {&e, &mn, &mx};
                    float* outs[3] = {mean, min_data, max_data};
                    for (int q = 0; q < 3; ++q) {
                        if (!outs[q])
                            continue;
                        outs[q][o] = ds[q]->occ;
                        outs[q][o + 1] = ds[q]->weight;
                        outs[q][o + 2] = ds[q]->observed ? 1.0f : 0.0f;
                    }
                }
            }
        }
        ++k;
    }
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_download_nodes(const se_gpu_map* map, int64_t capacity, int32_t* coords, float* min_data,
                                        float* max_data, int32_t* leaf, int64_t* count)
{
    se_gpu_status st = occ_args(map, "se_gpu_map_download_nodes");
    if (st != SE_GPU_OK)
        return st;
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    const OccDevice& m = map->occ->dev;
    int nn = 0;
    SE_CUDA_TRY(cudaMemcpy(&nn, m.counters + kOccNodes, sizeof(int), cudaMemcpyDeviceToHost));
    nn = nn < m.node_capacity ? nn : m.node_capacity;
    std::vector<int4> nc((size_t) nn);
    std::vector<int> ch((size_t) nn * 8);
    std::vector<OccD> nmin((size_t) nn), nmax((size_t) nn);
    SE_CUDA_TRY(cudaMemcpy(nc.data(), m.node_coord, (size_t) nn * sizeof(int4), cudaMemcpyDeviceToHost));
    SE_CUDA_TRY(cudaMemcpy(ch.data(), m.node_child, (size_t) nn * 8 * sizeof(int), cudaMemcpyDeviceToHost));
    SE_CUDA_TRY(cudaMemcpy(nmin.data(), m.node_min, (size_t) nn * sizeof(OccD), cudaMemcpyDeviceToHost));
    SE_CUDA_TRY(cudaMemcpy(nmax.data(), m.node_max, (size_t) nn * sizeof(OccD), cudaMemcpyDeviceToHost));
    std::vector<int> stack{0};
    int64_t k = 0;
    while (!stack.empty()) {
        const int n = stack.back();
        stack.pop_back();
        if (k < capacity) {
            if (coords) {
                coords[4 * k] = nc[(size_t) n].x;
                coords[4 * k + 1] = nc[(size_t) n].y;
                coords[4 * k + 2] = nc[(size_t) n].z;
                coords[4 * k + 3] = nc[(size_t) n].w;
            }
            const OccD* ds[2] = {&nmin[(size_t) n], &nmax[(size_t) n]};
            float* outs[2] = {min_data, max_data};
            for (int q = 0; q < 2; ++q) {
                if (!outs[q])
                    continue;
                outs[q][3 * k] = ds[q]->occ;
                outs[q][3 * k + 1] = ds[q]->weight;
                outs[q][3 * k + 2] = ds[q]->observed ? 1.0f : 0.0f;
            }
            if (leaf) {
                bool is_leaf = true;
                for (int i = 0; i < 8; ++i)
                    is_leaf = is_leaf && ch[(size_t) n * 8 + i] == -1;
                leaf[k] = is_leaf ? 1 : 0;
            }
        }
        ++k;
        for (int i = 7; i >= 0; --i) {
            const int c = ch[(size_t) n * 8 + i];
            if (c >= 0)
                stack.push_back(c);
        }
    }
    if (count)
        *count = k;
    return SE_GPU_OK;
}

} // extern "C"
