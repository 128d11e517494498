// ray_integrate.cu — MapIntegrator::integrateRayBatch for multi-res occupancy maps and a
// LeicaLidar (include/se/integrator/impl/map_integrator_impl.hpp:137-176): se::RayIntegrator
// (ray_integrator_impl.hpp, ray_integrator_core_impl.hpp) over a batch of (pose, ray) pairs.
//
// The reference integrates the rays one after the other. A ray's samples depend on the blocks it
// passes (their scales decide the sample step), so rays that share a block must update it in
// batch order; rays that share none are independent. The batch runs as:
//   1. ri_prep_kernel    per ray: poses, tau / sigma, and a conservative list of the blocks the
//                        ray can touch (its segment widened by a bound on the float error of the
//                        sample positions), counted, then written by ri_fill_kernel;
//   2. a radix sort of (block, ray) pairs gives every list entry its rank among the rays that
//      list the block, and every block one ticket counter;
//   3. ri_rays_kernel    one warp per ray, rays taken in batch order: before touching a block the
//                        ray waits until the ticket equals its rank, and it advances the ticket
//                        once its samples are past the block (an untouched listed block is passed
//                        the same way). A ray waits only for earlier rays, and the earliest
//                        unfinished ray is always running, so the batch always progresses; every
//                        wait is bounded and ends the batch with an error when it runs out;
//   4. the updated blocks up to their coarsest scale, then the nodes above them depth by depth
//      (propagateBlocksToCoarsestScale, propagateToRoot), then the updated octants.
// Within one block the updates happen in batch order, so the map equals the serial result.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>

#include <cub/cub.cuh>

#include "occupancy.cuh"
#include "pipeline.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr unsigned long long kRiWaitNs = 2000000000ull; // 2 s per wait
constexpr int kRiErrTimeout = 1, kRiErrList = 2, kRiErrEntry = 4, kRiErrTree = 8;
constexpr int kRiMaxDepth = 32;

// One ray of the batch after resetIntegrator (ray_integrator_impl.hpp:45-78).
struct RiRay {
    Tf T_SW;          // T_WS.inverse()
    Tf T_WS;          // T_SW.inverse(), as operator()() recomputes it
    F3 dir;           // ray.normalized()
    float ray_dist, tau, three_sigma, max_dist;
    int active;       // ray_dist >= near_plane
    // the sample positions in map voxel units lie within delta of A + t D, t in [t0, t1]
    double A[3], D[3];
    double t0, t1, delta;
};

// One block a ray may touch.
struct RiEntry {
    int bx, by, bz;     // block origin in voxels
    float t_enter, t_exit; // sample distances (|r_S|) over which the ray can be in the block
    int slot;           // ticket counter of the block
    int rank;           // rays before this one that list the block
    int held;           // the ray holds the block (ray kernel only)
};

struct RiCtl {
    int next_ray;
    int abort;
    int err;
    int n_updated;
    int n_out_nodes;
    int pad[3];
    int list_n[kRiMaxDepth];
};

struct RiArgs {
    OccDevice m;
    const float* poses;
    const float* rays;
    int n;
    int timestamp;
    int stamp;
    float near_plane, far_plane, pixel_dim_tan, pv_den;
    float sigma_min, sigma_max, tau_min, tau_max;
    int ray_bits;
    int nb; // blocks per map side
    RiRay* R;
    int* counts;
    long long* offsets;
    RiEntry* entries;
    unsigned long long* keys;
    int* vals;
    int* done;
    int* block_mark;
    int* updated;
    int updated_cap;
    int* node_lock;
    int* node_mark;
    int* lists[2];
    int* out_nodes;
    unsigned char* out_erased;
    RiCtl* ctl;
};

__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int* p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long globaltimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ OccD ldcg_occ(const OccD* p)
{
    OccD d;
    d.occ = __ldcg(&p->occ);
    d.weight = __ldcg(&p->weight);
    d.observed = __ldcg(&p->observed);
    return d;
}

__device__ __forceinline__ float clamp_std(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }

// ----------------------------------------------------------------------- the sensor --

// LeicaLidar::computeIntegrationScaleImpl (leica_lidar.cpp:87-129), ratios {1.5, 3, 6}
__device__ int leica_scale(const RiArgs& A, F3 c, int last_scale, int min_scale)
{
    for (int pass = 0; pass < 2; ++pass) {
        const float dist = norm(c);
        const float pixel_dim = dist * A.pixel_dim_tan;
        const float pv = pixel_dim * A.pv_den;
        const int scale = pv < 1.5f ? 0 : pv < 3.0f ? 1 : pv < 6.0f ? 2 : 3;
        if (pass == 0 && min_scale != -1 && scale != last_scale) {
            const F3 n = normalized(c);
            c = scale > last_scale ? sub(c, mul(0.25f, n)) : add(c, mul(0.25f, n));
            continue;
        }
        return scale;
    }
    return 0;
}

// --------------------------------------------------------------- block lists per ray --

__device__ bool ri_box(const RiRay& R, const double lo[3], const double hi[3], double& ta, double& tb)
{
    ta = R.t0;
    tb = R.t1;
    for (int a = 0; a < 3; ++a) {
        if (R.D[a] == 0.0) {
            if (R.A[a] < lo[a] || R.A[a] > hi[a])
                return false;
            continue;
        }
        double u = (lo[a] - R.A[a]) / R.D[a], w = (hi[a] - R.A[a]) / R.D[a];
        if (u > w) {
            const double x = u;
            u = w;
            w = x;
        }
        ta = u > ta ? u : ta;
        tb = w < tb ? w : tb;
        if (ta > tb)
            return false;
    }
    return true;
}

__device__ __forceinline__ int block_floor(double v, int nb)
{
    const double f = floor(v / 8.0);
    return f < 0.0 ? 0 : (f > (double) (nb - 1) ? nb - 1 : (int) f);
}

// Every block whose box, widened by delta, meets the segment: slab by slab along the axis the
// ray moves most along (so each block comes from one slab only), in the order the ray meets
// the slabs. emit(bx, by, bz, t_enter, t_exit).
template <class F>
__device__ int ri_enumerate(const RiRay& R, int nb, F emit)
{
    int a = 0;
    if (fabs(R.D[1]) > fabs(R.D[a]))
        a = 1;
    if (fabs(R.D[2]) > fabs(R.D[a]))
        a = 2;
    const int b = (a + 1) % 3, c = (a + 2) % 3;
    const double dl = R.delta;
    for (int i = 0; i < 3; ++i)
        if (!isfinite(R.A[i]) || !isfinite(R.D[i]))
            return 0;
    if (!isfinite(R.t0) || !isfinite(R.t1) || !isfinite(dl) || R.D[a] == 0.0)
        return 0;
    const double pa0 = R.A[a] + R.t0 * R.D[a], pa1 = R.A[a] + R.t1 * R.D[a];
    const double amin = pa0 < pa1 ? pa0 : pa1, amax = pa0 < pa1 ? pa1 : pa0;
    if (amax + dl < 0.0 || amin - dl >= 8.0 * nb)
        return 0;
    const int klo = block_floor(amin - dl, nb), khi = block_floor(amax + dl, nb);
    const int step = R.D[a] >= 0.0 ? 1 : -1;
    const int first = step > 0 ? klo : khi, last = step > 0 ? khi : klo;
    int count = 0;
    for (int k = first;; k += step) {
        double ts = (8.0 * k - dl - R.A[a]) / R.D[a], te = (8.0 * k + 8.0 + dl - R.A[a]) / R.D[a];
        if (ts > te) {
            const double x = ts;
            ts = te;
            te = x;
        }
        ts = ts > R.t0 ? ts : R.t0;
        te = te < R.t1 ? te : R.t1;
        if (ts <= te) {
            const double pb0 = R.A[b] + ts * R.D[b], pb1 = R.A[b] + te * R.D[b];
            const double pc0 = R.A[c] + ts * R.D[c], pc1 = R.A[c] + te * R.D[c];
            const double bmin = (pb0 < pb1 ? pb0 : pb1) - dl, bmax = (pb0 < pb1 ? pb1 : pb0) + dl;
            const double cmin = (pc0 < pc1 ? pc0 : pc1) - dl, cmax = (pc0 < pc1 ? pc1 : pc0) + dl;
            if (!(bmax < 0.0 || bmin >= 8.0 * nb || cmax < 0.0 || cmin >= 8.0 * nb)) {
                const int kb0 = block_floor(bmin, nb), kb1 = block_floor(bmax, nb);
                const int kc0 = block_floor(cmin, nb), kc1 = block_floor(cmax, nb);
                for (int kb = kb0; kb <= kb1; ++kb)
                    for (int kc = kc0; kc <= kc1; ++kc) {
                        int blk[3];
                        blk[a] = k;
                        blk[b] = kb;
                        blk[c] = kc;
                        double lo[3], hi[3];
                        for (int i = 0; i < 3; ++i) {
                            lo[i] = 8.0 * blk[i] - dl;
                            hi[i] = 8.0 * blk[i] + 8.0 + dl;
                        }
                        double ta, tb;
                        if (ri_box(R, lo, hi, ta, tb)) {
                            emit(8 * blk[0], 8 * blk[1], 8 * blk[2], ta, tb);
                            ++count;
                        }
                    }
            }
        }
        if (k == last)
            break;
    }
    return count;
}

// resetIntegrator (ray_integrator_impl.hpp:45-78) and the conservative segment of the ray.
__global__ void ri_prep_kernel(RiArgs A)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > A.n)
        return;
    if (i == A.n) {
        A.counts[i] = 0;
        return;
    }
    const OccDevice& m = A.m;
    RiRay R;
    const Tf T_in = tf_from16(A.poses + 16 * (size_t) i);
    const F3 ray = f3(A.rays[3 * (size_t) i], A.rays[3 * (size_t) i + 1], A.rays[3 * (size_t) i + 2]);
    R.T_SW = inverse_iso(T_in);
    R.T_WS = inverse_iso(R.T_SW);
    R.ray_dist = norm(ray);
    R.tau = clamp_std(m.cfg.k_tau * R.ray_dist, A.tau_min, A.tau_max);
    R.three_sigma = 3.0f * clamp_std(m.cfg.k_sigma * R.ray_dist, A.sigma_min, A.sigma_max);
    R.dir = normalized(ray);
    const float reach = R.ray_dist + R.tau;
    R.max_dist = A.far_plane < reach ? A.far_plane : reach;
    // a ray or pose with a NaN or an infinity samples nothing (its first distance test fails)
    bool finite = isfinite(R.ray_dist);
    for (int k = 0; k < 9; ++k)
        finite &= isfinite(R.T_WS.R[k]) && isfinite(R.T_SW.R[k]);
    for (int k = 0; k < 3; ++k)
        finite &= isfinite(R.T_WS.t[k]) && isfinite(R.T_SW.t[k]);
    R.active = finite && !(R.ray_dist < A.near_plane);
    // the segment in map voxel units: p_M / res = (T_MW (T_WS (t dir))) / res
    const double inv_res = 1.0 / (double) m.res;
    double o[3], d[3];
    for (int r = 0; r < 3; ++r) {
        o[r] = R.T_WS.t[r];
        d[r] = (double) R.T_WS.R[3 * r] * R.dir.x + (double) R.T_WS.R[3 * r + 1] * R.dir.y
            + (double) R.T_WS.R[3 * r + 2] * R.dir.z;
    }
    double tw = 0.0, tm = 0.0;
    for (int r = 0; r < 3; ++r) {
        R.A[r] = ((double) m.T_MW.R[3 * r] * o[0] + (double) m.T_MW.R[3 * r + 1] * o[1]
                  + (double) m.T_MW.R[3 * r + 2] * o[2] + (double) m.T_MW.t[r])
            * inv_res;
        R.D[r] = ((double) m.T_MW.R[3 * r] * d[0] + (double) m.T_MW.R[3 * r + 1] * d[1]
                  + (double) m.T_MW.R[3 * r + 2] * d[2])
            * inv_res;
        tw += fabs(o[r]);
        tm += fabs((double) m.T_MW.t[r]);
    }
    // Float error of a sample position: each of the n steps r += s dir rounds every component by
    // at most 2^-24 |r|, and the two transforms and the division by res add a few 2^-24 relative
    // errors of the coordinates; twice that bound, plus a floor, in voxels.
    const double n_steps = ((double) R.max_dist - (double) A.near_plane) / (0.5 * (double) m.res) + 4.0;
    const double mag = (double) R.max_dist + tw + tm + (double) m.dim;
    R.delta = 0.02 + (n_steps + 16.0) * 0x1p-23 * mag * inv_res;
    const double tpad = 0x1p-20 * ((double) R.max_dist + 1.0) + R.delta * (double) m.res;
    R.t0 = (double) A.near_plane - tpad;
    R.t1 = (double) (R.max_dist > A.near_plane ? R.max_dist : A.near_plane) + tpad;
    A.R[i] = R;
    A.counts[i] = R.active ? ri_enumerate(R, A.nb, [](int, int, int, double, double) {}) : 0;
}

__global__ void ri_fill_kernel(RiArgs A)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n)
        return;
    const RiRay& R = A.R[i];
    if (!R.active)
        return;
    long long e = A.offsets[i];
    const long long end = A.offsets[i + 1];
    const int nb = A.nb;
    ri_enumerate(R, nb, [&](int bx, int by, int bz, double ta, double tb) {
        if (e >= end)
            return;
        RiEntry E;
        E.bx = bx;
        E.by = by;
        E.bz = bz;
        E.t_enter = __double2float_rd(ta);
        E.t_exit = __double2float_ru(tb);
        E.slot = 0;
        E.rank = 0;
        E.held = 0;
        A.entries[e] = E;
        const unsigned long long lin =
            ((unsigned long long) (bz >> 3) * nb + (unsigned long long) (by >> 3)) * nb + (unsigned long long) (bx >> 3);
        A.keys[e] = (lin << A.ray_bits) | (unsigned long long) i;
        A.vals[e] = (int) e;
        ++e;
    });
}

// After the sort: the first position of a block's run is its ticket counter, the position within
// the run the ray's rank.
__global__ void ri_rank_kernel(RiArgs A, const unsigned long long* __restrict__ sorted_keys,
                               const int* __restrict__ sorted_vals, long long total)
{
    for (long long p = blockIdx.x * (long long) blockDim.x + threadIdx.x; p < total;
         p += (long long) gridDim.x * blockDim.x) {
        const unsigned long long blk = sorted_keys[p] >> A.ray_bits;
        long long lo = 0, hi = p;
        while (lo < hi) {
            const long long mid = (lo + hi) >> 1;
            if ((sorted_keys[mid] >> A.ray_bits) < blk)
                lo = mid + 1;
            else
                hi = mid;
        }
        RiEntry& E = A.entries[sorted_vals[p]];
        E.slot = (int) lo;
        E.rank = (int) (p - lo);
        A.done[p] = 0;
    }
}

// ------------------------------------------------------------------ octree in the loop --

__device__ void ri_abort(const RiArgs& A, int err)
{
    atomicOr(&A.ctl->err, err);
    atomicExch(&A.ctl->abort, 1);
}

__device__ __forceinline__ bool ri_aborted(const RiArgs& A)
{
    return *((volatile int*) &A.ctl->abort) != 0;
}

// Waits (lane 0, bounded) until the ticket *p reaches want, polling with acquire semantics. A
// ray far back in a block's queue polls rarely, the next in line often.
__device__ bool ri_wait_eq(const RiArgs& A, const int* p, int want, int lane)
{
    int ok = 1;
    if (lane == 0) {
        const unsigned long long t0 = globaltimer();
        int v = ld_acquire(p);
        while (v != want) {
            if (ri_aborted(A)) {
                ok = 0;
                break;
            }
            if (globaltimer() - t0 > kRiWaitNs) {
                ri_abort(A, kRiErrTimeout);
                ok = 0;
                break;
            }
            const int gap = want - v;
            __nanosleep(gap <= 1 ? 20u : (unsigned) min(gap, 512) * 128u);
            v = ld_acquire(p);
        }
    }
    ok = __shfl_sync(kFull, ok, 0);
    // the warp barrier orders lane 0's acquire before every lane's later loads
    __syncwarp();
    return ok != 0;
}

// Sets *p = v after the warp's writes: the warp barrier orders every lane's writes before lane
// 0's store, whose release semantics carry them to the next acquirer.
__device__ __forceinline__ void ri_release(int* p, int v, int lane)
{
    __syncwarp();
    if (lane == 0)
        st_release(p, v);
    __syncwarp();
}

// Octree::allocateChildren (octree_impl.hpp:200-233) under node n's lock, by the whole warp:
// the winner of the lock allocates all eight children at once, initialised with the node's data
// as it was while the node had no children.
__device__ bool ri_allocate_children(const RiArgs& A, int n, int lane)
{
    const OccDevice& m = A.m;
    int got = 0;
    if (lane == 0) {
        const unsigned long long t0 = globaltimer();
        unsigned ns = 32;
        for (;;) {
            if (atomicCAS(&A.node_lock[n], 0, 1) == 0) {
                got = 1;
                break;
            }
            if (ri_aborted(A))
                break;
            if (globaltimer() - t0 > kRiWaitNs) {
                ri_abort(A, kRiErrTimeout);
                break;
            }
            __nanosleep(ns);
            ns = ns < 1024 ? 2 * ns : ns;
        }
        __threadfence();
    }
    got = __shfl_sync(kFull, got, 0);
    if (!got)
        return false;
    int* child = m.node_child + 8 * (size_t) n;
    const int mine = lane < 8 ? ld_acquire(&child[lane]) : -1;
    const unsigned present = __ballot_sync(kFull, lane < 8 && mine != -1);
    if (present == 0u) {
        // NodeData::data(): the max data when observed and the node is a leaf (it is, here)
        OccD init = ldcg_occ(&m.node_max[n]);
        if (!init.observed)
            init = occ_default();
        const int4 nc = make_int4(__ldcg(&m.node_coord[n].x), __ldcg(&m.node_coord[n].y), __ldcg(&m.node_coord[n].z),
                                  __ldcg(&m.node_coord[n].w));
        const int csize = nc.w / 2;
        const bool blocks_below = nc.w == 16;
        int base = 0;
        if (lane == 0)
            base = atomicAdd(&m.counters[blocks_below ? kOccBlocks : kOccNodes], 8);
        base = __shfl_sync(kFull, base, 0);
        const int cap = blocks_below ? m.block_capacity : m.node_capacity;
        if (base + 8 > cap) {
            if (lane == 0)
                atomicOr(&m.counters[kOccError], blocks_below ? kOccErrBlockPool : kOccErrNodePool);
            ri_abort(A, kRiErrTree);
        }
        else if (lane < 8) {
            const int i = lane, idx = base + lane;
            const int cx = nc.x + csize * (i & 1), cy = nc.y + csize * ((i >> 1) & 1), cz = nc.z + csize * (i >> 2);
            if (blocks_below) {
                m.block_coord[3 * idx] = cx;
                m.block_coord[3 * idx + 1] = cy;
                m.block_coord[3 * idx + 2] = cz;
                OccBlockState st;
                st.init_data = init;
                st.min_scale = -1;
                st.current_scale = kOccMaxScale;
                st.finest = kOccMaxScale;
                st.buffer_scale = -1;
                st.curr_integr = st.curr_obs = st.buf_integr = st.buf_obs = 0ull;
                st.parent = n;
                st.live = 1;
                m.block_state[idx] = st;
                blk_mean(m, idx, kOccMaxScale)[0] = init;
                m.block_ts[idx] = -1;
            }
            else {
                m.node_coord[idx] = make_int4(cx, cy, cz, csize);
                m.node_parent[idx] = n;
                for (int k = 0; k < 8; ++k)
                    m.node_child[8 * (size_t) idx + k] = -1;
                m.node_min[idx] = init;
                m.node_max[idx] = init;
                m.node_mark[idx] = -1;
                m.node_ts[idx] = -1;
            }
            __threadfence();
            st_release(&child[i], blocks_below ? -2 - idx : idx);
        }
        __syncwarp();
        if (blocks_below && lane == 0) {
            atomicMin(&m.aabb[0], nc.x);
            atomicMin(&m.aabb[1], nc.y);
            atomicMin(&m.aabb[2], nc.z);
            atomicMax(&m.aabb[3], nc.x + nc.w - 1);
            atomicMax(&m.aabb[4], nc.y + nc.w - 1);
            atomicMax(&m.aabb[5], nc.z + nc.w - 1);
            m.aabb[6] = 0;
        }
    }
    else if (present != 0xffu) {
        // an occupancy node has no children or all eight
        ri_abort(A, kRiErrTree);
    }
    ri_release(&A.node_lock[n], 0, lane);
    return !ri_aborted(A);
}

// fetcher::finest_octant(voxel, 0, root) with allocateChildren on the way down
// (ray_integrator_impl.hpp:168-224): the block holding the voxel, or -1 after an abort.
__device__ int ri_block(const RiArgs& A, int x, int y, int z, int lane)
{
    const OccDevice& m = A.m;
    for (int guard = 0; guard < 64; ++guard) {
        int n = 0, slot = -1;
        for (int cs = m.size >> 1; cs >= 8; cs >>= 1) {
            const int idx = ((x & cs) > 0) + 2 * ((y & cs) > 0) + 4 * ((z & cs) > 0);
            const int ch = ld_acquire(&m.node_child[8 * (size_t) n + idx]);
            if (ch == -1) {
                slot = n;
                break;
            }
            if (slot_is_block(ch))
                return slot_block(ch);
            n = ch;
        }
        if (slot < 0) {
            ri_abort(A, kRiErrTree);
            return -1;
        }
        if (!ri_allocate_children(A, slot, lane))
            return -1;
    }
    ri_abort(A, kRiErrTree);
    return -1;
}

// ------------------------------------------------------------------- block operations --

// A held block's state, kept in registers (uniform across the warp) while the ray holds it.
struct RiBlock {
    int b;
    int min_scale, current_scale, finest;
    int ts;
    OccD init;
    int cx, cy, cz;
    int marked; // in this batch's updated-block list
};

__device__ void ri_load_block(const RiArgs& A, int b, RiBlock& B)
{
    const OccBlockState* st = A.m.block_state + b;
    B.b = b;
    B.min_scale = __ldcg(&st->min_scale);
    B.current_scale = __ldcg(&st->current_scale);
    B.finest = __ldcg(&st->finest);
    B.init = ldcg_occ(&st->init_data);
    B.ts = __ldcg(&A.m.block_ts[b]);
    B.cx = __ldcg(&A.m.block_coord[3 * b]);
    B.cy = __ldcg(&A.m.block_coord[3 * b + 1]);
    B.cz = __ldcg(&A.m.block_coord[3 * b + 2]);
    B.marked = __ldcg(&A.block_mark[b]) == A.stamp;
}

__device__ void ri_store_scales(const RiArgs& A, const RiBlock& B, int lane)
{
    if (lane == 0) {
        OccBlockState* st = A.m.block_state + B.b;
        st->min_scale = B.min_scale;
        st->current_scale = B.current_scale;
        st->finest = B.finest;
    }
}

__device__ __forceinline__ OccD* ri_min(const OccDevice& m, const RiBlock& B, int s)
{
    return blk_min(m, B.b, B.finest, s);
}
__device__ __forceinline__ OccD* ri_max(const OccDevice& m, const RiBlock& B, int s)
{
    return blk_max(m, B.b, B.finest, s);
}

// BlockMultiRes<Occupancy>::allocateDownTo (block_impl.hpp:540-590)
__device__ void ri_allocate_down_to(const RiArgs& A, RiBlock& B, int new_min, int lane)
{
    const OccDevice& m = A.m;
    if (new_min >= B.current_scale)
        return;
    for (int s = B.current_scale; s >= new_min; --s) {
        OccD* d = blk_mean(m, B.b, s);
        const int nv = (8 >> s) * (8 >> s) * (8 >> s);
        if (s != B.current_scale)
            for (int i = lane; i < nv; i += 32)
                d[i] = B.init;
        __syncwarp();
        if (s != new_min) {
            OccD* mn = m.block_min + (size_t) B.b * 585 + occ_scale_offset(s);
            OccD* mx = m.block_max + (size_t) B.b * 585 + occ_scale_offset(s);
            for (int i = lane; i < nv; i += 32) {
                const OccD v = ldcg_occ(&d[i]);
                mn[i] = v;
                mx[i] = v;
            }
        }
        __syncwarp();
    }
    B.finest = new_min;
    B.current_scale = new_min;
    B.min_scale = new_min;
    ri_store_scales(A, B, lane);
}

// ray_integrator::propagate_block_down_to_scale (ray_integrator_core_impl.hpp:358-426)
__device__ void ri_propagate_down(const RiArgs& A, RiBlock& B, int desired, int lane)
{
    const OccDevice& m = A.m;
    int cur = B.current_scale;
    while (cur > desired) {
        ri_allocate_down_to(A, B, cur - 1, lane);
        B.current_scale = cur - 1;
        ri_store_scales(A, B, lane);
        const int cs = cur - 1, ps = cur;
        const int nc = 8 >> cs, np = 8 >> ps;
        const OccD* pd = blk_mean(m, B.b, ps);
        OccD* cd = blk_mean(m, B.b, cs);
        for (int p = lane; p < np * np * np; p += 32) {
            const OccD par = ldcg_occ(&pd[p]);
            if (!par.observed)
                continue;
            const int x = p % np, y = (p / np) % np, z = p / (np * np);
            for (int k = 0; k < 8; ++k) {
                OccD& c = cd[(2 * x + (k & 1)) + (2 * y + ((k >> 1) & 1)) * nc + (2 * z + (k >> 2)) * nc * nc];
                c.weight = par.weight;
                c.occ = par.occ;
                c.observed = 0;
            }
        }
        __syncwarp();
        cur--;
    }
}

struct RiAcc {
    float mean_occ, mean_w, min_mean, min_w, min_o, max_mean, max_w, max_o;
    int count, observed;
};

__device__ __forceinline__ void ri_acc_init(RiAcc& a)
{
    a.mean_occ = a.mean_w = a.min_mean = a.min_w = a.max_mean = a.max_w = 0.0f;
    a.min_o = FLT_MAX;
    a.max_o = -FLT_MAX;
    a.count = a.observed = 0;
}

__device__ __forceinline__ void ri_acc_store(const RiAcc& a, OccD* pmean, OccD* pmin, OccD* pmax)
{
    if (a.count > 0) {
        pmean->occ = a.mean_occ / (float) a.count;
        pmean->weight = ceilf(a.mean_w) / (float) a.count;
        pmean->observed = 0;
        pmin->occ = a.min_mean;
        pmin->weight = a.min_w;
        pmax->occ = a.max_mean;
        pmax->weight = a.max_w;
        if (a.observed == 8) {
            pmax->observed = 1;
            pmin->observed = 1;
        }
    }
}

// ray_integrator::propagate_block_to_scale (ray_integrator_core_impl.hpp:206-352)
__device__ void ri_propagate_to_scale(const OccDevice& m, const RiBlock& B, int desired, int lane)
{
    int cs = B.current_scale;
    int ps = cs + 1;
    {
        const int nc = 8 >> cs, np = 8 >> ps;
        const OccD* cmean = blk_mean(m, B.b, cs);
        OccD *pmean = blk_mean(m, B.b, ps), *pmin = ri_min(m, B, ps), *pmax = ri_max(m, B, ps);
        for (int p = lane; p < np * np * np; p += 32) {
            const int x = p % np, y = (p / np) % np, z = p / (np * np);
            RiAcc a;
            ri_acc_init(a);
            for (int k = 0; k < 8; ++k) {
                const OccD c =
                    ldcg_occ(&cmean[(2 * x + (k & 1)) + (2 * y + ((k >> 1) & 1)) * nc + (2 * z + (k >> 2)) * nc * nc]);
                if (c.weight > 0.0f) {
                    a.count++;
                    a.mean_occ += c.occ;
                    a.mean_w += c.weight;
                    const float o = occ_field(c);
                    if (o > a.max_o) {
                        a.max_mean = c.occ;
                        a.max_w = c.weight;
                        a.max_o = o;
                    }
                    else if (o < a.min_o) {
                        a.min_mean = c.occ;
                        a.min_w = c.weight;
                        a.min_o = o;
                    }
                }
                if (c.observed)
                    a.observed++;
            }
            ri_acc_store(a, &pmean[p], &pmin[p], &pmax[p]);
        }
        __syncwarp();
    }
    for (ps += 1; ps <= desired; ++ps) {
        cs = ps - 1;
        const int nc = 8 >> cs, np = 8 >> ps;
        const OccD *cmean = blk_mean(m, B.b, cs), *cmin = ri_min(m, B, cs), *cmax = ri_max(m, B, cs);
        OccD *pmean = blk_mean(m, B.b, ps), *pmin = ri_min(m, B, ps), *pmax = ri_max(m, B, ps);
        for (int p = lane; p < np * np * np; p += 32) {
            const int x = p % np, y = (p / np) % np, z = p / (np * np);
            RiAcc a;
            ri_acc_init(a);
            for (int k = 0; k < 8; ++k) {
                const int ci = (2 * x + (k & 1)) + (2 * y + ((k >> 1) & 1)) * nc + (2 * z + (k >> 2)) * nc * nc;
                const OccD cx = ldcg_occ(&cmax[ci]);
                if (cx.weight > 0.0f) {
                    const OccD ce = ldcg_occ(&cmean[ci]);
                    const OccD cn = ldcg_occ(&cmin[ci]);
                    a.count++;
                    a.mean_occ += ce.occ;
                    a.mean_w += ce.weight;
                    const float mo = occ_field(cx);
                    if (mo > a.max_o) {
                        a.max_mean = cx.occ;
                        a.max_w = cx.weight;
                        a.max_o = mo;
                    }
                    const float no = occ_field(cn);
                    if (no < a.min_o) {
                        a.min_mean = cn.occ;
                        a.min_w = cn.weight;
                        a.min_o = no;
                    }
                }
                if (cx.observed)
                    a.observed++;
            }
            ri_acc_store(a, &pmean[p], &pmin[p], &pmax[p]);
        }
        __syncwarp();
    }
}

// updater::update_voxel (multires_ofusion_core_impl.hpp:46-77), as ray_integrator::update_voxel
__device__ __forceinline__ void ri_update_voxel(OccD& d, float range_diff, float tau, float three_sigma,
                                                const OccFieldConfig& c)
{
    float sample;
    if (range_diff < -three_sigma)
        sample = c.log_odd_min;
    else if (range_diff < tau / 2.0f) {
        const float v = c.log_odd_min - c.log_odd_min / three_sigma * (range_diff + three_sigma);
        sample = c.log_odd_max < v ? c.log_odd_max : v;
    }
    else if (range_diff < tau) {
        const float v = -c.log_odd_min * tau / (2.0f * three_sigma);
        sample = c.log_odd_max < v ? c.log_odd_max : v;
    }
    else
        return;
    if (d.weight < c.max_weight)
        d.weight = d.weight + 1.0f;
    d.occ = (d.occ * (d.weight - 1.0f) + sample) / d.weight;
    d.observed = 1;
}

// updateBlock (ray_integrator_impl.hpp:232-300)
__device__ void ri_update_block(const RiArgs& A, const RiRay& R, RiBlock& B, int vx, int vy, int vz, int desired,
                                float sample_dist, int lane)
{
    const OccDevice& m = A.m;
    if ((double) sample_dist < 1e-08)
        return;
    const bool already = B.ts == A.timestamp;
    if (!already) {
        B.ts = A.timestamp;
        if (lane == 0)
            m.block_ts[B.b] = A.timestamp;
    }
    const int last_scale = B.min_scale == -1 ? desired : B.current_scale;
    int s = last_scale;
    if (B.min_scale == -1) {
        ri_allocate_down_to(A, B, s, lane);
        B.init = occ_default();
        if (lane == 0)
            m.block_state[B.b].init_data = B.init;
    }
    else if (desired < last_scale) {
        ri_propagate_down(A, B, desired, lane);
        s = desired;
    }
    else if (!already && desired > last_scale) {
        ri_propagate_to_scale(m, B, desired, lane);
        s = desired;
        // deleteUpTo(s) (block_impl.hpp:595-627), then the current scale
        if (!(s <= B.min_scale || B.min_scale == -1)) {
            B.finest = s;
            B.min_scale = s;
        }
        B.current_scale = s;
        ri_store_scales(A, B, lane);
    }
    __syncwarp();
    if (lane == 0) {
        const int n = 8 >> s;
        const int idx = ((vx - B.cx) >> s) + n * ((vy - B.cy) >> s) + n * n * ((vz - B.cz) >> s);
        OccD* p = blk_mean(m, B.b, s) + idx;
        OccD d = ldcg_occ(p);
        ri_update_voxel(d, sample_dist - R.ray_dist, R.tau, R.three_sigma, m.cfg);
        *p = d;
    }
    __syncwarp();
}

// ------------------------------------------------------------------------ the rays --

// Passes list entry e: waits for the ray's turn if it does not hold the block yet, then hands
// the block to the next ray.
__device__ bool ri_pass(const RiArgs& A, long long e, int lane)
{
    RiEntry& E = A.entries[e];
    const int held = E.held, slot = E.slot, rank = E.rank;
    if (!held && !ri_wait_eq(A, &A.done[slot], rank, lane))
        return false;
    ri_release(&A.done[slot], rank + 1, lane);
    return true;
}

// updated_blocks_set_ / updated_blocks_vector_: the block joins this batch's list once.
__device__ __forceinline__ void ri_mark(const RiArgs& A, RiBlock& B, int lane)
{
    if (B.marked)
        return;
    B.marked = 1;
    if (lane == 0) {
        A.block_mark[B.b] = A.stamp;
        const int k = atomicAdd(&A.ctl->n_updated, 1);
        if (k < A.updated_cap)
            A.updated[k] = B.b;
        else
            ri_abort(A, kRiErrList);
    }
    __syncwarp();
}

// The samples that follow in a held, already integrated block, one per lane: lane k takes the
// sample k steps ahead (its position accumulated step by step, as the serial loop does). The run
// ends before the first sample that leaves the block, the map or the update distance, or whose
// scale would change the block (a finer integration scale); a sample whose scale changes the step
// ends it after itself. The updates are applied in sample order per voxel (the lowest lane of
// each voxel's group applies its group's updates in turn), so the result is the serial one.
// Returns the samples processed; r, the last voxel and the computed scale advance past them.
__device__ int ri_run(const RiArgs& A, const RiRay& R, const RiBlock& B, F3& r, int& lx, int& ly, int& lz,
                      int& computed, float* s_rd, int lane)
{
    const OccDevice& m = A.m;
    const float st = (float) (0.5 * (double) m.res * (double) (1 << computed));
    const float sx = st * R.dir.x, sy = st * R.dir.y, sz = st * R.dir.z;
    F3 q = r;
    for (int k = 0; k < lane; ++k)
        q = f3(q.x + sx, q.y + sy, q.z + sz);
    const float rn = norm(q);
    const F3 p_M = apply(m.T_MW, apply(R.T_WS, q));
    const bool inside = p_M.x >= 0.0f && p_M.x < m.dim && p_M.y >= 0.0f && p_M.y < m.dim && p_M.z >= 0.0f
        && p_M.z < m.dim;
    const int vx = inside ? (int) (p_M.x / m.res) : -1, vy = inside ? (int) (p_M.y / m.res) : -1,
              vz = inside ? (int) (p_M.z / m.res) : -1;
    const bool in_block = inside && (vx & ~7) == B.cx && (vy & ~7) == B.cy && (vz & ~7) == B.cz;
    // the block's scale decision (the same block centre and state for every lane)
    const F3 c_M = f3(((float) B.cx + 4.0f) * m.res, ((float) B.cy + 4.0f) * m.res, ((float) B.cz + 4.0f) * m.res);
    const int s0 = leica_scale(A, apply(R.T_SW, apply(m.T_WM, c_M)), B.current_scale, B.min_scale);
    const int fs = m.cfg.fs_integr_scale;
    const bool free_space = rn - R.ray_dist < -R.three_sigma;
    const int desired = (free_space && s0 < fs) ? (fs < B.current_scale ? fs : B.current_scale) : s0;
    // the previous sample's voxel, for the serial loop's repeat test
    int px = __shfl_up_sync(kFull, vx, 1), py = __shfl_up_sync(kFull, vy, 1), pz = __shfl_up_sync(kFull, vz, 1);
    if (lane == 0) {
        px = lx;
        py = ly;
        pz = lz;
    }
    const bool dup = vx == px && vy == py && vz == pz;
    const bool stop = !(rn < R.max_dist) || !in_block || !((double) rn >= 1e-08)
        || (!dup && desired < B.current_scale);
    const unsigned stops = __ballot_sync(kFull, stop);
    int len = stops ? __ffs(stops) - 1 : 32;
    const unsigned changes = __ballot_sync(kFull, !dup && desired != computed) & ((len >= 32) ? kFull : ((1u << len) - 1u));
    if (changes)
        len = __ffs(changes); // include the sample whose scale changes the step
    if (len == 0)
        return 0;
    const bool upd = lane < len && !dup;
    const int s = B.current_scale, n = 8 >> s;
    const int idx = upd ? ((vx - B.cx) >> s) + n * ((vy - B.cy) >> s) + n * n * ((vz - B.cz) >> s) : -1;
    s_rd[lane] = rn - R.ray_dist;
    __syncwarp();
    const unsigned upd_mask = __ballot_sync(kFull, upd);
    const unsigned group = __match_any_sync(kFull, idx) & upd_mask;
    if (upd && (group & ((1u << lane) - 1u)) == 0u) {
        OccD* p = blk_mean(m, B.b, s) + idx;
        OccD d = ldcg_occ(p);
        for (unsigned g = group; g; g &= g - 1u)
            ri_update_voxel(d, s_rd[__ffs(g) - 1], R.tau, R.three_sigma, m.cfg);
        *p = d;
    }
    __syncwarp();
    // the state after the run's last sample
    const int last = len - 1;
    const unsigned upd_in = upd_mask & ((len >= 32) ? kFull : ((1u << len) - 1u));
    if (upd_in)
        computed = __shfl_sync(kFull, desired, 31 - __clz(upd_in));
    lx = __shfl_sync(kFull, vx, last);
    ly = __shfl_sync(kFull, vy, last);
    lz = __shfl_sync(kFull, vz, last);
    const float qx = __shfl_sync(kFull, q.x, last), qy = __shfl_sync(kFull, q.y, last),
                qz = __shfl_sync(kFull, q.z, last);
    const float st2 = (float) (0.5 * (double) m.res * (double) (1 << computed));
    r = f3(qx + st2 * R.dir.x, qy + st2 * R.dir.y, qz + st2 * R.dir.z);
    return len;
}

// RayIntegrator::operator()() (ray_integrator_impl.hpp:82-129) for one ray, by one warp.
__device__ void ri_ray(const RiArgs& A, int ray, int lane, float* s_rd)
{
    const OccDevice& m = A.m;
    const RiRay& R = A.R[ray];
    const long long e0 = A.offsets[ray], e1 = A.offsets[ray + 1];
    long long rel = e0;  // entries before rel are passed
    if (R.active) {
        F3 r = mul(A.near_plane, R.dir);
        int computed = 0;
        int lx = -1, ly = -1, lz = -1;
        long long cur_e = -1;
        RiBlock B;
        B.b = -1;
        for (;;) {
            const float rn = norm(r);
            if (!(rn < R.max_dist))
                break;
            // the blocks the samples have left go to the next rays
            while (rel < e1 && A.entries[rel].t_exit < rn) {
                if (!ri_pass(A, rel, lane))
                    return;
                if (rel == cur_e) {
                    cur_e = -1;
                    B.b = -1;
                }
                ++rel;
            }
            // computeVariance (ray_integrator_impl.hpp:135-158)
            const float z_diff = rn - R.ray_dist;
            const bool free_space = z_diff < -R.three_sigma;
            const F3 r_W = apply(R.T_WS, r);
            const F3 p_M = apply(m.T_MW, r_W);
            if (!(p_M.x >= 0.0f && p_M.x < m.dim && p_M.y >= 0.0f && p_M.y < m.dim && p_M.z >= 0.0f && p_M.z < m.dim))
                break;
            const int vx = (int) (p_M.x / m.res), vy = (int) (p_M.y / m.res), vz = (int) (p_M.z / m.res);
            if (vx != lx || vy != ly || vz != lz) {
                const int bx = vx & ~7, by = vy & ~7, bz = vz & ~7;
                if (cur_e < 0 || A.entries[cur_e].bx != bx || A.entries[cur_e].by != by || A.entries[cur_e].bz != bz) {
                    long long e = -1;
                    for (long long k = rel; k < e1; ++k) {
                        const RiEntry& E = A.entries[k];
                        if (E.bx == bx && E.by == by && E.bz == bz) {
                            e = k;
                            break;
                        }
                    }
                    if (e < 0) {
                        ri_abort(A, kRiErrEntry);
                        return;
                    }
                    // the descent (and any allocation) does not depend on the batch order
                    const int b = ri_block(A, vx, vy, vz, lane);
                    if (b < 0)
                        return;
                    if (!A.entries[e].held) {
                        if (!ri_wait_eq(A, &A.done[A.entries[e].slot], A.entries[e].rank, lane))
                            return;
                        __syncwarp();
                        if (lane == 0)
                            A.entries[e].held = 1;
                        __syncwarp();
                    }
                    cur_e = e;
                    ri_load_block(A, b, B);
                }
                // a block an earlier sample of this batch integrated: this sample and the ones
                // after it in the block as one run
                if (B.min_scale != -1 && B.ts == A.timestamp) {
                    int k = ri_run(A, R, B, r, lx, ly, lz, computed, s_rd, lane);
                    if (k > 0) {
                        ri_mark(A, B, lane);
                        while (k == 32)
                            k = ri_run(A, R, B, r, lx, ly, lz, computed, s_rd, lane);
                        continue;
                    }
                }
                lx = vx;
                ly = vy;
                lz = vz;
                // operator()(ray_sample, voxel, state, octant) at block level (:174-214)
                const int last_scale = B.min_scale == -1 ? 0 : B.current_scale;
                const F3 c_M = f3(((float) B.cx + 4.0f) * m.res, ((float) B.cy + 4.0f) * m.res, ((float) B.cz + 4.0f) * m.res);
                const F3 c_S = apply(R.T_SW, apply(m.T_WM, c_M));
                int scale = leica_scale(A, c_S, last_scale, B.min_scale);
                const int fs = m.cfg.fs_integr_scale;
                if (free_space && scale < fs)
                    scale = B.min_scale == -1 ? fs : (fs < B.current_scale ? fs : B.current_scale);
                ri_update_block(A, R, B, vx, vy, vz, scale, rn, lane);
                computed = scale;
                ri_mark(A, B, lane);
            }
            const float step = (float) (0.5 * (double) m.res * (double) (1 << computed));
            r = f3(r.x + step * R.dir.x, r.y + step * R.dir.y, r.z + step * R.dir.z);
            // the rest of the samples in this block, one per lane
            if (B.b >= 0 && B.min_scale != -1 && B.ts == A.timestamp)
                while (ri_run(A, R, B, r, lx, ly, lz, computed, s_rd, lane) == 32) {
                }
        }
    }
    for (; rel < e1; ++rel)
        if (!ri_pass(A, rel, lane))
            return;
}

__global__ void __launch_bounds__(256) ri_rays_kernel(RiArgs A)
{
    __shared__ float s_rd[8][32];
    const int lane = threadIdx.x & 31;
    for (;;) {
        int ray = 0;
        if (lane == 0)
            ray = ri_aborted(A) ? A.n : atomicAdd(&A.ctl->next_ray, 1);
        ray = __shfl_sync(kFull, ray, 0);
        if (ray >= A.n)
            return;
        ri_ray(A, ray, lane, s_rd[threadIdx.x >> 5]);
    }
}

// Octree::allocateChildren(root) opens every ray's operator()().
__global__ void ri_root_kernel(RiArgs A)
{
    ri_allocate_children(A, 0, threadIdx.x & 31);
}

// ------------------------------------------------------------------------ propagation --

// propagateBlocksToCoarsestScale (ray_integrator_impl.hpp:124-132): one warp per updated block.
__global__ void __launch_bounds__(256) ri_blocks_kernel(RiArgs A)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int n_warps = (gridDim.x * blockDim.x) >> 5;
    const int n = min(A.ctl->n_updated, A.updated_cap);
    for (int i = warp; i < n; i += n_warps) {
        RiBlock B;
        ri_load_block(A, A.updated[i], B);
        if (B.current_scale != kOccMaxScale)
            ri_propagate_to_scale(A.m, B, kOccMaxScale, lane);
    }
}

__device__ __forceinline__ void ri_list_insert(const RiArgs& A, int n, int depth)
{
    if (n < 0)
        return;
    if (atomicExch(&A.node_mark[n], A.stamp) == A.stamp)
        return;
    const int k = atomicAdd(&A.ctl->list_n[depth], 1);
    if (k < A.m.node_capacity)
        A.lists[depth & 1][k] = n;
    else
        atomicOr(&A.ctl->err, kRiErrList);
}

// the parents of the updated blocks: node_set_[block_depth - 1]
__global__ void ri_seed_kernel(RiArgs A)
{
    const int n = min(A.ctl->n_updated, A.updated_cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        ri_list_insert(A, A.m.block_state[A.updated[i]].parent, A.m.block_depth - 1);
}

// ray_integrator::propagate_to_parent_node (ray_integrator_core_impl.hpp:104-176)
__device__ OccD ri_propagate_node(const OccDevice& m, int n, int timestamp)
{
    m.node_ts[n] = timestamp;
    float max_o = -FLT_MAX, max_mean = 0.0f, max_w = 0.0f;
    float min_o = FLT_MAX, min_mean = 0.0f, min_w = 0.0f;
    int max_cnt = 0, min_cnt = 0, observed = 0;
    for (int i = 0; i < 8; ++i) {
        const int c = m.node_child[8 * (size_t) n + i];
        if (c == -1)
            continue;
        OccD cmin, cmax;
        if (slot_is_block(c)) {
            const int b = slot_block(c);
            const int fin = m.block_state[b].finest;
            cmin = blk_min(m, b, fin, kOccMaxScale)[0];
            cmax = blk_max(m, b, fin, kOccMaxScale)[0];
        }
        else {
            cmin = m.node_min[c];
            cmax = m.node_max[c];
        }
        if (cmin.weight > 0.0f) {
            const float o = occ_field(cmin);
            if (o < min_o) {
                min_mean = cmin.occ;
                min_w = cmin.weight;
                min_o = o;
                min_cnt++;
            }
        }
        if (cmax.weight > 0.0f) {
            const float o = occ_field(cmax);
            if (o > max_o) {
                max_mean = cmax.occ;
                max_w = cmax.weight;
                max_o = o;
                max_cnt++;
            }
        }
        if (cmax.observed)
            observed++;
    }
    OccD mn = m.node_min[n], mx = m.node_max[n];
    if (min_cnt > 0) {
        mn.occ = min_mean;
        mn.weight = min_w;
        if (observed == 8)
            mn.observed = 1;
    }
    if (max_cnt > 0) {
        mx.occ = max_mean;
        mx.weight = max_w;
        if (observed == 8)
            mx.observed = 1;
    }
    m.node_min[n] = mn;
    m.node_max[n] = mx;
    return mx;
}

// Octree::deleteChildren: detach the subtree; its blocks stop being live
__device__ void ri_delete_children(const RiArgs& A, int n)
{
    const OccDevice& m = A.m;
    int stack[64];
    int sp = 0;
    stack[sp++] = n;
    while (sp > 0) {
        const int q = stack[--sp];
        for (int i = 0; i < 8; ++i) {
            const int c = m.node_child[8 * (size_t) q + i];
            if (c == -1)
                continue;
            if (slot_is_block(c))
                m.block_state[slot_block(c)].live = 0;
            else if (sp < 64)
                stack[sp++] = c;
            else
                atomicOr(&A.ctl->err, kRiErrList);
            m.node_child[8 * (size_t) q + i] = -1;
        }
    }
}

// One depth of propagateToRoot (ray_integrator_impl.hpp:314-350).
__global__ void ri_nodes_kernel(RiArgs A, int depth)
{
    const OccDevice& m = A.m;
    const int count = min(A.ctl->list_n[depth], m.node_capacity);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int n = A.lists[depth & 1][i];
        if (m.node_ts[n] == A.timestamp)
            continue;
        if (m.node_parent[n] < 0)
            continue;
        const OccD nd = ri_propagate_node(m, n, A.timestamp);
        ri_list_insert(A, m.node_parent[n], depth - 1);
        const int k = atomicAdd(&A.ctl->n_out_nodes, 1);
        if (k < m.node_capacity) {
            A.out_nodes[k] = n;
            A.out_erased[k] = 0;
        }
        if (nd.observed && (double) occ_field(nd) <= 0.95 * -100.0) {
            bool leaf = true;
            for (int c = 0; c < 8; ++c)
                leaf &= m.node_child[8 * (size_t) n + c] == -1;
            if (!leaf && k < m.node_capacity)
                A.out_erased[k] = 1; // updated_octants_->erase(octant_ptr)
            ri_delete_children(A, n);
        }
    }
}

__global__ void ri_root_prop_kernel(RiArgs A) { ri_propagate_node(A.m, 0, A.timestamp); }

// The updated octants (x, y, z, size): the updated blocks, then the propagated nodes that were
// not pruned.
__global__ void ri_out_kernel(RiArgs A, int32_t* __restrict__ out, long long capacity, int* count)
{
    const OccDevice& m = A.m;
    const int nb = min(A.ctl->n_updated, A.updated_cap);
    const int nn = min(A.ctl->n_out_nodes, m.node_capacity);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb + nn; i += gridDim.x * blockDim.x) {
        int4 o;
        if (i < nb) {
            const int b = A.updated[i];
            o = make_int4(m.block_coord[3 * b], m.block_coord[3 * b + 1], m.block_coord[3 * b + 2], 8);
        }
        else {
            if (A.out_erased[i - nb])
                continue;
            o = m.node_coord[A.out_nodes[i - nb]];
        }
        const int k = atomicAdd(count, 1);
        if (out && k < capacity) {
            out[4 * (size_t) k] = o.x;
            out[4 * (size_t) k + 1] = o.y;
            out[4 * (size_t) k + 2] = o.z;
            out[4 * (size_t) k + 3] = o.w;
        }
    }
}

} // namespace

// ------------------------------------------------------------------------ host side --

struct RiScratch {
    int ray_cap = 0;
    long long entry_cap = 0;
    int node_cap = 0, block_cap = 0;
    int stamp = 0;
    RiRay* rays = nullptr;
    int* counts = nullptr;
    long long* offsets = nullptr;
    RiEntry* entries = nullptr;
    unsigned long long* keys[2] = {nullptr, nullptr};
    int* vals[2] = {nullptr, nullptr};
    int* done = nullptr;
    void* cub_tmp = nullptr;
    size_t cub_bytes = 0;
    int* block_mark = nullptr;
    int* updated = nullptr;
    int* node_lock = nullptr;
    int* node_mark = nullptr;
    int* lists[2] = {nullptr, nullptr};
    int* out_nodes = nullptr;
    unsigned char* out_erased = nullptr;
    RiCtl* ctl = nullptr;
    int* out_count = nullptr;
};

void ri_scratch_free(RiScratch* s)
{
    if (!s)
        return;
    cudaFree(s->rays);
    cudaFree(s->counts);
    cudaFree(s->offsets);
    cudaFree(s->entries);
    for (int i = 0; i < 2; ++i) {
        cudaFree(s->keys[i]);
        cudaFree(s->vals[i]);
        cudaFree(s->lists[i]);
    }
    cudaFree(s->done);
    cudaFree(s->cub_tmp);
    cudaFree(s->block_mark);
    cudaFree(s->updated);
    cudaFree(s->node_lock);
    cudaFree(s->node_mark);
    cudaFree(s->out_nodes);
    cudaFree(s->out_erased);
    cudaFree(s->ctl);
    cudaFree(s->out_count);
    delete s;
}

namespace {

template <class T>
cudaError_t ri_grow(T*& p, size_t n)
{
    cudaFree(p);
    p = nullptr;
    return cudaMalloc(&p, n * sizeof(T) + 16);
}

se_gpu_status ri_prepare(se_gpu_occ_map* om, int n, cudaStream_t stream)
{
    if (!om->ri) {
        om->ri = new RiScratch();
        RiScratch& s = *om->ri;
        const OccDevice& m = om->dev;
        s.node_cap = m.node_capacity;
        s.block_cap = m.block_capacity;
        SE_CUDA_TRY(ri_grow(s.block_mark, (size_t) s.block_cap));
        SE_CUDA_TRY(ri_grow(s.updated, (size_t) s.block_cap));
        SE_CUDA_TRY(ri_grow(s.node_lock, (size_t) s.node_cap));
        SE_CUDA_TRY(ri_grow(s.node_mark, (size_t) s.node_cap));
        SE_CUDA_TRY(ri_grow(s.lists[0], (size_t) s.node_cap));
        SE_CUDA_TRY(ri_grow(s.lists[1], (size_t) s.node_cap));
        SE_CUDA_TRY(ri_grow(s.out_nodes, (size_t) s.node_cap));
        SE_CUDA_TRY(ri_grow(s.out_erased, (size_t) s.node_cap));
        SE_CUDA_TRY(ri_grow(s.ctl, 1));
        SE_CUDA_TRY(ri_grow(s.out_count, 1));
        SE_CUDA_TRY(cudaMemsetAsync(s.block_mark, 0, (size_t) s.block_cap * sizeof(int), stream));
        SE_CUDA_TRY(cudaMemsetAsync(s.node_lock, 0, (size_t) s.node_cap * sizeof(int), stream));
        SE_CUDA_TRY(cudaMemsetAsync(s.node_mark, 0, (size_t) s.node_cap * sizeof(int), stream));
    }
    RiScratch& s = *om->ri;
    if (n > s.ray_cap) {
        const int cap = n + n / 4 + 64;
        SE_CUDA_TRY(ri_grow(s.rays, (size_t) cap));
        SE_CUDA_TRY(ri_grow(s.counts, (size_t) cap + 1));
        SE_CUDA_TRY(ri_grow(s.offsets, (size_t) cap + 1));
        s.ray_cap = cap;
    }
    return SE_GPU_OK;
}

se_gpu_status ri_prepare_entries(RiScratch& s, long long total)
{
    if (total > s.entry_cap) {
        const long long cap = total + total / 4 + 1024;
        SE_CUDA_TRY(ri_grow(s.entries, (size_t) cap));
        for (int i = 0; i < 2; ++i) {
            SE_CUDA_TRY(ri_grow(s.keys[i], (size_t) cap));
            SE_CUDA_TRY(ri_grow(s.vals[i], (size_t) cap));
        }
        SE_CUDA_TRY(ri_grow(s.done, (size_t) cap));
        s.entry_cap = cap;
    }
    return SE_GPU_OK;
}

} // namespace

} // namespace se_gpu

using namespace se_gpu;

extern "C" se_gpu_status se_gpu_occ_integrate_ray_batch(se_gpu_map* map, const se_gpu_leica_lidar* sensor,
                                                        const float* poses_dev, const float* rays_dev, int64_t n,
                                                        int32_t timestamp, int32_t* octants_dev, int64_t capacity,
                                                        int64_t* n_octants, void* stream_p)
{
    if (!map || !map->occ || !sensor || !n_octants || n < 0 || n > (1ll << 30) || (n > 0 && (!poses_dev || !rays_dev))
        || capacity < 0 || (capacity > 0 && !octants_dev)) {
        set_last_error("se_gpu_occ_integrate_ray_batch: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (!(sensor->near_plane > 0.0f) || !(sensor->far_plane > sensor->near_plane)
        || !(sensor->elevation_resolution_deg > 0.0f) || !(sensor->azimuth_resolution_deg > 0.0f)) {
        set_last_error("se_gpu_occ_integrate_ray_batch: invalid LeicaLidar configuration");
        return SE_GPU_ERR_BAD_ARG;
    }
    *n_octants = 0;
    if (n == 0)
        return SE_GPU_OK;
    se_gpu_occ_map* om = map->occ;
    cudaStream_t stream = (cudaStream_t) stream_p;
    se_gpu_status st = ri_prepare(om, (int) n, stream);
    if (st != SE_GPU_OK)
        return st;
    RiScratch& s = *om->ri;
    const OccDevice& m = om->dev;
    s.stamp = s.stamp == INT_MAX ? 1 : s.stamp + 1;
    if (s.stamp == 1) {
        SE_CUDA_TRY(cudaMemsetAsync(s.block_mark, 0, (size_t) s.block_cap * sizeof(int), stream));
        SE_CUDA_TRY(cudaMemsetAsync(s.node_mark, 0, (size_t) s.node_cap * sizeof(int), stream));
    }
    RiArgs A;
    A.m = m;
    A.poses = poses_dev;
    A.rays = rays_dev;
    A.n = (int) n;
    A.timestamp = timestamp;
    A.stamp = s.stamp;
    A.near_plane = sensor->near_plane;
    A.far_plane = sensor->far_plane;
    // LeicaLidar's ctor (leica_lidar.cpp:53-73) and computeIntegrationScaleImpl's denominator
    const float min_ray_angle = std::min(sensor->azimuth_resolution_deg, sensor->elevation_resolution_deg);
    const float deg_to_rad = (float) (M_PI / 180.0);
    A.pixel_dim_tan = 2.0f * std::tan(min_ray_angle * 0.5f * deg_to_rad);
    A.pv_den = 1.0f / (std::sqrt(3.0f) * m.res);
    // RayIntegratorConfig (ray_integrator.hpp:60-72)
    A.sigma_min = m.cfg.sigma_min_factor * m.res;
    A.sigma_max = m.cfg.sigma_max_factor * m.res;
    A.tau_min = m.cfg.tau_min_factor * m.res;
    A.tau_max = m.cfg.tau_max_factor * m.res;
    A.nb = m.size / 8;
    int rb = 1;
    while ((1ll << rb) < n)
        ++rb;
    int lb = 0;
    while ((1 << lb) < A.nb)
        ++lb;
    if (3 * lb + rb > 64) {
        set_last_error("se_gpu_occ_integrate_ray_batch: %lld rays exceed the sort key of a map of %d voxels",
                       (long long) n, m.size);
        return SE_GPU_ERR_BAD_ARG;
    }
    A.ray_bits = rb;
    A.R = s.rays;
    A.counts = s.counts;
    A.offsets = s.offsets;
    A.block_mark = s.block_mark;
    A.updated = s.updated;
    A.updated_cap = s.block_cap;
    A.node_lock = s.node_lock;
    A.node_mark = s.node_mark;
    A.lists[0] = s.lists[0];
    A.lists[1] = s.lists[1];
    A.out_nodes = s.out_nodes;
    A.out_erased = s.out_erased;
    A.ctl = s.ctl;
    SE_CUDA_TRY(cudaMemsetAsync(s.ctl, 0, sizeof(RiCtl), stream));
    SE_CUDA_TRY(cudaMemsetAsync(s.out_count, 0, sizeof(int), stream));

    const int sms = device_sm_count();
    ri_prep_kernel<<<(int) ((n + 1 + 127) / 128), 128, 0, stream>>>(A);
    SE_CUDA_TRY(cudaGetLastError());
    size_t bytes = 0;
    SE_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, bytes, s.counts, s.offsets, (int) n + 1, stream));
    if (bytes > s.cub_bytes) {
        cudaFree(s.cub_tmp);
        s.cub_tmp = nullptr;
        SE_CUDA_TRY(cudaMalloc(&s.cub_tmp, bytes));
        s.cub_bytes = bytes;
    }
    SE_CUDA_TRY(cub::DeviceScan::ExclusiveSum(s.cub_tmp, bytes, s.counts, s.offsets, (int) n + 1, stream));
    long long total = 0;
    SE_CUDA_TRY(cudaMemcpyAsync(&total, s.offsets + n, sizeof(long long), cudaMemcpyDeviceToHost, stream));
    SE_CUDA_TRY(cudaStreamSynchronize(stream));
    if (total >= (1ll << 31)) {
        set_last_error("se_gpu_occ_integrate_ray_batch: %lld ray-block pairs exceed the batch limit", total);
        return SE_GPU_ERR_BAD_ARG;
    }
    st = ri_prepare_entries(s, total);
    if (st != SE_GPU_OK)
        return st;
    A.entries = s.entries;
    A.keys = s.keys[0];
    A.vals = s.vals[0];
    A.done = s.done;
    if (total > 0) {
        ri_fill_kernel<<<(int) ((n + 127) / 128), 128, 0, stream>>>(A);
        SE_CUDA_TRY(cudaGetLastError());
        cub::DoubleBuffer<unsigned long long> dk(s.keys[0], s.keys[1]);
        cub::DoubleBuffer<int> dv(s.vals[0], s.vals[1]);
        const int end_bit = 3 * lb + rb;
        bytes = 0;
        SE_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, bytes, dk, dv, (int) total, 0, end_bit, stream));
        if (bytes > s.cub_bytes) {
            cudaFree(s.cub_tmp);
            s.cub_tmp = nullptr;
            SE_CUDA_TRY(cudaMalloc(&s.cub_tmp, bytes));
            s.cub_bytes = bytes;
        }
        SE_CUDA_TRY(cub::DeviceRadixSort::SortPairs(s.cub_tmp, bytes, dk, dv, (int) total, 0, end_bit, stream));
        ri_rank_kernel<<<sms * 4, 256, 0, stream>>>(A, dk.Current(), dv.Current(), total);
        SE_CUDA_TRY(cudaGetLastError());
    }
    ri_root_kernel<<<1, 32, 0, stream>>>(A);
    SE_CUDA_TRY(cudaGetLastError());
    ri_rays_kernel<<<sms * 4, 256, 0, stream>>>(A);
    SE_CUDA_TRY(cudaGetLastError());
    RiCtl ctl;
    SE_CUDA_TRY(cudaMemcpyAsync(&ctl, s.ctl, sizeof(RiCtl), cudaMemcpyDeviceToHost, stream));
    SE_CUDA_TRY(cudaStreamSynchronize(stream));
    if (ctl.err) {
        se_gpu_status pool = occ_check(om);
        if (pool != SE_GPU_OK)
            return pool;
        set_last_error("se_gpu_occ_integrate_ray_batch: %s",
                       (ctl.err & kRiErrTimeout) ? "a ray waited too long for a block (the batch was abandoned)"
                       : (ctl.err & kRiErrList) ? "the updated-block list overflowed"
                       : (ctl.err & kRiErrEntry) ? "a sample fell outside its ray's block list"
                                                 : "the octree is inconsistent");
        return SE_GPU_ERR_CUDA;
    }
    ri_blocks_kernel<<<sms * 4, 256, 0, stream>>>(A);
    ri_seed_kernel<<<sms, 256, 0, stream>>>(A);
    for (int d = m.block_depth - 1; d > 0; --d) {
        ri_nodes_kernel<<<sms * 2, 256, 0, stream>>>(A, d);
        // the next depth's list is filled by this launch; the one after reuses this depth's array
    }
    ri_root_prop_kernel<<<1, 1, 0, stream>>>(A);
    ri_out_kernel<<<sms * 2, 256, 0, stream>>>(A, octants_dev, capacity, s.out_count);
    SE_CUDA_TRY(cudaGetLastError());
    int cnt = 0;
    SE_CUDA_TRY(cudaMemcpyAsync(&cnt, s.out_count, sizeof(int), cudaMemcpyDeviceToHost, stream));
    SE_CUDA_TRY(cudaMemcpyAsync(&ctl, s.ctl, sizeof(RiCtl), cudaMemcpyDeviceToHost, stream));
    SE_CUDA_TRY(cudaStreamSynchronize(stream));
    *n_octants = cnt;
    if (ctl.err) {
        set_last_error("se_gpu_occ_integrate_ray_batch: a propagation list overflowed");
        return SE_GPU_ERR_POOL_FULL;
    }
    return occ_check(om);
}
