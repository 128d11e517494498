// track.cu — se::Tracker::track: projective point-to-plane ICP over a 3-level depth pyramid.
//
// Per frame: half_sample_robust_image x2, depth_to_point_cloud and point_cloud_to_normal for the
// three levels, then the ICP iterations (coarse to fine, {4, 5, 10} by default):
//   - every thread evaluates trackKernel for a strided set of pixels (icp_impl.hpp:16-102) and
//     accumulates the 32 reduction values of newReduce (icp.cpp:45-184) in FP32 with two-sum
//     compensation (hi, lo pairs);
//   - shared memory gives one compensated partial per CTA, which the CTA adds exactly (integer
//     fixed point, order-independent) into global accumulators;
//   - the totals give the 6x6 normal equations, solved by FP64 elimination; the FP64 se(3)
//     exponential is applied and the pose composed in FP64 (icp.cpp:15-41,208-223,
//     math_util_impl.hpp:117-174), and the level stops when |x| < threshold.
// By default one cooperative launch per frame runs every iteration (icp_persistent_kernel: each
// CTA waits for the complete totals and solves redundantly) and checkPoseKernel
// (icp.cpp:227-246) at its end. Where that grid cannot be resident at once, one launch per
// iteration (icp_iter_kernel: the last CTA to finish, by an atomic ticket, solves; later
// iterations of a converged level return at entry, so the launch sequence is fixed and can be
// captured in a CUDA graph) and a final check kernel give the same poses bit for bit.
#include <cmath>
#include <cstddef>
#include <cstring>
#include <mutex>

#include "pipeline.cuh"
#include "profile.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

int device_sm_count();

constexpr int kTrackThreads = 256;
constexpr int kMaxTrackCtas = 1024;

enum {
    kFlagDone0 = 0,  // level converged flags 0..2
    kFlagIters0 = 3, // iterations run per level 3..5
    kFlagAccepted = 6,
    kFlagBarrierTimeout = 7, // the persistent ICP kernel's wait for an iteration's merged totals gave up
    kFlagOverflow = 8,       // a CTA partial outside the exact merge's range (|v| >= 2^38)
    kNumFlags = 9
};

struct TrackState {
    // the 80 bytes a synchronous track() reads back: pose_f then flags
    float pose_f[12];    // FP32 copy of T_WS used by the per-pixel kernel
    int flags[kNumFlags];
    double pose[12];     // T_WS, row-major 3x4, FP64
    float ref_inv[12];   // (T_WS_ref)^-1 in FP32
    float ref_f[12];     // T_WS_ref
    float last_red[32];  // final reduction of the last iteration run
    unsigned int ticket;
    unsigned int end_ticket; // CTAs done with the persistent kernel (the last one runs the check)
};
constexpr size_t kTrackReadback = sizeof(float) * 12 + sizeof(int) * kNumFlags;

struct LevelImages {
    const float* depth[3];
    float* pts[3];
    float* nrm[3];
    int w[3], h[3];
    Pinhole s[3];
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

struct CSum {
    float hi, lo;
    __device__ __forceinline__ void add(float v)
    {
        float s, e;
        two_sum(hi, v, s, e);
        hi = s;
        lo = lo + e;
    }
    __device__ __forceinline__ void merge(float h2, float l2)
    {
        float s, e;
        two_sum(hi, h2, s, e);
        hi = s;
        lo = (lo + l2) + e;
    }
};

// ------------------------------------------------------------- exact partial merge --
// Each CTA's compensated sum (hi, lo) of a reduction term is split, by integer operations on the
// float bits, into a fixed-point integer part in units of 2^-10 and a fraction in units of 2^-50
// (bits below 2^-50 are dropped), and both are added with 64-bit integer atomics into one of four
// copies of the term (by CTA index, each copy on its own 128-byte line, to spread the atomics
// over L2). Integer sums do not depend on the order of arrival, so the merged totals, and the
// poses computed from them, are the same run to run and between the persistent and the
// per-iteration kernels. A partial of magnitude 2^38 or more (or not finite) raises
// kFlagOverflow: the pose is then rejected and the call reports an error. The persistent kernel
// adds 2^56 to both words with every partial: the top byte of a word counts the partials it has
// received (at most 128 CTAs per copy, so the values stay below 2^55 in magnitude), and a CTA
// knows the totals of an iteration are complete when every word's count is, without a
// separate barrier (icp_await_totals).
constexpr int kAccCopies = 4;
constexpr int kAccStride = 16;                                // u64 words per (copy, term)
constexpr size_t kAccBufWords = (size_t) kAccCopies * 32 * kAccStride;
constexpr int kAccBuffers = 3;                                // the persistent kernel rotates

__device__ __forceinline__ void fixed_split(float f, long long& I, unsigned long long& F, bool& bad)
{
    const unsigned b = __float_as_uint(f);
    const int e = (int) ((b >> 23) & 0xffu);
    const unsigned long long m = (b & 0x7fffffu) | (e ? 0x800000u : 0u);
    const int ee = e ? e : 1; // |f| = m 2^(ee - 150)
    I = 0;
    F = 0;
    if (e == 0xff || ee > 164) { // |f| >= 2^38: |I| could reach 2^48
        bad = true;
        return;
    }
    if (ee >= 140) {
        I = (long long) (m << (ee - 140)); // < 2^52
    }
    else if (ee >= 100) {
        const unsigned long long x = m << (ee - 100); // units of 2^-50, < 2^64
        I = (long long) (x >> 40);
        F = x & ((1ull << 40) - 1);
    }
    else if (100 - ee < 24) {
        F = m >> (100 - ee);
    }
    if (b >> 31) { // -(I 2^40 + F) with F in [0, 2^40)
        if (F) {
            I = -I - 1;
            F = (1ull << 40) - F;
        }
        else {
            I = -I;
        }
    }
}

__device__ __forceinline__ void acc_add(unsigned long long* buf, int copy, int term, float hi, float lo, bool& bad,
                                        unsigned long long count = 0)
{
    long long I1, I2;
    unsigned long long F1, F2;
    fixed_split(hi, I1, F1, bad);
    fixed_split(lo, I2, F2, bad);
    unsigned long long* p = buf + ((size_t) copy * 32 + term) * kAccStride;
    // reductions without a returned value: the issuing thread does not wait for them (the grid
    // barrier's release orders them before the arrival)
    asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"((unsigned long long) (I1 + I2) + count)
                 : "memory");
    asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p + 1), "l"(F1 + F2 + count) : "memory");
}

// The total A 2^-10 + B 2^-50 of a term's merged integer sums.
__device__ __forceinline__ double acc_total_of(long long A, unsigned long long B)
{
    // A 2^-10 and B 2^-50 as doubles without a 64-bit integer conversion: an integer added to the
    // bits of 1.5 2^k (|integer| < 2^51) gives 1.5 2^k + integer 2^(k-52) exactly, and subtracting
    // 1.5 2^k leaves the scaled integer (k = 42: units of 2^-10; k = 2: units of 2^-50). The sum of
    // the two rounds once, like fma((double) B, 2^-50, (double) A 2^-10).
    const long long kMagic10 = 0x4298000000000000LL, kMagic50 = 0x4018000000000000LL;
    const double hi = (A > -(1LL << 51) && A < (1LL << 51))
        ? __longlong_as_double(kMagic10 + A) - __longlong_as_double(kMagic10)
        : (double) A * 0x1p-10;
    const double lo = B < (1ULL << 51) ? __longlong_as_double(kMagic50 + (long long) B) - __longlong_as_double(kMagic50)
                                       : (double) B * 0x1p-50;
    return hi + lo;
}

__device__ __forceinline__ double acc_total(const unsigned long long* buf, int term)
{
    long long A = 0;
    unsigned long long B = 0;
#pragma unroll
    for (int c = 0; c < kAccCopies; ++c) {
        const unsigned long long* p = buf + ((size_t) c * 32 + term) * kAccStride;
        A += (long long) __ldcg(p);
        B += __ldcg(p + 1);
    }
    return acc_total_of(A, B);
}

// Zeroes the two words of every (copy, term) of a buffer, threads tid of nthreads.
__device__ __forceinline__ void acc_clear(unsigned long long* buf, int tid, int nthreads)
{
    for (int i = tid; i < kAccCopies * 32 * 2; i += nthreads)
        buf[(size_t) (i >> 1) * kAccStride + (i & 1)] = 0ull;
}

// half_sample_robust_image (src/map/preprocessor.cpp:156-195) for output pixel (x, y) with
// radius 1: the mean of the 2 x 2 input pixels within e_d of the top-left one.
__device__ __forceinline__ float half_sample_px(const float* __restrict__ in, int in_w, int ow, int oh, float e_d,
                                                int x, int y)
{
    const int px = 2 * x, py = 2 * y;
    float count = 0.0f, sum = 0.0f;
    const float centre = in[px + py * in_w];
    for (int i = 0; i <= 1; ++i) {
        for (int j = 0; j <= 1; ++j) {
            int qx = px + j, qy = py + i;
            qx = min(max(qx, 0), 2 * ow - 1);
            qy = min(max(qy, 0), 2 * oh - 1);
            const float v = in[qx + qy * in_w];
            if (fabsf(v - centre) < e_d) {
                count += 1.0f;
                sum += v;
            }
        }
    }
    return sum / count;
}

__device__ __forceinline__ F3 ld3(const float* p, size_t i) { return f3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

// depth_to_point_cloud and point_cloud_to_normal<NegY> for one pixel (x, y), straight from the
// depth image (the points of the pixel and of its four neighbours are formed on the fly with
// the same float operations as the point image would hold).
__device__ __forceinline__ F3 depth_point(const float* __restrict__ depth, const Pinhole& s, int w, int x, int y)
{
    const float d = depth[x + w * y];
    if (d > 0.0f)
        return mul(d, back_project(s, (float) x, (float) y));
    return f3(0.0f, 0.0f, 0.0f);
}

// point_cloud_to_normal<NegY> for pixel (x, y), reading the neighbours' points from the depth
// image
__device__ __forceinline__ F3 depth_normal(const float* __restrict__ depth, const Pinhole& s, int w, int h, int x,
                                           int y, int neg_y)
{
    const F3 p = depth_point(depth, s, w, x, y);
    if (p.z == 0.0f)
        return f3(0.0f, 0.0f, 0.0f);
    const int lx = max(x - 1, 0), rx = min(x + 1, w - 1);
    int uy, dy;
    if (neg_y) {
        uy = max(y - 1, 0);
        dy = min(y + 1, h - 1);
    }
    else {
        dy = max(y - 1, 0);
        uy = min(y + 1, h - 1);
    }
    const F3 left = depth_point(depth, s, w, lx, y), right = depth_point(depth, s, w, rx, y);
    const F3 up = depth_point(depth, s, w, x, uy), down = depth_point(depth, s, w, x, dy);
    if (left.z == 0.0f || right.z == 0.0f || up.z == 0.0f || down.z == 0.0f)
        return f3(0.0f, 0.0f, 0.0f);
    return normalized(cross(sub(right, left), sub(up, down)));
}

// depth_to_point_cloud (include/se/map/impl/preprocessor_impl.hpp:18-40) and
// point_cloud_to_normal<NegY> (src/map/preprocessor.cpp:109-152) for every level, one launch.
__global__ void points_normals_kernel(LevelImages li, int levels, int neg_y)
{
    grid_dep_wait();
    const int l = blockIdx.z;
    if (l >= levels)
        return;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int w = li.w[l], h = li.h[l];
    if (x >= w || y >= h)
        return;
    const int i = x + w * y;
    const F3 p = depth_point(li.depth[l], li.s[l], w, x, y);
    const F3 n = depth_normal(li.depth[l], li.s[l], w, h, x, y, neg_y);
    float* op = li.pts[l] + 3 * (size_t) i;
    float* on = li.nrm[l] + 3 * (size_t) i;
    op[0] = p.x;
    op[1] = p.y;
    op[2] = p.z;
    on[0] = n.x;
    on[1] = n.y;
    on[2] = n.z;
}

struct TrackInit {
    float T_WS[12];
    float ref_inv[12];
};

// With pose12_in the start pose is read from the device (row-major 3x4) and its inverse is
// formed here with the same float operations the host would use. One thread.
__device__ void track_init(TrackState* st, TrackInit init, const float* pose12_in)
{
    if (pose12_in) {
        const Tf T = tf_from12(pose12_in);
        const Tf Ti = inverse_iso(T);
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) {
                init.T_WS[4 * i + j] = T.R[3 * i + j];
                init.ref_inv[4 * i + j] = Ti.R[3 * i + j];
            }
            init.T_WS[4 * i + 3] = T.t[i];
            init.ref_inv[4 * i + 3] = Ti.t[i];
        }
    }
    for (int i = 0; i < 12; ++i) {
        st->pose[i] = (double) init.T_WS[i];
        st->pose_f[i] = init.T_WS[i];
        st->ref_f[i] = init.T_WS[i];
        st->ref_inv[i] = init.ref_inv[i];
    }
    for (int i = 0; i < 32; ++i)
        st->last_red[i] = 0.0f;
    for (int i = 0; i < kNumFlags; ++i)
        st->flags[i] = 0;
    st->ticket = 0;
    st->end_ticket = 0;
}

__global__ void track_init_kernel(TrackState* st, TrackInit init, const float* pose12_in)
{
    track_init(st, init, pose12_in);
}

// The first launch of a track(): block 0 initialises the state and clears the merge
// accumulators; every thread forms the depth of one level-1 pixel and, with three levels, the
// first thread of each 2 x 2 group forms the level-2 depth from the group's values
// (half_sample_robust_image twice, the second pass on the first's values). A warp covers 16 x 2
// level-1 pixels (lane & 15, lane >> 4), so a group's values meet by shuffles; a CTA of 32 x 8
// threads covers 16 x 16. Grid: ceil(w1 / 16) x ceil(h1 / 16) (one block when there is no
// pyramid).
__global__ void pyramid_init_kernel(TrackState* st, TrackInit init, const float* pose12_in, unsigned long long* acc,
                                    LevelImages li, int levels, float e_d, float* __restrict__ d1,
                                    float* __restrict__ d2)
{
    grid_dep_wait();
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    if (blockIdx.x == 0 && blockIdx.y == 0) {
        for (int b = 0; b < kAccBuffers; ++b)
            acc_clear(acc + (size_t) b * kAccBufWords, tid, blockDim.x * blockDim.y);
        if (tid == 0)
            track_init(st, init, pose12_in);
    }
    if (levels < 2)
        return;
    const int lane = tid & 31, warp = tid >> 5;
    const int x1 = blockIdx.x * 16 + (lane & 15), y1 = blockIdx.y * 16 + 2 * warp + (lane >> 4);
    const int w1 = li.w[1], h1 = li.h[1];
    float v = 0.0f;
    if (x1 < w1 && y1 < h1) {
        v = half_sample_px(li.depth[0], li.w[0], w1, h1, e_d, x1, y1);
        d1[x1 + y1 * w1] = v;
    }
    if (levels < 3)
        return;
    // the group of (x1, y1) with x1, y1 even: (x1 + 1, y1), (x1, y1 + 1), (x1 + 1, y1 + 1)
    float q[2][2];
    q[0][0] = v;
    q[0][1] = __shfl_down_sync(0xffffffffu, v, 1);
    q[1][0] = __shfl_down_sync(0xffffffffu, v, 16);
    q[1][1] = __shfl_down_sync(0xffffffffu, v, 17);
    if ((lane & 1) != 0 || lane >= 16)
        return;
    const int x2 = x1 >> 1, y2 = y1 >> 1;
    if (x2 >= li.w[2] || y2 >= li.h[2])
        return;
    // the 2 x 2 level-1 pixels of this output are in range (2 x2 + 1 <= 2 w2 - 1): no clamping
    const float centre = q[0][0];
    float count = 0.0f, sum = 0.0f;
#pragma unroll
    for (int i = 0; i <= 1; ++i)
#pragma unroll
        for (int j = 0; j <= 1; ++j)
            if (fabsf(q[i][j] - centre) < e_d) {
                count += 1.0f;
                sum += q[i][j];
            }
    d2[x2 + y2 * li.w[2]] = sum / count;
}

// ---------------------------------------------------------------------- FP64 solve --
// Measured on GB300: the FP64 pipe of an SM sub-partition completes one warp instruction
// (DFMA, DMUL, DADD, or a conversion to or from FP64) every ~63 cycles, with any number of
// active lanes, and a dependent one follows after as long; warps on different sub-partitions
// run their FP64 instructions in parallel. The solve and update are therefore arranged by the
// number of FP64 instructions each warp issues on the critical path:
//   - the 6x6 system [C | b] is eliminated by two warps, one entry per lane, in six
//     division-free steps (row_i <- d_j row_i - a_ij row_j for every row i != j: LDL^T's
//     trailing update with the back substitution folded in), two FP64 instructions per step;
//   - the six divisions x_i = b_i / D_i at the end use one reciprocal each, seeded in FP32 on
//     the mantissa (the pivots' products outgrow FP32's range) and refined by one FP64 Newton
//     step (relative error ~1e-14);
//   - the exponential's coefficients (one warp), the cross products it multiplies (another)
//     and the convergence test (a third) run side by side, and the new pose follows from them
//     in four FP64 instructions.

__device__ __forceinline__ double drcp(double x)
{
    const float xf = (float) x;
    if (!(fabsf(xf) > 1e-30f && fabsf(xf) < 1e30f))
        return 1.0 / x;
    const double r = (double) (1.0f / xf);
    return fma(r, fma(-x, r, 1.0), r);
}

// d > 0 and finite, from the bits (no FP64 instruction): positive sign, nonzero, exponent not
// all ones. A pivot failing it makes the reference's LLT fail and its update zero
// (icp.cpp:33-41).
__device__ __forceinline__ bool pivot_ok(double d)
{
    const long long b = __double_as_longlong(d);
    return b > 0 && (b >> 52) < 0x7ff;
}

// b / d for a finite d > 0 of any magnitude: d = m 2^e with m in [1, 2), 1 / m from drcp, the
// quotient b (1 / m) rescaled by 2^-e through its exponent field.
__device__ __forceinline__ double div_pos(double b, double d)
{
    const int hi = __double2hiint(d), lo = __double2loint(d);
    const int e = ((hi >> 20) & 0x7ff) - 1023;
    const double m = __hiloint2double((hi & 0x800fffff) | 0x3ff00000, lo);
    const double q = b * drcp(m);
    const long long qb = __double_as_longlong(q);
    const int qe = (int) ((qb >> 52) & 0x7ff);
    if (qe == 0 || qe == 0x7ff || qe - e <= 0 || qe - e >= 0x7ff)
        return b / d; // zero, subnormal, or a result outside the normal range: the IEEE division
    return __longlong_as_double(qb - (long long) e * (1LL << 52));
}

// x < y for x, y >= 0 (or x NaN: false), by the bits: no FP64 instruction.
__device__ __forceinline__ bool lt_nonneg(double x, double y) { return __double_as_longlong(x) < __double_as_longlong(y); }

// Series coefficients (Horner, highest first) of A = sin t / t, B = (1 - cos t) / t^2 and
// C = (t - sin t) / t^3 in x = t^2.
__constant__ double kExpSeries[3][5] = {{1.0 / 362880, -1.0 / 5040, 1.0 / 120, -1.0 / 6, 1.0},
                                        {1.0 / 3628800, -1.0 / 40320, 1.0 / 720, -1.0 / 24, 0.5},
                                        {1.0 / 39916800, -1.0 / 362880, 1.0 / 5040, -1.0 / 120, 1.0 / 6}};

__device__ __forceinline__ double pick3(int k, double a, double b, double c) { return k == 0 ? a : (k == 1 ? b : c); }

// Named barrier of the first `nthreads` threads (whole warps) of the CTA.
__device__ __forceinline__ void bar_named(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Solves C x = b (C symmetric, the packed upper triangle of the newReduce layout in sh_val[7..27],
// b = sh_val[1..6], icp.cpp:15-41), forms exp(x) (math_util_impl.hpp:117-174 in Rodrigues form:
// R = I + A W + B W^2, V = I + B W + C W^2, W = hat(omega), translation V rho) and composes
// T <- exp(x) T with the pose sh_pose (row-major 3x4): R T applied column by column as
// c + A (omega x c) + B (omega x (omega x c)), the translation plus V rho. Writes the new pose to
// sh_new / sh_newf and |x| < threshold to *sh_conv. Called by every thread of the CTA; warps 0
// and 1 (two sub-partitions, so their FP64 instructions run side by side) do the work and
// synchronise among themselves with a named barrier, the other warps wait at the CTA barrier at
// the end.
__device__ __noinline__ void icp_tail(const double* sh_val, const double* sh_pose, double* sh_new, float* sh_newf,
                                      int* sh_conv, float icp_threshold)
{
    __shared__ double M[2][42];
    __shared__ double sh_x[6];
    __shared__ double sh_coef[3];
    __shared__ double sh_u[16], sh_u2[16];
    __shared__ int sh_ok;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp < 2) {
        // elimination: entry e = 21 warp + lane (lanes < 21) is (r, c) of the 6 x 7 system; each
        // lane keeps its entry in a register and publishes it for the other rows each step
        const bool gj = lane < 21;
        const int e = warp * 21 + lane, r = e / 7, c = e % 7;
        double a = 0.0;
        if (gj) {
            const int lo = r < c ? r : c, hi = r < c ? c : r;
            a = c == 6 ? sh_val[1 + r] : sh_val[7 + lo * 6 - lo * (lo - 1) / 2 + (hi - lo)];
            M[0][e] = a;
        }
        if (threadIdx.x == 0)
            sh_ok = 1;
        bar_named(1, 64);
#pragma unroll 1
        for (int j = 0; j < 6; ++j) {
            const double* Mi = M[j & 1];
            double* Mo = M[(j + 1) & 1];
            if (gj) {
                const double d = Mi[7 * j + j];
                if (r != j)
                    a = c == j ? 0.0 : fma(d, a, -(Mi[7 * r + j] * Mi[7 * j + c]));
                Mo[e] = a;
                if (e == 0 && !pivot_ok(d))
                    sh_ok = 0;
            }
            bar_named(1, 64);
        }
        if (gj && c == 6)
            sh_x[r] = sh_ok ? div_pos(a, M[0][7 * r + r]) : 0.0;
        bar_named(1, 64);

        const double wx = sh_x[3], wy = sh_x[4], wz = sh_x[5];
        if (warp == 0) {
            // lanes 0, 1, 2: the coefficients A, B, C
            const double xx = fma(wz, wz, fma(wy, wy, wx * wx));
            const int k = lane < 3 ? lane : 0;
            double coef;
            if (lt_nonneg(xx, 0.01)) {
                // Horner in x; below 1e-5 (1e-7) the terms past x^2 (x) are under 1e-18 relative
                const int first = lt_nonneg(xx, 1e-7) ? 3 : (lt_nonneg(xx, 1e-5) ? 2 : 0);
                coef = kExpSeries[k][first];
#pragma unroll 1
                for (int u = first + 1; u < 5; ++u)
                    coef = fma(coef, xx, kExpSeries[k][u]);
            }
            else {
                const double t = sqrt(xx);
                double sn, cs;
                sincos(t, &sn, &cs);
                const double it = drcp(t), it2 = it * it;
                coef = k == 0 ? sn * it : (k == 1 ? (1.0 - cs) * it2 : (t - sn) * it2 * it);
            }
            if (lane < 3)
                sh_coef[lane] = coef;
        }
        else {
            // lanes 0..11: column lane / 3, row lane % 3 of the pose; lanes 12..14: rho
            const int l = lane < 15 ? lane : 14;
            const int col = l / 3, i = l % 3, i1 = i == 2 ? 0 : i + 1, i2 = i == 0 ? 2 : i - 1;
            const double v1 = l < 12 ? sh_pose[4 * i1 + col] : sh_x[i1];
            const double v2 = l < 12 ? sh_pose[4 * i2 + col] : sh_x[i2];
            const double u = fma(pick3(i1, wx, wy, wz), v2, -(pick3(i2, wx, wy, wz) * v1)); // (omega x v)_i
            const int base = l - i;
            const double u1 = __shfl_sync(0xffffffffu, u, base + i1), u2 = __shfl_sync(0xffffffffu, u, base + i2);
            const double uu = fma(pick3(i1, wx, wy, wz), u2, -(pick3(i2, wx, wy, wz) * u1));
            if (lane < 15) {
                sh_u[lane] = u;
                sh_u2[lane] = uu;
            }
            // the convergence test in FP32, as the reference's x.norm() < icp_threshold on its
            // FP32 x (icp.cpp:218)
            const float xf = lane < 6 ? (float) sh_x[lane] : 0.0f;
            float q = xf * xf;
            q += __shfl_down_sync(0xffffffffu, q, 4);
            q += __shfl_down_sync(0xffffffffu, q, 2);
            q += __shfl_down_sync(0xffffffffu, q, 1);
            if (lane == 0)
                *sh_conv = sqrtf(q) < icp_threshold;
        }
        bar_named(1, 64);
        if (warp == 1) {
            const int l = lane < 15 ? lane : 14;
            const int col = l / 3, i = l % 3;
            const double c1 = l < 12 ? sh_coef[0] : sh_coef[1], c2 = l < 12 ? sh_coef[1] : sh_coef[2];
            const double v = l < 12 ? sh_pose[4 * i + col] : sh_x[i];
            double val = fma(c2, sh_u2[l], fma(c1, sh_u[l], v));
            const double vrho = __shfl_down_sync(0xffffffffu, val, 3); // lanes 9..11 take V rho from 12..14
            if (lane >= 9 && lane < 12)
                val += vrho;
            if (lane < 12) {
                sh_new[4 * i + col] = val;
                sh_newf[4 * i + col] = (float) val;
            }
        }
    }
    __syncthreads();
}

struct IterParams {
    const float* ref_pts;
    const float* ref_nrm;
    const float* pts;
    const float* nrm;
    int w, h;          // level size
    int W;             // full-resolution width (row stride of the reference images)
    int level;
    float dist_threshold, normal_threshold, icp_threshold;
    int ncta, nthr;    // ICP pass partition: CTAs and threads per CTA that hold pixels at this level
};

// trackKernel for one pixel (icp_impl.hpp:16-102) given its input normal and point, its 32
// reduction terms of newReduce (icp.cpp:45-184) added into sum: [e^2, e*J (6), upper J^T J (21),
// inlier, dist-reject, normal-reject, other reject].
__device__ __forceinline__ void icp_pixel_add(const Pinhole& s, const IterParams& ip, const Tf& T, const Tf& Tri,
                                              bool in_range, F3 n_in, F3 p_S, float sum[32])
{
    if (!in_range)
        return;
    int result;
    float e = 0.0f;
    float J[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (n_in.x == 0.0f && n_in.y == 0.0f && n_in.z == 0.0f) {
        result = -1;
    }
    else {
        const F3 p_W = apply(T, p_S);
        const F3 p_ref = apply(Tri, p_W);
        float u, vv;
        if (!project(s, p_ref, u, vv)) {
            result = -2;
        }
        else {
            const int px = (int) (u + 0.5f), py = (int) (vv + 0.5f);
            const size_t ri = (size_t) px + (size_t) py * ip.W;
            const F3 rn = ld3(ip.ref_nrm, ri);
            const F3 rp = ld3(ip.ref_pts, ri);
            const F3 n_ref = f3(-rn.x, -rn.y, -rn.z);
            if (n_ref.x == 0.0f && n_ref.y == 0.0f && n_ref.z == 0.0f) {
                result = -3;
            }
            else {
                const F3 diff = sub(rp, p_W);
                const F3 n_W = rot(T, n_in);
                if (norm(diff) > ip.dist_threshold) {
                    result = -4;
                }
                else if (dot(n_W, n_ref) < ip.normal_threshold) {
                    result = -5;
                }
                else {
                    result = 1;
                    e = dot(n_ref, diff);
                    const F3 c = cross(p_W, n_ref);
                    J[0] = n_ref.x;
                    J[1] = n_ref.y;
                    J[2] = n_ref.z;
                    J[3] = c.x;
                    J[4] = c.y;
                    J[5] = c.z;
                }
            }
        }
    }
    if (result < 1) {
        sum[29] += result == -4 ? 1.0f : 0.0f;
        sum[30] += result == -5 ? 1.0f : 0.0f;
        sum[31] += result > -4 ? 1.0f : 0.0f;
        return;
    }
    sum[0] += e * e;
#pragma unroll
    for (int k = 0; k < 6; ++k)
        sum[1 + k] += e * J[k];
    int q = 7;
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int c = r; c < 6; ++c)
            sum[q++] += J[r] * J[c];
    sum[28] += 1.0f;
}

// Lane k of the warp adds term k of the 32 lanes' sums into its compensated accumulators
// (the 32 x 32 term matrix goes through shared memory, stride 33: conflict-free), and the sums
// restart from zero.
__device__ __forceinline__ void icp_flush_terms(float sum[32], float (*sh_t)[33], CSum acc[4])
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 32; ++k) {
        sh_t[lane][k] = sum[k];
        sum[k] = 0.0f;
    }
    __syncwarp();
#pragma unroll 4
    for (int j = 0; j < 32; ++j)
        acc[j & 3].add(sh_t[j][lane]);
    __syncwarp();
}

// Pixels a thread adds in plain FP32 before its sums go into the compensated accumulators.
constexpr int kIcpFlushRounds = 8;

// ------------------------------------------------------------------ ICP main pass --
// One CTA per SM, kIcpThreads threads. Each thread takes pixels i, i + S, i + 2S, ... of the
// level (S = CTAs x threads) two at a time: both pixels' inputs, then both projections, then
// both reference gathers in flight together, then both pixels' terms (the next pair's inputs
// are loaded meanwhile). trackKernel's decisions (icp_impl.hpp:16-102) use the same float
// operations as the oracle; the 28 reduction sums of newReduce (icp.cpp:45-184) are
// accumulated per thread with fused multiply-adds over at most 8 pixels, then lane k of the
// warp adds term k of the 32 lanes into two-sum compensated accumulators; the four counters
// (inliers, distance rejects, normal rejects, other rejects) are integers.
constexpr int kIcpThreads = 512;
constexpr int kIcpWarps = kIcpThreads / 32;
constexpr int kIcpPairRounds = 4; // pairs a thread adds before its sums go to the compensated accumulators

struct IcpIn {
    F3 n, p;
    bool in;
};

__device__ __forceinline__ IcpIn icp_load(const IterParams& ip, int i, int npix)
{
    IcpIn a;
    a.in = i < npix;
    if (a.in) {
        a.n = ld3(ip.nrm, (size_t) i);
        a.p = ld3(ip.pts, (size_t) i);
    }
    else {
        a.n = f3(0.0f, 0.0f, 0.0f);
        a.p = a.n;
    }
    return a;
}

// A pixel after its projection: code 0 = gather the reference pixel ri; -1 / -2 = rejected
// (invalid input normal / projection outside); 2 = no pixel.
struct IcpPre {
    int code;
    int ri;
    F3 p_W, n_in;
};

__device__ __forceinline__ IcpPre icp_pre(const Pinhole& s, const IterParams& ip, const Tf& T, const Tf& Tri,
                                          const IcpIn& a)
{
    IcpPre q;
    q.code = 2;
    q.ri = 0;
    q.p_W = f3(0.0f, 0.0f, 0.0f);
    q.n_in = a.n;
    if (!a.in)
        return q;
    if (a.n.x == 0.0f && a.n.y == 0.0f && a.n.z == 0.0f) {
        q.code = -1;
        return q;
    }
    q.p_W = apply(T, a.p);
    const F3 p_ref = apply(Tri, q.p_W);
    float u, v;
    if (!project(s, p_ref, u, v)) {
        q.code = -2;
        return q;
    }
    q.ri = (int) (u + 0.5f) + (int) (v + 0.5f) * ip.W;
    q.code = 0;
    return q;
}

struct IcpRef {
    F3 rn, rp;
};

__device__ __forceinline__ IcpRef icp_ref(const IterParams& ip, const IcpPre& q)
{
    IcpRef r;
    if (q.code == 0) {
        r.rn = ld3(ip.ref_nrm, (size_t) q.ri);
        r.rp = ld3(ip.ref_pts, (size_t) q.ri);
    }
    else {
        r.rn = f3(0.0f, 0.0f, 0.0f);
        r.rp = r.rn;
    }
    return r;
}

// The rest of trackKernel for one projected pixel, and its terms added.
__device__ __forceinline__ void icp_finish(const IterParams& ip, const Tf& T, const IcpPre& q, const IcpRef& r,
                                           float sum[28], int cnt[4])
{
    if (q.code == 2)
        return;
    int result = q.code;
    float e = 0.0f;
    float J[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (result == 0) {
        const F3 n_ref = f3(-r.rn.x, -r.rn.y, -r.rn.z);
        if (n_ref.x == 0.0f && n_ref.y == 0.0f && n_ref.z == 0.0f) {
            result = -3;
        }
        else {
            const F3 diff = sub(r.rp, q.p_W);
            const F3 n_W = rot(T, q.n_in);
            if (norm(diff) > ip.dist_threshold) {
                result = -4;
            }
            else if (dot(n_W, n_ref) < ip.normal_threshold) {
                result = -5;
            }
            else {
                result = 1;
                e = dot(n_ref, diff);
                const F3 c = cross(q.p_W, n_ref);
                J[0] = n_ref.x;
                J[1] = n_ref.y;
                J[2] = n_ref.z;
                J[3] = c.x;
                J[4] = c.y;
                J[5] = c.z;
            }
        }
    }
    if (result < 1) {
        cnt[1] += result == -4 ? 1 : 0;
        cnt[2] += result == -5 ? 1 : 0;
        cnt[3] += result > -4 ? 1 : 0;
        return;
    }
    cnt[0] += 1;
    sum[0] = __fmaf_rn(e, e, sum[0]);
#pragma unroll
    for (int k = 0; k < 6; ++k)
        sum[1 + k] = __fmaf_rn(e, J[k], sum[1 + k]);
    int q2 = 7;
#pragma unroll
    for (int rr = 0; rr < 6; ++rr)
#pragma unroll
        for (int cc = rr; cc < 6; ++cc) {
            sum[q2] = __fmaf_rn(J[rr], J[cc], sum[q2]);
            ++q2;
        }
}

// Lane k (< 28) of the warp sums term k of the 32 lanes' sums (the 32 x 28 term matrix goes
// through this warp's slice of shared memory, stride 29: conflict-free) in plain FP32, pairwise
// over four partial sums of eight, and adds the result into its compensated accumulator; the
// sums restart from zero.
constexpr int kIcpTermStride = 29;
constexpr size_t kIcpDynSmem = (size_t) kIcpWarps * 32 * kIcpTermStride * sizeof(float);

__device__ __forceinline__ void icp_flush28(float sum[28], float* sh_t, CSum& acc)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 28; ++k) {
        sh_t[lane * kIcpTermStride + k] = sum[k];
        sum[k] = 0.0f;
    }
    __syncwarp();
    if (lane < 28) {
        float p[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int j = 0; j < 32; ++j)
            p[j & 3] += sh_t[j * kIcpTermStride + lane];
        acc.add((p[0] + p[1]) + (p[2] + p[3]));
    }
    __syncwarp();
}

// The first pair of pixels a thread of CTA cta takes at a level (loaded ahead of the pass).
__device__ __forceinline__ void icp_first_pair(const IterParams& ip, int cta, IcpIn& a, IcpIn& b)
{
    const int npix = ip.w * ip.h;
    const int i = cta < ip.ncta && (int) threadIdx.x < ip.nthr ? cta * ip.nthr + (int) threadIdx.x : npix;
    a = icp_load(ip, i, npix);
    b = icp_load(ip, i + ip.ncta * ip.nthr, npix);
}

// This CTA's share of one ICP iteration: its pixels' terms summed and merged exactly into the
// global accumulators buf (copy cta % kAccCopies). Threads tid < ip.nthr of CTAs cta < ip.ncta
// hold pixels (one per thread at the coarse levels, about four at full resolution); (a, b) is
// the thread's first pair (icp_first_pair). Every thread of the CTA calls it; ends with a CTA
// barrier. Warp 0 merges the warps' compensated partials of term k (lane k) in warp order. With
// counted set (the persistent kernel) every CTA adds, those without pixels zeros, and each
// addition carries the count kAccCount.
constexpr unsigned long long kAccCount = 1ull << 56;

__device__ __forceinline__ void icp_cta_pass(const Pinhole& s, const IterParams& ip, const Tf T, const Tf Tri,
                                             int cta, unsigned long long* buf, int* overflow_flag, IcpIn a, IcpIn b,
                                             bool counted)
{
    extern __shared__ float icp_dyn_smem[]; // kIcpDynSmem bytes: the warps' term matrices
    __shared__ float2 sh_warp[kIcpWarps][32];
    __shared__ int sh_cnt[4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool active = cta < ip.ncta && (int) threadIdx.x < ip.nthr; // uniform per warp
    if (threadIdx.x < 4)
        sh_cnt[threadIdx.x] = 0;
    CSum acc{0.0f, 0.0f};
    int cnt[4] = {0, 0, 0, 0};
    if (active) {
        float sum[28];
#pragma unroll
        for (int k = 0; k < 28; ++k)
            sum[k] = 0.0f;
        const int npix = ip.w * ip.h;
        const int stride = ip.ncta * ip.nthr;
        int i = cta * ip.nthr + threadIdx.x;
        int rounds = 0;
        for (int base = cta * ip.nthr; base < npix; base += 2 * stride) { // uniform across the active warps
            const int inext = i + 2 * stride;
            const IcpIn a2 = icp_load(ip, inext, npix), b2 = icp_load(ip, inext + stride, npix);
            const IcpPre qa = icp_pre(s, ip, T, Tri, a), qb = icp_pre(s, ip, T, Tri, b);
            const IcpRef ra = icp_ref(ip, qa), rb = icp_ref(ip, qb);
            icp_finish(ip, T, qa, ra, sum, cnt);
            icp_finish(ip, T, qb, rb, sum, cnt);
            if (++rounds == kIcpPairRounds || base + 2 * stride >= npix) {
                icp_flush28(sum, icp_dyn_smem + warp * 32 * kIcpTermStride, acc);
                rounds = 0;
            }
            a = a2;
            b = b2;
            i = inext;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            cnt[k] = __reduce_add_sync(0xffffffffu, cnt[k]);
        sh_warp[warp][lane] = make_float2(acc.hi, acc.lo);
    }
    __syncthreads();
    if (active && lane < 4 && cnt[lane] != 0)
        atomicAdd(&sh_cnt[lane], cnt[lane]);
    __syncthreads();
    if (warp == 0 && (counted || cta < ip.ncta)) {
        float hi = 0.0f, lo = 0.0f;
        if (cta >= ip.ncta) {
            // no pixels at this level: zeros, so that the counts stay those of the whole grid
        }
        else if (lane < 28) {
            CSum t{0.0f, 0.0f};
            const int nw = ip.nthr >> 5;
            for (int wi = 0; wi < nw; ++wi)
                t.merge(sh_warp[wi][lane].x, sh_warp[wi][lane].y);
            hi = t.hi;
            lo = t.lo;
        }
        else {
            hi = (float) sh_cnt[lane - 28]; // exact: at most 2^24 pixels per CTA
            lo = 0.0f;
        }
        bool bad = false;
        acc_add(buf, cta % kAccCopies, lane, hi, lo, bad, counted ? kAccCount : 0ull);
        if (bad)
            atomicExch(overflow_flag, 1);
    }
    __syncthreads();
}

// The merged totals of buf in sh_val (warp 0), and the final reduction in st->last_red when
// record is set.
__device__ __forceinline__ void icp_read_totals(const unsigned long long* buf, double* sh_val, TrackState* st,
                                                bool record)
{
    if (threadIdx.x < 32) {
        const double v = acc_total(buf, threadIdx.x);
        sh_val[threadIdx.x] = v;
        if (record)
            st->last_red[threadIdx.x] = (float) v;
    }
}

__device__ __forceinline__ void icp_pose_to_shared(const TrackState* st, Tf& T, Tf& Tri, double* sh_pose)
{
    if (threadIdx.x < 12) {
        const int i = threadIdx.x, r = i >> 2, c = i & 3;
        if (c < 3) {
            T.R[3 * r + c] = st->pose_f[i];
            Tri.R[3 * r + c] = st->ref_inv[i];
        }
        else {
            T.t[r] = st->pose_f[i];
            Tri.t[r] = st->ref_inv[i];
        }
        if (sh_pose)
            sh_pose[i] = st->pose[i];
    }
}

// One ICP iteration (the fallback when the persistent grid cannot be resident at once):
// every CTA adds its partial; the last CTA to finish (atomic ticket, no waiting) solves and
// updates the pose. Same partition, merge and tail as the persistent kernel: bit-identical poses.
__global__ void __launch_bounds__(kIcpThreads, 1) icp_iter_kernel(Pinhole s, IterParams ip, TrackState* st,
                                                                 unsigned long long* __restrict__ acc_buf)
{
    __shared__ Tf T, Tri;
    __shared__ int sh_last;
    if (st->flags[kFlagDone0 + ip.level])
        return;
    icp_pose_to_shared(st, T, Tri, nullptr);
    __syncthreads();
    const Tf Tl = T, Tril = Tri;
    IcpIn a, b;
    icp_first_pair(ip, blockIdx.x, a, b);
    icp_cta_pass(s, ip, Tl, Tril, blockIdx.x, acc_buf, &st->flags[kFlagOverflow], a, b, false);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0)
        sh_last = (atomicAdd(&st->ticket, 1u) == gridDim.x - 1) ? 1 : 0;
    __syncthreads();
    if (!sh_last)
        return;
    __threadfence();

    // ---- last CTA
    __shared__ double sh_pose[12];
    __shared__ double sh_val[32];
    __shared__ double sh_new[12];
    __shared__ float sh_newf[12];
    __shared__ int sh_conv;
    if (threadIdx.x < 12)
        sh_pose[threadIdx.x] = __ldcg(&st->pose[threadIdx.x]);
    icp_read_totals(acc_buf, sh_val, st, true);
    __syncthreads();
    icp_tail(sh_val, sh_pose, sh_new, sh_newf, &sh_conv, ip.icp_threshold);
    acc_clear(acc_buf, threadIdx.x, blockDim.x); // for the next launch (every CTA has added)
    if (threadIdx.x < 12) {
        st->pose[threadIdx.x] = sh_new[threadIdx.x];
        st->pose_f[threadIdx.x] = sh_newf[threadIdx.x];
    }
    if (threadIdx.x == 0) {
        st->ticket = 0;
        st->flags[kFlagIters0 + ip.level] += 1;
        if (sh_conv)
            st->flags[kFlagDone0 + ip.level] = 1;
    }
}

// checkPoseKernel (icp.cpp:227-246): revert to the reference pose on a poor final alignment.
__device__ void icp_check(TrackState* st, int W, int H, float track_threshold, float* pose12_out)
{
    const float* v = st->last_red;
    // a timed-out wait for the totals of the persistent ICP leaves no trustworthy pose: reject it
    const bool reject = ((double) sqrtf(v[0] / v[28]) > 2e-2) || (v[28] / (float) (W * H) < track_threshold)
        || st->flags[kFlagBarrierTimeout] != 0 || st->flags[kFlagOverflow] != 0;
    if (reject) {
        for (int i = 0; i < 12; ++i) {
            st->pose_f[i] = st->ref_f[i];
            st->pose[i] = (double) st->ref_f[i];
        }
    }
    st->flags[kFlagAccepted] = reject ? 0 : 1;
    if (pose12_out)
        for (int i = 0; i < 12; ++i)
            pose12_out[i] = st->pose_f[i];
}

__global__ void icp_check_kernel(TrackState* st, int W, int H, float track_threshold, float* pose12_out)
{
    icp_check(st, W, H, track_threshold, pose12_out);
}

// ------------------------------------------------------- persistent ICP (all iterations) --
// The per-iteration launches above, fused into one cooperative launch per frame, one CTA per
// SM: every CTA runs every iteration of every level; after each iteration's pass every CTA waits
// until the merged totals are complete (the count bytes of the accumulator words, no separate
// barrier), reads them and solves redundantly (the same operations on the same values, so every
// CTA holds the same new pose) instead of one last CTA solving and the next launch reading its
// result. The pixel partition, the exact merge's integer totals and the FP64 tail are those of
// icp_iter_kernel, so the poses are bit-identical to it.

struct IcpLevels {
    IterParams ip[3];
    int nctas[3];
    int iters[3];
    int levels;
    int W, H;           // checkPoseKernel's image size and threshold, and where the pose goes
    float track_threshold;
    float* pose12_out;
    int missing_ctas;   // test aid: CTAs the barrier waits for beyond the grid (0 in use)
};

constexpr unsigned kIcpSpinLimit = 1u << 24;                // polls at most, and
constexpr unsigned long long kIcpWaitNs = 500000000ull;     // half a second at most, then the timeout flag

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The merged totals of one iteration of the persistent kernel, awaited by warp 0 of every CTA in
// place of a grid barrier: lane k reads the two words of term k in the four copies (relaxed
// loads at GPU scope, all in flight together) until every word's count byte has advanced, since
// this buffer's previous use (prev, this CTA's copy of the words then, in shared memory), by the
// number of CTAs that add into that copy (the grid's CTAs of that residue; copy 0 waits for
// `missing` more, a test aid); the totals are the advances less their counts. The buffers are
// never cleared within a launch: a CTA adds to a buffer again only three iterations later, after
// every CTA's additions of the two iterations between, which every CTA makes only after it has
// read this one. Bounded: on timeout (or when another CTA timed out) the flag is set and the CTA
// goes on with what has arrived, so a stuck launch ends with an error instead of hanging.
__device__ __forceinline__ void icp_await_totals(const unsigned long long* buf, unsigned long long (*prev)[32],
                                                 int ngrid, int missing, double* sh_val, TrackState* st,
                                                 bool record, int* timeout)
{
    if (threadIdx.x >= 32)
        return;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x;
    unsigned long long w[kAccCopies][2];
    long long A = 0;
    unsigned long long B = 0;
    unsigned spins = 0;
    const unsigned long long t0 = global_ns();
    while (true) {
#pragma unroll
        for (int c = 0; c < kAccCopies; ++c) {
            const unsigned long long* p = buf + ((size_t) c * 32 + lane) * kAccStride;
            asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(w[c][0]) : "l"(p) : "memory");
            asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(w[c][1]) : "l"(p + 1) : "memory");
        }
        bool ok = true;
        A = 0;
        B = 0;
#pragma unroll
        for (int c = 0; c < kAccCopies; ++c) {
            const unsigned long long n =
                (unsigned long long) ((ngrid - c + kAccCopies - 1) / kAccCopies + (c == 0 ? missing : 0)) & 0xffull;
            const unsigned long long dI = w[c][0] - prev[2 * c][lane], dF = w[c][1] - prev[2 * c + 1][lane];
            const unsigned long long cI = (dI + (kAccCount >> 1)) >> 56, cF = (dF + (kAccCount >> 1)) >> 56;
            ok = ok && cI == n && cF == n;
            A += (long long) (dI - (cI << 56));
            B += dF - (cF << 56);
        }
        if (__all_sync(full, ok))
            break;
        // uniform across the warp: spins is, and the decision is the warp's
        if ((++spins & 15u) == 0u) {
            const bool give_up = *((volatile int*) timeout) != 0 || spins > kIcpSpinLimit
                || global_ns() - t0 > kIcpWaitNs;
            if (__any_sync(full, give_up)) {
                if (lane == 0)
                    atomicExch(timeout, 1);
                break;
            }
        }
    }
#pragma unroll
    for (int c = 0; c < kAccCopies; ++c) {
        prev[2 * c][lane] = w[c][0];
        prev[2 * c + 1][lane] = w[c][1];
    }
    const double v = acc_total_of(A, B);
    sh_val[lane] = v;
    if (record)
        st->last_red[lane] = (float) v;
}

__global__ void __launch_bounds__(kIcpThreads, 1) icp_persistent_kernel(Pinhole s, IcpLevels L, TrackState* st,
                                                                       unsigned long long* __restrict__ acc_base)
{
    __shared__ Tf T, Tri;
    __shared__ double sh_pose[12];
    __shared__ double sh_new[12];
    __shared__ float sh_newf[12];
    __shared__ double sh_val[32];
    __shared__ int sh_conv;
    // the accumulator words as this CTA last read them, per buffer (zero: the tracker's state
    // init clears the buffers before the launch)
    __shared__ unsigned long long sh_prev[kAccBuffers][2 * kAccCopies][32];
    for (int i = threadIdx.x; i < kAccBuffers * 2 * kAccCopies * 32; i += blockDim.x)
        (&sh_prev[0][0][0])[i] = 0ull;
    icp_pose_to_shared(st, T, Tri, sh_pose);
    // the first pair of the next pass is loaded before the wait for the totals and the tail of the
    // current iteration (its inputs do not depend on the pose), assuming the level goes on; a
    // level that converges early reloads it
    int pf_level = L.levels - 1;
    IcpIn pa, pb;
    icp_first_pair(L.ip[pf_level], blockIdx.x, pa, pb);
    __syncthreads();
    unsigned phase = 0;
    for (int level = L.levels - 1; level >= 0; --level) {
        const IterParams& ip = L.ip[level];
        for (int iter = 0; iter < L.iters[level]; ++iter) {
            unsigned long long* buf = acc_base + (size_t) (phase % kAccBuffers) * kAccBufWords;
            if (pf_level != level)
                icp_first_pair(ip, blockIdx.x, pa, pb);
            {
                const Tf Tl = T, Tril = Tri; // the poses in registers for the pass
                icp_cta_pass(s, ip, Tl, Tril, blockIdx.x, buf, &st->flags[kFlagOverflow], pa, pb, true);
            }
            pf_level = iter + 1 < L.iters[level] ? level : level - 1;
            if (pf_level >= 0)
                icp_first_pair(L.ip[pf_level], blockIdx.x, pa, pb);
            // every CTA: the merged totals, once complete, then the solve and update
            icp_await_totals(buf, sh_prev[phase % kAccBuffers], gridDim.x, L.missing_ctas, sh_val, st,
                             blockIdx.x == 0, &st->flags[kFlagBarrierTimeout]);
            ++phase;
            __syncthreads();
            icp_tail(sh_val, sh_pose, sh_new, sh_newf, &sh_conv, ip.icp_threshold);
            if (blockIdx.x == 0 && threadIdx.x == 0)
                st->flags[kFlagIters0 + level] = iter + 1; // a store: no global read on the critical path
            if (threadIdx.x < 12) {
                const int i = threadIdx.x, r = i >> 2, c = i & 3;
                sh_pose[i] = sh_new[i];
                if (c < 3)
                    T.R[3 * r + c] = sh_newf[i];
                else
                    T.t[r] = sh_newf[i];
            }
            __syncthreads();
            if (sh_conv) {
                if (blockIdx.x == 0 && threadIdx.x == 0)
                    st->flags[kFlagDone0 + level] = 1;
                break;
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < 12) {
        st->pose[threadIdx.x] = sh_pose[threadIdx.x];
        const int i = threadIdx.x, r = i >> 2, c = i & 3;
        st->pose_f[i] = c < 3 ? T.R[3 * r + c] : T.t[r];
    }
    // checkPoseKernel by the last CTA to finish: it sees the final pose and every flag
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0 && atomicAdd(&st->end_ticket, 1u) == gridDim.x - 1) {
        __threadfence();
        icp_check(st, L.W, L.H, L.track_threshold, L.pose12_out);
        st->end_ticket = 0;
    }
}

} // namespace se_gpu


using namespace se_gpu;

struct se_gpu_tracker {
    se_gpu_pinhole sensor;
    se_gpu_tracker_config config;
    Pinhole s;
    LevelImages li;
    int levels;
    float* pyr_depth[3]; // levels 1, 2 (index 0 unused: the input is level 0)
    float* pts[3];
    float* nrm[3];
    unsigned long long* acc; // kAccBuffers exact-merge accumulators (the persistent kernel rotates)
    TrackState* state;
    int nctas[3];        // CTAs that hold pixels at each level (at most one per SM)
    int nthrs[3];        // threads per CTA that hold pixels at each level
    int persistent;      // one cooperative launch per frame (when the grid fits on the GPU)
    int missing_ctas;    // se_gpu_tracker_test_barrier_timeout
    int persistent_ctas; // its grid: one CTA per SM
};

namespace se_gpu {
// The ICP kernels' dynamic shared memory (above the 48 KiB default), set once per process.
static cudaError_t icp_kernel_attributes()
{
    static std::once_flag once;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        err = cudaFuncSetAttribute(icp_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int) kIcpDynSmem);
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(icp_iter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int) kIcpDynSmem);
    });
    return err;
}

// Whether the persistent ICP's grid (one CTA per SM) can be resident at once.
static cudaError_t icp_persistent_fits(int ctas, bool& fits)
{
    int per_sm = 0;
    const cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, icp_persistent_kernel, kIcpThreads, kIcpDynSmem);
    // the count byte of the exact merge's words holds at most 128 CTAs per copy
    fits = e == cudaSuccess && per_sm * device_sm_count() >= ctas && ctas <= kAccCopies * 128;
    return e;
}
} // namespace se_gpu

extern "C" {

se_gpu_status se_gpu_tracker_create(const se_gpu_pinhole* sensor, const se_gpu_tracker_config* config,
                                    se_gpu_tracker** out)
{
    if (!sensor || !config || !out || sensor->width <= 0 || sensor->height <= 0 || config->num_levels < 1
        || config->num_levels > 3) {
        set_last_error("se_gpu_tracker_create: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    se_gpu_tracker* t = new se_gpu_tracker();
    std::memset(t, 0, sizeof(*t));
    t->sensor = *sensor;
    t->config = *config;
    t->s = make_pinhole(*sensor);
    t->levels = config->num_levels;
    auto fail = [&](cudaError_t e, const char* what) {
        se_gpu_status st = cuda_status(e, what);
        se_gpu_tracker_destroy(t);
        return st;
    };
    cudaError_t e;
    for (int l = 0; l < t->levels; ++l) {
        const int w = sensor->width / (1 << l), h = sensor->height / (1 << l);
        t->li.w[l] = w;
        t->li.h[l] = h;
        t->li.s[l] = downsampled(t->s, (float) (1 << l));
        if (l > 0 && (e = cudaMalloc(&t->pyr_depth[l], (size_t) w * h * sizeof(float))) != cudaSuccess)
            return fail(e, "cudaMalloc(pyramid)");
        if ((e = cudaMalloc(&t->pts[l], (size_t) w * h * 3 * sizeof(float))) != cudaSuccess)
            return fail(e, "cudaMalloc(points)");
        if ((e = cudaMalloc(&t->nrm[l], (size_t) w * h * 3 * sizeof(float))) != cudaSuccess)
            return fail(e, "cudaMalloc(normals)");
        t->li.pts[l] = t->pts[l];
        t->li.nrm[l] = t->nrm[l];
        t->li.depth[l] = t->pyr_depth[l];
        // one pixel per thread where the level allows, at most one CTA of kIcpThreads per SM:
        // every pixel's chain (projection, reference gather, terms) is latency-bound, so the
        // coarse levels run fastest with all their pixels in flight at once (measured at
        // 640x480 on GB300, ICP per frame: 4 pixels per thread at every level 118 us, 2 at
        // levels 1-2 106 us, 1 at levels 1-2 104 us); the full-resolution level fills the
        // grid with about four pixels per thread
        const long long want = (long long) w * h;
        const int sms = device_sm_count() < kMaxTrackCtas ? device_sm_count() : kMaxTrackCtas;
        const long long warps = (want + 31) / 32;
        t->nctas[l] = (int) (warps < sms ? (warps > 0 ? warps : 1) : sms);
        const long long per = (want + t->nctas[l] - 1) / t->nctas[l];
        const long long thr = (per + 31) / 32 * 32;
        t->nthrs[l] = (int) (thr < 32 ? 32 : (thr > kIcpThreads ? kIcpThreads : thr));
    }
    if ((e = cudaMalloc(&t->acc, kAccBuffers * kAccBufWords * sizeof(unsigned long long))) != cudaSuccess
        || (e = cudaMemset(t->acc, 0, kAccBuffers * kAccBufWords * sizeof(unsigned long long))) != cudaSuccess)
        return fail(e, "cudaMalloc(acc)");
    if ((e = icp_kernel_attributes()) != cudaSuccess)
        return fail(e, "cudaFuncSetAttribute(ICP shared memory)");
    {
        // the persistent kernel needs its whole grid resident at once
        t->persistent_ctas = 0;
        for (int l = 0; l < t->levels; ++l)
            t->persistent_ctas = t->nctas[l] > t->persistent_ctas ? t->nctas[l] : t->persistent_ctas;
        bool fits = false;
        if ((e = icp_persistent_fits(t->persistent_ctas, fits)) != cudaSuccess)
            return fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        t->persistent = fits ? 1 : 0;
    }
    if ((e = cudaMalloc(&t->state, sizeof(TrackState))) != cudaSuccess)
        return fail(e, "cudaMalloc(state)");
    if ((e = cudaMemset(t->state, 0, sizeof(TrackState))) != cudaSuccess)
        return fail(e, "cudaMemset(state)");
    *out = t;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_tracker_destroy(se_gpu_tracker* t)
{
    if (!t)
        return SE_GPU_OK;
    for (int l = 0; l < 3; ++l) {
        cudaFree(t->pyr_depth[l]);
        cudaFree(t->pts[l]);
        cudaFree(t->nrm[l]);
    }
    cudaFree(t->acc);
    cudaFree(t->state);
    delete t;
    return SE_GPU_OK;
}

// Enqueue the whole track on `stream` from a host pose. Asynchronous.
} // extern "C"

namespace se_gpu {

se_gpu_status enqueue_track(se_gpu_tracker* t, const float* depth_dev, const float* ref_pts, const float* ref_nrm,
                            const float* T_WS, float* pose12_io, cudaStream_t stream)
{
    TrackInit init;
    std::memset(&init, 0, sizeof(init));
    if (T_WS) {
        const Tf T = tf_from16(T_WS);
        const Tf Ti = inverse_iso(T);
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) {
                init.T_WS[4 * i + j] = T.R[3 * i + j];
                init.ref_inv[4 * i + j] = Ti.R[3 * i + j];
            }
            init.T_WS[4 * i + 3] = T.t[i];
            init.ref_inv[4 * i + 3] = Ti.t[i];
        }
    }
    const float* pose_in = T_WS ? nullptr : pose12_io;
    LevelImages li = t->li;
    li.depth[0] = depth_dev;
    {
    ProfScope ps(kProfTrackPrep, stream);
    const float e_d = 0.1f * 3;
    {
        // one thread per level-1 pixel, 16 x 16 per block (a single block without a pyramid)
        const dim3 b(32, 8);
        const dim3 g(t->levels > 1 ? (li.w[1] + 15) / 16 : 1, t->levels > 1 ? (li.h[1] + 15) / 16 : 1);
        launch_chained(pyramid_init_kernel, g, b, stream, t->state, init, pose_in, t->acc, li, t->levels, e_d,
                       t->pyr_depth[1], t->pyr_depth[2]);
    }
    {
        const dim3 b(32, 8), g((li.w[0] + 31) / 32, (li.h[0] + 7) / 8, t->levels);
        launch_chained(points_normals_kernel, g, b, stream, li, t->levels, t->s.left_hand);
    }
    }
    IcpLevels L;
    std::memset(&L, 0, sizeof(L));
    L.levels = t->levels;
    L.W = t->sensor.width;
    L.H = t->sensor.height;
    L.track_threshold = t->config.track_threshold;
    L.pose12_out = T_WS ? nullptr : pose12_io;
    L.missing_ctas = t->missing_ctas;
    for (int level = t->levels - 1; level >= 0; --level) {
        IterParams& ip = L.ip[level];
        ip.ref_pts = ref_pts;
        ip.ref_nrm = ref_nrm;
        ip.pts = t->pts[level];
        ip.nrm = t->nrm[level];
        ip.w = li.w[level];
        ip.h = li.h[level];
        ip.W = t->sensor.width;
        ip.level = level;
        ip.dist_threshold = t->config.dist_threshold;
        ip.normal_threshold = t->config.normal_threshold;
        ip.icp_threshold = t->config.icp_threshold;
        L.nctas[level] = t->nctas[level];
        ip.ncta = t->nctas[level];
        ip.nthr = t->nthrs[level];
        L.iters[level] = t->config.iterations[level];
    }
    if (t->persistent) {
        ProfScope ps(kProfIcpIter, stream);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(t->persistent_ctas);
        cfg.blockDim = dim3(kIcpThreads);
        cfg.dynamicSmemBytes = kIcpDynSmem;
        cfg.stream = stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        SE_CUDA_TRY(cudaLaunchKernelEx(&cfg, icp_persistent_kernel, t->s, L, t->state, t->acc));
    }
    else {
        for (int level = t->levels - 1; level >= 0; --level)
            for (int it = 0; it < t->config.iterations[level]; ++it) {
                ProfScope ps(kProfIcpIter, stream);
                icp_iter_kernel<<<t->nctas[level], kIcpThreads, kIcpDynSmem, stream>>>(t->s, L.ip[level], t->state,
                                                                                       t->acc);
            }
    }
    if (!t->persistent) { // the persistent kernel runs the check itself
        ProfScope ps(kProfIcpCheck, stream);
        icp_check_kernel<<<1, 1, 0, stream>>>(t->state, t->sensor.width, t->sensor.height,
                                              t->config.track_threshold, T_WS ? nullptr : pose12_io);
    }
    SE_CUDA_TRY(cudaGetLastError());
    return SE_GPU_OK;
}

int tracker_accepted_offset() { return (int) offsetof(TrackState, flags) + 4 * kFlagAccepted; }
void* tracker_state(se_gpu_tracker* t) { return t->state; }

} // namespace se_gpu

extern "C" {

se_gpu_status se_gpu_track(se_gpu_tracker* t, const float* depth_dev, const float* ref_pts, const float* ref_nrm,
                           float T_WS[16], int* accepted, void* stream_p)
{
    if (!t || !depth_dev || !ref_pts || !ref_nrm || !T_WS) {
        set_last_error("se_gpu_track: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    cudaStream_t stream = (cudaStream_t) stream_p;
    se_gpu_status st = enqueue_track(t, depth_dev, ref_pts, ref_nrm, T_WS, nullptr, stream);
    if (st != SE_GPU_OK)
        return st;
    TrackState hs;
    SE_CUDA_TRY(cudaMemcpyAsync(&hs, t->state, kTrackReadback, cudaMemcpyDeviceToHost, stream));
    SE_CUDA_TRY(cudaStreamSynchronize(stream));
    for (int i = 0; i < 12; ++i)
        T_WS[i] = hs.pose_f[i];
    T_WS[12] = T_WS[13] = T_WS[14] = 0.0f;
    T_WS[15] = 1.0f;
    if (accepted)
        *accepted = hs.flags[kFlagAccepted];
    if (hs.flags[kFlagBarrierTimeout]) {
        set_last_error("se_gpu_track: the ICP's wait for the merged totals timed out (the pose was reverted)");
        return SE_GPU_ERR_CUDA;
    }
    if (hs.flags[kFlagOverflow]) {
        set_last_error("se_gpu_track: an ICP partial sum exceeded the exact merge's range (the pose was reverted)");
        return SE_GPU_ERR_CUDA;
    }
    return SE_GPU_OK;
}

se_gpu_status se_gpu_tracker_set_persistent(se_gpu_tracker* t, int enable)
{
    if (!t) {
        set_last_error("se_gpu_tracker_set_persistent: null tracker");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (enable) {
        bool fits = false;
        SE_CUDA_TRY(icp_persistent_fits(t->persistent_ctas, fits));
        if (!fits) {
            set_last_error("se_gpu_tracker_set_persistent: %d CTAs do not fit on the device at once",
                           t->persistent_ctas);
            return SE_GPU_ERR_NOT_SUPPORTED;
        }
    }
    t->persistent = enable ? 1 : 0;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_tracker_test_barrier_timeout(se_gpu_tracker* t, int enable)
{
    if (!t) {
        set_last_error("se_gpu_tracker_test_barrier_timeout: null tracker");
        return SE_GPU_ERR_BAD_ARG;
    }
    t->missing_ctas = enable ? 1 : 0;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_tracker_level_images(se_gpu_tracker* t, int level, float* depth_dev, float* pts_dev,
                                          float* nrm_dev, void* stream_p)
{
    if (!t || level < 0 || level >= t->levels) {
        set_last_error("se_gpu_tracker_level_images: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    cudaStream_t stream = (cudaStream_t) stream_p;
    const size_t n = (size_t) t->li.w[level] * (size_t) t->li.h[level];
    if (depth_dev && level > 0)
        SE_CUDA_TRY(cudaMemcpyAsync(depth_dev, t->pyr_depth[level], n * sizeof(float), cudaMemcpyDeviceToDevice,
                                    stream));
    if (pts_dev)
        SE_CUDA_TRY(cudaMemcpyAsync(pts_dev, t->pts[level], 3 * n * sizeof(float), cudaMemcpyDeviceToDevice, stream));
    if (nrm_dev)
        SE_CUDA_TRY(cudaMemcpyAsync(nrm_dev, t->nrm[level], 3 * n * sizeof(float), cudaMemcpyDeviceToDevice, stream));
    return SE_GPU_OK;
}

se_gpu_status se_gpu_tracker_last_reduction(se_gpu_tracker* t, float reduction[32], int iterations_run[3])
{
    if (!t) {
        set_last_error("se_gpu_tracker_last_reduction: null tracker");
        return SE_GPU_ERR_BAD_ARG;
    }
    TrackState hs;
    SE_CUDA_TRY(cudaMemcpy(&hs, t->state, sizeof(TrackState), cudaMemcpyDeviceToHost));
    if (reduction)
        for (int i = 0; i < 32; ++i)
            reduction[i] = hs.last_red[i];
    if (iterations_run)
        for (int l = 0; l < 3; ++l)
            iterations_run[l] = hs.flags[kFlagIters0 + l];
    return SE_GPU_OK;
}

} // extern "C"

namespace se_gpu {

// ================================================== allocation-free single-level tracking ==
//
// Some callers cannot allocate device memory when they track: a host that has handed all
// free device memory to its own pool allocator, a real-time or certified loop whose memory
// budget is fixed at start-up, or a process that must not let cudaMalloc's implicit device
// synchronisation stall its other streams. se_gpu_track_noalloc serves them: the caller passes
// only its depth image, the reference raycast and the pose, and the ICP's scratch (the
// iteration state and the per-CTA partial sums) lives in the file-scope array below, which
// every GPU that loads this library keeps for the life of the process.
//
// It tracks at full resolution only (config->num_levels == 1): the input point cloud and
// normals are formed on the fly from the depth image, with the arithmetic of
// depth_to_point_cloud and point_cloud_to_normal, so no pyramid images are needed.

constexpr int kNoAllocMaxCtas = 300;                  // the tracker's largest ICP grid
constexpr long long kNoAllocMaxPixels = 4096LL * 4096LL; // largest depth image accepted

struct NoAllocScratch {
    TrackState state;
    float2 partials[kNoAllocMaxCtas * 32];
};

// 256-byte aligned scratch of sizeof(NoAllocScratch) bytes (about 77 KiB) per device. All
// calls share it and it keeps the last call's contents: each call clears what must start at
// zero (flags, ticket, reduction) in track_init_kernel, and calls that overlap on the GPU
// (two streams, or two host threads) race on it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

// depth_to_point_cloud for pixel i of the full-resolution image

// icp_iter_kernel with its inputs formed from the depth image and its scratch in the static
// array (same per-pixel terms, reduction order and FP64 tail).
__global__ void __launch_bounds__(kTrackThreads, 3) icp_iter_noalloc_kernel(Pinhole s, IterParams ip, const float* __restrict__ depth,
                                                                          int neg_y, NoAllocScratch* scratch)
{
    constexpr int kWarps = kTrackThreads / 32;
    TrackState* st = &scratch->state;
    float2* __restrict__ partials = scratch->partials;
    __shared__ float sh_terms[kWarps][32][33];
    __shared__ float2 sh_warp[kWarps][32];
    __shared__ int sh_last;
    __shared__ Tf T, Tri; // the poses live in shared memory: fewer live registers per thread
    if (st->flags[kFlagDone0 + ip.level])
        return;
    if (threadIdx.x < 12) {
        const int i = threadIdx.x, r = i >> 2, c = i & 3;
        if (c < 3) {
            T.R[3 * r + c] = st->pose_f[i];
            Tri.R[3 * r + c] = st->ref_inv[i];
        }
        else {
            T.t[r] = st->pose_f[i];
            Tri.t[r] = st->ref_inv[i];
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    CSum acc[4] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
    const int npix = ip.w * ip.h;
    const int stride = gridDim.x * kTrackThreads;
    int i = blockIdx.x * kTrackThreads + threadIdx.x;
    bool in_range = i < npix;
    // (x, y) of pixel i, advanced with i by the grid stride
    const int sdy = stride / ip.w, sdx = stride - sdy * ip.w;
    int x = i % ip.w, y = i / ip.w;
    F3 n_cur = in_range ? depth_normal(depth, s, ip.w, ip.h, x, y, neg_y) : f3(0.0f, 0.0f, 0.0f);
    F3 p_cur = in_range ? depth_point(depth, s, ip.w, x, y) : f3(0.0f, 0.0f, 0.0f);
    float sum[32];
#pragma unroll
    for (int k = 0; k < 32; ++k)
        sum[k] = 0.0f;
    int rounds = 0;
    for (int base = blockIdx.x * kTrackThreads; base < npix; base += stride) {
        const int i_next = i + stride;
        const bool next_in = i_next < npix;
        int x_next = x + sdx, y_next = y + sdy;
        if (x_next >= ip.w) {
            x_next -= ip.w;
            ++y_next;
        }
        const F3 n_next = next_in ? depth_normal(depth, s, ip.w, ip.h, x_next, y_next, neg_y) : f3(0.0f, 0.0f, 0.0f);
        const F3 p_next = next_in ? depth_point(depth, s, ip.w, x_next, y_next) : f3(0.0f, 0.0f, 0.0f);
        icp_pixel_add(s, ip, T, Tri, in_range, n_cur, p_cur, sum);
        if (++rounds == kIcpFlushRounds || base + stride >= npix) { // uniform across the CTA
            icp_flush_terms(sum, sh_terms[warp], acc);
            rounds = 0;
        }
        i = i_next;
        x = x_next;
        y = y_next;
        in_range = next_in;
        n_cur = n_next;
        p_cur = p_next;
    }
    acc[0].merge(acc[1].hi, acc[1].lo);
    acc[2].merge(acc[3].hi, acc[3].lo);
    acc[0].merge(acc[2].hi, acc[2].lo);
    sh_warp[warp][lane] = make_float2(acc[0].hi, acc[0].lo);
    __syncthreads();
    if (threadIdx.x < 32) {
        CSum t{0.0f, 0.0f};
        for (int wi = 0; wi < kWarps; ++wi)
            t.merge(sh_warp[wi][threadIdx.x].x, sh_warp[wi][threadIdx.x].y);
        partials[blockIdx.x * 32 + threadIdx.x] = make_float2(t.hi, t.lo);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0)
        sh_last = (atomicAdd(&st->ticket, 1u) == gridDim.x - 1) ? 1 : 0;
    __syncthreads();
    if (!sh_last)
        return;
    __threadfence();

    // ---- last CTA
    __shared__ double sh_pose[12];
    __shared__ double sh_val[32];
    __shared__ double sh_new[12];
    __shared__ float sh_newf[12];
    __shared__ int sh_conv;
    if (threadIdx.x < 12)
        sh_pose[threadIdx.x] = __ldcg(&st->pose[threadIdx.x]); // overlaps the merge below
    {
        // warp w merges rows w, w + 8, ...; loads are issued 16 at a time so that the L2
        // latency is paid once per batch, not once per row
        CSum t{0.0f, 0.0f};
        const int nb = (int) gridDim.x;
        for (int b0 = warp; b0 < nb; b0 += 16 * kWarps) {
            float2 pr[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                const int b = b0 + u * kWarps;
                pr[u] = b < nb ? __ldcg(&partials[b * 32 + lane]) : make_float2(0.0f, 0.0f);
            }
#pragma unroll
            for (int u = 0; u < 16; ++u)
                t.merge(pr[u].x, pr[u].y);
        }
        sh_warp[warp][lane] = make_float2(t.hi, t.lo);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        CSum t{0.0f, 0.0f};
        for (int c = 0; c < kWarps; ++c)
            t.merge(sh_warp[c][threadIdx.x].x, sh_warp[c][threadIdx.x].y);
        const double v = (double) t.hi + (double) t.lo;
        sh_val[threadIdx.x] = v;
        st->last_red[threadIdx.x] = (float) v;
    }
    __syncthreads();
    icp_tail(sh_val, sh_pose, sh_new, sh_newf, &sh_conv, ip.icp_threshold);
    if (threadIdx.x < 12) {
        st->pose[threadIdx.x] = sh_new[threadIdx.x];
        st->pose_f[threadIdx.x] = sh_newf[threadIdx.x];
    }
    if (threadIdx.x == 0) {
        st->ticket = 0;
        st->flags[kFlagIters0 + ip.level] += 1;
        if (sh_conv)
            st->flags[kFlagDone0 + ip.level] = 1;
    }
}


} // namespace se_gpu

// Device address of the static scratch, looked up once per device (cudaGetSymbolAddress with
// that device current) by the first call made on the device.
static void* g_noalloc_addr[64];
static std::mutex g_noalloc_mu;

static se_gpu_status noalloc_scratch(NoAllocScratch** out)
{
    int dev = 0;
    SE_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_last_error("se_gpu_track_noalloc: device ordinal %d out of range", dev);
        return SE_GPU_ERR_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr)
            return cuda_status(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress(scratch)");
        g_noalloc_addr[dev] = p;
    }
    *out = (NoAllocScratch*) g_noalloc_addr[dev];
    return SE_GPU_OK;
}

extern "C" se_gpu_status se_gpu_track_noalloc(const se_gpu_pinhole* sensor, const se_gpu_tracker_config* config,
                                              const float* depth_dev, const float* ref_pts, const float* ref_nrm,
                                              float T_WS[16], int* accepted, float reduction[32],
                                              void* stream_p)
{
    if (!sensor || !config || !depth_dev || !ref_pts || !ref_nrm || !T_WS || sensor->width <= 0
        || sensor->height <= 0) {
        set_last_error("se_gpu_track_noalloc: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (config->num_levels != 1) {
        set_last_error("se_gpu_track_noalloc: tracks one full-resolution level only (num_levels = %d; a pyramid "
                       "would need scratch images)", config->num_levels);
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    const long long npix = (long long) sensor->width * sensor->height;
    if (npix > kNoAllocMaxPixels) {
        set_last_error("se_gpu_track_noalloc: a %dx%d image exceeds the allocation-free limit of %lld pixels",
                       sensor->width, sensor->height, kNoAllocMaxPixels);
        return SE_GPU_ERR_BAD_ARG;
    }
    if (config->iterations[0] < 0 || config->iterations[0] > 1000) {
        set_last_error("se_gpu_track_noalloc: iterations[0] = %d out of range", config->iterations[0]);
        return SE_GPU_ERR_BAD_ARG;
    }
    NoAllocScratch* scratch = nullptr;
    se_gpu_status st = noalloc_scratch(&scratch);
    if (st != SE_GPU_OK)
        return st;
    cudaStream_t stream = (cudaStream_t) stream_p;
    const Pinhole s = make_pinhole(*sensor);

    TrackInit init;
    std::memset(&init, 0, sizeof(init));
    const Tf T = tf_from16(T_WS);
    const Tf Ti = inverse_iso(T);
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) {
            init.T_WS[4 * i + j] = T.R[3 * i + j];
            init.ref_inv[4 * i + j] = Ti.R[3 * i + j];
        }
        init.T_WS[4 * i + 3] = T.t[i];
        init.ref_inv[4 * i + 3] = Ti.t[i];
    }
    track_init_kernel<<<1, 1, 0, stream>>>(&scratch->state, init, nullptr);
    IterParams ip;
    ip.ref_pts = ref_pts;
    ip.ref_nrm = ref_nrm;
    ip.pts = nullptr;
    ip.nrm = nullptr;
    ip.w = sensor->width;
    ip.h = sensor->height;
    ip.W = sensor->width;
    ip.level = 0;
    ip.dist_threshold = config->dist_threshold;
    ip.normal_threshold = config->normal_threshold;
    ip.icp_threshold = config->icp_threshold;
    ip.ncta = 0; // the allocation-free kernel partitions by its own grid
    ip.nthr = 0;
    const long long tiles = (npix + kTrackThreads - 1) / kTrackThreads;
    int ctas = (int) (tiles < kNoAllocMaxCtas ? tiles : kNoAllocMaxCtas);
    if (ctas > 2 * device_sm_count())
        ctas = 2 * device_sm_count();
    for (int it = 0; it < config->iterations[0]; ++it)
        icp_iter_noalloc_kernel<<<ctas, kTrackThreads, 0, stream>>>(s, ip, depth_dev, s.left_hand, scratch);
    icp_check_kernel<<<1, 1, 0, stream>>>(&scratch->state, sensor->width, sensor->height, config->track_threshold,
                                          nullptr);
    SE_CUDA_TRY(cudaGetLastError());
    float head[12 + kNumFlags];
    float red[32];
    SE_CUDA_TRY(cudaMemcpyAsync(head, &scratch->state, kTrackReadback, cudaMemcpyDeviceToHost, stream));
    SE_CUDA_TRY(cudaMemcpyAsync(red, scratch->state.last_red, sizeof(red), cudaMemcpyDeviceToHost, stream));
    SE_CUDA_TRY(cudaStreamSynchronize(stream));
    for (int i = 0; i < 12; ++i)
        T_WS[i] = head[i];
    T_WS[12] = T_WS[13] = T_WS[14] = 0.0f;
    T_WS[15] = 1.0f;
    if (accepted) {
        int flags[kNumFlags];
        std::memcpy(flags, &head[12], sizeof(flags));
        *accepted = flags[kFlagAccepted];
    }
    if (reduction)
        std::memcpy(reduction, red, sizeof(red));
    return SE_GPU_OK;
}
