// preprocess.cu — the project-defined bilateral pre-filter of the tracking input. The
// reference has no bilateral filter (it feeds the downsampled depth straight to the tracker,
// app/src/main.cpp:119-128); the benchmark configuration of the tracked TSDF path asks for a
// bilateral-filtered tracking input, defined here as: invalid (<= 0 or NaN) centres stay 0;
// the valid taps of the (2r+1)^2 window inside the image are weighted by a spatial Gaussian
// (sigma_space pixels, weights computed in double on the host and rounded to float) times
// exp(-(d - c)^2 / (2 sigma_range^2)); the weighted mean is summed dy outer, dx inner, the
// numerator by fused multiply-adds. The exponential is evaluated in float operations only (Cody &
// Waite reduction and a degree-7 Taylor polynomial by Horner's rule in fused multiply-adds), the
// same operations as the CPU oracle, so both give identical images.
#include <cmath>

#include "pipeline.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

constexpr int kBilateralMaxRadius = 7;

struct BilateralParams {
    int w, h, radius;
    float k; // 1 / (2 sigma_range^2)
    float ws[(2 * kBilateralMaxRadius + 1) * (2 * kBilateralMaxRadius + 1)];
};

// e^x for x <= 0: x = n ln2 + r with ln2 split into a head exact in 12 bits and a tail
// (Cody & Waite, 1980), e^r by its degree-7 Taylor polynomial (|r| <= ln2/2, relative error
// below 3e-8) by Horner's rule in fused multiply-adds, then 2^n exactly.
__device__ __forceinline__ float exp_cw(float x)
{
    if (x < -87.0f)
        return 0.0f;
    const float n = rintf(x * 1.44269504f);
    const float r = fmaf(-n, 1.42860677e-06f, fmaf(-n, 0.693145751953125f, x));
    float p = 0.000198412701f;
    p = fmaf(p, r, 0.00138888892f);
    p = fmaf(p, r, 0.00833333377f);
    p = fmaf(p, r, 0.0416666679f);
    p = fmaf(p, r, 0.166666672f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    // p * 2^n: n >= -126 here, so 2^n is a normal float and the product is the correctly
    // rounded value ldexp gives
    return p * __int_as_float(((int) n + 127) << 23);
}

constexpr int kTileX = 32, kTileY = 8;

template <int R>
__global__ void __launch_bounds__(kTileX * kTileY) bilateral_kernel(const float* __restrict__ in,
                                                                    float* __restrict__ out,
                                                                    const __grid_constant__ BilateralParams P)
{
    constexpr int kMaxW = kTileX + 2 * R, kMaxH = kTileY + 2 * R;
    __shared__ float tile[kMaxH][kMaxW];
    constexpr int r = R;
    const int tw = kTileX + 2 * r, th = kTileY + 2 * r;
    const int x0 = blockIdx.x * kTileX - r, y0 = blockIdx.y * kTileY - r;
    for (int i = threadIdx.y * kTileX + threadIdx.x; i < tw * th; i += kTileX * kTileY) {
        const int tx = i % tw, ty = i / tw;
        const int gx = x0 + tx, gy = y0 + ty;
        // taps outside the image are skipped; 0 marks them invalid like a missing depth
        tile[ty][tx] = (gx >= 0 && gx < P.w && gy >= 0 && gy < P.h) ? in[gx + gy * P.w] : 0.0f;
    }
    __syncthreads();
    const int x = blockIdx.x * kTileX + threadIdx.x, y = blockIdx.y * kTileY + threadIdx.y;
    if (x >= P.w || y >= P.h)
        return;
    const float c = tile[threadIdx.y + r][threadIdx.x + r];
    if (!(c > 0.0f)) {
        out[x + y * P.w] = 0.0f;
        return;
    }
    constexpr int n = 2 * r + 1;
    float num = 0.0f, den = 0.0f;
#pragma unroll
    for (int dy = -r; dy <= r; ++dy) {
#pragma unroll
        for (int dx = -r; dx <= r; ++dx) {
            const float d = tile[threadIdx.y + r + dy][threadIdx.x + r + dx];
            if (!(d > 0.0f))
                continue;
            const float diff = d - c;
            const float wgt = P.ws[(dy + r) * n + (dx + r)] * exp_cw(-(diff * diff) * P.k);
            num = fmaf(wgt, d, num);
            den = den + wgt;
        }
    }
    out[x + y * P.w] = num / den;
}

se_gpu_status check_bilateral(const se_gpu_bilateral_config* c)
{
    if (!c || c->radius < 0 || c->radius > kBilateralMaxRadius || !(c->sigma_space_px > 0.0f)
        || !(c->sigma_range_m > 0.0f)) {
        set_last_error("bilateral: radius in [0, %d], sigma_space_px > 0, sigma_range_m > 0", kBilateralMaxRadius);
        return SE_GPU_ERR_BAD_ARG;
    }
    return SE_GPU_OK;
}

se_gpu_status enqueue_bilateral(const float* in, float* out, int w, int h, const se_gpu_bilateral_config& c,
                                cudaStream_t stream)
{
    BilateralParams P;
    P.w = w;
    P.h = h;
    P.radius = c.radius;
    P.k = 1.0f / (2.0f * c.sigma_range_m * c.sigma_range_m);
    const int n = 2 * c.radius + 1;
    const double s = (double) c.sigma_space_px;
    for (int dy = -c.radius; dy <= c.radius; ++dy)
        for (int dx = -c.radius; dx <= c.radius; ++dx)
            P.ws[(dy + c.radius) * n + (dx + c.radius)] = (float) std::exp(-(double) (dx * dx + dy * dy) / (2.0 * s * s));
    const dim3 grid((w + kTileX - 1) / kTileX, (h + kTileY - 1) / kTileY);
    const dim3 block(kTileX, kTileY);
    switch (c.radius) {
    case 0: bilateral_kernel<0><<<grid, block, 0, stream>>>(in, out, P); break;
    case 1: bilateral_kernel<1><<<grid, block, 0, stream>>>(in, out, P); break;
    case 2: bilateral_kernel<2><<<grid, block, 0, stream>>>(in, out, P); break;
    case 3: bilateral_kernel<3><<<grid, block, 0, stream>>>(in, out, P); break;
    case 4: bilateral_kernel<4><<<grid, block, 0, stream>>>(in, out, P); break;
    case 5: bilateral_kernel<5><<<grid, block, 0, stream>>>(in, out, P); break;
    case 6: bilateral_kernel<6><<<grid, block, 0, stream>>>(in, out, P); break;
    default: bilateral_kernel<7><<<grid, block, 0, stream>>>(in, out, P); break;
    }
    SE_CUDA_TRY(cudaGetLastError());
    return SE_GPU_OK;
}

} // namespace se_gpu

using namespace se_gpu;

extern "C" se_gpu_status se_gpu_bilateral_filter(const float* in_dev, float* out_dev, int width, int height,
                                                 const se_gpu_bilateral_config* config, void* stream)
{
    if (!in_dev || !out_dev || width <= 0 || height <= 0 || in_dev == out_dev) {
        set_last_error("se_gpu_bilateral_filter: invalid argument (the filter is not in place)");
        return SE_GPU_ERR_BAD_ARG;
    }
    const se_gpu_status st = check_bilateral(config);
    if (st != SE_GPU_OK)
        return st;
    return enqueue_bilateral(in_dev, out_dev, width, height, *config, (cudaStream_t) stream);
}

// ------------------------------------------------------------------ depth downsampling --

namespace se_gpu {

constexpr int kDownsampleMaxRatio = 8;

// preprocessor::downsample_depth (src/map/preprocessor.cpp:19-84), one thread per output pixel:
// the region's depths >= 1e-5 in scan order, then the element of stable rank count / 2 (rank =
// the smaller depths plus the equal ones earlier in the scan), i.e. the stable sort's middle
// element; 0 and the region's first pixel when no depth is valid.
__global__ void downsample_depth_kernel(const float* __restrict__ in, int w_in, float* __restrict__ out, int w_out,
                                        int h_out, int ratio, long long* __restrict__ map)
{
    const int x_out = blockIdx.x * blockDim.x + threadIdx.x, y_out = blockIdx.y * blockDim.y + threadIdx.y;
    if (x_out >= w_out || y_out >= h_out)
        return;
    const int xb = x_out * ratio, yb = y_out * ratio;
    float v[kDownsampleMaxRatio * kDownsampleMaxRatio];
    int idx[kDownsampleMaxRatio * kDownsampleMaxRatio];
    int n = 0;
    for (int yr = 0; yr < ratio; ++yr)
        for (int xr = 0; xr < ratio; ++xr) {
            const float d = in[(xb + xr) + (size_t) (yb + yr) * w_in];
            if (d >= 1e-5f) {
                v[n] = d;
                idx[n] = xr + yr * ratio;
                ++n;
            }
        }
    const size_t o = (size_t) x_out + (size_t) y_out * w_out;
    if (n == 0) {
        out[o] = 0.0f;
        if (map)
            map[o] = (long long) xb + (long long) yb * w_in;
        return;
    }
    const int want = n / 2;
    int pick = 0;
    for (int i = 0; i < n; ++i) {
        int rank = 0;
        for (int j = 0; j < n; ++j)
            rank += (v[j] < v[i] || (v[j] == v[i] && j < i)) ? 1 : 0;
        if (rank == want)
            pick = i;
    }
    out[o] = v[pick];
    if (map)
        map[o] = (long long) (xb + idx[pick] % ratio) + (long long) (yb + idx[pick] / ratio) * w_in;
}

} // namespace se_gpu

extern "C" se_gpu_status se_gpu_downsample_depth(const float* in_dev, int w_in, int h_in, float* out_dev, int w_out,
                                                 int h_out, int64_t* map_dev, void* stream)
{
    if (!in_dev || !out_dev || w_out <= 0 || h_out <= 0 || w_in < w_out || h_in < h_out || w_in % w_out != 0
        || h_in % h_out != 0 || w_in / w_out != h_in / h_out || w_in / w_out > se_gpu::kDownsampleMaxRatio) {
        se_gpu::set_last_error("se_gpu_downsample_depth: the input must be 1..%d times the output in both axes",
                               se_gpu::kDownsampleMaxRatio);
        return SE_GPU_ERR_BAD_ARG;
    }
    const dim3 block(32, 8), grid((w_out + 31) / 32, (h_out + 7) / 8);
    se_gpu::downsample_depth_kernel<<<grid, block, 0, (cudaStream_t) stream>>>(
        in_dev, w_in, out_dev, w_out, h_out, w_in / w_out, reinterpret_cast<long long*>(map_dev));
    SE_CUDA_TRY(cudaGetLastError());
    return SE_GPU_OK;
}
