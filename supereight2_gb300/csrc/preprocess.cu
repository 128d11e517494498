// preprocess.cu — the project-defined bilateral pre-filter of the tracking input. The
// reference has no bilateral filter (it feeds the downsampled depth straight to the tracker,
// app/src/main.cpp:119-128); the benchmark configuration of the tracked TSDF path asks for a
// bilateral-filtered tracking input, defined here as: invalid (<= 0 or NaN) centres stay 0;
// the valid taps of the (2r+1)^2 window inside the image are weighted by a spatial Gaussian
// (sigma_space pixels, weights computed in double on the host and rounded to float) times
// exp(-(d - c)^2 / (2 sigma_range^2)); the weighted mean is summed dy outer, dx inner. The
// exponential is evaluated in float operations only (Cody & Waite reduction and a degree-7
// Taylor polynomial), the same operations as the CPU oracle, so both give identical images.
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
// below 3e-8), then 2^n exactly.
__device__ __forceinline__ float exp_cw(float x)
{
    if (x < -87.0f)
        return 0.0f;
    const float n = rintf(x * 1.44269504f);
    const float r = (x - n * 0.693145751953125f) - n * 1.42860677e-06f;
    const float p = 1.0f
        + r * (1.0f + r * (0.5f + r * (0.166666672f + r * (0.0416666679f + r * (0.00833333377f
                                                     + r * (0.00138888892f + r * 0.000198412701f))))));
    return ldexpf(p, (int) n);
}

constexpr int kTileX = 32, kTileY = 8;

__global__ void __launch_bounds__(kTileX * kTileY) bilateral_kernel(const float* __restrict__ in,
                                                                    float* __restrict__ out,
                                                                    const __grid_constant__ BilateralParams P)
{
    constexpr int kMaxW = kTileX + 2 * kBilateralMaxRadius, kMaxH = kTileY + 2 * kBilateralMaxRadius;
    __shared__ float tile[kMaxH][kMaxW];
    const int r = P.radius;
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
    const int n = 2 * r + 1;
    float num = 0.0f, den = 0.0f;
    for (int dy = -r; dy <= r; ++dy) {
        for (int dx = -r; dx <= r; ++dx) {
            const float d = tile[threadIdx.y + r + dy][threadIdx.x + r + dx];
            if (!(d > 0.0f))
                continue;
            const float diff = d - c;
            const float wgt = P.ws[(dy + r) * n + (dx + r)] * exp_cw(-(diff * diff) * P.k);
            num = num + wgt * d;
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
    bilateral_kernel<<<grid, dim3(kTileX, kTileY), 0, stream>>>(in, out, P);
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
