// common.cu — error reporting, sensor set-up shared by the host entry points.
#include <cmath>
#include <cstdarg>
#include <cstdio>

#include "se_gpu_internal.cuh"

namespace se_gpu {

static thread_local char g_last_error[512] = "";

void set_last_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

se_gpu_status cuda_status(cudaError_t e, const char* what)
{
    set_last_error("%s: %s", what, cudaGetErrorString(e));
    return SE_GPU_ERR_CUDA;
}

/* se::math::plane_normal (include/se/common/impl/math_util_impl.hpp:88-101) */
static F3 plane_normal(F3 p1, F3 p2, F3 p3) { return normalized(cross(sub(p2, p1), sub(p3, p2))); }

Pinhole make_pinhole(int w, int h, float fx, float fy, float cx, float cy, float near_p, float far_p)
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
    // computeFrustumVertices / computeFrustumNormals (src/sensor/pinhole_camera.cpp:246-310)
    const F3 tl = back_project(s, 0.0f, 0.0f);
    const F3 tr = back_project(s, (float) w, 0.0f);
    const F3 br = back_project(s, (float) w, (float) h);
    const F3 bl = back_project(s, 0.0f, (float) h);
    const F3 tl_n = mul(near_p, tl), tl_f = mul(far_p, tl), tr_n = mul(near_p, tr), tr_f = mul(far_p, tr);
    const F3 br_n = mul(near_p, br), br_f = mul(far_p, br), bl_n = mul(near_p, bl), bl_f = mul(far_p, bl);
    const F3 ns[4] = {plane_normal(tl_f, tl_n, bl_n), plane_normal(tr_n, tr_f, br_f),
                      plane_normal(bl_f, bl_n, br_n), plane_normal(tr_f, tr_n, tl_n)};
    float sign = fx * fy;
    sign = sign / fabsf(sign);
    for (int i = 0; i < 4; ++i) {
        s.planes[i][0] = ns[i].x * sign;
        s.planes[i][1] = ns[i].y * sign;
        s.planes[i][2] = ns[i].z * sign;
        s.planes[i][3] = 0.0f;
    }
    s.planes[4][0] = 0.0f;
    s.planes[4][1] = 0.0f;
    s.planes[4][2] = 1.0f;
    s.planes[4][3] = -near_p;
    s.planes[5][0] = 0.0f;
    s.planes[5][1] = 0.0f;
    s.planes[5][2] = -1.0f;
    s.planes[5][3] = far_p;
    return s;
}

Pinhole make_pinhole(const se_gpu_pinhole& p)
{
    return make_pinhole(p.width, p.height, p.fx, p.fy, p.cx, p.cy, p.near_plane, p.far_plane);
}

Pinhole downsampled(const Pinhole& s, float dsf)
{
    return make_pinhole((int) ((float) s.w / dsf), (int) ((float) s.h / dsf), s.fx / dsf, s.fy / dsf,
                        (s.cx + 0.5f) / dsf - 0.5f, (s.cy + 0.5f) / dsf - 0.5f, s.near_plane, s.far_plane);
}

static int num_sms_cached()
{
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0)
            n = 152;
    }
    return n;
}

int device_sm_count() { return num_sms_cached(); }

} // namespace se_gpu

using namespace se_gpu;

extern "C" {

const char* se_gpu_last_error(void) { return se_gpu::g_last_error; }

const char* se_gpu_status_string(se_gpu_status s)
{
    switch (s) {
    case SE_GPU_OK: return "ok";
    case SE_GPU_ERR_BAD_ARG: return "bad argument";
    case SE_GPU_ERR_CUDA: return "CUDA error";
    case SE_GPU_ERR_POOL_FULL: return "block pool full";
    case SE_GPU_ERR_HASH_PROBE_LIMIT: return "block hash probe limit reached";
    case SE_GPU_ERR_NOT_SUPPORTED: return "not supported";
    case SE_GPU_ERR_NO_DEVICE: return "no compute capability 10.3 device";
    }
    return "unknown status";
}

int se_gpu_abi_version(void) { return 1; }

} // extern "C"
