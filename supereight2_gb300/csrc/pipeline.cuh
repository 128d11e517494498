// pipeline.cuh — stream-ordered building blocks shared by the C entry points and the captured
// frame pipeline. A pose is given either on the host (row-major float[16]) or on the device
// (float[12], row-major 3x4); exactly one of the two pointers is non-null.
#pragma once

#include "se_gpu_internal.cuh"

struct se_gpu_tracker;

namespace se_gpu {

se_gpu_status enqueue_integrate(se_gpu_map* map, const float* depth_dev, const se_gpu_pinhole& sensor,
                                const float* T_WC_host16, const float* pose12_dev, int timestamp,
                                cudaStream_t stream);
se_gpu_status enqueue_raycast(const se_gpu_map* map, const se_gpu_pinhole& sensor, const float* T_WS_host16,
                              const float* pose12_dev, float* pts_dev, float* nrm_dev, int8_t* scale_dev,
                              cudaStream_t stream);
// Multi-res TSDF update over the frame's block list (after carve and frustum).
void enqueue_update_multires(const MapDevice& m, const Pinhole& s, const float* depth_dev,
                             const IntegrateParams* params, cudaStream_t stream);
// Occupancy maps (occupancy.cu).
se_gpu_status occ_map_create(const se_gpu_map_config* cfg, const se_gpu_occupancy_config* occ, int size,
                             se_gpu_occ_map** out);
void occ_map_destroy(se_gpu_occ_map* om);
se_gpu_status occ_check(se_gpu_occ_map* om);
se_gpu_status occ_aabb(const se_gpu_occ_map* om, int32_t mn[3], int32_t mx[3], int* empty);
se_gpu_status occ_raycast_volume(const se_gpu_occ_map* om, const se_gpu_pinhole& sensor, const float* T_WS16,
                                 float* pts, float* nrm, int8_t* scale, cudaStream_t stream);
se_gpu_status occ_integrate(se_gpu_occ_map* om, const float* depth_dev, const se_gpu_pinhole& sensor,
                            const float* T_WC16, int timestamp, cudaStream_t stream);
se_gpu_status occ_integrate_range(se_gpu_occ_map* om, const float* range_dev, const se_gpu_lidar& sensor,
                                  const float* T_WS16, int timestamp, cudaStream_t stream);
void occ_scratch_free(se_gpu_occ_map* om);
// The bilateral pre-filter of the tracking input (preprocess.cu).
se_gpu_status check_bilateral(const se_gpu_bilateral_config* c);
se_gpu_status enqueue_bilateral(const float* in, float* out, int w, int h, const se_gpu_bilateral_config& c,
                                cudaStream_t stream);
// With pose12_dev_io the tracker starts from, and writes its result to, that device pose.
se_gpu_status enqueue_track(se_gpu_tracker* t, const float* depth_dev, const float* ref_pts, const float* ref_nrm,
                            const float* T_WS_host16, float* pose12_dev_io, cudaStream_t stream);

} // namespace se_gpu
