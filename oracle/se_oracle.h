/*
 * se_oracle.h — C interface of the CPU oracle for the supereight2 dense-mapping hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the GPU product is compared
 * against, and the timed CPU baseline. Only tests, the smoke check and the benchmark's CPU
 * baseline leg may load it. The product library (libse_gpu) never links or calls it.
 *
 * It is a CPU restatement, in C++17 + OpenMP, of these reference paths (paths relative to the
 * supereight2 source tree):
 *   - Morton key operations        include/se/map/utils/impl/key_util_impl.hpp:44-436
 *   - Map transforms / octree size include/se/map/impl/map_impl.hpp:37-55,494-590;
 *                                  include/se/map/octree/impl/octree_impl.hpp:14-19
 *   - RaycastCarver allocation     include/se/integrator/allocator/impl/raycast_carver_impl.hpp:17-128
 *   - octree allocation            include/se/map/octree/impl/allocator_impl.hpp:68-147,
 *                                  include/se/map/octree/impl/octree_impl.hpp:171-199
 *   - FrustumIterator              include/se/map/octree/iterator.hpp:197-235,
 *                                  include/se/map/octree/impl/iterator_impl.hpp:88-160
 *   - single-res TSDF update       include/se/integrator/updater/impl/singleres_tsdf_updater_impl.hpp:14-132,
 *                                  include/se/map/impl/data_field_impl.hpp:39-54
 *   - multi-res TSDF update        include/se/integrator/updater/impl/multires_tsdf_updater_impl.hpp:14-250,
 *                                  src/sensor/pinhole_camera.cpp:115-152,
 *                                  include/se/map/octree/impl/propagator_impl.hpp:17-117,
 *                                  include/se/map/impl/data_impl.hpp:13-50,
 *                                  include/se/map/octant/impl/block_impl.hpp:80-202
 *   - raycast_volume (TSDF)        include/se/map/impl/raycaster_impl.hpp:456-627
 *   - VoxelBlockRayIterator        include/se/map/octree/impl/voxel_block_ray_iterator_impl.hpp:19-249
 *   - visitor interp / gradient    include/se/map/octree/impl/visitor_impl.hpp:67-302,704-717,976-1251
 *                                  (multi-res: :398-697,740-790,906-972,1257-1497)
 *   - Tracker / ICP                include/se/tracker/impl/tracker_impl.hpp:30-116,
 *                                  include/se/tracker/impl/icp_impl.hpp:16-102, src/tracker/icp.cpp:15-246
 *   - preprocessing                src/map/preprocessor.cpp:109-195,
 *                                  include/se/map/impl/preprocessor_impl.hpp:18-40
 *   - se(3) exponential            include/se/common/impl/math_util_impl.hpp:104-174
 *   - PinholeCamera                src/sensor/pinhole_camera.cpp:29-39,95-111,189-310,
 *                                  include/se/sensor/impl/pinhole_camera_impl.hpp:15-32
 *
 * All matrices cross this interface as row-major float[16] (4x4 homogeneous).
 * Images are row-major, pixel (x, y) at index x + y * width; 3-vectors are packed xyz floats.
 */
#ifndef SE_ORACLE_H
#define SE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct so_map so_map;

typedef struct {
    int width;
    int height;
    float fx, fy, cx, cy;
    float near_plane;
    float far_plane;
} so_pinhole;

typedef struct {
    int num_levels;     /* pyramid levels, at most 3 */
    int iterations[3];  /* per level, finest first: reference default {10, 5, 4} */
    float dist_threshold;
    float normal_threshold;
    float track_threshold;
    float icp_threshold;
} so_tracker_config;

typedef struct {
    long long n_valid_pixels;   /* pixels that passed the near/far test of the carver */
    long long n_new_blocks;     /* blocks allocated by this call */
    long long n_frustum_blocks; /* previously allocated blocks returned by the frustum fetch */
    long long n_updated_voxels; /* voxels whose field update returned true */
} so_integrate_stats;

typedef struct {
    int converged_iterations[3]; /* iterations actually run per level */
    int accepted;                /* checkPoseKernel result */
    float reduction[32];         /* final 32-float reduction (row 0 of the 8x32 buffer) */
} so_track_stats;

void so_set_num_threads(int n);
int so_get_num_threads(void);

/* Map<Data<TSDF>, Res::Single, 8>. T_MW may be NULL (reference default: translation dim/2). */
so_map* so_map_create(const float dim[3], float res, float truncation_boundary_factor,
                      float max_weight, const float* T_MW);
/* Map<Data<TSDF>, Res::Multi, 8> (multires_tsdf_updater_impl.hpp:14-250). */
so_map* so_map_create_multires(const float dim[3], float res, float truncation_boundary_factor,
                               float max_weight, const float* T_MW);
int so_map_is_multires(const so_map* map);
void so_map_destroy(so_map* map);
int so_map_size(const so_map* map);
float so_map_dim(const so_map* map);

/* se::MapIntegrator::integrateDepth for a TSDF single-res map and a pinhole camera. */
void so_integrate_depth(so_map* map, const float* depth, const so_pinhole* sensor,
                        const float T_WC[16], int timestamp, so_integrate_stats* stats);

/* se::raycaster::raycast_volume. pts/nrm are width*height*3 floats, scale width*height. */
/* Distinct voxels the single-res raycast reads at T_WS (a measurement aid). */
long long so_raycast_touched(const so_map* map, const so_pinhole* sensor, const float T_WS[16]);
void so_raycast_volume(const so_map* map, const so_pinhole* sensor, const float T_WS[16],
                       float* pts_W, float* nrm_W, int8_t* scale);

/* se::Tracker::track(depth, T_WS, pts, nrm). T_WS is updated in place; returns acceptance. */
int so_track(const so_pinhole* sensor, const so_tracker_config* config, const float* depth,
             float T_WS[16], const float* ref_pts_W, const float* ref_nrm_W,
             so_track_stats* stats);

/* Map inspection. */
long long so_map_num_blocks(const so_map* map);
/* keys: uint64 block keys (Morton code << 5 | scale 3); coords: 3 ints per block;
 * tsdf / weight: 512 floats per block in x + 8y + 64z order. Any pointer may be NULL. */
void so_map_blocks(const so_map* map, uint64_t* keys, int32_t* coords, float* tsdf,
                   float* weight, int32_t* timestamps);
/* Multi-res blocks: 585 values per block (scale 0: 512 in x + 8y + 64z order, scale 1: 64,
 * scale 2: 8, scale 3: 1) of data and past data; scales: (current_scale, min_scale) per block.
 * so_map_blocks reports a multi-res map's scale-0 level. */
void so_map_mr_blocks(const so_map* map, uint64_t* keys, int32_t* coords, float* tsdf, float* weight,
                      float* past_tsdf, float* past_weight, int32_t* scales);
/* Allocated-block AABB in voxel coordinates, inclusive; returns 0 when empty. */
int so_map_aabb(const so_map* map, int32_t mn[3], int32_t mx[3]);
/* Allocate the block containing voxel_coord (through the normal allocator) and overwrite its
 * 512 voxels. */
/* Test set-up of a multi-res map block: data pyramid (585 entries, past data set equal), scales. */
void so_map_set_mr_block(so_map* map, const int32_t voxel_coord[3], const float* tsdf585,
                         const float* weight585, int current_scale, int min_scale);
void so_map_set_block(so_map* map, const int32_t voxel_coord[3], const float* tsdf512,
                      const float* weight512);
int so_map_get_data(const so_map* map, const float point_W[3], float* tsdf, float* weight);
int so_map_get_field_interp(const so_map* map, const float point_W[3], float* value);
int so_map_get_field_grad(const so_map* map, const float point_W[3], float grad[3]);
/* Distance (metres) to the first allocated block along a ray, as VoxelBlockRayIterator::tcmin()
 * reports it after the first next(); returns 0 if next() returned no block. */
int so_first_block_tmin(const so_map* map, const float origin_W[3], const float dir_W[3],
                        float t_near, float t_far, float* tcmin);

/* Differentiable depth render of a single-res map in FP64 (no reference counterpart; the
 * checker of se_gpu_render_depth / se_gpu_raycast_adjoint): depth = z of the root of the
 * trilinear TSDF on each pixel's ray after the raycast march (0 where there is none).
 * The adjoint accumulates sum_i grad_depth[i] * d depth_i / d xi for the left perturbation
 * T = exp(xi) T_WS, xi = [rho; omega]; voxel_grad (num_blocks * 512, in so_map_blocks order)
 * and jac (width * height * 6: d depth_i / d xi) may be NULL. */
void so_render_depth_f64(const so_map* map, const so_pinhole* sensor, const double T_WS[16], double* depth);
void so_raycast_adjoint_f64(const so_map* map, const so_pinhole* sensor, const double T_WS[16],
                            const double* grad_depth, double twist_grad[6], double* voxel_grad, double* jac);
/* Overwrite one voxel of an allocated single-res block (no-op elsewhere). */
void so_map_set_voxel(so_map* map, const int32_t voxel_coord[3], float tsdf, float weight);

/* --------------------------------------------------------- multi-res occupancy maps -- */
/* Map<Data<Occupancy>, Res::Multi, 8> with the reference's default field configuration
 * (data_field.hpp:52-71). T_MW may be NULL (translation dim/2). */
typedef struct so_occ_map so_occ_map;
typedef struct {
    long long n_blocks_listed; /* blocks the VolumeCarver returned for update */
    long long n_nodes_listed;  /* free-space nodes the VolumeCarver returned */
    long long n_blocks_freed;  /* blocks freed below those nodes */
    long long n_nodes_pruned;  /* nodes whose children were deleted by the propagation */
} so_occ_stats;
so_occ_map* so_occ_map_create(const float dim[3], float res, const float* T_MW);
/* The same with the field configuration of a YAML "data" node: cfg = {k_sigma,
 * sigma_min_factor, sigma_max_factor, k_tau, tau_min_factor, tau_max_factor, log_odd_min,
 * log_odd_max, fs_integr_scale}. */
so_occ_map* so_occ_map_create_cfg(const float dim[3], float res, const float* T_MW, const float cfg[9]);
void so_occ_map_destroy(so_occ_map* map);
/* Map::getData / Map::getFieldInterp for occupancy maps; data as (occupancy, weight,
 * observed); the interpolation returns 0 for nullopt. */
void so_occ_get_data(const so_occ_map* map, const float point_W[3], float out[3]);
int so_occ_get_field_interp(const so_occ_map* map, const float point_W[3], float* value, int* scale);
int so_occ_get_field_grad(const so_occ_map* map, const float point_W[3], float grad[3]);
int so_occ_map_size(const so_occ_map* map);
/* MapIntegrator<OccupancyMap<Res::Multi>>::integrateDepth for a pinhole camera. */
void so_occ_integrate_depth(so_occ_map* map, const float* depth, const so_pinhole* sensor,
                            const float T_WC[16], int timestamp, so_occ_stats* stats);
long long so_occ_num_blocks(const so_occ_map* map);
long long so_occ_num_nodes(const so_occ_map* map);
/* Test set-up: the block holding voxel c with the given scales and mean pyramid (585 x 3). */
void so_occ_set_block(so_occ_map* map, const int32_t c[3], int current_scale, int min_scale,
                      const float* mean585);
/* Dual marching cubes of an occupancy map: faces (9 floats each, voxel units) and face scales. */
long long so_occ_dual_marching_cubes(const so_occ_map* map, int min_desired_scale, float* faces,
                                     int8_t* scales, long long capacity);
/* Live blocks in allocation order; every pointer may be NULL. coords: 3 ints; scales:
 * (current, min, buffer); counts: (curr_integr, curr_observed, buffer_integr,
 * buffer_observed); mean / min / max: 585 entries of (occupancy, weight, observed). */
void so_occ_blocks(const so_occ_map* map, int32_t* coords, int32_t* scales, int64_t* counts,
                   float* mean, float* min_data, float* max_data);
/* Nodes reachable from the root (depth first): coords (x, y, z, size), min / max data as
 * (occupancy, weight, observed), leaf flag. Returns the count (pass NULLs to count). */
long long so_occ_nodes(const so_occ_map* map, int32_t* coords, float* min_data, float* max_data,
                       int32_t* leaf);
int so_occ_aabb(const so_occ_map* map, int32_t mn[3], int32_t mx[3]);
/* raycaster::raycast_volume for an occupancy map (raycaster_impl.hpp:32-452,537-627). */
void so_occ_raycast_volume(const so_occ_map* map, const so_pinhole* sensor, const float T_WS[16],
                           float* pts_W, float* nrm_W, int8_t* scale);
/* A spinning LiDAR (the reference's OusterLidar): equiangular columns over 360 degrees of azimuth
 * (clockwise from +x), rows linear in elevation from elevation_max_deg (row 0) down to
 * elevation_min_deg; the range image holds ranges in metres (<= 0: no return). */
typedef struct {
    int width, height;
    float elevation_min_deg, elevation_max_deg;
    float near_plane, far_plane;
} so_lidar;
/* MapIntegrator<OccupancyMap<Res::Multi>>::integrateDepth for an OusterLidar range image. */
/* LeicaLidar (include/se/sensor/leica_lidar.hpp): the ray-batch sensor of the ray integrator. */
typedef struct {
    int width, height;
    float near_plane, far_plane;
    float elevation_resolution_deg, azimuth_resolution_deg;
} so_leica;
/* MapIntegrator::integrateRayBatch (multi-res occupancy, LeicaLidar): rays (n x 3, sensor
 * frame) with their poses (n x 16 T_WS, row-major) in order; up to capacity updated octants
 * (x, y, z, size) written to octants; returns the number of updated octants. */
long long so_occ_integrate_ray_batch(so_occ_map* map, const so_leica* sensor, const float* poses,
                                     const float* rays, long long n, int timestamp, int32_t* octants,
                                     long long capacity);
int so_leica_integration_scale(const so_leica* sensor, const float c_S[3], float res, int last_scale,
                               int min_scale);
void so_occ_block_timestamps(const so_occ_map* map, int32_t* ts);
void so_occ_integrate_lidar(so_occ_map* map, const float* range, const so_lidar* sensor,
                            const float T_WS[16], int timestamp, so_occ_stats* stats);
int so_lidar_project(const so_lidar* sensor, const float p_S[3], float uv[2]);
float so_atan2(float y, float x);
float so_lidar_tan_half_min_angle(const so_lidar* sensor);
int so_occ_lidar_integration_scale(const so_lidar* sensor, const float c_S[3], float res, int last_scale,
                                   int min_scale);
int so_occ_pooling_image_lidar(const float* depth, int w, int h, float* out, float* max_value);
/* uncert::depth_sigma with the default linear model. */
void so_occ_depth_sigma(const float* depth, int n, float res, float* sigma);
/* DensePoolingImage<PinholeCamera>: (max_level + 1) * w * h pixels of (min, max, crossing,
 * known) into out (may be NULL); returns max_level. */
int so_occ_pooling_image(const float* depth, int w, int h, float* out, float* max_value);

/* Morton key operations (key_util_impl.hpp). */
uint64_t so_expand(uint64_t value);
uint64_t so_compact(uint64_t value);
uint64_t so_encode_code(int32_t x, int32_t y, int32_t z);
void so_decode_code(uint64_t code, int32_t coord[3]);
/* Returns 1 when no detail is lost at that scale (encode_key's bool). */
int so_encode_key(int32_t x, int32_t y, int32_t z, uint64_t scale, uint64_t* key);
void so_decode_key(uint64_t key, int32_t coord[3], uint64_t* scale);
uint64_t so_code_to_child_idx(uint64_t code, uint64_t child_scale);
uint64_t so_parent_key(uint64_t key);
int so_key_at_scale(uint64_t key, uint64_t scale, uint64_t* key_at_scale);
int so_code_at_scale(uint64_t key, uint64_t scale, uint64_t* code_at_scale);
uint64_t so_block_key(uint64_t key, uint64_t max_block_scale);
uint64_t so_block_code(uint64_t key, uint64_t max_block_scale);
int so_is_child(uint64_t parent_key, uint64_t child_key);
int so_is_siblings(uint64_t a, uint64_t b);
/* The unique_* helpers sort keys in place; they return the number of unique keys written. */
long long so_unique_keys(uint64_t* keys, long long n, uint64_t* out);
long long so_unique_codes(uint64_t* keys, long long n, uint64_t* out);
long long so_unique_allocation(uint64_t* keys, long long n, uint64_t max_block_scale,
                               uint64_t* out);
long long so_unique_at_scale(uint64_t* keys, long long n, uint64_t scale, uint64_t* out);

/* se(3) exponential of a twist [rho; omega] as a row-major 4x4 (math_util_impl.hpp:117-174). */
void so_se3_exp(const float twist[6], float T[16]);

/* The project-defined bilateral pre-filter of the tracking input (no reference counterpart):
 * spatial weights and the filter itself; exp_cw is its float exponential. */
void so_bilateral_weights(int radius, float sigma_space, float* ws);
void so_bilateral_filter(const float* in, int w, int h, int radius, float sigma_space, float sigma_range, float* out);
float so_exp_cw(float x);

/* preprocessor::downsample_depth: median downsampling by the integer ratio w_in / w_out
 * (equal in both axes); map (may be NULL) receives the chosen input pixel per output pixel. */
void so_downsample_depth(const float* in, int w_in, int h_in, float* out, int w_out, int h_out, int64_t* map);

/* Marching cubes of a single-res map: faces (9 floats each, voxel units), returns the count;
 * the case table it triangulates with (ntri[256], tri[256 * 24], -1 padded). */
long long so_marching_cubes(const so_map* map, float* faces, long long capacity);
void so_mc_table(int32_t* ntri, int32_t* tri);
/* Dual marching cubes of a multi-res TSDF map: faces (9 floats each, voxel units) and the scale
 * of each face; returns the face count (-1 for a single-res map). */
long long so_dual_marching_cubes(const so_map* map, int min_desired_scale, float* faces, int8_t* scales,
                                 long long capacity);
/* The partition of the 8 dual corners of a block-relative primal corner into blocks. */
void so_dual_groups(const int32_t rel[3], int32_t group_of[8], int32_t above[8], int32_t* n_groups);

/* Preprocessing helpers exposed for tests. */
void so_half_sample_robust(const float* in, int w, int h, float e_d, int radius, float* out);
void so_depth_to_point_cloud(const float* depth, const so_pinhole* sensor, float* pts);
void so_point_cloud_to_normal(const float* pts, int w, int h, int neg_y, float* nrm);
void so_tracker_pyramid(const so_pinhole* sensor, const float* depth, int levels, float* depth_out,
                        float* pts_out, float* nrm_out);

#ifdef __cplusplus
}
#endif

#endif /* SE_ORACLE_H */
