/*
 * se_gpu.h — C ABI of the GB300 (sm_103a) implementation of supereight2's per-frame
 * dense-mapping hot path: TSDF block allocation, voxel update, raycast and ICP tracking.
 *
 * Conventions
 *   - Matrices are row-major float[16] (4x4 homogeneous transforms), e.g. T_WC maps camera
 *     coordinates to world coordinates. Eigen's Isometry3f::matrix() is column-major: transpose
 *     it (or map it with Eigen::RowMajor) when crossing this boundary.
 *   - Images are device pointers, row-major, pixel (x, y) at index x + y * width, exactly the
 *     memory layout of se::Image<T> (include/se/image/image.hpp:19-70). 3-vector images are
 *     packed xyz float triplets (the layout of se::Image<Eigen::Vector3f>).
 *   - Every call that takes a stream is stream-ordered and asynchronous unless stated. Calls on
 *     one map are not re-entrant: issue them on one stream (the reference's calls on one map are
 *     not re-entrant either).
 *   - Errors: every function returns se_gpu_status. Device-side failures (block pool full, hash
 *     probe limit) are latched in the map and reported by se_gpu_map_check(), which
 *     synchronises the stream. The reference asserts or silently drops in these cases.
 *
 * Pinhole projection convention (the reference delegates it to the un-vendored srl_projection
 * module): rz = 1/z, u = fx*(x*rz) + cx, v = fy*(y*rz) + cy; a projection is Successful iff
 * z > 0 and (u, v) lies in [-0.5, w-0.5) x [-0.5, h-0.5); round_pixel is int(p + 0.5).
 * backProject(u, v) = ((u - cx) * (1/fx), (v - cy) * (1/fy), 1).
 */
#ifndef SE_GPU_H
#define SE_GPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SE_GPU_API __attribute__((visibility("default")))
#else
#define SE_GPU_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SE_GPU_OK = 0,
    SE_GPU_ERR_BAD_ARG = 1,        /* invalid argument (null pointer, size mismatch, ...) */
    SE_GPU_ERR_CUDA = 2,           /* a CUDA runtime call failed; see se_gpu_last_error() */
    SE_GPU_ERR_POOL_FULL = 3,      /* the block pool ran out; some blocks were not allocated */
    SE_GPU_ERR_HASH_PROBE_LIMIT = 4, /* the block hash hit its probe limit */
    SE_GPU_ERR_NOT_SUPPORTED = 5,  /* the map type does not support this call */
    SE_GPU_ERR_NO_DEVICE = 6       /* no CUDA device of compute capability 10.3 */
} se_gpu_status;

typedef enum { SE_GPU_FIELD_TSDF = 0, SE_GPU_FIELD_OCCUPANCY = 1 } se_gpu_field;
typedef enum { SE_GPU_RES_SINGLE = 0, SE_GPU_RES_MULTI = 1 } se_gpu_res;
typedef enum {
    SE_GPU_STORAGE_F32 = 0, /* float tsdf + float weight per voxel (the reference layout) */
    SE_GPU_STORAGE_F16 = 1  /* 4 bytes per voxel, FP32 arithmetic: the tsdf as FP16 with 8 more
                             * significand bits (bits 31..8; bits 31..16 are the binary16 value
                             * truncated toward zero) and an 8-bit integer weight (bits 7..0,
                             * max_weight <= 255). Within max_weight * 2^-19 truncation units
                             * of the F32 layout (1.9e-4 at max_weight 100). */
} se_gpu_storage;

/* se::Map<Data<TSDF>, Res::Single, 8>::Config + FieldData<TSDF>::Config
 * (include/se/map/map.hpp:41-57, include/se/map/data_field.hpp:76-84) plus pool sizing. */
typedef struct {
    float dim[3];      /* metres; the octree side is pow2ceil(max(dim)/res) voxels, >= 16 */
    float res;         /* metres per voxel */
    float T_MW[16];    /* world-to-map transform; set has_T_MW = 0 for translation(dim/2) */
    int has_T_MW;
    int field;         /* se_gpu_field: TSDF, or occupancy (multi-res only) */
    int res_type;      /* se_gpu_res: single-res (Map<.., Res::Single>) or multi-res TSDF */
    int storage;       /* se_gpu_storage */
    float truncation_boundary_factor; /* reference default 8 */
    float max_weight;  /* reference default 100; an integer <= 65535 (<= 255 with F16 storage) */
    int64_t max_blocks; /* block pool capacity (8^3-voxel blocks) */
} se_gpu_map_config;

/* se::FieldData<Occupancy>::Config (include/se/map/data_field.hpp:52-71): the parameters a YAML
 * "data" node sets. max_weight keeps the reference's default floor(|-100 / (0.97 * -5.015)|). */
typedef struct {
    float k_sigma;          /* 0.052 */
    float sigma_min_factor; /* 1.5 */
    float sigma_max_factor; /* 6 */
    float k_tau;            /* 0.026 */
    float tau_min_factor;   /* 6 */
    float tau_max_factor;   /* 16 */
    float log_odd_min;      /* -5.015 */
    float log_odd_max;      /* 5.015 */
    int fs_integr_scale;    /* 1 */
} se_gpu_occupancy_config;

/* se::PinholeCamera::Config (include/se/sensor/sensor.hpp:29-57, pinhole_camera.hpp). */
typedef struct {
    int width;
    int height;
    float fx, fy, cx, cy;
    float near_plane;
    float far_plane;
} se_gpu_pinhole;

/* se::OusterLidar::Config (include/se/sensor/ouster_lidar.hpp:25-60) for an equiangular spinning
 * LiDAR. The reference delegates the projection to the un-vendored srl_projection module; this
 * ABI fixes it: column u sweeps 360 degrees of azimuth clockwise from +x, u = (pi - atan2(y, x))
 * * width / 2pi - 0.5 wrapped into [-0.5, width - 0.5); row v = (el_max - el) * (height - 1) /
 * (el_max - el_min) with el = atan2(z, |xy|), row 0 the highest beam, Successful iff v lies in
 * [-0.5, height - 0.5). Angles use an arctangent of documented accuracy (1e-5 rad,
 * Abramowitz-Stegun 4.4.49) so that every platform rounds alike. Range images hold the range
 * (metres, <= 0: no return); measurementFromPoint is the point's norm. The beam elevations are
 * linear from elevation_max_deg (row 0) to elevation_min_deg; min_ray_angle = min(beam spacing,
 * 360 / width) (src/sensor/ouster_lidar.cpp:59-85). */
typedef struct {
    int width;                  /* columns (azimuth steps) */
    int height;                 /* beams */
    float elevation_min_deg;
    float elevation_max_deg;
    float near_plane;
    float far_plane;
} se_gpu_lidar;

/* se::LeicaLidar::Config (include/se/sensor/leica_lidar.hpp): the ray-batch sensor of
 * se_gpu_occ_integrate_ray_batch. The integration scale uses pixel_dim_tan =
 * 2 tan(min(elevation, azimuth resolution) / 2) (src/sensor/leica_lidar.cpp:53-73, 87-129);
 * width and height are kept for the sensor's image model, which the ray integrator does not use. */
typedef struct {
    int width;
    int height;
    float near_plane;
    float far_plane;
    float elevation_resolution_deg;
    float azimuth_resolution_deg;
} se_gpu_leica_lidar;

/* The bilateral pre-filter of the tracking input. No counterpart in the reference (it feeds
 * the depth straight to the tracker); defined by this library: invalid (<= 0 or NaN) centres
 * stay 0, the valid taps of the (2 radius + 1)^2 window inside the image are weighted by
 * exp(-(dx^2 + dy^2) / (2 sigma_space_px^2)) * exp(-(d - c)^2 / (2 sigma_range_m^2)). The
 * benchmark's tracked TSDF configuration uses radius 2, 4 px, 0.03 m. radius <= 7. */
typedef struct {
    int radius;
    float sigma_space_px;
    float sigma_range_m;
} se_gpu_bilateral_config;

/* se::TrackerConfig (include/se/tracker/tracker.hpp:22-33). */
typedef struct {
    int num_levels;    /* at most 3 */
    int iterations[3]; /* finest level first; reference default {10, 5, 4} */
    float dist_threshold;   /* 0.1 */
    float normal_threshold; /* 0.8 */
    float track_threshold;  /* 0.15 */
    float icp_threshold;    /* 1e-5 */
} se_gpu_tracker_config;

/* Per-call counters of the last integrate_depth (read with se_gpu_map_integrate_stats). */
typedef struct {
    int64_t n_new_blocks;      /* blocks allocated by the carver */
    int64_t n_listed_blocks;   /* new + previously allocated blocks in the frustum */
    int64_t n_updated_voxels;  /* voxels whose field update returned true */
    int64_t n_valid_pixels;    /* pixels in [near, far + band/2] */
} se_gpu_integrate_stats;

typedef struct se_gpu_map se_gpu_map;
typedef struct se_gpu_tracker se_gpu_tracker;

/* Last error message of this thread (CUDA error string or argument check). */
SE_GPU_API const char* se_gpu_last_error(void);
SE_GPU_API const char* se_gpu_status_string(se_gpu_status status);
/* ABI version, bumped on any incompatible change. */
SE_GPU_API int se_gpu_abi_version(void);

/* ------------------------------------------------------------------------------ maps -- */

/* Replaces se::Map ctor (include/se/map/impl/map_impl.hpp:37-55) and the Octree ctor
 * (include/se/map/octree/impl/octree_impl.hpp:14-19). Allocates the block pool and hash on the
 * current CUDA device. */
SE_GPU_API se_gpu_status se_gpu_map_create(const se_gpu_map_config* config, se_gpu_map** map);
/* The same for an occupancy map (field SE_GPU_FIELD_OCCUPANCY, res_type SE_GPU_RES_MULTI) with
 * its field configuration (NULL: the reference's defaults); se_gpu_map_create uses the defaults.
 * max_blocks bounds the block pool; the node pool holds max_blocks / 2 + 4096 nodes. */
SE_GPU_API se_gpu_status se_gpu_map_create_occupancy(const se_gpu_map_config* config,
                                                     const se_gpu_occupancy_config* occupancy,
                                                     se_gpu_map** map);
SE_GPU_API se_gpu_status se_gpu_map_destroy(se_gpu_map* map);
/* Octree side in voxels (Octree::getSize()) and map side in metres (Map::getDim()). */
SE_GPU_API se_gpu_status se_gpu_map_size(const se_gpu_map* map, int* size, float* dim_m);
/* Synchronise the map's last stream and return any latched device-side error, then clear it. */
SE_GPU_API se_gpu_status se_gpu_map_check(se_gpu_map* map);

/* Replaces se::MapIntegrator<TSDFMap<Res::Single | Res::Multi>>::integrateDepth(timestamp,
 * Measurements{Measurement{depth, sensor, T_WC}}) (include/se/integrator/map_integrator.hpp:78-81,
 * impl/map_integrator_impl.hpp:52-84): RaycastCarver allocation (allocator/impl/
 * raycast_carver_impl.hpp:56-128) then the single-res TSDF update (updater/impl/
 * singleres_tsdf_updater_impl.hpp:14-132) or the multi-res one (updater/impl/
 * multires_tsdf_updater_impl.hpp:14-250). depth_dev: width*height floats on the device. */
SE_GPU_API se_gpu_status se_gpu_integrate_depth(se_gpu_map* map, const float* depth_dev,
                                     const se_gpu_pinhole* sensor, const float T_WC[16],
                                     int timestamp, void* stream);
/* Replaces se::MapIntegrator<OccupancyMap<Res::Multi>>::integrateDepth(timestamp,
 * Measurements{Measurement{range, OusterLidar, T_WS}}) (impl/map_integrator_impl.hpp:90-130)
 * with the Ouster variants of the pooling image (allocator/impl/dense_pooling_image_impl.hpp:
 * 395-784), of the VolumeCarver (allocator/impl/volume_carver_impl.hpp:339-537) and of the
 * integration scale (src/sensor/ouster_lidar.cpp:107-146). Occupancy maps only. range_dev:
 * width*height floats on the device. */
SE_GPU_API se_gpu_status se_gpu_integrate_range(se_gpu_map* map, const float* range_dev,
                                                const se_gpu_lidar* sensor, const float T_WS[16],
                                                int timestamp, void* stream);

/* Replaces se::MapIntegrator::integrateRayBatch(timestamp, rayPoseBatch, sensor, updated_octants)
 * for multi-res occupancy maps with a LeicaLidar (include/se/integrator/impl/
 * map_integrator_impl.hpp:137-176, se::RayIntegrator in impl/ray_integrator_impl.hpp and
 * impl/ray_integrator_core_impl.hpp): the n rays rays_dev[3 i] (sensor frame) with their poses
 * poses_dev[16 i] (T_WS, row-major), all on the device, are integrated in batch order, then the
 * updated blocks are propagated to their coarsest scale and the nodes above them to the root.
 * The map equals the one the reference's serial loop leaves: rays run concurrently, but rays
 * that may touch the same block update it in batch order. octants_dev (may be NULL) receives up
 * to capacity updated octants as (x, y, z, size) in voxels, size 8 for a block, in any order:
 * the updated blocks and the propagated nodes, less the nodes whose children were pruned (the
 * reference's updated_octants set); *n_octants their number. A wait of a ray for a block that
 * runs past 2 s abandons the batch (SE_GPU_ERR_CUDA, the map then partly updated). Synchronous.
 * Occupancy maps only. */
SE_GPU_API se_gpu_status se_gpu_occ_integrate_ray_batch(se_gpu_map* map, const se_gpu_leica_lidar* sensor,
                                                        const float* poses_dev, const float* rays_dev,
                                                        int64_t n, int32_t timestamp, int32_t* octants_dev,
                                                        int64_t capacity, int64_t* n_octants, void* stream);

/* Batched occupancy integration; no counterpart in the reference, which integrates one map per
 * call. n (<= 16) occupancy maps with one sensor (a pinhole camera or a LiDAR: exactly one of
 * the two pointers non-NULL) integrate one frame each per call, every stage of the pipeline in
 * one launch over all maps' work (uneven block and node counts share the grid). The maps stay owned by the caller and must
 * outlive the batch; calls on a batch are not re-entrant and none of its maps may be used by
 * another call in flight. */
typedef struct se_gpu_occ_batch se_gpu_occ_batch;
/* flags: SE_GPU_OCC_BATCH_GRAPH (capture and replay, as above) and SE_GPU_OCC_BATCH_AUTOTUNE:
 * the first 4 calls run the default geometry (the maps grow from empty), the next 12 run in turn
 * 4 candidate launch geometries (CTAs per SM of the carver, list and block stages) three times,
 * timed with events (these calls synchronise the stream), and the batch keeps per stage the
 * candidate with the least time in its best round; the graph is captured after tuning. Results
 * do not depend on the geometry. */
#define SE_GPU_OCC_BATCH_GRAPH 1
#define SE_GPU_OCC_BATCH_AUTOTUNE 2
/* SE_GPU_OCC_BATCH_PERSISTENT: each call runs as one cooperative launch, every stage a
 * grid-stride loop over the whole batch separated by grid barriers (a barrier that waits past
 * 1 s abandons the frame and se_gpu_map_check reports it); with AUTOTUNE the tuned geometry is
 * its CTAs per SM (1 or 2; tiles[0]). Results equal the multi-launch path's. */
#define SE_GPU_OCC_BATCH_PERSISTENT 4
SE_GPU_API se_gpu_status se_gpu_occ_batch_create(se_gpu_map* const* maps, int n,
                                                 const se_gpu_pinhole* pinhole,
                                                 const se_gpu_lidar* lidar, int flags,
                                                 se_gpu_occ_batch** batch);
/* The launch geometry in use (CTAs per SM: carver, lists, blocks) and the tuning calls left. */
SE_GPU_API se_gpu_status se_gpu_occ_batch_tiles(const se_gpu_occ_batch* batch, int tiles[3],
                                                int* tuning_calls_left);
/* images_dev[i]: map i's depth / range image on the device; T_WS: n row-major 4x4 poses
 * (host); timestamps: n frame numbers (host). Stream-ordered. */
SE_GPU_API se_gpu_status se_gpu_occ_batch_integrate(se_gpu_occ_batch* batch,
                                                    const float* const* images_dev,
                                                    const float* T_WS, const int* timestamps,
                                                    void* stream);
/* The four per-frame counters of every map of the batch (as se_gpu_map_occupancy_stats: blocks
 * listed, free-space nodes listed, blocks freed, nodes pruned), 4 int32 per map into stats_host
 * (pinned for an asynchronous copy), enqueued on stream: valid once the stream passes this call,
 * so that a caller reads step k's counters while step k + 1 runs. */
SE_GPU_API se_gpu_status se_gpu_occ_batch_stats_async(const se_gpu_occ_batch* batch, int32_t* stats_host,
                                                      void* stream);
SE_GPU_API se_gpu_status se_gpu_occ_batch_destroy(se_gpu_occ_batch* batch);

/* Counters of the last integrate_depth; synchronises the stream. */
SE_GPU_API se_gpu_status se_gpu_map_integrate_stats(se_gpu_map* map, se_gpu_integrate_stats* stats);

/* Replaces se::raycaster::raycast_volume(map, sensor, T_WS, points_W, normals_W, scale)
 * (include/se/map/raycaster.hpp:56-64, impl/raycaster_impl.hpp:456-627; occupancy maps:
 * impl/raycaster_impl.hpp:32-452 with normals against the field gradient). Output device
 * images: pts_W and nrm_W are width*height*3 floats, scale is width*height int8 (may be NULL). */
SE_GPU_API se_gpu_status se_gpu_raycast(const se_gpu_map* map, const se_gpu_pinhole* sensor,
                             const float T_WS[16], float* pts_W_dev, float* nrm_W_dev,
                             int8_t* scale_dev, void* stream);

/* Replaces se::algorithms::marching_cube(octree) for single-res TSDF maps
 * (include/se/map/algorithms/impl/marching_cube_impl.hpp:830-890, 1175-1201): the faces of the
 * surface between observed inside (tsdf < 0) and observed outside voxels, 9 floats each (three
 * vertices in voxel units of the map frame, the reference's Face::vertexes; world = T_WM *
 * (res * v)). Vertices follow meshing::compute_intersection exactly and each crossing pattern
 * is triangulated by the reference's case table (edge_tables.hpp, triTable; see
 * se_gpu_mc_case_table), so the faces are the reference's face for face. Faces point away from
 * the inside. Writes up to capacity faces (any order) to faces_dev and the total to
 * *count (call again with a larger buffer when *count > capacity). Synchronous. Multi-res TSDF
 * and occupancy maps: se_gpu_dual_marching_cube with min_desired_scale 0, without the scales. */
SE_GPU_API se_gpu_status se_gpu_marching_cube(se_gpu_map* map, float* faces_dev, int64_t capacity,
                                              int64_t* count, void* stream);
/* Replaces se::algorithms::marching_cube(octree, min_desired_scale) for multi-res TSDF and
 * occupancy maps (dual_marching_cube_kernel, marching_cube_impl.hpp:895-975): each block is
 * meshed on its dual grid at clamp(min_desired_scale, current_scale, 3), across block faces at
 * the coarser of the two blocks' scales (gather_dual_data :683-758); inside = tsdf < 0, or
 * occupancy * weight > 0 (faces point away from occupied space). faces_dev as for
 * se_gpu_marching_cube (may be NULL to count); scales_dev (may be NULL) receives each face's
 * scale (Face::scale). min_desired_scale in [0, 3]. Single-res maps: SE_GPU_ERR_NOT_SUPPORTED.
 * Synchronous. */
SE_GPU_API se_gpu_status se_gpu_dual_marching_cube(se_gpu_map* map, int min_desired_scale,
                                                   float* faces_dev, int8_t* scales_dev,
                                                   int64_t capacity, int64_t* count, void* stream);
/* The case table: ntri[c] faces for case c (bit i = corner i inside, corners (0,0,0), (1,0,0),
 * (1,0,1), (0,0,1), (0,1,0), (1,1,0), (1,1,1), (0,1,1)), tri[15 c + 3 f + j] the edge (as
 * meshing::edge_to_corners) of vertex j of face f, -1 padded: the reference's triTable
 * (include/se/map/algorithms/edge_tables.hpp) row for row. Host only. */
SE_GPU_API se_gpu_status se_gpu_mc_case_table(int32_t ntri[256], int32_t tri[256 * 15]);

/* ------------------------------------------------------------------------------- IO -- */
/* The reference's on-disk outputs (the headers of include/se/map/io), written by this library's own host code
 * in the same standard ASCII formats. io::save_mesh (mesh_io_impl.hpp): faces (host, 9 floats
 * each) transformed by T_OV (row-major 4x4 affine), format by extension: .ply (faces coloured
 * by scale), .vtk (polydata with a per-face scale and scale colour), .obj; scales (host, one per
 * face) may be NULL for scale 0. */
SE_GPU_API se_gpu_status se_gpu_save_mesh(const float* faces, const int8_t* scales, int64_t n,
                                          const float T_OV[16], const char* filename);
/* Map::mesh's transform T_OV = T_OW * T_WM * Scaling(res) (map_impl.hpp:454-459). */
SE_GPU_API se_gpu_status se_gpu_map_mesh_transform(const se_gpu_map* map, const float T_OW[16],
                                                   float T_OV[16]);
/* Map::saveMesh(filename, T_OW, min_desired_scale) (map_impl.hpp:464-469): marching cubes on the
 * GPU (dual for multi-res and occupancy maps, which take min_desired_scale), then
 * se_gpu_save_mesh. Synchronous. */
SE_GPU_API se_gpu_status se_gpu_map_save_mesh(se_gpu_map* map, const float T_OW[16],
                                              int min_desired_scale, const char* filename,
                                              void* stream);
/* io::save_point_cloud_vtk (point_cloud_io_impl.hpp): n points (host, xyz) transformed by T_WC. */
SE_GPU_API se_gpu_status se_gpu_save_point_cloud_vtk(const float* points, int64_t n,
                                                     const float T_WC[16], const char* filename);
/* get_field(getData(coord)) of a single-res TSDF map over the voxel box [lo, hi), x fastest,
 * into out_host ((hi - lo) product floats). Synchronous. */
SE_GPU_API se_gpu_status se_gpu_map_field_box(const se_gpu_map* map, const int32_t lo[3],
                                              const int32_t hi[3], float* out_host);
/* Map::saveFieldSlices(fx, fy, fz, point_W) (map_impl.hpp:273-320 with io::save_3d_slice_vtk,
 * octree_io_impl.hpp): the x, y and z slices of the field through the voxel of point_W as VTK
 * rectilinear grids (an empty or NULL name skips that slice). Single-res TSDF maps. */
SE_GPU_API se_gpu_status se_gpu_map_save_field_slices(const se_gpu_map* map, const char* filename_x,
                                                      const char* filename_y,
                                                      const char* filename_z,
                                                      const float point_W[3]);

/* Block download for checking and checkpointing. Writes up to capacity blocks:
 * keys (Morton code << 5 | 3), coords (3 ints: the block's minimum voxel), tsdf and weight
 * (512 floats per block, x + 8y + 64z), timestamps. Host pointers, any may be NULL.
 * Synchronous. *count receives the number of allocated blocks. */
SE_GPU_API se_gpu_status se_gpu_map_download_blocks(const se_gpu_map* map, int64_t capacity,
                                         uint64_t* keys, int32_t* coords, float* tsdf,
                                         float* weight, int32_t* timestamps, int64_t* count);
/* Multi-resolution maps: per block the 585-entry voxel pyramid of BlockMultiRes
 * (include/se/map/octant/block.hpp:66-166; scale 0: 512 entries x + 8y + 64z at offset 0,
 * scale 1: 64 at 512, scale 2: 8 at 576, scale 3: 1 at 584) of data (tsdf, weight) and past
 * data (past_tsdf, past_weight), and scales (2 ints per block: current_scale, min_scale; -1
 * before the first update). se_gpu_map_download_blocks returns a multi-res map's scale-0
 * level. Host pointers, any may be NULL; synchronous. */
SE_GPU_API se_gpu_status se_gpu_map_download_multires(const se_gpu_map* map, int64_t capacity,
                                           uint64_t* keys, int32_t* coords, float* tsdf,
                                           float* weight, float* past_tsdf, float* past_weight,
                                           int32_t* scales, int64_t* count);
/* Occupancy maps. Counters of the last integrate_depth: {blocks the VolumeCarver listed,
 * free-space nodes it listed, blocks freed below those nodes, nodes pruned}; synchronises. */
SE_GPU_API se_gpu_status se_gpu_map_occupancy_stats(se_gpu_map* map, int64_t stats[4]);
/* Live blocks (pool order), up to capacity: coords (3 ints), scales (current, min, buffer),
 * counts (current integrations, current observed, buffer integrations, buffer observed), and
 * the 585-entry mean / min / max pyramids (offsets as for multi-res TSDF) of (occupancy,
 * weight, observed) with min / max at the finest scale equal to the mean data and the block's
 * init data below it (BlockMultiRes<Occupancy>, include/se/map/octant/impl/block_impl.hpp:
 * 206-855). Host pointers, any may be NULL; synchronous; *count receives the live blocks. */
SE_GPU_API se_gpu_status se_gpu_map_download_occupancy(const se_gpu_map* map, int64_t capacity,
                                                       int32_t* coords, int32_t* scales,
                                                       int64_t* counts, float* mean, float* min_data,
                                                       float* max_data, int64_t* count);
/* Nodes reachable from the root, depth first in child order: (x, y, z, size), min / max data
 * as (occupancy, weight, observed), leaf flag. Synchronous; *count receives the number. */
SE_GPU_API se_gpu_status se_gpu_map_download_nodes(const se_gpu_map* map, int64_t capacity,
                                                   int32_t* coords, float* min_data, float* max_data,
                                                   int32_t* leaf, int64_t* count);
/* Block upload (checkpoint restore, test set-up, single-res maps only): allocates the blocks with the given keys
 * (Morton code << 5 | 3, as written by se_gpu_map_download_blocks) if they are not allocated,
 * then overwrites their 512 voxels from tsdf / weight (host, 512 floats per block; weights are
 * rounded to integers). Synchronous. */
SE_GPU_API se_gpu_status se_gpu_map_upload_blocks(se_gpu_map* map, int64_t n, const uint64_t* keys,
                                       const float* tsdf, const float* weight);
/* Replaces Map::getFieldInterp(point_W) and Map::getFieldGrad(point_W)
 * (include/se/map/impl/map_impl.hpp:154-172,236-262) for a batch of n device points
 * (3 floats each). valid_dev (n ints) receives 1 where the reference returns a value. */
SE_GPU_API se_gpu_status se_gpu_map_field_interp(const se_gpu_map* map, int64_t n, const float* points_W_dev,
                                      float* values_dev, int* valid_dev, void* stream);
SE_GPU_API se_gpu_status se_gpu_map_field_grad(const se_gpu_map* map, int64_t n, const float* points_W_dev,
                                    float* grads_dev, int* valid_dev, void* stream);
/* Allocated-block AABB in voxels (Octree::aabb(), inclusive). Synchronous; returns
 * SE_GPU_OK with *empty = 1 when no block is allocated. */
SE_GPU_API se_gpu_status se_gpu_map_aabb(const se_gpu_map* map, int32_t mn[3], int32_t mx[3], int* empty);

/* ---------------------------------------------------------- differentiable raycast -- */

/* Differentiable depth render of a single-res map. No counterpart in the reference. Per
 * pixel, the march of raycast_volume (include/se/map/impl/raycaster_impl.hpp:456-533) up to
 * the first sample below the surface, then regula falsi on the trilinear TSDF inside that
 * last step: depth_dev[x + y*width] = z (camera frame) of the root, 0 where the march finds
 * no crossing or the interpolation is undefined at the bracket. */
SE_GPU_API se_gpu_status se_gpu_render_depth(const se_gpu_map* map, const se_gpu_pinhole* sensor,
                                             const float T_WS[16], float* depth_dev, void* stream);
/* Adjoint of se_gpu_render_depth, recomputing each ray's march. No counterpart in the
 * reference. With the pose perturbed on the left, T = exp(xi) T_WS, xi = [rho; omega] (the
 * reference's se(3) update, src/tracker/icp.cpp:208-223):
 *   twist_grad_dev[6] += sum_i grad_depth_dev[i] * d depth_i / d xi     (device doubles)
 *   voxel_grad_dev[b*512 + v] += sum_i grad_depth_dev[i] * d depth_i / d tsdf(b, v)
 *       (b the pool index, the block order of se_gpu_map_download_blocks; may be NULL)
 *   jac_dev[6*i + j] = d depth_i / d xi_j  (width*height*6 floats; may be NULL)
 * grad_depth_dev (width*height floats) may be NULL when jac_dev is given. Asynchronous. */
SE_GPU_API se_gpu_status se_gpu_raycast_adjoint(const se_gpu_map* map, const se_gpu_pinhole* sensor,
                                                const float T_WS[16], const float* grad_depth_dev,
                                                double* twist_grad_dev, float* voxel_grad_dev,
                                                float* jac_dev, void* stream);

/* --------------------------------------------------------------------------- tracker -- */

/* Replaces se::preprocessor::downsample_depth(input, output) (src/map/preprocessor.cpp:19-84):
 * each output pixel is the median (upper middle for an even count) of the depths >= 1e-5 of its
 * ratio x ratio input region (ratio = w_in / w_out = h_in / h_out, at most 8), or 0 when none is
 * valid; map_dev (may be NULL) receives the chosen input pixel x + y * w_in as the reference's
 * Image<size_t>. Equal depths keep their region scan order (the reference's std::sort leaves
 * that order unspecified), which decides map_dev only. Device pointers; stream-ordered. The
 * matching sensor is se::PinholeCamera(config, ratio): fx / ratio, fy / ratio,
 * (cx + 0.5) / ratio - 0.5, (cy + 0.5) / ratio - 0.5 (src/sensor/pinhole_camera.cpp:29-39). */
SE_GPU_API se_gpu_status se_gpu_downsample_depth(const float* in_dev, int w_in, int h_in,
                                                 float* out_dev, int w_out, int h_out,
                                                 int64_t* map_dev, void* stream);

/* The bilateral pre-filter (see se_gpu_bilateral_config) of a device depth image into another
 * device image (not in place). Stream-ordered. */
SE_GPU_API se_gpu_status se_gpu_bilateral_filter(const float* in_dev, float* out_dev, int width,
                                                 int height, const se_gpu_bilateral_config* config,
                                                 void* stream);

/* Replaces se::Tracker ctor (include/se/tracker/tracker.hpp:42-48): device buffers for the
 * depth pyramid, per-level point clouds and normals and the ICP partial sums. */
SE_GPU_API se_gpu_status se_gpu_tracker_create(const se_gpu_pinhole* sensor,
                                    const se_gpu_tracker_config* config,
                                    se_gpu_tracker** tracker);
SE_GPU_API se_gpu_status se_gpu_tracker_destroy(se_gpu_tracker* tracker);

/* Replaces se::Tracker::track(depth, T_WS, surface_point_cloud_W, surface_normals_W)
 * (include/se/tracker/impl/tracker_impl.hpp:30-116): 3-level projective point-to-plane ICP
 * against the raycast (ref_pts/ref_nrm, width*height*3 device floats) taken at the input T_WS.
 * T_WS is read and written on the host; *accepted receives the checkPoseKernel result (a
 * rejected track leaves T_WS unchanged, as in the reference). Synchronous. */
SE_GPU_API se_gpu_status se_gpu_track(se_gpu_tracker* tracker, const float* depth_dev,
                           const float* ref_pts_W_dev, const float* ref_nrm_W_dev,
                           float T_WS[16], int* accepted, void* stream);
/* ICP launch shape (no counterpart in the reference): 1 (the default when the grid fits on the
 * device) runs all levels and iterations of a track() in one cooperative launch whose CTAs wait,
 * bounded, for each iteration's merged totals to be complete; 0 launches one kernel per
 * iteration. Both give bit-identical poses. A wait that times out rejects the frame's pose
 * (accepted = 0) and se_gpu_track returns SE_GPU_ERR_CUDA. */
SE_GPU_API se_gpu_status se_gpu_tracker_set_persistent(se_gpu_tracker* tracker, int enable);
/* Test aid for the failure path: with enable != 0 the persistent ICP waits for the partial of
 * one CTA more than the grid holds, so its bounded wait runs out (half a second), the frame's
 * pose is rejected and se_gpu_track returns SE_GPU_ERR_CUDA; the context stays usable. */
SE_GPU_API se_gpu_status se_gpu_tracker_test_barrier_timeout(se_gpu_tracker* tracker, int enable);
/* Final 32-float reduction of the last track (icp.cpp:45-204 layout: [sum e^2, J^T e (6),
 * upper J^T J (21), inliers, distance rejects, normal rejects, other]) and the iterations run
 * per level. Synchronous. */
SE_GPU_API se_gpu_status se_gpu_tracker_last_reduction(se_gpu_tracker* tracker, float reduction[32],
                                            int iterations_run[3]);

/* The tracker's input pyramid of the last track at one level (0 = full resolution): the
 * half-sampled depth (half_sample_robust_image, src/map/preprocessor.cpp:156-195; levels >= 1
 * only, level 0's depth is the caller's input), the point cloud (depth_to_point_cloud,
 * include/se/map/impl/preprocessor_impl.hpp:18-40) and the normals (point_cloud_to_normal,
 * src/map/preprocessor.cpp:109-152), copied into caller device buffers of (W >> level) x
 * (H >> level) floats, and 3 floats per pixel for points and normals. Any pointer may be NULL.
 * Stream-ordered, asynchronous. */
SE_GPU_API se_gpu_status se_gpu_tracker_level_images(se_gpu_tracker* tracker, int level,
                                                     float* depth_dev, float* pts_dev,
                                                     float* nrm_dev, void* stream);

/* Allocation-free tracking. No counterpart in the reference. For callers that cannot
 * allocate device memory while they track (a host whose pool allocator owns the free device
 * memory, a loop with a memory budget fixed at start-up, or code that must not let
 * cudaMalloc's implicit device synchronisation stall its other streams): one full-resolution
 * ICP level (config->num_levels must be 1, config->iterations[0] iterations), with the
 * tracker's scratch in a static device array of about 77 KiB that the library holds on every
 * GPU that loads it. Depth images larger than 4096 x 4096 pixels are rejected. The first call
 * on a device looks up the array's device address, and with CUDA's lazy module loading (the
 * default since CUDA 12.2) that lookup is also when the driver loads this part of the
 * library onto the device, which allocates the static array and the kernels' code there: make
 * the first call at start-up, before a pool allocator takes the free memory and before any
 * stream capture. Later calls allocate nothing. Calls share the array: calls that overlap on
 * the GPU race. T_WS is read and
 * written on the host; accepted and reduction (32 floats, se_gpu_tracker_last_reduction's
 * layout) may be NULL. Synchronous. */
SE_GPU_API se_gpu_status se_gpu_track_noalloc(const se_gpu_pinhole* sensor,
                                              const se_gpu_tracker_config* config,
                                              const float* depth_dev, const float* ref_pts_W_dev,
                                              const float* ref_nrm_W_dev, float T_WS[16],
                                              int* accepted, float reduction[32], void* stream);

/* ---------------------------------------------------------------- captured pipeline -- */

/* The per-frame loop of the reference application (app/src/main.cpp:126-160: track the new
 * depth against the previous raycast, integrate it at the tracked pose, raycast the map at
 * that pose) as one CUDA graph, with the pose and the frame counter kept on the device. The
 * frame owns its input depth buffer and the raycast images, which are the tracking reference
 * of the next frame. tracker may be NULL (integrate + raycast only). No counterpart exists in
 * the reference, which runs these steps as separate blocking calls. */
typedef struct se_gpu_frame se_gpu_frame;
SE_GPU_API se_gpu_status se_gpu_frame_create(se_gpu_map* map, se_gpu_tracker* tracker,
                                             const se_gpu_pinhole* sensor, se_gpu_frame** frame);
SE_GPU_API se_gpu_status se_gpu_frame_destroy(se_gpu_frame* frame);
/* Device buffers owned by the frame: the input depth (width*height floats, written by the
 * caller before se_gpu_frame_run) and the raycast outputs (width*height*3 floats each, and
 * width*height int8). Any pointer may be NULL. */
SE_GPU_API se_gpu_status se_gpu_frame_buffers(se_gpu_frame* frame, float** depth_dev,
                                              float** pts_W_dev, float** nrm_W_dev,
                                              int8_t** scale_dev);
/* Track on the bilateral-filtered input (config) or on the input itself (NULL, the default);
 * integration always uses the unfiltered depth. The next run recaptures the graph. */
SE_GPU_API se_gpu_status se_gpu_frame_set_bilateral(se_gpu_frame* frame,
                                                    const se_gpu_bilateral_config* config);
/* Set the device pose T_WS and the integration timestamp of the next run. Synchronous. */
SE_GPU_API se_gpu_status se_gpu_frame_set_pose(se_gpu_frame* frame, const float T_WS[16],
                                               int timestamp);
/* Launch one frame on stream: [track (if track != 0)] + integrate + raycast. Asynchronous;
 * the first call per mode captures the graph (call it before any capture of your own). */
SE_GPU_API se_gpu_status se_gpu_frame_run(se_gpu_frame* frame, int track, void* stream);
/* The frame path's autotuner (no counterpart in the reference): the next `runs` runs of the
 * frame (runs >= 6; 0 stops tuning) are launched directly on the stream instead of from the
 * graph, each with one candidate launch geometry of the voxel update (4, 8 or 16 CTAs per SM; 4
 * or 2 voxels per lane per round) and of the raycast (8 x 4 or 16 x 2 pixels per warp), timed
 * with events (these runs synchronise the stream); afterwards the map keeps per kernel the
 * candidate with the least time seen and the graphs are captured again with it. Results do not
 * depend on the geometry. Run it on a grown map. */
SE_GPU_API se_gpu_status se_gpu_frame_autotune(se_gpu_frame* frame, int runs);
/* The geometry in use: tiles[0] update CTAs per SM, tiles[1] voxels per lane per round,
 * tiles[2] raycast warp tile (0: 8 x 4, 1: 16 x 2); tuning_left (may be NULL) the tuning runs
 * still to come. */
SE_GPU_API se_gpu_status se_gpu_frame_tiles(const se_gpu_frame* frame, int tiles[3], int* tuning_left);
/* se_gpu_frame_run with the frame's depth image taken from host memory (width*height floats),
 * as integrateDepth / track take a host Image<float>. The host copy runs on the frame's own copy
 * stream into one of two device staging buffers, so the next call's copy overlaps this frame's
 * work; the frame's stream then waits for it and copies the staging buffer into the input
 * buffer. Pinned memory keeps the copy asynchronous; the host buffer must stay unchanged until
 * the frame's stream has passed this call. */
SE_GPU_API se_gpu_status se_gpu_frame_run_host(se_gpu_frame* frame, const float* depth_host, int track,
                                               void* stream);
/* Read the device pose (after the runs enqueued on stream) and the last run's acceptance (the
 * checkPoseKernel result; 1 when the last run did not track). Synchronous. */
SE_GPU_API se_gpu_status se_gpu_frame_get_pose(se_gpu_frame* frame, float T_WS[16],
                                               int* accepted, void* stream);
/* The same read without waiting: the row-major 3x4 pose and the acceptance are copied into the
 * caller's host memory (pinned, for the copies to stay asynchronous) on stream; they are valid
 * once the stream has reached this point (an event or a synchronisation). A caller that reads
 * each frame's pose while the next frame runs keeps two sets of buffers. */
SE_GPU_API se_gpu_status se_gpu_frame_get_pose_async(se_gpu_frame* frame, float pose12_host[12],
                                                     int* accepted_host, void* stream);

/* ------------------------------------------------------------------------- profiling -- */

/* Per-kernel device time: when enabled, each public call records CUDA events on its stream
 * around every kernel it launches. se_gpu_profiling_read synchronises on the recorded events
 * and returns, for the first n kernels in se_gpu_profiling_name order, the accumulated
 * milliseconds and launch counts (reset != 0 clears them). Off by default. */
SE_GPU_API se_gpu_status se_gpu_profiling_enable(int enable);
SE_GPU_API se_gpu_status se_gpu_profiling_read(int n, double* total_ms, int64_t* launches,
                                               int reset);
SE_GPU_API const char* se_gpu_profiling_name(int index);
SE_GPU_API int se_gpu_profiling_count(void);

#ifdef __cplusplus
}
#endif

#endif /* SE_GPU_H */
