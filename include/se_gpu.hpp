/*
 * se_gpu.hpp — C++17 mirror of supereight2's dense-mapping API over the C ABI of se_gpu.h.
 *
 * Names and argument meaning follow the reference so that calling code reads the same:
 *   se::gpu::TSDFMap                    se::TSDFMap<se::Res::Single>  (include/se/map/map.hpp)
 *   se::gpu::MapIntegrator::integrateDepth(ts, Measurement{depth, sensor, T_WC})
 *                                       include/se/integrator/map_integrator.hpp:78-81
 *   se::gpu::raycaster::raycast_volume(map, sensor, T_WS, pts, nrm, scale)
 *                                       include/se/map/raycaster.hpp:56-64
 *   se::gpu::Tracker(map, sensor, config).track(depth, T_WS, pts, nrm) -> bool
 *                                       include/se/tracker/tracker.hpp:42-73
 * Images are device buffers with se::Image's layout (row-major, x + y * width; 3-vectors
 * packed). Poses are row-major 4x4 float arrays (Pose). Errors throw se::gpu::Error carrying
 * the status and se_gpu_last_error(); the reference asserts instead.
 */
#ifndef SE_GPU_HPP
#define SE_GPU_HPP

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "se_gpu.h"

namespace se {
namespace gpu {

class Error : public std::runtime_error {
  public:
    Error(se_gpu_status s, const std::string& what)
        : std::runtime_error(what + ": " + se_gpu_status_string(s) + " (" + se_gpu_last_error() + ")"), status(s)
    {
    }
    se_gpu_status status;
};

inline void check(se_gpu_status s, const char* what)
{
    if (s != SE_GPU_OK)
        throw Error(s, what);
}

/** Row-major 4x4 transform (Eigen::Isometry3f::matrix() transposed). */
using Pose = std::array<float, 16>;

inline Pose identity()
{
    return Pose{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
}

/** se::PinholeCamera::Config (width, height, fx, fy, cx, cy, near_plane, far_plane). */
struct PinholeCamera {
    se_gpu_pinhole c;
    PinholeCamera(int width, int height, float fx, float fy, float cx, float cy, float near_plane = 0.01f,
                  float far_plane = 10.0f)
        : c{width, height, fx, fy, cx, cy, near_plane, far_plane}
    {
    }
};

/** A device image of T with se::Image's memory layout; not owned. */
template <typename T>
struct DeviceImage {
    T* data;
    int width;
    int height;
};

/** se::TSDFMap<se::Res::Single>: block hash + block pool on the current CUDA device. */
class TSDFMap {
  public:
    struct Config {
        std::array<float, 3> dim{10.0f, 10.0f, 10.0f};
        float res = 0.1f;
        float truncation_boundary_factor = 8.0f;
        float max_weight = 100.0f;
        se_gpu_storage storage = SE_GPU_STORAGE_F32;
        int64_t max_blocks = 1 << 20;
    };

    explicit TSDFMap(const Config& cfg)
    {
        se_gpu_map_config c{};
        for (int i = 0; i < 3; ++i)
            c.dim[i] = cfg.dim[i];
        c.res = cfg.res;
        c.has_T_MW = 0;
        c.field = SE_GPU_FIELD_TSDF;
        c.res_type = SE_GPU_RES_SINGLE;
        c.storage = cfg.storage;
        c.truncation_boundary_factor = cfg.truncation_boundary_factor;
        c.max_weight = cfg.max_weight;
        c.max_blocks = cfg.max_blocks;
        check(se_gpu_map_create(&c, &h_), "se_gpu_map_create");
    }
    TSDFMap(const TSDFMap&) = delete;
    TSDFMap& operator=(const TSDFMap&) = delete;
    ~TSDFMap() { se_gpu_map_destroy(h_); }

    /** Octree::getSize() */
    int size() const
    {
        int s = 0;
        check(se_gpu_map_size(h_, &s, nullptr), "se_gpu_map_size");
        return s;
    }
    /** Synchronise and throw on a latched device-side failure (pool full, probe limit). */
    void check_errors() { check(se_gpu_map_check(h_), "se_gpu_map_check"); }
    int64_t num_blocks() const
    {
        int64_t n = 0;
        check(se_gpu_map_download_blocks(h_, 0, nullptr, nullptr, nullptr, nullptr, nullptr, &n), "download");
        return n;
    }
    se_gpu_map* handle() const { return h_; }

  private:
    se_gpu_map* h_ = nullptr;
};

/** se::Measurement<PinholeCamera, float>: a depth image, its sensor and T_WC. */
struct Measurement {
    DeviceImage<const float> image;
    const PinholeCamera& sensor;
    Pose T_WC;
};

class MapIntegrator {
  public:
    explicit MapIntegrator(TSDFMap& map) : map_(map) {}
    void integrateDepth(int timestamp, const Measurement& m, void* stream = nullptr)
    {
        check(se_gpu_integrate_depth(map_.handle(), m.image.data, &m.sensor.c, m.T_WC.data(), timestamp, stream),
              "se_gpu_integrate_depth");
    }

  private:
    TSDFMap& map_;
};

namespace raycaster {
inline void raycast_volume(const TSDFMap& map, const PinholeCamera& sensor, const Pose& T_WS,
                           DeviceImage<float> surface_point_cloud_W, DeviceImage<float> surface_normals_W,
                           DeviceImage<int8_t> surface_scale, void* stream = nullptr)
{
    check(se_gpu_raycast(map.handle(), &sensor.c, T_WS.data(), surface_point_cloud_W.data, surface_normals_W.data,
                         surface_scale.data, stream),
          "se_gpu_raycast");
}
} // namespace raycaster

/** se::TrackerConfig defaults (include/se/tracker/tracker.hpp:22-33). */
struct TrackerConfig {
    std::vector<int> iterations{10, 5, 4};
    float dist_threshold = 0.1f;
    float normal_threshold = 0.8f;
    float track_threshold = 0.15f;
    float icp_threshold = 0.00001f;
};

class Tracker {
  public:
    Tracker(TSDFMap& map, const PinholeCamera& sensor, const TrackerConfig& config = TrackerConfig())
        : map_(map), sensor_(sensor)
    {
        se_gpu_tracker_config c{};
        c.num_levels = (int) config.iterations.size();
        for (int i = 0; i < c.num_levels && i < 3; ++i)
            c.iterations[i] = config.iterations[i];
        c.dist_threshold = config.dist_threshold;
        c.normal_threshold = config.normal_threshold;
        c.track_threshold = config.track_threshold;
        c.icp_threshold = config.icp_threshold;
        check(se_gpu_tracker_create(&sensor.c, &c, &h_), "se_gpu_tracker_create");
    }
    Tracker(const Tracker&) = delete;
    Tracker& operator=(const Tracker&) = delete;
    ~Tracker() { se_gpu_tracker_destroy(h_); }

    /** Track depth against the raycast taken at T_WS; T_WS is updated (kept on failure). */
    bool track(DeviceImage<const float> depth, Pose& T_WS, DeviceImage<float> surface_point_cloud_W,
               DeviceImage<float> surface_normals_W, void* stream = nullptr)
    {
        int accepted = 0;
        check(se_gpu_track(h_, depth.data, surface_point_cloud_W.data, surface_normals_W.data, T_WS.data(), &accepted,
                           stream),
              "se_gpu_track");
        return accepted != 0;
    }

  private:
    TSDFMap& map_;
    const PinholeCamera& sensor_;
    se_gpu_tracker* h_ = nullptr;
};

} // namespace gpu
} // namespace se

#endif // SE_GPU_HPP
