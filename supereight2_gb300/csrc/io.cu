// io.cu — the map's on-disk outputs (include/se/map/io/*): triangle meshes as PLY, VTK polydata
// or OBJ (io::save_mesh, mesh_io_impl.hpp), point clouds as VTK polydata (io::save_point_cloud_vtk,
// point_cloud_io_impl.hpp) and axis-aligned field slices as VTK rectilinear grids
// (Map::saveFieldSlices, map_impl.hpp:273-320 with io::save_3d_slice_vtk, octree_io_impl.hpp).
// The formats are the standard ASCII ones the reference writes, so its files and these open in
// the same viewers; the writers are this library's own host code. Slices are gathered on the
// GPU (one thread per voxel of the slice through the dense block index).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pipeline.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

namespace {

bool ends_with(const std::string& s, const char* suffix)
{
    const size_t n = std::strlen(suffix);
    return s.size() >= n && s.compare(s.size() - n, n, suffix) == 0;
}

// T (row-major 4x4 affine) applied to a point
void apply16(const float* T, const float* p, float* q)
{
    for (int r = 0; r < 3; ++r)
        q[r] = ((T[4 * r] * p[0] + T[4 * r + 1] * p[1]) + T[4 * r + 2] * p[2]) + T[4 * r + 3];
}

struct File {
    FILE* f;
    explicit File(const char* path) : f(std::fopen(path, "w")) {}
    ~File()
    {
        if (f)
            std::fclose(f);
    }
};

// A face colour per integration scale (single-res meshes are all scale 0; io::save_mesh colours
// faces by scale_colour(face.scale), mesh_io_impl.hpp).
void scale_rgb(int scale, int rgb[3])
{
    static const int palette[8][3] = {{102, 194, 165}, {252, 141, 98}, {141, 160, 203}, {231, 138, 195},
                                      {166, 216, 84},  {255, 217, 47}, {229, 196, 148}, {179, 179, 179}};
    const int* c = palette[scale < 0 ? 7 : (scale > 7 ? 7 : scale)];
    rgb[0] = c[0];
    rgb[1] = c[1];
    rgb[2] = c[2];
}

// io::has_supported_mesh_extension (src/map/io/mesh_io.cpp:13-21): .ply, .vtk, .obj
bool supported_mesh_extension(const std::string& path)
{
    return ends_with(path, ".ply") || ends_with(path, ".vtk") || ends_with(path, ".obj");
}

se_gpu_status write_mesh(const float* faces, const int8_t* scales, int64_t n, const float* T, const std::string& path)
{
    // an unsupported name is refused before any file is created
    if (!supported_mesh_extension(path)) {
        set_last_error("unknown mesh file extension (.ply, .vtk or .obj): %s", path.c_str());
        return SE_GPU_ERR_BAD_ARG;
    }
    File out(path.c_str());
    if (!out.f) {
        set_last_error("cannot write %s", path.c_str());
        return SE_GPU_ERR_BAD_ARG;
    }
    FILE* f = out.f;
    std::vector<float> v((size_t) n * 9);
    for (int64_t i = 0; i < 3 * n; ++i)
        apply16(T, faces + 3 * i, v.data() + 3 * i);
    const auto face_scale = [scales](int64_t i) { return scales ? (int) scales[i] : 0; };
    int rgb[3];
    if (ends_with(path, ".ply")) {
        std::fprintf(f, "ply\nformat ascii 1.0\ncomment supereight2_gb300 mesh\n");
        std::fprintf(f, "element vertex %lld\nproperty float x\nproperty float y\nproperty float z\n", (long long) (3 * n));
        std::fprintf(f, "element face %lld\nproperty list uchar int vertex_index\n", (long long) n);
        std::fprintf(f, "property uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n");
        for (int64_t i = 0; i < 3 * n; ++i)
            std::fprintf(f, "%.9g %.9g %.9g\n", v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        for (int64_t i = 0; i < n; ++i) {
            scale_rgb(face_scale(i), rgb);
            std::fprintf(f, "3 %lld %lld %lld %d %d %d\n", (long long) (3 * i), (long long) (3 * i + 1),
                         (long long) (3 * i + 2), rgb[0], rgb[1], rgb[2]);
        }
    }
    else if (ends_with(path, ".vtk")) {
        std::fprintf(f, "# vtk DataFile Version 3.0\nsupereight2_gb300 mesh\nASCII\nDATASET POLYDATA\n\n");
        std::fprintf(f, "POINTS %lld float\n", (long long) (3 * n));
        for (int64_t i = 0; i < 3 * n; ++i)
            std::fprintf(f, "%.9g %.9g %.9g\n", v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        std::fprintf(f, "\nPOLYGONS %lld %lld\n", (long long) n, (long long) (4 * n));
        for (int64_t i = 0; i < n; ++i)
            std::fprintf(f, "3 %lld %lld %lld\n", (long long) (3 * i), (long long) (3 * i + 1), (long long) (3 * i + 2));
        std::fprintf(f, "\nCELL_DATA %lld\nSCALARS scale unsigned_char\nLOOKUP_TABLE default\n", (long long) n);
        for (int64_t i = 0; i < n; ++i)
            std::fprintf(f, "%d\n", face_scale(i));
        std::fprintf(f, "COLOR_SCALARS scale_colour 3\n");
        for (int64_t i = 0; i < n; ++i) {
            scale_rgb(face_scale(i), rgb);
            std::fprintf(f, "%.9g %.9g %.9g\n", rgb[0] / 255.0f, rgb[1] / 255.0f, rgb[2] / 255.0f);
        }
    }
    else if (ends_with(path, ".obj")) {
        std::fprintf(f, "# supereight2_gb300 mesh\n");
        for (int64_t i = 0; i < 3 * n; ++i)
            std::fprintf(f, "v %.9g %.9g %.9g\n", v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        for (int64_t i = 0; i < n; ++i)
            std::fprintf(f, "f %lld %lld %lld\n", (long long) (3 * i + 1), (long long) (3 * i + 2), (long long) (3 * i + 3));
    }
    else {
        set_last_error("unknown mesh file extension (.ply, .vtk or .obj): %s", path.c_str());
        return SE_GPU_ERR_BAD_ARG;
    }
    return std::ferror(f) ? (set_last_error("write error on %s", path.c_str()), SE_GPU_ERR_BAD_ARG) : SE_GPU_OK;
}

} // namespace

// get_field(getData(coord)) over a box [lo, hi) of voxel coordinates, x fastest
template <int S>
__global__ void field_box_kernel(MapDevice m, int3 lo, int3 dim, float* __restrict__ out)
{
    const long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long) dim.x * dim.y * dim.z;
    if (i >= n)
        return;
    const int x = lo.x + (int) (i % dim.x), y = lo.y + (int) ((i / dim.x) % dim.y), z = lo.z + (int) (i / ((long long) dim.x * dim.y));
    float t = 1.0f, w = 0.0f;
    const int b = m.block_index[((size_t) (z >> 3) << (2 * m.log2_bps)) | ((size_t) (y >> 3) << m.log2_bps) | (size_t) (x >> 3)];
    if (b >= 0)
        load_voxel<S>(m, b, (x & 7) + 8 * (y & 7) + 64 * (z & 7), t, w);
    out[i] = t;
}

} // namespace se_gpu

using namespace se_gpu;

extern "C" {

se_gpu_status se_gpu_save_mesh(const float* faces, const int8_t* scales, int64_t n, const float T_OV[16],
                               const char* filename)
{
    if ((!faces && n > 0) || n < 0 || !T_OV || !filename) {
        set_last_error("se_gpu_save_mesh: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    return write_mesh(faces, scales, n, T_OV, filename);
}

se_gpu_status se_gpu_map_mesh_transform(const se_gpu_map* map, const float T_OW[16], float T_OV[16])
{
    if (!map || !T_OW || !T_OV) {
        set_last_error("se_gpu_map_mesh_transform: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    // T_OV = T_OW * T_WM * Scaling(res) (map_impl.hpp:457)
    const Tf& W = map->dev.T_WM; // occupancy maps keep their geometry here too
    const float res = map->dev.res;
    float A[16];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c)
            A[4 * r + c] = W.R[3 * r + c] * res;
        A[4 * r + 3] = W.t[r];
    }
    A[12] = A[13] = A[14] = 0.0f;
    A[15] = 1.0f;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c)
            T_OV[4 * r + c] = ((T_OW[4 * r] * A[c] + T_OW[4 * r + 1] * A[4 + c]) + T_OW[4 * r + 2] * A[8 + c])
                + T_OW[4 * r + 3] * A[12 + c];
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_save_mesh(se_gpu_map* map, const float T_OW[16], int min_desired_scale, const char* filename,
                                   void* stream)
{
    if (!map || !T_OW || !filename) {
        set_last_error("se_gpu_map_save_mesh: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    const bool dual = map->occ || map->dev.res_type == SE_GPU_RES_MULTI;
    const auto extract = [&](float* f, int8_t* sc, int64_t cap, int64_t* cnt) {
        return dual ? se_gpu_dual_marching_cube(map, min_desired_scale, f, sc, cap, cnt, stream)
                    : se_gpu_marching_cube(map, f, cap, cnt, stream);
    };
    int64_t n = 0;
    se_gpu_status st = extract(nullptr, nullptr, 0, &n);
    if (st != SE_GPU_OK)
        return st;
    std::vector<float> h((size_t) n * 9);
    std::vector<int8_t> hs(dual ? (size_t) n : 0);
    if (n > 0) {
        float* d = nullptr;
        int8_t* ds = nullptr;
        SE_CUDA_TRY(cudaMalloc(&d, (size_t) n * 9 * sizeof(float) + (size_t) n));
        ds = reinterpret_cast<int8_t*>(d + (size_t) n * 9);
        int64_t n2 = 0;
        st = extract(d, dual ? ds : nullptr, n, &n2);
        if (st == SE_GPU_OK && (cudaMemcpy(h.data(), d, h.size() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess
                                || (dual && cudaMemcpy(hs.data(), ds, hs.size(), cudaMemcpyDeviceToHost) != cudaSuccess)))
            st = cuda_status(cudaGetLastError(), "cudaMemcpy(mesh)");
        cudaFree(d);
        if (st != SE_GPU_OK)
            return st;
    }
    float T_OV[16];
    se_gpu_map_mesh_transform(map, T_OW, T_OV);
    return write_mesh(h.data(), dual ? hs.data() : nullptr, n, T_OV, filename);
}

se_gpu_status se_gpu_save_point_cloud_vtk(const float* points, int64_t n, const float T_WC[16], const char* filename)
{
    if ((!points && n > 0) || n < 0 || !T_WC || !filename) {
        set_last_error("se_gpu_save_point_cloud_vtk: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    File out(filename);
    if (!out.f) {
        set_last_error("cannot write %s", filename);
        return SE_GPU_ERR_BAD_ARG;
    }
    std::fprintf(out.f, "# vtk DataFile Version 1.0\nsupereight2_gb300 point cloud\nASCII\nDATASET POLYDATA\n");
    std::fprintf(out.f, "POINTS %lld FLOAT\n", (long long) n);
    for (int64_t i = 0; i < n; ++i) {
        float q[3];
        apply16(T_WC, points + 3 * i, q);
        std::fprintf(out.f, "%.9g %.9g %.9g\n", q[0], q[1], q[2]);
    }
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_field_box(const se_gpu_map* map, const int32_t lo[3], const int32_t hi[3], float* out_host)
{
    if (!map || !lo || !hi || !out_host || map->occ || map->dev.res_type == SE_GPU_RES_MULTI) {
        set_last_error("se_gpu_map_field_box: invalid argument (single-res TSDF maps)");
        return SE_GPU_ERR_BAD_ARG;
    }
    const MapDevice& m = map->dev;
    for (int a = 0; a < 3; ++a)
        if (lo[a] < 0 || hi[a] > m.size || hi[a] <= lo[a]) {
            set_last_error("se_gpu_map_field_box: box outside the map");
            return SE_GPU_ERR_BAD_ARG;
        }
    const int3 l = make_int3(lo[0], lo[1], lo[2]);
    const int3 dim = make_int3(hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]);
    const long long n = (long long) dim.x * dim.y * dim.z;
    SE_CUDA_TRY(cudaStreamSynchronize(map->last_stream));
    float* d = nullptr;
    SE_CUDA_TRY(cudaMalloc(&d, (size_t) n * sizeof(float)));
    const unsigned grid = (unsigned) ((n + 255) / 256);
    if (m.storage == SE_GPU_STORAGE_F32)
        field_box_kernel<SE_GPU_STORAGE_F32><<<grid, 256>>>(m, l, dim, d);
    else
        field_box_kernel<SE_GPU_STORAGE_F16><<<grid, 256>>>(m, l, dim, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpy(out_host, d, (size_t) n * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess)
        return cuda_status(e, "se_gpu_map_field_box");
    return SE_GPU_OK;
}

se_gpu_status se_gpu_map_save_field_slices(const se_gpu_map* map, const char* filename_x, const char* filename_y,
                                           const char* filename_z, const float point_W[3])
{
    if (!map || !point_W || map->occ || map->dev.res_type == SE_GPU_RES_MULTI) {
        set_last_error("se_gpu_map_save_field_slices: invalid argument (single-res TSDF maps)");
        return SE_GPU_ERR_BAD_ARG;
    }
    const MapDevice& m = map->dev;
    int v[3];
    // pointToVoxel (map_impl.hpp:538-550); a point outside the map gives the slices at -1, empty
    if (!point_to_voxel(m, f3(point_W[0], point_W[1], point_W[2]), v[0], v[1], v[2])) {
        set_last_error("se_gpu_map_save_field_slices: the point is outside the map");
        return SE_GPU_ERR_BAD_ARG;
    }
    const char* names[3] = {filename_x, filename_y, filename_z};
    for (int axis = 0; axis < 3; ++axis) {
        if (!names[axis] || !names[axis][0])
            continue;
        int32_t lo[3] = {0, 0, 0}, hi[3] = {m.size, m.size, m.size};
        lo[axis] = v[axis];
        hi[axis] = v[axis] + 1;
        std::vector<float> vals((size_t) (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]));
        se_gpu_status st = se_gpu_map_field_box(map, lo, hi, vals.data());
        if (st != SE_GPU_OK)
            return st;
        File out(names[axis]);
        if (!out.f) {
            set_last_error("cannot write %s", names[axis]);
            return SE_GPU_ERR_BAD_ARG;
        }
        FILE* f = out.f;
        std::fprintf(f, "# vtk DataFile Version 1.0\nsupereight2_gb300 field slice\nASCII\nDATASET RECTILINEAR_GRID\n");
        std::fprintf(f, "DIMENSIONS %d %d %d\n", hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]);
        const char* axis_names[3] = {"X", "Y", "Z"};
        for (int a = 0; a < 3; ++a) {
            std::fprintf(f, "%s_COORDINATES %d int\n", axis_names[a], hi[a] - lo[a]);
            for (int c = lo[a]; c < hi[a]; ++c)
                std::fprintf(f, "%d ", c);
            std::fprintf(f, "\n");
        }
        std::fprintf(f, "POINT_DATA %zu\nSCALARS scalars float 1\nLOOKUP_TABLE default\n", vals.size());
        for (float x : vals)
            std::fprintf(f, "%.9g\n", x);
    }
    return SE_GPU_OK;
}

} // extern "C"
