// mesh.cu — se::algorithms::marching_cube for single-res TSDF maps
// (include/se/map/algorithms/impl/marching_cube_impl.hpp:830-890, 1175-1201) with the
// isosurface::occupied case index (:25-41).
//
// The reference triangulates each cube with a third-party case table (edge_tables.hpp). This
// library builds its case table on the host from a stated rule instead:
//  - corners in the order of meshing::gather_data: c0 (0,0,0), c1 (1,0,0), c2 (1,0,1),
//    c3 (0,0,1), c4 (0,1,0), c5 (1,1,0), c6 (1,1,1), c7 (0,1,1); edges as edge_to_corners
//    (:96-127); case bit i = corner i inside (tsdf < 0);
//  - on each cube face the crossed edges are joined into segments; a face with four crossed
//    edges (inside corners on a diagonal) gets the two segments that cut off its inside corners
//    (a neighbouring cube sees the same face and makes the same choice: the mesh is closed);
//  - the segments close into loops; a loop is walked from its lowest edge towards the lower of
//    that edge's two neighbours, reversed when its Newell normal points from outside corners to
//    inside ones (faces point away from the inside), and fanned from its first edge.
// Vertex positions follow meshing::compute_intersection exactly; only the triangulation of a
// crossing pattern can differ from the reference's table.
//
// One thread per cube: the 8 corner values (one block or the dense block index), the case, up
// to 5 faces with checkVertex, written through one atomic per warp.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "pipeline.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

namespace {

constexpr int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}};
constexpr int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {0, 3}, {4, 5}, {5, 6}, {6, 7}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
constexpr int kFace[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}, {0, 1, 5, 4}, {3, 2, 6, 7}};
constexpr int kMaxTri = 5;

struct CaseTable {
    signed char ntri[256];
    signed char tri[256][3 * kMaxTri];
};

int edge_between(int a, int b)
{
    for (int e = 0; e < 12; ++e)
        if ((kEdge[e][0] == a && kEdge[e][1] == b) || (kEdge[e][0] == b && kEdge[e][1] == a))
            return e;
    return -1;
}

// Builds the triangulation of every case; false if a case needs more than kMaxTri faces.
bool build_case_table(CaseTable& T)
{
    std::memset(&T, 0, sizeof(T));
    for (int cfg = 0; cfg < 256; ++cfg) {
        const auto inside = [cfg](int c) { return ((cfg >> c) & 1) != 0; };
        int adj[12][2], deg[12] = {0};
        const auto join = [&](int ea, int eb) {
            adj[ea][deg[ea]++] = eb;
            adj[eb][deg[eb]++] = ea;
        };
        for (const auto& f : kFace) {
            int cross[4], nc = 0;
            for (int k = 0; k < 4; ++k)
                if (inside(f[k]) != inside(f[(k + 1) % 4]))
                    cross[nc++] = edge_between(f[k], f[(k + 1) % 4]);
            if (nc == 2) {
                join(cross[0], cross[1]);
            }
            else if (nc == 4) {
                for (int k = 0; k < 4; ++k)
                    if (inside(f[k])) // the edges before and after an inside corner
                        join(edge_between(f[(k + 3) % 4], f[k]), edge_between(f[k], f[(k + 1) % 4]));
            }
        }
        bool seen[12] = {false};
        int nt = 0;
        for (int start = 0; start < 12; ++start) {
            if (!deg[start] || seen[start])
                continue;
            int loop[12], len = 0, prev = -1, cur = start;
            do {
                loop[len++] = cur;
                seen[cur] = true;
                const int next = prev < 0 ? std::min(adj[cur][0], adj[cur][1])
                                          : (adj[cur][0] == prev ? adj[cur][1] : adj[cur][0]);
                prev = cur;
                cur = next;
            } while (cur != start);
            double nrm[3] = {0.0, 0.0, 0.0}, dir[3] = {0.0, 0.0, 0.0};
            for (int i = 0; i < len; ++i) {
                const int e = loop[i], e2 = loop[(i + 1) % len];
                double a[3], b[3];
                for (int k = 0; k < 3; ++k) {
                    a[k] = 0.5 * (kCorner[kEdge[e][0]][k] + kCorner[kEdge[e][1]][k]);
                    b[k] = 0.5 * (kCorner[kEdge[e2][0]][k] + kCorner[kEdge[e2][1]][k]);
                }
                nrm[0] += (a[1] - b[1]) * (a[2] + b[2]);
                nrm[1] += (a[2] - b[2]) * (a[0] + b[0]);
                nrm[2] += (a[0] - b[0]) * (a[1] + b[1]);
                const int in_c = inside(kEdge[e][0]) ? kEdge[e][0] : kEdge[e][1];
                const int out_c = in_c == kEdge[e][0] ? kEdge[e][1] : kEdge[e][0];
                for (int k = 0; k < 3; ++k)
                    dir[k] += kCorner[out_c][k] - kCorner[in_c][k];
            }
            if (nrm[0] * dir[0] + nrm[1] * dir[1] + nrm[2] * dir[2] < 0.0)
                std::reverse(loop + 1, loop + len);
            for (int i = 1; i + 1 < len; ++i) {
                if (nt == kMaxTri)
                    return false;
                T.tri[cfg][3 * nt] = (signed char) loop[0];
                T.tri[cfg][3 * nt + 1] = (signed char) loop[i];
                T.tri[cfg][3 * nt + 2] = (signed char) loop[i + 1];
                ++nt;
            }
        }
        T.ntri[cfg] = (signed char) nt;
    }
    return true;
}

} // namespace

__constant__ CaseTable c_case_table;
__constant__ signed char c_edge[12][2];
__constant__ signed char c_corner[8][3];

// meshing::compute_intersection (marching_cube_impl.hpp:82-93) from the gathered corner values
__device__ __forceinline__ F3 mc_vertex(int x, int y, int z, int e, const float* val)
{
    const int a = c_edge[e][0], b = c_edge[e][1];
    const int ax = x + c_corner[a][0], ay = y + c_corner[a][1], az = z + c_corner[a][2];
    const int bx = x + c_corner[b][0], by = y + c_corner[b][1], bz = z + c_corner[b][2];
    const float v0 = val[a], v1 = val[b];
    const F3 p0 = f3((float) ax + 0.5f, (float) ay + 0.5f, (float) az + 0.5f);
    const F3 p1 = f3((float) bx + 0.5f, (float) by + 0.5f, (float) bz + 0.5f);
    const float s = (0.0f - v0) / (v1 - v0);
    return f3(p0.x + s * (p1.x - p0.x), p0.y + s * (p1.y - p0.y), p0.z + s * (p1.z - p0.z));
}

template <int S>
__global__ void __launch_bounds__(256) marching_cube_kernel(MapDevice m, int n_blocks, float* __restrict__ out,
                                                            long long capacity, unsigned long long* count)
{
    const long long gid = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    const int blk = (int) (gid >> 9), vi = (int) (gid & 511);
    float faces[kMaxTri][9];
    int nf = 0;
    if (blk < n_blocks) {
        const int lx = vi & 7, ly = (vi >> 3) & 7, lz = vi >> 6;
        const int x = m.block_coord[3 * blk] + lx, y = m.block_coord[3 * blk + 1] + ly, z = m.block_coord[3 * blk + 2] + lz;
        const int top = m.size - 1;
        // cubes [coord, min(coord + 8, size - 1)) per axis
        if (x < top && y < top && z < top) {
            float val[8];
            bool valid = true;
            if (lx < 7 && ly < 7 && lz < 7) {
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int cx = (k == 1 || k == 2 || k == 5 || k == 6) ? 1 : 0, cy = k >= 4 ? 1 : 0,
                              cz = (k == 2 || k == 3 || k == 6 || k == 7) ? 1 : 0;
                    float w;
                    load_voxel<S>(m, blk, vi + cx + 8 * cy + 64 * cz, val[k], w);
                    valid = valid && (w != 0.0f);
                }
            }
            else {
#pragma unroll 1
                for (int k = 0; k < 8; ++k) {
                    const int cx = (k == 1 || k == 2 || k == 5 || k == 6) ? 1 : 0, cy = k >= 4 ? 1 : 0,
                              cz = (k == 2 || k == 3 || k == 6 || k == 7) ? 1 : 0;
                    const int X = x + cx, Y = y + cy, Z = z + cz;
                    const int b = m.block_index[((size_t) (Z >> 3) << (2 * m.log2_bps))
                                                | ((size_t) (Y >> 3) << m.log2_bps) | (size_t) (X >> 3)];
                    float w = 0.0f;
                    val[k] = 1.0f;
                    if (b >= 0)
                        load_voxel<S>(m, b, (X & 7) + 8 * (Y & 7) + 64 * (Z & 7), val[k], w);
                    valid = valid && (w != 0.0f);
                }
            }
            int cfg = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                cfg |= (val[k] < 0.0f ? 1 : 0) << k;
            const int nt = valid ? c_case_table.ntri[cfg] : 0;
            const float lim = (float) m.size;
            for (int t = 0; t < nt; ++t) {
                bool keep = true;
                float f[9];
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const F3 v = mc_vertex(x, y, z, c_case_table.tri[cfg][3 * t + j], val);
                    // checkVertex (marching_cube_impl.hpp:814-818)
                    keep = keep && !(v.x <= 0.0f || v.y <= 0.0f || v.z <= 0.0f || v.x > lim || v.y > lim || v.z > lim);
                    f[3 * j] = v.x;
                    f[3 * j + 1] = v.y;
                    f[3 * j + 2] = v.z;
                }
                if (keep) {
#pragma unroll
                    for (int k = 0; k < 9; ++k)
                        faces[nf][k] = f[k];
                    ++nf;
                }
            }
        }
    }
    // one atomic per warp for the warp's faces
    const int lane = threadIdx.x & 31;
    int incl = nf;
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o)
            incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    unsigned long long base = 0;
    if (lane == 31 && total > 0)
        base = atomicAdd(count, (unsigned long long) total);
    base = __shfl_sync(0xffffffffu, base, 31);
    const unsigned long long first = base + (unsigned long long) (incl - nf);
    for (int i = 0; i < nf; ++i) {
        const unsigned long long slot = first + (unsigned long long) i;
        if ((long long) slot < capacity)
#pragma unroll
            for (int k = 0; k < 9; ++k)
                out[slot * 9 + k] = faces[i][k];
    }
}

static se_gpu_status upload_case_table()
{
    static std::mutex mu;
    static int done_device = -1;
    std::lock_guard<std::mutex> lock(mu);
    int dev = 0;
    SE_CUDA_TRY(cudaGetDevice(&dev));
    if (done_device == dev)
        return SE_GPU_OK;
    CaseTable T;
    if (!build_case_table(T)) {
        set_last_error("marching cubes: a case needs more than %d faces", kMaxTri);
        return SE_GPU_ERR_CUDA;
    }
    signed char e[12][2];
    for (int i = 0; i < 12; ++i) {
        e[i][0] = (signed char) kEdge[i][0];
        e[i][1] = (signed char) kEdge[i][1];
    }
    SE_CUDA_TRY(cudaMemcpyToSymbol(c_case_table, &T, sizeof(T)));
    SE_CUDA_TRY(cudaMemcpyToSymbol(c_edge, e, sizeof(e)));
    signed char c[8][3];
    for (int i = 0; i < 8; ++i)
        for (int k = 0; k < 3; ++k)
            c[i][k] = (signed char) kCorner[i][k];
    SE_CUDA_TRY(cudaMemcpyToSymbol(c_corner, c, sizeof(c)));
    done_device = dev;
    return SE_GPU_OK;
}

} // namespace se_gpu

using namespace se_gpu;

extern "C" {

se_gpu_status se_gpu_mc_case_table(int32_t ntri[256], int32_t tri[256 * 15])
{
    CaseTable T;
    if (!ntri || !tri || !build_case_table(T)) {
        set_last_error("se_gpu_mc_case_table: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    for (int c = 0; c < 256; ++c) {
        ntri[c] = T.ntri[c];
        for (int k = 0; k < 3 * kMaxTri; ++k)
            tri[15 * c + k] = k < 3 * T.ntri[c] ? T.tri[c][k] : -1;
    }
    return SE_GPU_OK;
}

se_gpu_status se_gpu_marching_cube(se_gpu_map* map, float* faces_dev, int64_t capacity, int64_t* count, void* stream_p)
{
    if (!map || !count || capacity < 0 || (capacity > 0 && !faces_dev)) {
        set_last_error("se_gpu_marching_cube: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (map->occ || map->dev.res_type == SE_GPU_RES_MULTI) {
        set_last_error("se_gpu_marching_cube: single-res TSDF maps only (multi-res maps use the reference's "
                       "dual marching cubes, not built)");
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    se_gpu_status st = upload_case_table();
    if (st != SE_GPU_OK)
        return st;
    const MapDevice& m = map->dev;
    cudaStream_t stream = (cudaStream_t) stream_p;
    int nb = 0;
    SE_CUDA_TRY(cudaMemcpyAsync(&nb, m.counters + kCntNumBlocks, sizeof(int), cudaMemcpyDeviceToHost, stream));
    unsigned long long* d_count = nullptr;
    SE_CUDA_TRY(cudaMallocAsync(&d_count, sizeof(unsigned long long), stream));
    SE_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), stream));
    SE_CUDA_TRY(cudaStreamSynchronize(stream));
    nb = nb < m.capacity ? nb : m.capacity;
    if (nb > 0) {
        const long long threads = (long long) nb * 512;
        const unsigned grid = (unsigned) ((threads + 255) / 256);
        if (m.storage == SE_GPU_STORAGE_F32)
            marching_cube_kernel<SE_GPU_STORAGE_F32><<<grid, 256, 0, stream>>>(m, nb, faces_dev, capacity, d_count);
        else
            marching_cube_kernel<SE_GPU_STORAGE_F16><<<grid, 256, 0, stream>>>(m, nb, faces_dev, capacity, d_count);
        SE_CUDA_TRY(cudaGetLastError());
    }
    unsigned long long n = 0;
    SE_CUDA_TRY(cudaMemcpyAsync(&n, d_count, sizeof(n), cudaMemcpyDeviceToHost, stream));
    SE_CUDA_TRY(cudaFreeAsync(d_count, stream));
    SE_CUDA_TRY(cudaStreamSynchronize(stream));
    *count = (int64_t) n;
    return SE_GPU_OK;
}

} // extern "C"
