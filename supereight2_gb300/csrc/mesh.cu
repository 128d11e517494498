// mesh.cu — se::algorithms::marching_cube (include/se/map/algorithms/impl/marching_cube_impl.hpp)
// with the isosurface::occupied case index (:25-41):
//  - single-res TSDF maps: marching_cube_kernel (:830-890);
//  - multi-res TSDF and occupancy maps: dual_marching_cube_kernel (:895-975), meshing the dual
//    grid of each block at its integration scale (gather_dual_data :269-289, :683-758).
//
// The case table is the reference's (edge_tables.hpp, triTable), in the encoding of
// mc_case_table.inc (generated from the reference's sources by make_mc_table.py): per case the
// face count and the cube edges of the faces in triTable's order. Corners in the order of
// meshing::gather_data: c0 (0,0,0), c1 (1,0,0), c2 (1,0,1), c3 (0,0,1), c4 (0,1,0), c5 (1,1,0),
// c6 (1,1,1), c7 (0,1,1); edges as edge_to_corners (:96-127); case bit i = corner i inside
// (tsdf < 0, or occupancy * weight > 0).
// Vertex positions follow meshing::compute_intersection / compute_dual_intersection exactly.
//
// Single-res: one thread per cube: the 8 corner values (one block or the dense block index), the
// case, up to 5 faces with checkVertex, written through one atomic per warp. Dual: one thread per
// primal corner of a block's dual grid ((8 / stride + 1)^3 per block, 768 thread slots per block).
#include <algorithm>
#include <cstring>
#include <mutex>

#include "multires.cuh"
#include "occupancy.cuh"
#include "pipeline.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {

namespace {

constexpr int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}};
constexpr int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {0, 3}, {4, 5}, {5, 6}, {6, 7}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
constexpr int kMaxTri = 5;

struct CaseTable {
    signed char ntri[256];
    signed char tri[256][3 * kMaxTri];
};

#include "mc_case_table.inc"

// Decodes the case table; false if a case had more than kMaxTri faces.
bool build_case_table(CaseTable& T)
{
    std::memset(&T, 0, sizeof(T));
    for (int cfg = 0; cfg < 256; ++cfg) {
        const unsigned long long w = kMcCaseWords[cfg];
        const int nt = (int) (w >> 60);
        if (nt > kMaxTri)
            return false;
        T.ntri[cfg] = (signed char) nt;
        for (int k = 0; k < 3 * nt; ++k)
            T.tri[cfg][k] = (signed char) ((w >> (4 * k)) & 0xf);
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

// Writes each thread's nf faces (and their scale) through one atomic per warp.
__device__ __forceinline__ void emit_faces(const float (*faces)[9], int nf, int scale, float* __restrict__ out,
                                           int8_t* __restrict__ out_scale, long long capacity,
                                           unsigned long long* count)
{
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
        if ((long long) slot < capacity) {
            if (out)
#pragma unroll
                for (int k = 0; k < 9; ++k)
                    out[slot * 9 + k] = faces[i][k];
            if (out_scale)
                out_scale[slot] = (int8_t) scale;
        }
    }
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
    emit_faces(faces, nf, 0, out, nullptr, capacity, count);
}

// ------------------------------------------------------------ dual marching cubes --
// A block store seen by the dual kernel: BlockT::data(voxel, scale) as (get_field, is_valid),
// fetcher::block, the block's current scale and coordinate.
template <int S>
struct MrTsdfStore {
    MapDevice m;
    __device__ int size() const { return m.size; }
    __device__ bool live(int) const { return true; }
    __device__ const int* coord(int b) const { return m.block_coord + 3 * (size_t) b; }
    __device__ int current_scale(int b) const { return (int) m.block_scale[2 * (size_t) b]; }
    __device__ int block_at(int x, int y, int z) const { return mr_block_of(m, x, y, z); }
    // BlockMultiRes<TSDF>::data(voxel, scale) (block_impl.hpp:164-170): the pyramid at any scale;
    // valid = weight != 0 (data_field_impl.hpp:32-35), field = tsdf
    __device__ bool data(int b, int x, int y, int z, int s, float& f) const
    {
        float w;
        mr_load_data<S>(m, b, mr_index(x & 7, y & 7, z & 7, s), f, w);
        return w != 0.0f;
    }
    __device__ static bool inside(float f) { return f < 0.0f; }
};

struct OccStore {
    OccDevice m;
    __device__ int size() const { return m.size; }
    __device__ bool live(int b) const { return m.block_state[b].live != 0; }
    __device__ const int* coord(int b) const { return m.block_coord + 3 * (size_t) b; }
    __device__ int current_scale(int b) const { return m.block_state[b].current_scale; }
    // fetcher::block (fetcher_impl.hpp:107-126) by descent from the root
    __device__ int block_at(int x, int y, int z) const
    {
        int n = 0;
        for (int cs = m.size >> 1; cs >= 8; cs >>= 1) {
            const int idx = ((x & cs) > 0) + 2 * ((y & cs) > 0) + 4 * ((z & cs) > 0);
            const int ch = m.node_child[8 * (size_t) n + idx];
            if (ch == -1)
                return -1;
            if (slot_is_block(ch))
                return slot_block(ch);
            n = ch;
        }
        return -1;
    }
    // BlockMultiRes<Occupancy>::data(voxel, scale) (block_impl.hpp:326-340): the init data
    // below the finest allocated scale; field = occupancy * weight, valid = weight != 0
    __device__ bool data(int b, int x, int y, int z, int s, float& f) const
    {
        const OccBlockState& st = m.block_state[b];
        const OccD d = s < st.finest ? st.init_data : blk_mean(m, b, s)[occ_voxel_idx(x & 7, y & 7, z & 7, s)];
        f = occ_field(d);
        return occ_valid(d);
    }
    __device__ static bool inside(float f) { return f > 0.0f; }
};

constexpr int kDualSlots = 768; // >= 9^3 primal corners of a block at scale 0

// algorithms::dual_marching_cube_kernel (marching_cube_impl.hpp:895-975). Thread slot k of block
// b takes the primal corner (x, y, z) = coord + stride (kx, ky, kz) of the block's dual grid at
// voxel_scale = clamp(min_desired_scale, current_scale, 3). Inside the block (no coordinate a
// multiple of 8) the 8 dual corners are p + (stride / 2) N_i at voxel_scale; on a block face,
// edge or corner, the dual corner i = p + L_i (L_i = c_i - 1) lies in the block offset by -1
// along an axis where p is on the lower face and L_i = -1, by +1 where p is on the upper face and
// L_i = 0. A neighbouring block ranks above the meshed one iff the first non-zero component of
// its offset (x, then y, then z) is +1 (the order norm_dual_corner_idxs tabulates, :311-680); a
// block ranking below must integrate at a strictly coarser scale, one ranking above at the same
// or a coarser scale, else the cell has no faces. Corners in a neighbour are read at
// max(its current scale, voxel_scale) at ((d / s) s + s / 2).
template <class Store>
__global__ void __launch_bounds__(256) dual_marching_cube_kernel(Store st, int n_blocks, int min_desired_scale,
                                                                 float* __restrict__ out, int8_t* __restrict__ out_scale,
                                                                 long long capacity, unsigned long long* count)
{
    const long long gid = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    const int blk = (int) (gid / kDualSlots), k = (int) (gid % kDualSlots);
    float faces[kMaxTri][9];
    int nf = 0;
    int voxel_scale = 0;
    if (blk < n_blocks && st.live(blk)) {
        const int cur = st.current_scale(blk);
        voxel_scale = min_desired_scale < cur ? cur : (min_desired_scale > 3 ? 3 : min_desired_scale);
        const int stride = 1 << voxel_scale;
        const int n = (8 >> voxel_scale) + 1;
        const int* bc = st.coord(blk);
        const int size = st.size();
        const int kx = k % n, ky = (k / n) % n, kz = k / (n * n);
        const int p[3] = {bc[0] + kx * stride, bc[1] + ky * stride, bc[2] + kz * stride};
        int last[3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
            last[a] = bc[a] + 8 < size - 1 ? bc[a] + 8 : size - 1;
        bool work = kz < n && p[0] <= last[0] && p[1] <= last[1] && p[2] <= last[2];
        if (work && (p[0] == last[0] || p[1] == last[1] || p[2] == last[2]))
            work = st.block_at(p[0], p[1], p[2]) >= 0;
        float val[8], pos[8][3];
        bool valid = work;
        if (work) {
            const int rel[3] = {p[0] - bc[0], p[1] - bc[1], p[2] - bc[2]};
            if (p[0] % 8 != 0 && p[1] % 8 != 0 && p[2] % 8 != 0) {
                const float h = (float) stride / 2;
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float nx = c_corner[i][0] ? 1.0f : -1.0f, ny = c_corner[i][1] ? 1.0f : -1.0f,
                                nz = c_corner[i][2] ? 1.0f : -1.0f;
                    pos[i][0] = (float) p[0] + h * nx;
                    pos[i][1] = (float) p[1] + h * ny;
                    pos[i][2] = (float) p[2] + h * nz;
                    valid = st.data(blk, (int) pos[i][0], (int) pos[i][1], (int) pos[i][2], voxel_scale, val[i]) && valid;
                }
            }
            else {
                int nb_of[8], off_key[8];
#pragma unroll 1
                for (int i = 0; i < 8 && valid; ++i) {
                    int off[3], c[3];
                    bool in_map = true;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const int ca = c_corner[i][a];
                        off[a] = (rel[a] == 0 && ca == 0) ? -1 : ((rel[a] == 8 && ca == 1) ? 1 : 0);
                        c[a] = p[a] + ca - 1;
                        in_map = in_map && c[a] >= 0 && c[a] < size;
                    }
                    off_key[i] = 9 * (off[0] + 1) + 3 * (off[1] + 1) + (off[2] + 1);
                    int nb = -2;
                    if (off_key[i] == 13) {
                        nb = blk;
                    }
                    else {
                        for (int j = 0; j < i; ++j)
                            if (off_key[j] == off_key[i])
                                nb = nb_of[j];
                        if (nb == -2) {
                            nb = in_map ? st.block_at(c[0], c[1], c[2]) : -1;
                            if (nb >= 0) {
                                const int lead = off[0] != 0 ? off[0] : (off[1] != 0 ? off[1] : off[2]);
                                const int ns = st.current_scale(nb);
                                if (lead > 0 ? ns < cur : ns <= cur)
                                    nb = -1;
                            }
                        }
                    }
                    nb_of[i] = nb;
                    if (nb < 0) {
                        valid = false;
                        break;
                    }
                    int gs = voxel_scale;
                    if (nb != blk) {
                        const int ns = st.current_scale(nb);
                        gs = ns > voxel_scale ? ns : voxel_scale;
                    }
                    const int s = 1 << gs;
                    int q[3];
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        pos[i][a] = (float) ((c[a] / s) * s) + (float) s * 0.5f;
                        q[a] = (int) pos[i][a];
                    }
                    valid = st.data(nb, q[0], q[1], q[2], gs, val[i]) && valid;
                }
            }
        }
        if (valid) {
            int cfg = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i)
                cfg |= (Store::inside(val[i]) ? 1 : 0) << i;
            const int nt = c_case_table.ntri[cfg];
            const float lim = (float) size;
            for (int t = 0; t < nt; ++t) {
                bool keep = true;
                float f[9];
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const int e = c_case_table.tri[cfg][3 * t + j];
                    const int a = c_edge[e][0], b = c_edge[e][1];
                    // compute_dual_intersection (marching_cube_impl.hpp:208-219)
                    const float sf = (0.0f - val[a]) / (val[b] - val[a]);
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        const float v = pos[a][q] + sf * (pos[b][q] - pos[a][q]);
                        keep = keep && !(v <= 0.0f || v > lim); // checkVertex (:814-818)
                        f[3 * j + q] = v;
                    }
                }
                if (keep) {
#pragma unroll
                    for (int q = 0; q < 9; ++q)
                        faces[nf][q] = f[q];
                    ++nf;
                }
            }
        }
    }
    emit_faces(faces, nf, voxel_scale, out, out_scale, capacity, count);
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

se_gpu_status se_gpu_dual_marching_cube(se_gpu_map* map, int min_desired_scale, float* faces_dev, int8_t* scales_dev,
                                        int64_t capacity, int64_t* count, void* stream_p)
{
    if (!map || !count || capacity < 0 || min_desired_scale < 0 || min_desired_scale > 3) {
        set_last_error("se_gpu_dual_marching_cube: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (!map->occ && map->dev.res_type != SE_GPU_RES_MULTI) {
        set_last_error("se_gpu_dual_marching_cube: multi-res TSDF or occupancy maps only");
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    se_gpu_status st = upload_case_table();
    if (st != SE_GPU_OK)
        return st;
    cudaStream_t stream = (cudaStream_t) stream_p;
    int nb = 0;
    if (map->occ) {
        SE_CUDA_TRY(cudaMemcpyAsync(&nb, map->occ->dev.counters + kOccBlocks, sizeof(int), cudaMemcpyDeviceToHost, stream));
    }
    else {
        SE_CUDA_TRY(cudaMemcpyAsync(&nb, map->dev.counters + kCntNumBlocks, sizeof(int), cudaMemcpyDeviceToHost, stream));
    }
    unsigned long long* d_count = nullptr;
    SE_CUDA_TRY(cudaMallocAsync(&d_count, sizeof(unsigned long long), stream));
    SE_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), stream));
    SE_CUDA_TRY(cudaStreamSynchronize(stream));
    const int cap_blocks = map->occ ? map->occ->dev.block_capacity : map->dev.capacity;
    nb = nb < cap_blocks ? nb : cap_blocks;
    float* out = capacity > 0 ? faces_dev : nullptr;
    int8_t* out_s = capacity > 0 ? scales_dev : nullptr;
    if (nb > 0) {
        const long long threads = (long long) nb * kDualSlots;
        const unsigned grid = (unsigned) ((threads + 255) / 256);
        if (map->occ)
            dual_marching_cube_kernel<<<grid, 256, 0, stream>>>(OccStore{map->occ->dev}, nb, min_desired_scale, out,
                                                                out_s, capacity, d_count);
        else if (map->dev.storage == SE_GPU_STORAGE_F32)
            dual_marching_cube_kernel<<<grid, 256, 0, stream>>>(MrTsdfStore<SE_GPU_STORAGE_F32>{map->dev}, nb,
                                                                min_desired_scale, out, out_s, capacity, d_count);
        else
            dual_marching_cube_kernel<<<grid, 256, 0, stream>>>(MrTsdfStore<SE_GPU_STORAGE_F16>{map->dev}, nb,
                                                                min_desired_scale, out, out_s, capacity, d_count);
        SE_CUDA_TRY(cudaGetLastError());
    }
    unsigned long long n = 0;
    SE_CUDA_TRY(cudaMemcpyAsync(&n, d_count, sizeof(n), cudaMemcpyDeviceToHost, stream));
    SE_CUDA_TRY(cudaFreeAsync(d_count, stream));
    SE_CUDA_TRY(cudaStreamSynchronize(stream));
    *count = (int64_t) n;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_marching_cube(se_gpu_map* map, float* faces_dev, int64_t capacity, int64_t* count, void* stream_p)
{
    if (!map || !count || capacity < 0 || (capacity > 0 && !faces_dev)) {
        set_last_error("se_gpu_marching_cube: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (map->occ || map->dev.res_type == SE_GPU_RES_MULTI)
        return se_gpu_dual_marching_cube(map, 0, faces_dev, nullptr, capacity, count, stream_p);
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
