/*
 * se_oracle_occ.cpp — CPU oracle for supereight2's multi-resolution occupancy (OFusion) maps.
 *
 * TEST INFRASTRUCTURE ONLY: the checker the GPU product is compared against. It is never linked
 * into or called by the product library.
 *
 * A restatement, with the reference's loop structure and float arithmetic, of (paths relative
 * to the supereight2 source tree):
 *   - depth uncertainty image          src/integrator/uncertainty.cpp:12-34
 *   - sigma / tau                      include/se/integrator/updater/impl/multires_ofusion_core_impl.hpp:17-40
 *   - DensePoolingImage<PinholeCamera> include/se/integrator/allocator/impl/dense_pooling_image_impl.hpp:56-347
 *   - VolumeCarver<.., PinholeCamera>  include/se/integrator/allocator/impl/volume_carver_impl.hpp:17-310
 *   - OFusion Updater                  include/se/integrator/updater/impl/multires_ofusion_updater_impl.hpp:18-606
 *   - voxel update / free / propagation include/se/integrator/updater/impl/multires_ofusion_core_impl.hpp:46-276
 *   - FieldData<Occupancy>::update     include/se/map/impl/data_field_impl.hpp:19-28
 *   - up_prop_mean / min / max         include/se/map/impl/data_impl.hpp:52-152
 *   - BlockMultiRes<Occupancy>         include/se/map/octant/impl/block_impl.hpp:206-855
 *   - Octree::allocateChildren / deleteChildren  include/se/map/octree/impl/octree_impl.hpp:200-255
 *
 * The octree is the reference's pointer octree with index-addressed nodes and blocks. A block's
 * voxel pyramid keeps the reference's storage semantics: mean data exists from the finest
 * allocated scale up; min / max data are separate arrays above the finest scale and alias the
 * mean data at it; the integration buffer is its own array when finer than the current scale
 * and aliases the mean data otherwise. Every order-dependent step (scale buffers, propagation,
 * pruning) runs per block or per node in the reference's order; the only parallel loops are over
 * independent blocks.
 */
#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <set>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_common.hpp"
#include "oracle_dual_mc.hpp"

namespace {

/* ------------------------------------------------------------------- occupancy data -- */

struct OccData {
    float occ = 0.0f;
    float weight = 0.0f;
    bool observed = false;
};

static inline bool occ_valid(const OccData& d) { return d.weight != 0.0f; }
static inline float occ_field(const OccData& d) { return d.occ * d.weight; }

/* FieldData<Occupancy>::update, data_field_impl.hpp:19-28 */
static inline void occ_update(OccData& d, float value, float max_weight)
{
    if (d.weight < max_weight)
        d.weight = d.weight + 1.0f;
    d.occ = (d.occ * (d.weight - 1.0f) + value) / d.weight;
    d.observed = true;
}

struct OccConfig {
    float k_sigma = 0.052f;
    float sigma_min_factor = 1.5f;
    float sigma_max_factor = 6.0f;
    float k_tau = 0.026f;
    float tau_min_factor = 6.0f;
    float tau_max_factor = 16.0f;
    float log_odd_min = (float) -5.015;
    float log_odd_max = (float) 5.015;
    float max_weight = 0.0f;
    int fs_integr_scale = 1;
};

static OccConfig default_occ_config()
{
    OccConfig c;
    /* max_weight = floor(|min_occupancy / (0.97 * log_odd_min)|), data_field.hpp:67 */
    c.max_weight = std::floor(std::fabs(-100.0f / (0.97f * c.log_odd_min)));
    return c;
}

constexpr float kMinOccupancy = -100.0f;

/* data::up_prop_mean, data_impl.hpp:52-90 */
static int up_prop_mean(OccData& parent, const OccData child[8])
{
    float occ_sum = 0.0f, w_sum = 0.0f;
    int n = 0;
    for (int i = 0; i < 8; ++i) {
        if (occ_valid(child[i])) {
            ++n;
            occ_sum += child[i].occ;
            w_sum += child[i].weight;
        }
    }
    if (n > 0) {
        parent.occ = occ_sum / (float) n;
        parent.weight = std::ceil(w_sum / (float) n);
        parent.observed = false;
    }
    return n;
}

/* data::detail::up_prop_best, data_impl.hpp:96-125 */
static int up_prop_best(OccData& parent, const OccData child[8], bool want_min)
{
    float best = want_min ? std::numeric_limits<float>::max() : std::numeric_limits<float>::lowest();
    int best_i = 0, n_valid = 0, n_obs = 0;
    for (int i = 0; i < 8; ++i) {
        const OccData& d = child[i];
        if (occ_valid(d)) {
            ++n_valid;
            n_obs += d.observed ? 1 : 0;
            const float f = occ_field(d);
            if (want_min ? (f < best) : (f > best)) {
                best = f;
                best_i = i;
            }
        }
    }
    if (n_valid > 0) {
        parent = child[best_i];
        parent.observed = (n_obs == 8);
    }
    return n_valid;
}

/* ------------------------------------------------------------------ octree and block -- */

constexpr int kOccMaxScale = 3;
constexpr int kOccScaleOffset[4] = {0, 512, 576, 584};

static inline int cube(int v) { return v * v * v; }

struct OccBlock {
    int32_t coord[3];
    int parent;
    int timestamp = -1;
    OccData init_data;
    int min_scale = -1;
    int current_scale = kOccMaxScale;
    int finest = kOccMaxScale; /* finest scale with mean data */
    OccData mean[585];
    OccData minv[585];
    OccData maxv[585];
    OccData buffer[512];
    int buffer_scale = -1;
    size_t curr_integr = 0, curr_obs = 0, buf_integr = 0, buf_obs = 0;

    OccData* mean_at(int s) { return &mean[kOccScaleOffset[s]]; }
    OccData* min_at(int s) { return s == finest ? mean_at(s) : &minv[kOccScaleOffset[s]]; }
    OccData* max_at(int s) { return s == finest ? mean_at(s) : &maxv[kOccScaleOffset[s]]; }
    const OccData& max_data() { return max_at(kOccMaxScale)[0]; }
    const OccData& min_data() { return min_at(kOccMaxScale)[0]; }
    OccData* curr_data() { return mean_at(current_scale); }
    OccData* buffer_data() { return buffer_scale >= current_scale ? mean_at(buffer_scale) : buffer; }
    int voxel_idx(const int32_t c[3], int s) const
    {
        const int n = 8 >> s;
        return ((c[0] - coord[0]) >> s) + n * ((c[1] - coord[1]) >> s) + n * n * ((c[2] - coord[2]) >> s);
    }
    /* BlockMultiRes::data(voxel, scale): init_data below the finest allocated scale */
    const OccData& data_at(const int32_t c[3], int s)
    {
        if (s < finest)
            return init_data;
        return mean_at(s)[voxel_idx(c, s)];
    }
    const OccData& max_data_at(const int32_t c[3], int s)
    {
        if (s < finest)
            return init_data;
        return max_at(s)[voxel_idx(c, s)];
    }

    /* BlockMultiRes ctor, block_impl.hpp:208-220 */
    void init(const OccData& init)
    {
        init_data = init;
        mean[kOccScaleOffset[3]] = init;
    }

    /* allocateDownTo, block_impl.hpp:540-586 */
    void allocate_down_to(int new_min)
    {
        if (new_min >= current_scale)
            return;
        for (int s = current_scale; s >= new_min; --s) {
            OccData* d = mean_at(s);
            const int nv = cube(8 >> s);
            if (s != current_scale)
                std::fill(d, d + nv, init_data);
            if (s != new_min) {
                std::copy(d, d + nv, &minv[kOccScaleOffset[s]]);
                std::copy(d, d + nv, &maxv[kOccScaleOffset[s]]);
            }
        }
        finest = new_min;
        current_scale = new_min;
        min_scale = new_min;
    }

    /* deleteUpTo, block_impl.hpp:592-624 */
    void delete_up_to(int new_min)
    {
        if (new_min <= min_scale || min_scale == -1)
            return;
        finest = new_min;
        min_scale = new_min;
    }

    void init_curr_count()
    {
        if (init_data.observed) {
            curr_integr = (size_t) init_data.weight;
            curr_obs = (size_t) cube(8 >> current_scale);
        }
        else {
            curr_integr = 0;
            curr_obs = 0;
        }
    }

    void incr_buffer_integr(bool do_increment)
    {
        if (do_increment
            || (double) (buf_obs * (size_t) cube(1 << buffer_scale))
                >= 0.90 * (double) (curr_obs * (size_t) cube(1 << current_scale)))
            ++buf_integr;
    }

    void reset_buffer()
    {
        buffer_scale = -1;
        buf_integr = 0;
        buf_obs = 0;
    }

    void init_buffer(int bs)
    {
        reset_buffer();
        buffer_scale = bs;
        if (bs < current_scale) {
            const OccData def;
            std::fill(buffer, buffer + cube(8 >> bs), def);
        }
    }

    /* switchData, block_impl.hpp:718-780 */
    bool switch_data()
    {
        if (buf_integr >= 20
            && (double) (buf_obs * (size_t) cube(1 << buffer_scale))
                >= 0.9 * (double) (curr_obs * (size_t) cube(1 << current_scale))) {
            const int bs = buffer_scale;
            if (bs < current_scale) {
                std::copy(buffer, buffer + cube(8 >> bs), mean_at(bs));
                const OccData def;
                const int nv = cube(8 >> (bs + 1));
                std::fill(&minv[kOccScaleOffset[bs + 1]], &minv[kOccScaleOffset[bs + 1]] + nv, def);
                std::fill(&maxv[kOccScaleOffset[bs + 1]], &maxv[kOccScaleOffset[bs + 1]] + nv, def);
                finest = bs;
            }
            else {
                delete_up_to(bs);
            }
            OccData* d = mean_at(bs);
            for (int i = 0; i < cube(8 >> bs); ++i) {
                if (d[i].weight > 0.0f && !d[i].observed) {
                    d[i].observed = true;
                    ++buf_obs;
                }
            }
            current_scale = bs;
            min_scale = bs;
            curr_integr = buf_integr;
            curr_obs = buf_obs;
            reset_buffer();
            return true;
        }
        return false;
    }
};

/* A child slot: -1 empty, node index n >= 0, or block index b encoded as -2 - b. */
static inline bool slot_is_block(int s) { return s <= -2; }
static inline int slot_block(int s) { return -2 - s; }

struct OccNode {
    int32_t coord[3];
    int size;
    int parent;
    int child[8];
    OccData min_data, max_data;
    int timestamp = -1;
    bool is_leaf() const
    {
        for (int i = 0; i < 8; ++i)
            if (child[i] != -1)
                return false;
        return true;
    }
    /* NodeData<Occupancy>::data(), node.hpp:53-57 */
    OccData data() const { return (max_data.observed && is_leaf()) ? max_data : OccData(); }
};

struct OccOctree {
    int size = 0;
    std::vector<OccNode> nodes;
    std::vector<OccBlock> blocks;
    std::vector<char> block_live;
    bool aabb_empty = true;
    int32_t aabb_min[3] = {0, 0, 0}, aabb_max[3] = {0, 0, 0};

    void init(int sz)
    {
        size = sz;
        nodes.clear();
        blocks.clear();
        block_live.clear();
        OccNode root;
        root.coord[0] = root.coord[1] = root.coord[2] = 0;
        root.size = sz;
        root.parent = -1;
        std::fill(root.child, root.child + 8, -1);
        nodes.push_back(root);
        aabb_empty = true;
    }
    int block_depth() const { return (int) std::lround(std::log2((double) size)) - 3; }

    void aabb_extend(const int32_t c[3], int sz)
    {
        for (int i = 0; i < 3; ++i) {
            const int lo = c[i], hi = c[i] + sz - 1;
            if (aabb_empty) {
                aabb_min[i] = lo;
                aabb_max[i] = hi;
            }
            else {
                aabb_min[i] = std::min(aabb_min[i], lo);
                aabb_max[i] = std::max(aabb_max[i], hi);
            }
        }
        aabb_empty = false;
    }

    /* Octree::allocateChildren, octree_impl.hpp:200-233 */
    void allocate_children(int n)
    {
        const OccData init = nodes[n].data();
        const bool blocks_below = nodes[n].size == 16;
        const int csize = nodes[n].size / 2;
        for (int i = 0; i < 8; ++i) {
            if (nodes[n].child[i] != -1)
                continue;
            int32_t cc[3];
            for (int a = 0; a < 3; ++a)
                cc[a] = nodes[n].coord[a] + csize * ((i >> a) & 1);
            if (blocks_below) {
                OccBlock b;
                std::memcpy(b.coord, cc, sizeof(cc));
                b.parent = n;
                b.init(init);
                blocks.push_back(b);
                block_live.push_back(1);
                nodes[n].child[i] = -2 - (int) (blocks.size() - 1);
            }
            else {
                OccNode c;
                std::memcpy(c.coord, cc, sizeof(cc));
                c.size = csize;
                c.parent = n;
                std::fill(c.child, c.child + 8, -1);
                c.min_data = init;
                c.max_data = init;
                nodes.push_back(c);
                nodes[n].child[i] = (int) nodes.size() - 1;
            }
        }
        if (blocks_below)
            aabb_extend(nodes[n].coord, nodes[n].size);
    }

    /* Octree::deleteChildren, octree_impl.hpp:238-255 */
    void delete_children(int n)
    {
        for (int i = 0; i < 8; ++i) {
            const int c = nodes[n].child[i];
            if (c == -1)
                continue;
            if (slot_is_block(c))
                block_live[slot_block(c)] = 0;
            else
                delete_children(c);
            nodes[n].child[i] = -1;
        }
    }

    /* fetcher::leaf: the block holding the voxel, or the deepest node on its path when that
     * node has no children at all; -1 (no octant) otherwise. Returns a slot code. */
    int leaf(const int32_t c[3]) const
    {
        int n = 0;
        for (int cs = size >> 1; cs >= 8; cs >>= 1) {
            const int idx = ((c[0] & cs) > 0) + 2 * ((c[1] & cs) > 0) + 4 * ((c[2] & cs) > 0);
            const int ch = nodes[n].child[idx];
            if (ch == -1)
                return nodes[n].is_leaf() ? n : -1;
            if (slot_is_block(ch))
                return ch;
            n = ch;
        }
        return n;
    }
};

/* ------------------------------------------------------------------ pooling image -- */

struct PPixel {
    float min, max;
    int crossing; /* 0 inside, 1 crossing, 2 outside */
    int known;    /* 0 known, 1 part known, 2 unknown */
};

static inline PPixel pix(float mn, float mx, int cr, int kn) { return PPixel{mn, mx, cr, kn}; }
static inline PPixel known_pixel() { return pix(FLT_MAX, FLT_MIN, 0, 0); }
static inline PPixel unknown_pixel() { return pix(FLT_MAX, FLT_MIN, 0, 2); }
static inline PPixel crossing_known_pixel() { return pix(FLT_MAX, FLT_MIN, 1, 0); }
static inline PPixel crossing_unknown_pixel() { return pix(FLT_MAX, FLT_MIN, 1, 2); }
static inline PPixel outside_pixel_batch() { return pix(0.0f, 0.0f, 2, 2); }

/* DensePoolingImage<PinholeCamera>, dense_pooling_image_impl.hpp:56-347 */
struct PoolingImage {
    int w = 0, h = 0, max_level = 0;
    bool wrap = false; /* DensePoolingImage<OusterLidar>: columns wrap around (360 degrees) */
    float max_value = 0.0f;
    std::vector<std::vector<PPixel>> img;

    void build(const float* depth, int w_, int h_, bool wrap_ = false)
    {
        w = w_;
        h = h_;
        wrap = wrap_;
        const int image_max_dim = std::min(w, h);
        max_level = (int) (std::log2((double) ((image_max_dim - 1) / 2)) + 2) - 1;
        img.assign(max_level + 1, std::vector<PPixel>((size_t) w * h));
        for (int v = 0; v < h; ++v)
            for (int u = 0; u < w; ++u) {
                const float d = depth[u + v * w];
                if (d <= 0)
                    img[0][u + v * w] = unknown_pixel();
                else {
                    PPixel p = known_pixel();
                    p.min = d;
                    p.max = d;
                    img[0][u + v * w] = p;
                }
            }
        const std::vector<PPixel> def((size_t) w * h, crossing_known_pixel());
        if (max_level >= 1) {
            img[1] = def;
            const std::vector<PPixel>& L0 = img[0];
            for (int y = 0; y < h; ++y)
                for (int x = 0; x < w; ++x) {
                    PPixel& p = img[1][x + w * y];
                    if (wrap ? (y >= 1 && y < h - 1) : (y >= 1 && y < h - 1 && x >= 1 && x < w - 1))
                        p.crossing = 0;
                    const int top = y > 0 ? y - 1 : 0, bottom = y < h - 1 ? y + 1 : h - 1;
                    /* dense_pooling_image_impl.hpp:436-437: the Ouster image wraps in x */
                    const int left = x > 0 ? x - 1 : (wrap ? w - 1 : 0);
                    const int right = x < w - 1 ? x + 1 : (wrap ? 0 : w - 1);
                    auto at = [&](int xx, int yy) -> const PPixel& { return L0[xx + yy * w]; };
                    p.min = std::min(at(x, y).min,
                                     std::min(std::min(std::min(at(left, top).min, at(x, top).min),
                                                       std::min(at(right, top).min, at(right, y).min)),
                                              std::min(std::min(at(right, bottom).min, at(x, bottom).min),
                                                       std::min(at(left, bottom).min, at(left, y).min))));
                    p.max = std::max(at(x, y).max,
                                     std::max(std::max(std::max(at(left, top).max, at(x, top).max),
                                                       std::max(at(right, top).max, at(right, y).max)),
                                              std::max(std::max(at(right, bottom).max, at(x, bottom).max),
                                                       std::max(at(left, bottom).max, at(left, y).max))));
                    const int uf = at(x, y).known + at(left, top).known + at(x, top).known + at(right, top).known
                        + at(right, y).known + at(right, bottom).known + at(x, bottom).known
                        + at(left, bottom).known + at(left, y).known;
                    if (uf == 18)
                        p.known = 2;
                    else if (uf > 0)
                        p.known = 1;
                }
        }
        for (int l = 2, s = 2; l <= max_level; ++l, s <<= 1) {
            img[l] = def;
            const int s_half = s / 2;
            const std::vector<PPixel>& P = img[l - 1];
            for (int y = 0; y < h; ++y)
                for (int x = 0; x < w; ++x) {
                    PPixel& p = img[l][x + y * w];
                    int left, right, top, bottom;
                    if (x - s_half < 0) {
                        left = wrap ? w + (x - s_half) : 0;
                        if (!wrap)
                            p.crossing = 1;
                    }
                    else
                        left = x - s_half;
                    if (x + s_half >= w) {
                        right = wrap ? (x + s_half) - w : w - 1;
                        if (!wrap)
                            p.crossing = 1;
                    }
                    else
                        right = x + s_half;
                    if (y - s_half < 0) {
                        top = 0;
                        p.crossing = 1;
                    }
                    else
                        top = y - s_half;
                    if (y + s_half >= h) {
                        bottom = h - 1;
                        p.crossing = 1;
                    }
                    else
                        bottom = y + s_half;
                    const PPixel &a = P[left + top * w], &b = P[right + top * w], &c = P[left + bottom * w],
                                 &d = P[right + bottom * w];
                    p.min = std::min(std::min(a.min, b.min), std::min(c.min, d.min));
                    p.max = std::max(std::max(a.max, b.max), std::max(c.max, d.max));
                    const int uf = a.known + b.known + c.known + d.known;
                    if (uf == 8)
                        p.known = 2;
                    else if (uf > 0)
                        p.known = 1;
                    if (y >= s && y < h - s && x >= s && x < w - s)
                        p.crossing = 0;
                }
        }
        const int s = 1 << (max_level - 1);
        max_value = 0.0f;
        for (int v = s; true; v += 2 * s) {
            if (v > h - s - 1)
                v = h - s - 1;
            for (int u = s; true; u += 2 * s) {
                if (u > w - s - 1)
                    u = w - s - 1;
                const PPixel& p = img[max_level][u + w * v];
                if (max_value < p.max)
                    max_value = p.max;
                if (u == w - s - 1)
                    break;
            }
            if (v == h - s - 1)
                break;
        }
    }

    PPixel pool_bounding_box(int u_min, int u_max, int v_min, int v_max) const
    {
        const int u_diff = u_max - u_min, v_diff = v_max - v_min;
        const int min_side = std::min(u_diff, v_diff);
        /* log2(0) is -inf, which the reference turns into level 0 through its clamps */
        const int half = min_side / 2;
        const int lc = half > 0 ? (int) std::ceil(std::log2((double) half)) : std::numeric_limits<int>::min();
        const int level = std::max(0, std::min(max_level, lc));
        const int s = level > 0 ? 1 << std::max(level - 1, 0) : 0;
        PPixel batch = known_pixel();
        size_t n = 0, n_unknown = 0, n_part = 0;
        const int step = 2 * s + 1;
        for (int v = v_min + s; true; v += step) {
            if (v > v_max - s)
                v = v_max - s;
            for (int u = u_min + s; true; u += step) {
                if (u > u_max - s)
                    u = u_max - s;
                int uf = u;
                if (wrap && (u_min < 0 || u_max > w - 1)) {
                    if (u < 0)
                        uf += w;
                    else if (u > w - 1)
                        uf -= w;
                }
                const PPixel& p = img[level][uf + w * v];
                if (batch.max < p.max)
                    batch.max = p.max;
                if (batch.min > p.min)
                    batch.min = p.min;
                if (p.known == 2) {
                    ++n_unknown;
                    ++n_part;
                }
                else if (p.known == 1)
                    ++n_part;
                ++n;
                if (u == u_max - s)
                    break;
            }
            if (v == v_max - s)
                break;
        }
        if (n == n_unknown)
            batch.known = 2;
        else if (n_part > 0)
            batch.known = 1;
        return batch;
    }

    /* DensePoolingImage<OusterLidar>::conservativeQuery, dense_pooling_image_impl.hpp:743-781 */
    PPixel conservative_query_lidar(int u_min, int v_min, int u_max, int v_max) const
    {
        bool v_in = true, v_out = false;
        if ((float) v_min < 0.0f) {
            v_in = false;
            v_min = 0;
            if ((float) v_max < 0.0f)
                v_out = true;
        }
        else if ((float) v_min > (float) (unsigned) (h - 1)) {
            v_out = true;
        }
        if ((float) v_max > (float) (unsigned) (h - 1)) {
            v_in = false;
            v_max = h - 1;
        }
        if (v_out || u_min == u_max || v_min == v_max)
            return outside_pixel_batch();
        PPixel p = pool_bounding_box(u_min, u_max, v_min, v_max);
        if (!v_in)
            p.crossing = 1;
        return p;
    }

    PPixel conservative_query(int u_min, int v_min, int u_max, int v_max) const
    {
        bool u_in = true, u_out = false, v_in = true, v_out = false;
        if ((float) u_min < 0.0f) {
            u_in = false;
            u_min = 0;
            if ((float) u_max < 0.0f)
                u_out = true;
        }
        else if ((float) u_min > (float) (unsigned) (w - 1)) {
            u_out = true;
        }
        if ((float) u_max > (float) (unsigned) (w - 1)) {
            u_in = false;
            u_max = w - 1;
        }
        if ((float) v_min < 0.0f) {
            v_in = false;
            v_min = 0;
            if ((float) v_max < 0.0f)
                v_out = true;
        }
        else if ((float) v_min > (float) (unsigned) (h - 1)) {
            v_out = true;
        }
        if ((float) v_max > (float) (unsigned) (h - 1)) {
            v_in = false;
            v_max = h - 1;
        }
        if (u_out || v_out || u_min == u_max || v_min == v_max)
            return outside_pixel_batch();
        PPixel p = pool_bounding_box(u_min, u_max, v_min, v_max);
        if (!u_in || !v_in)
            p.crossing = 1;
        return p;
    }
};

/* ----------------------------------------------------------------- LiDAR model -- */
/* The Ouster projection lives in the un-vendored srl_projection module; this is a
 * project-defined equiangular model (parity unpinned), the same in the oracle and the GPU:
 * columns sweep the azimuth clockwise from +x (u = (pi - az) * w / (2 pi) - 0.5, wrapped into
 * [-0.5, w - 0.5)), rows sweep the elevation linearly from el_max (row 0) to el_min (row h-1),
 * projection succeeds for rows in [-0.5, h - 0.5). Angles use atan2 built on the
 * Abramowitz-Stegun 4.4.49 polynomial for atan on [0, 1] (|error| <= 1e-5 rad), in plain float
 * operations, so every platform rounds the same way. */
static inline float atan01_as(float x)
{
    const float x2 = x * x;
    return x * (0.9998660f + x2 * (-0.3302995f + x2 * (0.1801410f + x2 * (-0.0851330f + x2 * 0.0208351f))));
}

static inline float atan2_as(float y, float x)
{
    const float ax = std::fabs(x), ay = std::fabs(y);
    if (ax == 0.0f && ay == 0.0f)
        return 0.0f;
    float a = ay <= ax ? atan01_as(ay / ax) : 1.57079637f - atan01_as(ax / ay);
    if (x < 0.0f)
        a = 3.14159274f - a;
    return y < 0.0f ? -a : a;
}

struct Lidar {
    int w, h;
    float el_min_rad, el_max_rad;
    float near_plane, far_plane;
    float u_scale, v_scale;   /* w / (2 pi), (h - 1) / (el_max - el_min) */
    float tan_half_min_angle; /* tan(min_ray_angle / 2 in radians) */
};

static Lidar make_lidar(const so_lidar* c)
{
    Lidar L;
    L.w = c->width;
    L.h = c->height;
    L.near_plane = c->near_plane;
    L.far_plane = c->far_plane;
    constexpr float deg_to_rad = (float) M_PI / 180.0f;
    /* the beam elevation angles of the model, then OusterLidar's constructor (ouster_lidar.cpp:59-85) */
    std::vector<float> el((size_t) c->height);
    const float step = (c->elevation_max_deg - c->elevation_min_deg) / (float) (c->height - 1);
    for (int i = 0; i < c->height; ++i)
        el[(size_t) i] = c->elevation_max_deg - (float) i * step;
    float min_el = std::fabs(el[1] - el[0]);
    for (int i = 2; i < c->height; ++i)
        min_el = std::min(min_el, std::fabs(el[(size_t) i - 1] - el[(size_t) i]));
    const float az = 360.0f / (float) c->width;
    const float min_ray_angle = std::min(min_el, az);
    L.tan_half_min_angle = std::tan(min_ray_angle / 2.0f * deg_to_rad);
    L.el_min_rad = *std::min_element(el.begin(), el.end()) * deg_to_rad;
    L.el_max_rad = *std::max_element(el.begin(), el.end()) * deg_to_rad;
    L.u_scale = (float) c->width / (2.0f * 3.14159274f);
    L.v_scale = (float) (c->height - 1) / (L.el_max_rad - L.el_min_rad);
    return L;
}

static inline bool lidar_project(const Lidar& L, V3 p, float& u, float& v)
{
    const float rxy = std::sqrt(p.x * p.x + p.y * p.y);
    if (rxy == 0.0f && p.z == 0.0f) {
        u = v = 0.0f;
        return false;
    }
    const float az = atan2_as(p.y, p.x);
    const float el = atan2_as(p.z, rxy);
    u = (3.14159274f - az) * L.u_scale - 0.5f;
    if (u < -0.5f)
        u += (float) L.w;
    if (u >= (float) L.w - 0.5f)
        u -= (float) L.w;
    v = (L.el_max_rad - el) * L.v_scale;
    return v >= -0.5f && v < (float) L.h - 0.5f;
}

} // namespace

/* ------------------------------------------------------------------------ the map -- */

struct so_occ_map {
    OccOctree octree;
    float res;
    float dim;
    Tf T_MW, T_WM;
    OccConfig cfg;
};

namespace {

static inline V3 occ_voxel_to_point(const so_occ_map& m, const int32_t c[3], int stride)
{
    const float off = (float) stride * 0.5f;
    return apply(m.T_WM, v3(((float) c[0] + off) * m.res, ((float) c[1] + off) * m.res, ((float) c[2] + off) * m.res));
}

/* computeIntegrationScaleImpl, pinhole_camera.cpp:115-152 (default ratios {1.5, 3, 6}) */
static int occ_integration_scale(const Pinhole& s, V3 c_S, float res, int last_scale, int min_scale, int max_scale)
{
    static const float kRatio[3] = {1.5f, 3.0f, 6.0f};
    const float pixel_dim = c_S.z * s.inv_fx;
    const float pv = pixel_dim / res;
    int scale = 0;
    for (float r : kRatio) {
        if (pv < r)
            break;
        scale++;
    }
    scale = std::min(scale, max_scale);
    if (scale > last_scale && min_scale != -1) {
        c_S.z -= 0.25f;
        return occ_integration_scale(s, c_S, res, last_scale, -1, max_scale);
    }
    if (scale < last_scale && min_scale != -1) {
        c_S.z += 0.25f;
        return occ_integration_scale(s, c_S, res, last_scale, -1, max_scale);
    }
    return scale;
}

static inline float compute_tau(float depth, float tau_min, float tau_max, const OccConfig& c)
{
    return std::clamp(c.k_tau * depth, tau_min, tau_max);
}

/* updater::update_voxel, multires_ofusion_core_impl.hpp:46-77 */
static bool update_voxel(OccData& d, float range_diff, float tau, float three_sigma, const OccConfig& c)
{
    float sample;
    if (range_diff < -three_sigma)
        sample = c.log_odd_min;
    else if (range_diff < tau / 2)
        sample = std::min(c.log_odd_min - c.log_odd_min / three_sigma * (range_diff + three_sigma), c.log_odd_max);
    else if (range_diff < tau)
        sample = std::min(-c.log_odd_min * tau / (2 * three_sigma), c.log_odd_max);
    else
        return false;
    const bool newly = !d.observed;
    occ_update(d, sample, c.max_weight);
    return newly;
}

static bool free_voxel(OccData& d, const OccConfig& c)
{
    const bool newly = !d.observed;
    occ_update(d, c.log_odd_min, c.max_weight);
    return newly;
}

/* OusterLidar::computeIntegrationScaleImpl, ouster_lidar.cpp:107-146 */
static int lidar_integration_scale(const Lidar& L, V3 c, float res, int last_scale, int min_scale, int max_scale)
{
    static const float kRatio[3] = {1.5f, 3.0f, 6.0f};
    const float dist = norm(c);
    const float pixel_dim = 2.0f * dist * L.tan_half_min_angle;
    const float pv = (float) ((double) pixel_dim / (std::sqrt(3.0) * (double) res));
    int scale = 0;
    for (float r : kRatio) {
        if (pv < r)
            break;
        scale++;
    }
    scale = std::min(scale, max_scale);
    if ((scale > last_scale || scale < last_scale) && min_scale != -1) {
        const V3 n = normalized(c);
        const V3 h = scale > last_scale ? c - 0.25f * n : c + 0.25f * n;
        return lidar_integration_scale(L, h, res, last_scale, -1, max_scale);
    }
    return scale;
}

enum class VarState { Constant, Gradient, Undefined };

struct Frame {
    const so_occ_map* m;
    bool lidar = false;
    Lidar L;
    int w, h; /* image size */
    Pinhole s;
    Tf T_WS, T_SW;
    const float* depth;
    std::vector<float> sigma;
    PoolingImage depth_pool, sigma_pool;
    float sigma_min, sigma_max, tau_min, tau_max;
    float max_depth_value;
};

struct Allocation {
    std::vector<int> node_list;
    std::vector<int> block_list;
    std::vector<VarState> var_list;
    std::vector<char> inside_list;
};

/* VolumeCarver::computeVariance, volume_carver_impl.hpp:100-126 */
static VarState compute_variance(const Frame& f, float d_min, float d_max, float n_min, float n_max, float std_max)
{
    const float z_diff_max = n_max - d_min;
    const float z_diff_min = n_min - d_max;
    const float tau_max = compute_tau(d_max, f.tau_min, f.tau_max, f.m->cfg);
    const float three_sigma_min = 3.0f * std_max;
    if ((double) z_diff_min > 1.25 * (double) tau_max)
        return VarState::Undefined;
    if ((double) z_diff_max < -1.25 * (double) three_sigma_min)
        return VarState::Constant;
    return VarState::Gradient;
}

static void carve_emit(so_occ_map& mm, Frame& f, int depth, int slot, bool should_split, VarState var,
                       bool projects_inside, Allocation& out);
static bool camera_in_node(const so_occ_map& mm, const Frame& f, const int32_t coord[3], int size);

/* VolumeCarver<.., PinholeCamera>::operator()(coord, size, depth, octant), volume_carver_impl.hpp:132-310.
 * `slot` is the octant: a node index or a block slot code. */
static void carve(so_occ_map& mm, Frame& f, const int32_t coord[3], int size, int depth, int slot, Allocation& out)
{
    OccOctree& oct = mm.octree;
    const float size_to_radius = std::sqrt(3.0f) / 2.0f;
    const float zero_depth_band = 1.0e-6f;
    const V3 centre_W = occ_voxel_to_point(mm, coord, size);
    const V3 centre_S = apply(f.T_SW, centre_W);
    const float rad = (float) size * size_to_radius * mm.res;
    const float approx_max = centre_S.z + rad;
    const float approx_min = centre_S.z - rad;
    if (approx_min > f.max_depth_value || approx_max < zero_depth_band)
        return;
    V3 corner_S[8];
    int n_front = 0;
    for (int k = 0; k < 8; ++k) {
        const float rx = (float) (k & 1), ry = (float) ((k >> 1) & 1), rz = (float) (k >> 2);
        const V3 p_M = v3(((float) size * rx + (float) coord[0]) * mm.res, ((float) size * ry + (float) coord[1]) * mm.res,
                          ((float) size * rz + (float) coord[2]) * mm.res);
        corner_S[k] = apply(f.T_SW, apply(mm.T_WM, p_M));
        if (!(corner_S[k].z < zero_depth_band))
            ++n_front;
    }
    if (n_front == 0)
        return;
    float pu[8], pv[8];
    bool ok[8];
    for (int k = 0; k < 8; ++k) {
        const V3 p = corner_S[k];
        if (std::fabs(p.z) < 1.0e-12f) {
            pu[k] = pv[k] = 0.0f;
            ok[k] = false;
            continue;
        }
        const float rz = 1.0f / p.z;
        pu[k] = f.s.fx * (p.x * rz) + f.s.cx;
        pv[k] = f.s.fy * (p.y * rz) + f.s.cy;
        ok[k] = p.z > 0.0f && pu[k] >= -0.5f && pu[k] < (float) f.s.w - 0.5f && pv[k] >= -0.5f
            && pv[k] < (float) f.s.h - 0.5f;
    }
    bool should_split = false, projects_inside = false;
    VarState var = VarState::Gradient;
    const bool is_block = slot_is_block(slot);
    if (depth < oct.block_depth() + 1) {
        if (n_front < 8) {
            const bool cam_in = camera_in_node(mm, f, coord, size);
            bool crosses = false;
            for (int k = 0; k < 8; ++k)
                crosses = crosses || ok[k];
            if (cam_in)
                should_split = true;
            else if (crosses)
                should_split = true;
            else {
                /* sphereInFrustumInf: the frustum planes without the far one */
                bool in = true;
                for (int i = 0; i < 5; ++i) {
                    const float d = ((centre_S.x * f.s.normals[i][0] + centre_S.y * f.s.normals[i][1])
                                     + centre_S.z * f.s.normals[i][2])
                        + f.s.normals[i][3];
                    if (d < -rad)
                        in = false;
                }
                if (in)
                    should_split = true;
                else
                    return;
            }
        }
        else {
            for (int k = 0; k < 8; ++k) {
                pu[k] = pu[k] > 1e7f ? 1e7f : pu[k];
                pv[k] = pv[k] > 1e7f ? 1e7f : pv[k];
                pu[k] = pu[k] < -1e7f ? -1e7f : pu[k];
                pv[k] = pv[k] < -1e7f ? -1e7f : pv[k];
            }
            float umin = pu[0], umax = pu[0], vmin = pv[0], vmax = pv[0], zmin = corner_S[0].z, zmax = corner_S[0].z;
            for (int k = 1; k < 8; ++k) {
                umin = std::min(umin, pu[k]);
                umax = std::max(umax, pu[k]);
                vmin = std::min(vmin, pv[k]);
                vmax = std::max(vmax, pv[k]);
                zmin = std::min(zmin, corner_S[k].z);
                zmax = std::max(zmax, corner_S[k].z);
            }
            const int bb_min[2] = {(int) umin, (int) vmin}, bb_max[2] = {(int) umax, (int) vmax};
            const PPixel pp = f.depth_pool.conservative_query(bb_min[0], bb_min[1], bb_max[0], bb_max[1]);
            if (pp.known == 2)
                return;
            if (zmin > pp.max + f.tau_max)
                return;
            const PPixel sp = f.sigma_pool.conservative_query(bb_min[0], bb_min[1], bb_max[0], bb_max[1]);
            var = compute_variance(f, pp.min, pp.max, zmin, zmax, sp.max);
            if (var != VarState::Gradient) {
                OccData cd = is_block ? oct.blocks[slot_block(slot)].max_data() : oct.nodes[slot].data();
                if (cd.observed && (double) occ_field(cd) <= 0.95 * (double) kMinOccupancy)
                    return;
            }
            if (pp.crossing == 1)
                should_split = true;
            else if (pp.known == 1)
                should_split = true;
            else if (var == VarState::Gradient)
                should_split = true;
            projects_inside = pp.known == 0;
        }
    }
    carve_emit(mm, f, depth, slot, should_split, var, projects_inside, out);
}

/* cameraInNode, volume_carver_impl.hpp:83-98 */
static bool camera_in_node(const so_occ_map& mm, const Frame& f, const int32_t coord[3], int size)
{
    V3 cam_v = v3(-1.0f, -1.0f, -1.0f);
    const V3 t = v3(f.T_WS.t[0], f.T_WS.t[1], f.T_WS.t[2]);
    const V3 p_M = apply(mm.T_MW, t);
    if (p_M.x >= 0.0f && p_M.x < mm.dim && p_M.y >= 0.0f && p_M.y < mm.dim && p_M.z >= 0.0f && p_M.z < mm.dim)
        cam_v = p_M / mm.res;
    return cam_v.x >= (float) coord[0] && cam_v.x <= (float) (coord[0] + size) && cam_v.y >= (float) coord[1]
        && cam_v.y <= (float) (coord[1] + size) && cam_v.z >= (float) coord[2] && cam_v.z <= (float) (coord[2] + size);
}

/* VolumeCarver<.., OusterLidar>::operator()(coord, size, depth, octant), volume_carver_impl.hpp:339-537:
 * range-based depth bounds, the camera-in-node test first, and corner columns unwrapped around
 * the centre's column before the bounding box goes to the wrap-around pooling image. */
static void carve_lidar(so_occ_map& mm, Frame& f, const int32_t coord[3], int size, int depth, int slot, Allocation& out)
{
    OccOctree& oct = mm.octree;
    const float size_to_radius = std::sqrt(3.0f) / 2.0f;
    const V3 centre_W = occ_voxel_to_point(mm, coord, size);
    const V3 centre_S = apply(f.T_SW, centre_W);
    const float rad = (float) size * size_to_radius * mm.res;
    const float range = norm(centre_S);
    const float approx_max = range + rad;
    const float approx_min = range - rad;
    if (approx_min > f.max_depth_value)
        return;
    bool should_split = false, projects_inside = false;
    VarState var = VarState::Gradient;
    const bool is_block = slot_is_block(slot);
    if (depth < oct.block_depth() + 1) {
        if (camera_in_node(mm, f, coord, size))
            should_split = true;
        else {
            float pu[8], pv[8];
            for (int k = 0; k < 8; ++k) {
                const float rx = (float) (k & 1), ry = (float) ((k >> 1) & 1), rz = (float) (k >> 2);
                const V3 p_M = v3(((float) size * rx + (float) coord[0]) * mm.res,
                                  ((float) size * ry + (float) coord[1]) * mm.res,
                                  ((float) size * rz + (float) coord[2]) * mm.res);
                lidar_project(f.L, apply(f.T_SW, apply(mm.T_WM, p_M)), pu[k], pv[k]);
            }
            float cu, cv;
            lidar_project(f.L, centre_S, cu, cv);
            const float W = (float) f.L.w;
            float cu_comp = cu + (float) (f.L.w / 2);
            if (cu_comp > W - 0.5f)
                cu_comp = cu_comp - W;
            for (int k = 0; k < 8; ++k) {
                if (cu < cu_comp && pu[k] > cu && pu[k] > cu_comp)
                    pu[k] = pu[k] - W;
                else if (cu > cu_comp && pu[k] < cu && pu[k] < cu_comp)
                    pu[k] = pu[k] + W;
            }
            float umin = pu[0], umax = pu[0], vmin = pv[0], vmax = pv[0];
            for (int k = 1; k < 8; ++k) {
                umin = std::min(umin, pu[k]);
                umax = std::max(umax, pu[k]);
                vmin = std::min(vmin, pv[k]);
                vmax = std::max(vmax, pv[k]);
            }
            const int bb_min[2] = {(int) umin, (int) vmin}, bb_max[2] = {(int) umax, (int) vmax};
            const PPixel pp = f.depth_pool.conservative_query_lidar(bb_min[0], bb_min[1], bb_max[0], bb_max[1]);
            if (pp.known == 2)
                return;
            if (approx_min > pp.max + f.tau_max)
                return;
            const PPixel sp = f.sigma_pool.conservative_query_lidar(bb_min[0], bb_min[1], bb_max[0], bb_max[1]);
            var = compute_variance(f, pp.min, pp.max, approx_min, approx_max, sp.max);
            if (var != VarState::Gradient) {
                OccData cd = is_block ? oct.blocks[slot_block(slot)].max_data() : oct.nodes[slot].data();
                if (cd.observed && (double) occ_field(cd) <= 0.95 * (double) kMinOccupancy)
                    return;
            }
            if (pp.crossing == 1)
                should_split = true;
            else if (pp.known == 1)
                should_split = true;
            else if (var == VarState::Gradient)
                should_split = true;
            projects_inside = pp.known == 0;
        }
    }
    carve_emit(mm, f, depth, slot, should_split, var, projects_inside, out);
}

/* the common tail of both carvers: split (allocate the children and recurse) or list the octant */
static void carve_emit(so_occ_map& mm, Frame& f, int depth, int slot, bool should_split, VarState var,
                       bool projects_inside, Allocation& out)
{
    OccOctree& oct = mm.octree;
    const bool is_block = slot_is_block(slot);
    if (should_split) {
        if (is_block) {
            out.block_list.push_back(slot_block(slot));
            out.var_list.push_back(var);
            out.inside_list.push_back(projects_inside ? 1 : 0);
        }
        else {
            oct.allocate_children(slot);
            const int csize = oct.nodes[slot].size / 2;
            for (int i = 0; i < 8; ++i) {
                int32_t cc[3];
                for (int a = 0; a < 3; ++a)
                    cc[a] = oct.nodes[slot].coord[a] + csize * ((i >> a) & 1);
                const int child = oct.nodes[slot].child[i];
                if (f.lidar)
                    carve_lidar(mm, f, cc, csize, depth + 1, child, out);
                else
                    carve(mm, f, cc, csize, depth + 1, child, out);
            }
        }
    }
    else {
        if (is_block) {
            out.block_list.push_back(slot_block(slot));
            out.var_list.push_back(var);
            out.inside_list.push_back(projects_inside ? 1 : 0);
        }
        else if (var == VarState::Constant) {
            out.node_list.push_back(slot);
        }
    }
}

/* the scale choice shared by updateBlock and freeBlock (multires_ofusion_updater_impl.hpp:183-205,
 * 308-330) */
static int recommended_scale(const so_occ_map& m, const Frame& f, OccBlock& b, V3 centre_C, bool free_min, int& last_scale)
{
    last_scale = (b.min_scale == -1) ? 0 : b.current_scale;
    const int computed = f.lidar ? lidar_integration_scale(f.L, centre_C, m.res, last_scale, b.min_scale, kOccMaxScale)
                                 : occ_integration_scale(f.s, centre_C, m.res, last_scale, b.min_scale, kOccMaxScale);
    const int min_integr = (free_min && (b.min_scale == -1 || (double) b.max_data().occ < 0.95 * (double) m.cfg.log_odd_min))
        ? m.cfg.fs_integr_scale
        : std::max(0, last_scale - 1);
    const int max_integr = (b.min_scale == -1) ? kOccMaxScale : std::min(kOccMaxScale, last_scale + 1);
    return std::min(std::max(min_integr, computed), max_integr);
}

/* the buffer set-up shared by updateBlock and freeBlock when the recommended scale differs */
static void prepare_buffer(OccBlock& b, int recommended, int last_scale)
{
    if (recommended == b.buffer_scale)
        return;
    b.init_buffer(recommended);
    if (recommended < last_scale) {
        const unsigned np = 8u >> last_scale, np2 = np * np;
        const unsigned nb = np << 1, nb2 = nb * nb;
        OccData* buf = b.buffer_data();
        const OccData* cur = b.curr_data();
        for (unsigned z = 0; z < np; z++)
            for (unsigned y = 0; y < np; y++)
                for (unsigned x = 0; x < np; x++) {
                    const OccData& pd = cur[x + y * np + z * np2];
                    for (unsigned k = 0; k < 2; k++)
                        for (unsigned j = 0; j < 2; j++)
                            for (unsigned i = 0; i < 2; i++) {
                                OccData& bd = buf[(2 * x + i) + (2 * y + j) * nb + (2 * z + k) * nb2];
                                bd.occ = pd.occ;
                                bd.weight = pd.weight;
                                bd.observed = false;
                            }
                }
    }
}

/* Updater::updateBlockData<UpdateBuffer>, multires_ofusion_updater_impl.hpp:413-545 */
static void update_block_data(const so_occ_map& m, const Frame& f, OccBlock& b, V3 centre_C, int scale, bool low_var,
                              bool inside, bool to_buffer)
{
    const int stride = 1 << scale;
    const int n = 8 >> scale, n2 = n * n;
    const V3 base_C = apply(f.T_SW, occ_voxel_to_point(m, b.coord, stride));
    const float rs = m.res * (float) stride;
    float D[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            D[i][j] = f.T_SW.R[i][j] * rs;
    const float tau = compute_tau(f.lidar ? norm(centre_C) : centre_C.z, f.tau_min, f.tau_max, m.cfg);
    OccData* data = to_buffer ? b.buffer_data() : b.curr_data();
    const float near_p = f.lidar ? f.L.near_plane : f.s.near_plane;
    const float far_p = f.lidar ? f.L.far_plane : f.s.far_plane;
    for (int z = 0; z < n; z++)
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++) {
                const float fx = (float) x, fy = (float) y, fz = (float) z;
                const V3 dlt = v3((D[0][0] * fx + D[0][1] * fy) + D[0][2] * fz, (D[1][0] * fx + D[1][1] * fy) + D[1][2] * fz,
                                  (D[2][0] * fx + D[2][1] * fy) + D[2][2] * fz);
                const V3 p = base_C + dlt;
                float u, v;
                if (!(f.lidar ? lidar_project(f.L, p, u, v) : project(f.s, p, u, v)))
                    continue;
                int px, py;
                round_pixel(u, v, px, py);
                const float dv = f.depth[px + py * f.w];
                if (dv < near_p)
                    continue;
                const float three_sigma = 3.0f * f.sigma[px + py * f.w];
                OccData& d = data[x + y * n + z * n2];
                bool newly;
                if (low_var) {
                    newly = free_voxel(d, m.cfg);
                }
                else {
                    const float pm = f.lidar ? norm(p) : p.z;
                    const float range = norm(p);
                    const float range_diff = (pm - dv) * (range / pm);
                    newly = update_voxel(d, range_diff, tau, three_sigma, m.cfg);
                    if (dv > far_p)
                        continue;
                }
                if (to_buffer) {
                    if (newly)
                        ++b.buf_obs;
                }
                else if (newly) {
                    ++b.curr_obs;
                }
            }
    if (to_buffer)
        b.incr_buffer_integr(inside);
    else
        ++b.curr_integr;
}

/* Updater::updateBlock, multires_ofusion_updater_impl.hpp:296-409 */
static void update_block(const so_occ_map& m, const Frame& f, OccBlock& b, bool low_var, bool inside)
{
    const V3 centre_C = apply(f.T_SW, occ_voxel_to_point(m, b.coord, 8));
    int last_scale;
    const int rec = recommended_scale(m, f, b, centre_C, low_var, last_scale);
    int integration_scale = last_scale;
    if (b.min_scale == -1) {
        integration_scale = rec;
        b.allocate_down_to(integration_scale);
        b.current_scale = integration_scale;
        b.init_curr_count();
        b.init_data = OccData();
    }
    else if (rec != last_scale) {
        prepare_buffer(b, rec, last_scale);
        update_block_data(m, f, b, centre_C, rec, low_var, inside, true);
        if (b.switch_data())
            return;
    }
    else {
        b.reset_buffer();
    }
    update_block_data(m, f, b, centre_C, integration_scale, low_var, inside, false);
}

/* Updater::freeBlock, multires_ofusion_updater_impl.hpp:168-292 */
static void free_block(const so_occ_map& m, const Frame& f, OccBlock& b)
{
    const V3 centre_C = apply(f.T_SW, occ_voxel_to_point(m, b.coord, 8));
    int last_scale;
    const int rec = recommended_scale(m, f, b, centre_C, true, last_scale);
    int integration_scale = last_scale;
    if (b.min_scale == -1) {
        integration_scale = rec;
        b.allocate_down_to(integration_scale);
        b.current_scale = integration_scale;
        b.init_curr_count();
        b.init_data = OccData();
    }
    else if (rec != last_scale) {
        prepare_buffer(b, rec, last_scale);
        const int n = cube(8 >> rec);
        OccData* buf = b.buffer_data();
        for (int i = 0; i < n; ++i)
            if (free_voxel(buf[i], m.cfg))
                ++b.buf_obs;
        b.incr_buffer_integr(true);
        if (b.switch_data())
            return;
    }
    else {
        b.reset_buffer();
    }
    const int n = cube(8 >> integration_scale);
    OccData* cur = b.curr_data();
    for (int i = 0; i < n; ++i)
        if (free_voxel(cur[i], m.cfg))
            ++b.curr_obs;
    ++b.curr_integr;
}

/* updater::propagate_block_to_coarsest_scale, multires_ofusion_core_impl.hpp:120-276 */
static void propagate_block(OccBlock& b)
{
    if (b.current_scale == kOccMaxScale)
        return;
    int cs = b.current_scale;
    int ps = cs + 1;
    auto gather = [](const OccData* src, int x, int y, int z, int nc, OccData out[8]) {
        int k8 = 0;
        for (int k = 0; k < 2; k++)
            for (int j = 0; j < 2; j++)
                for (int i = 0; i < 2; i++)
                    out[k8++] = src[(2 * x + i) + (2 * y + j) * nc + (2 * z + k) * nc * nc];
    };
    {
        const int np = 8 >> ps, nc = 8 >> cs;
        OccData* pmin = b.min_at(ps);
        OccData* pmax = b.max_at(ps);
        OccData* pmean = b.mean_at(ps);
        const OccData* cmean = b.mean_at(cs);
        for (int z = 0; z < np; z++)
            for (int y = 0; y < np; y++)
                for (int x = 0; x < np; x++) {
                    const int pi = x + y * np + z * np * np;
                    OccData ch[8];
                    gather(cmean, x, y, z, nc, ch);
                    if (b.buffer_scale > b.current_scale) {
                        up_prop_best(pmin[pi], ch, true);
                        up_prop_best(pmax[pi], ch, false);
                    }
                    else {
                        up_prop_mean(pmean[pi], ch);
                        up_prop_best(pmin[pi], ch, true);
                        up_prop_best(pmax[pi], ch, false);
                    }
                }
    }
    for (ps += 1; ps <= kOccMaxScale; ++ps) {
        cs = ps - 1;
        const int np = 8 >> ps, nc = 8 >> cs;
        OccData *pmin = b.min_at(ps), *pmax = b.max_at(ps), *pmean = b.mean_at(ps);
        const OccData *cmin = b.min_at(cs), *cmax = b.max_at(cs), *cmean = b.mean_at(cs);
        for (int z = 0; z < np; z++)
            for (int y = 0; y < np; y++)
                for (int x = 0; x < np; x++) {
                    const int pi = x + y * np + z * np * np;
                    OccData c0[8], c1[8], c2[8];
                    gather(cmean, x, y, z, nc, c0);
                    gather(cmin, x, y, z, nc, c1);
                    gather(cmax, x, y, z, nc, c2);
                    up_prop_mean(pmean[pi], c0);
                    up_prop_best(pmin[pi], c1, true);
                    up_prop_best(pmax[pi], c2, false);
                }
    }
}

/* updater::propagate_to_parent_node, multires_ofusion_core_impl.hpp:88-117 */
static OccData propagate_to_parent_node(OccOctree& oct, int n, int timestamp)
{
    OccNode& node = oct.nodes[n];
    node.timestamp = timestamp;
    OccData cmin[8], cmax[8];
    for (int i = 0; i < 8; ++i) {
        const int c = node.child[i];
        if (c == -1)
            continue;
        if (slot_is_block(c)) {
            OccBlock& b = oct.blocks[slot_block(c)];
            cmin[i] = b.min_data();
            cmax[i] = b.max_data();
        }
        else {
            cmin[i] = oct.nodes[c].min_data;
            cmax[i] = oct.nodes[c].max_data;
        }
    }
    up_prop_best(node.min_data, cmin, true);
    up_prop_best(node.max_data, cmax, false);
    return node.max_data;
}

struct UpdaterState {
    std::vector<std::set<int>> node_set;
    std::vector<int> freed_blocks;
};

/* Updater::freeNodeRecurse, multires_ofusion_updater_impl.hpp:550-600 */
static void free_node_recurse(so_occ_map& m, const Frame& f, int n, int depth, UpdaterState& st)
{
    OccOctree& oct = m.octree;
    if (oct.nodes[n].is_leaf()) {
        OccData d = oct.nodes[n].data();
        occ_update(d, m.cfg.log_odd_min, m.cfg.max_weight);
        oct.nodes[n].min_data = d;
        oct.nodes[n].max_data = d;
        st.node_set[depth - 1].insert(oct.nodes[n].parent);
    }
    else {
        for (int i = 0; i < 8; ++i) {
            const int c = oct.nodes[n].child[i];
            if (slot_is_block(c)) {
                free_block(m, f, oct.blocks[slot_block(c)]);
                st.node_set[depth].insert(n);
                st.freed_blocks.push_back(slot_block(c));
            }
            else {
                free_node_recurse(m, f, c, depth + 1, st);
            }
        }
    }
}

/* depthToSigma, uncertainty.cpp:12-34 (linear model) */
static void depth_sigma(const float* depth, int n, float res, const OccConfig& c, float* sigma)
{
    const float smin = res * c.sigma_min_factor, smax = res * c.sigma_max_factor;
    for (int i = 0; i < n; ++i) {
        const float d = depth[i];
        if (d <= 0.0f || std::isnan(d))
            sigma[i] = 0.0f;
        else
            sigma[i] = std::clamp(c.k_sigma * d, smin, smax);
    }
}

/* visitor::getData(octree, voxel) for occupancy maps (visitor_impl.hpp:704-717) */
static OccData occ_get_data_voxel(const so_occ_map& m, const int32_t c[3])
{
    const int slot = m.octree.leaf(c);
    if (slot == -1)
        return OccData();
    if (slot_is_block(slot)) {
        OccBlock& b = const_cast<OccBlock&>(m.octree.blocks[slot_block(slot)]);
        return b.data_at(c, b.current_scale);
    }
    return m.octree.nodes[slot].data();
}

static OccData occ_get_data(const so_occ_map& m, V3 p_W)
{
    const V3 v = apply(m.T_MW, p_W) / m.res;
    const int32_t c[3] = {(int) v.x, (int) v.y, (int) v.z};
    return occ_get_data_voxel(m, c);
}

/* visitor::getInterp multi-res (visitor_impl.hpp:906-972) with detail::get_neighbours
 * (:398-697) on an occupancy octree: a corner whose leaf is a node takes the node's data;
 * a scale is skipped when a corner has no octant or its block integrates at a coarser scale. */
static bool occ_interp(const so_occ_map& m, V3 vf, int desired_scale, float& out, int* returned_scale)
{
    const OccOctree& o = m.octree;
    const int32_t c0[3] = {(int) vf.x, (int) vf.y, (int) vf.z};
    const int q = o.leaf(c0);
    if (q == -1)
        return false;
    const bool q_block = slot_is_block(q);
    const int init = q_block ? std::max(o.blocks[slot_block(q)].current_scale, desired_scale) : 0;
    for (int scale = init; scale <= kOccMaxScale; ++scale) {
        const int stride = 1 << scale;
        const float inv = 1.0f / (float) stride;
        const V3 bf = v3(inv * vf.x - 0.5f, inv * vf.y - 0.5f, inv * vf.z - 0.5f);
        const int32_t base[3] = {stride * (int) bf.x, stride * (int) bf.y, stride * (int) bf.z};
        if (o.aabb_empty)
            return false;
        for (int i = 0; i < 3; ++i)
            if (base[i] < o.aabb_min[i] || base[i] > o.aabb_max[i])
                return false;
        bool ok = true;
        for (int i = 0; i < 3; ++i)
            if (base[i] + stride >= o.size || base[i] < 0)
                ok = false;
        OccData d[8];
        for (int n = 0; ok && n < 8; ++n) {
            const int32_t c[3] = {base[0] + stride * (n & 1), base[1] + stride * ((n >> 1) & 1),
                                  base[2] + stride * ((n >> 2) & 1)};
            const int slot = o.leaf(c);
            if (slot == -1) {
                ok = false;
                break;
            }
            if (slot_is_block(slot)) {
                OccBlock& b = const_cast<OccBlock&>(o.blocks[slot_block(slot)]);
                if (b.current_scale > scale) {
                    ok = false;
                    break;
                }
                d[n] = b.data_at(c, scale);
            }
            else {
                d[n] = o.nodes[slot].data();
            }
        }
        if (!ok)
            continue;
        for (int n = 0; n < 8; ++n)
            if (!occ_valid(d[n]))
                return false;
        if (returned_scale)
            *returned_scale = q_block ? scale : (int) std::lround(std::log2((double) o.nodes[q].size));
        float f[8];
        for (int n = 0; n < 8; ++n)
            f[n] = occ_field(d[n]);
        const V3 t = v3(bf.x - std::floor(bf.x), bf.y - std::floor(bf.y), bf.z - std::floor(bf.z));
        const V3 tc = v3(1.0f - t.x, 1.0f - t.y, 1.0f - t.z);
        out = ((f[0] * tc.x + f[1] * t.x) * tc.y + (f[2] * tc.x + f[3] * t.x) * t.y) * tc.z
            + ((f[4] * tc.x + f[5] * t.x) * tc.y + (f[6] * tc.x + f[7] * t.x) * t.y) * t.z;
        return true;
    }
    return false;
}

/* fetcher::finest_octant (fetcher_impl.hpp:69-94) as a slot: the octant of size
 * max(2^scale, 8) on the voxel's path, the deepest node when that node has no children, or -1. */
static int occ_finest_octant(const OccOctree& o, const int32_t c[3], int scale_desired)
{
    const int size_desired = std::max(1 << scale_desired, 8);
    int n = 0, child = -1;
    for (int cs = o.size >> 1; cs >= size_desired; cs >>= 1) {
        const int idx = ((c[0] & cs) > 0) + 2 * ((c[1] & cs) > 0) + 4 * ((c[2] & cs) > 0);
        child = o.nodes[n].child[idx];
        if (child == -1)
            return o.nodes[n].is_leaf() ? n : -1;
        if (slot_is_block(child))
            return child;
        n = child;
    }
    return child;
}

/* visitor::getMaxData (visitor_impl.hpp:815-835) */
static OccData occ_max_data(const so_occ_map& m, const int32_t c[3], int scale_desired)
{
    const int slot = occ_finest_octant(m.octree, c, scale_desired);
    if (slot == -1)
        return OccData();
    if (slot_is_block(slot)) {
        OccBlock& b = const_cast<OccBlock&>(m.octree.blocks[slot_block(slot)]);
        const int so = std::max(scale_desired, b.current_scale);
        return b.max_at(so)[b.voxel_idx(c, so)];
    }
    return m.octree.nodes[slot].max_data;
}

/* visitor::getData(octree, block_ptr, voxel, scale_desired, scale_returned) for occupancy maps;
 * false for no octant (the default data). */
static bool occ_data_at(const so_occ_map& m, int hint_block, const int32_t c[3], int scale_desired, OccData& d,
                        int& scale_returned)
{
    const OccBlock* hb = &m.octree.blocks[hint_block];
    int slot = -2 - hint_block;
    if (!(c[0] >= hb->coord[0] && c[0] <= hb->coord[0] + 7 && c[1] >= hb->coord[1] && c[1] <= hb->coord[1] + 7
          && c[2] >= hb->coord[2] && c[2] <= hb->coord[2] + 7))
        slot = m.octree.leaf(c);
    if (slot == -1) {
        d = OccData();
        return false;
    }
    if (slot_is_block(slot)) {
        OccBlock& b = const_cast<OccBlock&>(m.octree.blocks[slot_block(slot)]);
        scale_returned = std::max(scale_desired, b.current_scale);
        d = b.mean_at(scale_returned)[b.voxel_idx(c, scale_returned)];
        return true;
    }
    scale_returned = scale_desired;
    d = m.octree.nodes[slot].data();
    return true;
}

/* visitor::getFieldGrad multi-res, desired scale 0 (visitor_impl.hpp:1257-1497), occupancy */
static bool occ_grad(const so_occ_map& m, V3 vf, V3& g)
{
    const OccOctree& o = m.octree;
    const int32_t c0[3] = {(int) vf.x, (int) vf.y, (int) vf.z};
    const int q = occ_finest_octant(o, c0, 0);
    if (q == -1)
        return false;
    if (!slot_is_block(q)) {
        if (occ_valid(o.nodes[q].data())) {
            g = v3(0.0f, 0.0f, 0.0f);
            return true;
        }
        return false;
    }
    const int init = std::max(0, o.blocks[slot_block(q)].current_scale);
    const int top = o.size - 1;
    for (int scale = init; scale <= kOccMaxScale; ++scale) {
        const int stride = 1 << scale;
        const float inv = 1.0f / (float) stride;
        const V3 sv = v3(inv * vf.x - 0.5f, inv * vf.y - 0.5f, inv * vf.z - 0.5f);
        const V3 fac = v3(sv.x - std::floor(sv.x), sv.y - std::floor(sv.y), sv.z - std::floor(sv.z));
        const int32_t base[3] = {stride * (int) sv.x, stride * (int) sv.y, stride * (int) sv.z};
        int32_t ll[3], lu[3], ul[3], uu[3];
        for (int i = 0; i < 3; ++i) {
            ll[i] = std::max(base[i] - stride, 0);
            lu[i] = std::max(base[i], 0);
            ul[i] = std::min(base[i] + stride, top);
            uu[i] = std::min(base[i] + 2 * stride, top);
        }
        const int oct = occ_finest_octant(o, base, scale);
        if (oct == -1)
            continue;
        if (!slot_is_block(oct)) {
            if (o.nodes[oct].is_leaf() && occ_valid(o.nodes[oct].data())) {
                g = v3(0.0f, 0.0f, 0.0f);
                return true;
            }
            continue;
        }
        const int32_t* X[32] = {ll, ll, ll, ll, lu, lu, lu, lu, lu, lu, lu, lu, lu, lu, lu, lu,
                                ul, ul, ul, ul, ul, ul, ul, ul, ul, ul, ul, ul, uu, uu, uu, uu};
        const int32_t* Y[32] = {lu, ul, lu, ul, ll, ll, lu, lu, lu, lu, ul, ul, ul, ul, uu, uu,
                                ll, ll, lu, lu, lu, lu, ul, ul, ul, ul, uu, uu, lu, ul, lu, ul};
        const int32_t* Z[32] = {lu, lu, ul, ul, lu, ul, ll, lu, ul, uu, ll, lu, ul, uu, lu, ul,
                                lu, ul, ll, lu, ul, uu, ll, lu, ul, uu, lu, ul, lu, lu, ul, ul};
        float v[32];
        bool ok = true;
        for (int i = 0; i < 32 && ok; ++i) {
            const int32_t c[3] = {X[i][0], Y[i][1], Z[i][2]};
            OccData d;
            int rs = -1;
            if (!occ_data_at(m, slot_block(oct), c, scale, d, rs) || !occ_valid(d) || rs != scale)
                ok = false;
            else
                v[i] = occ_field(d);
        }
        if (!ok)
            continue;
        const float rx = 1.0f - fac.x, ry = 1.0f - fac.y, rz = 1.0f - fac.z;
        const float gx = (((v[19] - v[0]) * rx + (v[28] - v[7]) * fac.x) * ry
                          + ((v[23] - v[1]) * rx + (v[29] - v[11]) * fac.x) * fac.y) * rz
            + (((v[20] - v[2]) * rx + (v[30] - v[8]) * fac.x) * ry
               + ((v[24] - v[3]) * rx + (v[31] - v[12]) * fac.x) * fac.y) * fac.z;
        const float gy = (((v[11] - v[4]) * rx + (v[23] - v[16]) * fac.x) * ry
                          + ((v[14] - v[7]) * rx + (v[26] - v[19]) * fac.x) * fac.y) * rz
            + (((v[12] - v[5]) * rx + (v[24] - v[17]) * fac.x) * ry
               + ((v[15] - v[8]) * rx + (v[27] - v[20]) * fac.x) * fac.y) * fac.z;
        const float gz = (((v[8] - v[6]) * rx + (v[20] - v[18]) * fac.x) * ry
                          + ((v[12] - v[10]) * rx + (v[24] - v[22]) * fac.x) * fac.y) * rz
            + (((v[9] - v[7]) * rx + (v[21] - v[19]) * fac.x) * ry
               + ((v[13] - v[11]) * rx + (v[25] - v[23]) * fac.x) * fac.y) * fac.z;
        const float sf = (float) stride;
        g = v3((0.5f * gx) / sf, (0.5f * gy) / sf, (0.5f * gz) / sf);
        return true;
    }
    return false;
}

static inline bool occ_contains(const so_occ_map& m, V3 p_W)
{
    const V3 p = apply(m.T_MW, p_W);
    return p.x >= 0.0f && p.x < m.dim && p.y >= 0.0f && p.y < m.dim && p.z >= 0.0f && p.z < m.dim;
}

static inline bool occ_interp_W(const so_occ_map& m, V3 p_W, float& out, int* scale)
{
    return occ_interp(m, apply(m.T_MW, p_W) / m.res, 0, out, scale);
}

/* find_valid_point (raycaster_impl.hpp:32-70) */
static bool find_valid_point(const so_occ_map& m, V3 o, V3 d, float step, float t_max, float& t, V3& point_W,
                             float& value)
{
    bool has = false;
    V3 p = o + t * d;
    if (occ_contains(m, p) && occ_valid(occ_get_data(m, p)))
        has = occ_interp_W(m, p, value, nullptr);
    while (!has) {
        t += step;
        if (t > t_max)
            return false;
        p = o + t * d;
        if (occ_contains(m, p) && occ_valid(occ_get_data(m, p)))
            has = occ_interp_W(m, p, value, nullptr);
    }
    point_W = p;
    return true;
}

/* compute_map_intersection (raycaster_impl.hpp:85-173) */
static float compute_map_intersection(const so_occ_map& m, V3 pos_W, V3 dir_W, float t_far, bool& valid)
{
    const V3 p = apply(m.T_MW, pos_W), dr = rot(m.T_MW, dir_W);
    const float pm[3] = {p.x, p.y, p.z}, dm[3] = {dr.x, dr.y, dr.z};
    const float mx = m.dim;
    bool inside = true;
    int quadrant[3];
    float cand[3] = {0.0f, 0.0f, 0.0f}, maxT[3];
    for (int i = 0; i < 3; ++i) {
        if (pm[i] < 0.0f) {
            quadrant[i] = 1;
            cand[i] = 0.0f;
            inside = false;
        }
        else if (pm[i] > mx) {
            quadrant[i] = 0;
            cand[i] = mx;
            inside = false;
        }
        else {
            quadrant[i] = 2;
        }
    }
    if (inside)
        return 0.0f;
    for (int i = 0; i < 3; ++i)
        maxT[i] = (quadrant[i] != 2 && (double) dm[i] != 0.) ? (cand[i] - pm[i]) / dm[i] : -1.0f;
    int which = 0;
    for (int i = 1; i < 3; ++i)
        if (maxT[which] < maxT[i])
            which = i;
    if (maxT[which] < 0.0f) {
        valid = false;
        return 0.0f;
    }
    float hit[3];
    for (int i = 0; i < 3; ++i) {
        if (which != i) {
            hit[i] = pm[i] + maxT[which] * dm[i];
            if (hit[i] < 0.0f || hit[i] > mx) {
                valid = false;
                return 0.0f;
            }
        }
        else {
            hit[i] = cand[i];
        }
    }
    const float t = norm(v3(hit[0] - pm[0], hit[1] - pm[1], hit[2] - pm[2]));
    if (t_far < t) {
        valid = false;
        return 0.0f;
    }
    return t;
}

/* advance_ray (raycaster_impl.hpp:189-338) */
static void advance_ray(const so_occ_map& m, V3 o, V3 d, float& t, float& t_far, int max_scale, bool& valid)
{
    const float voxel_dim = m.res;
    int scale = max_scale;
    float v_add = 0.0f;
    const float v = 1.0f / voxel_dim * t;
    float v_far = 1.0f / voxel_dim * t_far;
    V3 oc = v3(-1.0f, -1.0f, -1.0f);
    if (occ_contains(m, o))
        oc = apply(m.T_MW, o) / m.res;
    const float sz = (float) m.octree.size;
    const float dv[3] = {d.x, d.y, d.z};
    const float ocv[3] = {oc.x, oc.y, oc.z};
    float vmap[3];
    for (int i = 0; i < 3; ++i) {
        const float dvm = sz / std::fabs(dv[i]);
        const float frac = ocv[i] / sz;
        vmap[i] = dv[i] < 0 ? frac * dvm : (1 - frac) * dvm;
    }
    v_far = std::min(std::min(std::min(vmap[0], vmap[1]), vmap[2]) + v, v_far);
    t_far = voxel_dim * v_far;
    auto max_field = [&](V3 c, int s) {
        const int32_t ci[3] = {(int) c.x, (int) c.y, (int) c.z};
        return occ_field(occ_max_data(m, ci, s));
    };
    float f = max_field(oc, scale);
    while (f > -0.2f && scale > 2) {
        scale -= 1;
        f = max_field(oc, scale);
    }
    V3 rc = oc;
    while ((v + v_add) < v_far) {
        if (scale <= 2) {
            t = voxel_dim * (v + v_add - 4);
            return;
        }
        const int node_size = 1 << scale;
        const float rcv[3] = {rc.x, rc.y, rc.z};
        float Vmax[3];
        for (int i = 0; i < 3; ++i) {
            const int curr = node_size * (int) (std::floor(rcv[i]) / (float) node_size);
            const float frac = (rcv[i] - (float) curr) / (float) node_size;
            const float dV = (float) node_size / std::fabs(dv[i]);
            Vmax[i] = dv[i] < 0 ? frac * dV : (1 - frac) * dV;
            if (std::fabs(dv[i]) < 1.0e-6f)
                Vmax[i] = std::numeric_limits<float>::infinity();
        }
        const float Vmin = std::min(std::min(Vmax[0], Vmax[1]), Vmax[2]);
        v_add = (float) ((double) v_add + ((double) Vmin + 0.01));
        rc = (v + v_add) * d + oc;
        f = max_field(rc, scale);
        if (f > -0.2f) {
            while (f > -0.2f && scale > 2) {
                scale -= 1;
                f = max_field(rc, scale);
            }
        }
        else {
            for (int s = scale + 1; s <= max_scale; s++) {
                f = max_field(rc, s);
                if (f > -0.2f)
                    break;
                scale += 1;
            }
        }
    }
    valid = false;
}

/* raycast<Occupancy> (raycaster_impl.hpp:352-452). Returns 0 no hit, 1 hit; *zero_hit is set
 * when the reference returns its all-zero intersection (a hit at the origin with scale 0). */
static int raycast_occ(const so_occ_map& m, V3 o, V3 d, float t_far, V3& hit, int& scale_out)
{
    bool valid = true;
    float t = compute_map_intersection(m, o, d, t_far, valid);
    if (!valid)
        return 0;
    const int max_scale = std::min(7, (int) std::lround(std::log2((double) m.octree.size)) - 1);
    advance_ray(m, o, d, t, t_far, max_scale, valid);
    if (!valid)
        return 0;
    const float step = m.res / 2;
    float value_t = 0.0f, value_tt = 0.0f;
    bool has_tt = false;
    V3 pt = v3(0.0f, 0.0f, 0.0f), ptt = v3(0.0f, 0.0f, 0.0f);
    int scale_tt = 0;
    if (!find_valid_point(m, o, d, step, t_far, t, pt, value_t))
        return 0;
    t += step;
    if (value_t <= 0.0f) {
        for (; t < t_far; t += step) {
            const V3 p = o + d * t;
            const OccData data = occ_get_data(m, p);
            if (!occ_valid(data)) {
                t += step;
                if (!find_valid_point(m, o, d, step, t_far, t, pt, value_t)) {
                    hit = v3(0.0f, 0.0f, 0.0f);
                    scale_out = 0;
                    return 1;
                }
                if (value_t > 0.0f)
                    break;
                continue;
            }
            value_tt = occ_field(data);
            has_tt = true;
            ptt = p;
            if (value_tt > -0.2f) {
                float vi;
                int sc = scale_tt;
                if (occ_interp_W(m, p, vi, &sc)) {
                    value_tt = vi;
                    scale_tt = sc;
                }
                else {
                    has_tt = false;
                    t += step;
                    if (!find_valid_point(m, o, d, step, t_far, t, pt, value_t))
                        return 0;
                    if (value_t > 0.0f)
                        break;
                    continue;
                }
            }
            if (value_tt > 0.0f)
                break;
            value_t = value_tt;
            pt = ptt;
        }
        /* an empty value_tt (no sample assigned it) gives no hit */
        if (has_tt && value_tt > 0.0f && value_t < 0.0f) {
            t = t - norm(ptt - pt) * (value_tt - 0.0f) / (value_tt - value_t);
            hit = o + d * t;
            scale_out = scale_tt;
            return 1;
        }
    }
    return 0;
}

} // namespace

/* ------------------------------------------------------------------------ C API -- */

namespace {

/* ------------------------------------------------------------------- ray integrator -- */
/* se::RayIntegrator<OccupancyMap<Res::Multi>, LeicaLidar> (include/se/integrator/
 * ray_integrator.hpp, impl/ray_integrator_impl.hpp, impl/ray_integrator_core_impl.hpp) as
 * IntegrateRayBatchImplD<Occupancy, Multi>::integrate drives it (map_integrator_impl.hpp:
 * 137-176): every ray of the batch in order, then the updated blocks up to their coarsest scale,
 * then the nodes above them up to the root. */

struct Leica {
    float near_plane, far_plane;
    float pixel_dim_tan; /* 2 tan(min(azimuth, elevation resolution) / 2), leica_lidar.cpp:53-73 */
};

static Leica make_leica(const so_leica* c)
{
    Leica L;
    L.near_plane = c->near_plane;
    L.far_plane = c->far_plane;
    const float min_ray_angle = std::min(c->azimuth_resolution_deg, c->elevation_resolution_deg);
    const float deg_to_rad = (float) (M_PI / 180.0);
    L.pixel_dim_tan = 2.0f * std::tan(min_ray_angle * 0.5f * deg_to_rad);
    return L;
}

/* LeicaLidar::computeIntegrationScaleImpl (leica_lidar.cpp:87-129), ratios {1.5, 3, 6}. */
static int leica_integration_scale(const Leica& L, V3 c, float res, int last_scale, int min_scale, int max_scale)
{
    static const float kRatio[3] = {1.5f, 3.0f, 6.0f};
    const float dist = norm(c);
    const float pixel_dim = dist * L.pixel_dim_tan;
    const float den = 1.0f / (std::sqrt(3.0f) * res);
    const float pv = pixel_dim * den;
    int scale = 0;
    for (float r : kRatio) {
        if (pv < r)
            break;
        scale++;
    }
    scale = std::min(scale, max_scale);
    if (scale > last_scale && min_scale != -1)
        return leica_integration_scale(L, c - 0.25f * normalized(c), res, last_scale, -1, max_scale);
    if (scale < last_scale && min_scale != -1)
        return leica_integration_scale(L, c + 0.25f * normalized(c), res, last_scale, -1, max_scale);
    return scale;
}

enum class RayState { FreeSpace, Transition, Occupied, Undefined };

/* ray_integrator::propagate_block_down_to_scale (ray_integrator_core_impl.hpp:358-426) */
static void ri_propagate_down(OccBlock& b, int desired)
{
    int cur = b.current_scale;
    while (cur > desired) {
        b.allocate_down_to(cur - 1);
        b.current_scale = cur - 1;
        const int cs = cur - 1, ps = cur;
        const int nc = 8 >> cs, np = 8 >> ps;
        const OccData* pd = b.mean_at(ps);
        OccData* cd = b.mean_at(cs);
        for (int z = 0; z < np; z++)
            for (int y = 0; y < np; y++)
                for (int x = 0; x < np; x++) {
                    const OccData& p = pd[x + y * np + z * np * np];
                    if (!p.observed)
                        continue;
                    for (int k = 0; k < 2; k++)
                        for (int j = 0; j < 2; j++)
                            for (int i = 0; i < 2; i++) {
                                OccData& c = cd[(2 * x + i) + (2 * y + j) * nc + (2 * z + k) * nc * nc];
                                c.weight = p.weight;
                                c.occ = p.occ;
                                c.observed = false;
                            }
                }
        cur--;
    }
}

/* The parent-entry tail shared by both loops of propagate_block_to_scale. */
struct RiAcc {
    float mean_occ = 0.0f, mean_w = 0.0f;
    float min_mean = 0.0f, min_w = 0.0f, min_o = std::numeric_limits<float>::max();
    float max_mean = 0.0f, max_w = 0.0f, max_o = std::numeric_limits<float>::lowest();
    int count = 0, observed = 0;
    void store(OccData& pmean, OccData& pmin, OccData& pmax) const
    {
        if (count > 0) {
            pmean.occ = mean_occ / (float) count;
            pmean.weight = std::ceil(mean_w) / (float) count;
            pmean.observed = false;
            pmin.occ = min_mean;
            pmin.weight = min_w;
            pmax.occ = max_mean;
            pmax.weight = max_w;
            if (observed == 8) {
                pmax.observed = true;
                pmin.observed = true;
            }
        }
    }
};

/* ray_integrator::propagate_block_to_scale (ray_integrator_core_impl.hpp:206-352): the first
 * coarser scale from the mean data (a child sets the minimum only when it did not set the
 * maximum), every further scale from the child min / max data. */
static void ri_propagate_to_scale(OccBlock& b, int desired)
{
    int cs = b.current_scale;
    int ps = cs + 1;
    {
        const int nc = 8 >> cs, np = 8 >> ps;
        const OccData* cmean = b.mean_at(cs);
        OccData *pmean = b.mean_at(ps), *pmin = b.min_at(ps), *pmax = b.max_at(ps);
        for (int z = 0; z < np; z++)
            for (int y = 0; y < np; y++)
                for (int x = 0; x < np; x++) {
                    RiAcc a;
                    for (int k = 0; k < 2; k++)
                        for (int j = 0; j < 2; j++)
                            for (int i = 0; i < 2; i++) {
                                const OccData& c = cmean[(2 * x + i) + (2 * y + j) * nc + (2 * z + k) * nc * nc];
                                if (c.weight > 0.0f) {
                                    a.count++;
                                    a.mean_occ += c.occ;
                                    a.mean_w += c.weight;
                                    const float o = occ_field(c);
                                    if (o > a.max_o) {
                                        a.max_mean = c.occ;
                                        a.max_w = c.weight;
                                        a.max_o = o;
                                    }
                                    else if (o < a.min_o) {
                                        a.min_mean = c.occ;
                                        a.min_w = c.weight;
                                        a.min_o = o;
                                    }
                                }
                                if (c.observed)
                                    a.observed++;
                            }
                    const int pi = x + y * np + z * np * np;
                    a.store(pmean[pi], pmin[pi], pmax[pi]);
                }
    }
    for (ps += 1; ps <= desired; ++ps) {
        cs = ps - 1;
        const int nc = 8 >> cs, np = 8 >> ps;
        const OccData *cmean = b.mean_at(cs), *cmin = b.min_at(cs), *cmax = b.max_at(cs);
        OccData *pmean = b.mean_at(ps), *pmin = b.min_at(ps), *pmax = b.max_at(ps);
        for (int z = 0; z < np; z++)
            for (int y = 0; y < np; y++)
                for (int x = 0; x < np; x++) {
                    RiAcc a;
                    for (int k = 0; k < 2; k++)
                        for (int j = 0; j < 2; j++)
                            for (int i = 0; i < 2; i++) {
                                const int ci = (2 * x + i) + (2 * y + j) * nc + (2 * z + k) * nc * nc;
                                if (cmax[ci].weight > 0.0f) {
                                    a.count++;
                                    a.mean_occ += cmean[ci].occ;
                                    a.mean_w += cmean[ci].weight;
                                    const float mo = occ_field(cmax[ci]);
                                    if (mo > a.max_o) {
                                        a.max_mean = cmax[ci].occ;
                                        a.max_w = cmax[ci].weight;
                                        a.max_o = mo;
                                    }
                                    const float no = occ_field(cmin[ci]);
                                    if (no < a.min_o) {
                                        a.min_mean = cmin[ci].occ;
                                        a.min_w = cmin[ci].weight;
                                        a.min_o = no;
                                    }
                                }
                                if (cmax[ci].observed)
                                    a.observed++;
                            }
                    const int pi = x + y * np + z * np * np;
                    a.store(pmean[pi], pmin[pi], pmax[pi]);
                }
    }
}

/* ray_integrator::propagate_to_parent_node (ray_integrator_core_impl.hpp:104-176) */
static OccData ri_propagate_node(OccOctree& oct, int n, int timestamp)
{
    OccNode& node = oct.nodes[(size_t) n];
    node.timestamp = timestamp;
    float max_o = std::numeric_limits<float>::lowest(), max_mean = 0.0f, max_w = 0.0f;
    float min_o = std::numeric_limits<float>::max(), min_mean = 0.0f, min_w = 0.0f;
    int max_cnt = 0, min_cnt = 0, observed = 0;
    for (int i = 0; i < 8; ++i) {
        const int c = node.child[i];
        if (c == -1)
            continue;
        OccData cmin, cmax;
        if (slot_is_block(c)) {
            OccBlock& b = oct.blocks[(size_t) slot_block(c)];
            cmin = b.min_data();
            cmax = b.max_data();
        }
        else {
            cmin = oct.nodes[(size_t) c].min_data;
            cmax = oct.nodes[(size_t) c].max_data;
        }
        if (cmin.weight > 0.0f) {
            const float o = occ_field(cmin);
            if (o < min_o) {
                min_mean = cmin.occ;
                min_w = cmin.weight;
                min_o = o;
                min_cnt++;
            }
        }
        if (cmax.weight > 0.0f) {
            const float o = occ_field(cmax);
            if (o > max_o) {
                max_mean = cmax.occ;
                max_w = cmax.weight;
                max_o = o;
                max_cnt++;
            }
        }
        if (cmax.observed)
            observed++;
    }
    if (min_cnt > 0) {
        node.min_data.occ = min_mean;
        node.min_data.weight = min_w;
        if (observed == 8)
            node.min_data.observed = true;
    }
    if (max_cnt > 0) {
        node.max_data.occ = max_mean;
        node.max_data.weight = max_w;
        if (observed == 8)
            node.max_data.observed = true;
    }
    return node.max_data;
}

/* An octant of the updated-octants set: (x, y, z, size), size 8 for a block. */
typedef std::array<int32_t, 4> OctKey;

struct RayIntegrator {
    so_occ_map& m;
    const Leica& L;
    float sigma_min, sigma_max, tau_min, tau_max;
    int timestamp;
    std::vector<int> updated_blocks;  /* updated_blocks_vector_ */
    std::set<int> updated_set;        /* updated_blocks_set_ */
    std::set<OctKey>* updated_octants;
    /* per ray (resetIntegrator) */
    Tf T_SW;
    V3 ray;
    float ray_dist = 0.0f, tau = 0.0f, three_sigma = 0.0f;
    int32_t last_voxel[3] = {-1, -1, -1};
    int computed_scale = 0;

    RayIntegrator(so_occ_map& mm, const Leica& LL, int ts, std::set<OctKey>* upd) : m(mm), L(LL), timestamp(ts),
                                                                                 updated_octants(upd)
    {
        /* RayIntegratorConfig (ray_integrator.hpp:60-72) */
        sigma_min = m.cfg.sigma_min_factor * m.res;
        sigma_max = m.cfg.sigma_max_factor * m.res;
        tau_min = m.cfg.tau_min_factor * m.res;
        tau_max = m.cfg.tau_max_factor * m.res;
    }

    /* resetIntegrator without the skip test (ray_integrator_impl.hpp:45-78) */
    void reset(V3 r, const Tf& T_WS)
    {
        ray = r;
        ray_dist = norm(r);
        T_SW = inverse_iso(T_WS);
        computed_scale = 0;
        tau = compute_tau(ray_dist, tau_min, tau_max, m.cfg);
        three_sigma = 3.0f * std::clamp(m.cfg.k_sigma * ray_dist, sigma_min, sigma_max);
        last_voxel[0] = last_voxel[1] = last_voxel[2] = -1;
    }

    /* computeVariance (ray_integrator_impl.hpp:135-158) */
    RayState variance(float depth) const
    {
        const float z_diff = depth - ray_dist;
        if (z_diff < -three_sigma)
            return RayState::FreeSpace;
        if ((double) z_diff < (double) tau / 2.0)
            return RayState::Transition;
        if (z_diff < tau)
            return RayState::Occupied;
        return RayState::Undefined;
    }

    /* updateBlock (ray_integrator_impl.hpp:232-300) */
    void update_block(int bi, const int32_t v[3], int desired, float sample_dist)
    {
        if ((double) sample_dist < 1e-08)
            return;
        OccBlock& b = m.octree.blocks[(size_t) bi];
        const bool already = b.timestamp == timestamp;
        if (!already)
            b.timestamp = timestamp;
        const int last_scale = b.min_scale == -1 ? desired : b.current_scale;
        int s = last_scale;
        if (b.min_scale == -1) {
            b.allocate_down_to(s);
            b.init_data = OccData();
        }
        else if (desired < last_scale) {
            ri_propagate_down(b, desired);
            s = desired;
        }
        else if (!already && desired > last_scale) {
            ri_propagate_to_scale(b, desired);
            s = desired;
            b.delete_up_to(s);
            b.current_scale = s;
        }
        const int stride = 1 << s, n = 8 >> s;
        const int ox = (v[0] - b.coord[0]) / stride, oy = (v[1] - b.coord[1]) / stride,
                  oz = (v[2] - b.coord[2]) / stride;
        OccData& d = b.mean_at(s)[ox + n * oy + n * n * oz];
        update_voxel(d, sample_dist - ray_dist, tau, three_sigma, m.cfg);
    }

    /* operator()(ray_sample, voxel_coord, rayState, octant) for LeicaLidar
     * (ray_integrator_impl.hpp:162-228): descend to the block, allocating on the way. */
    void sample(V3 r_S, const int32_t v[3], RayState state)
    {
        OccOctree& o = m.octree;
        int slot;
        for (;;) {
            slot = occ_finest_octant(o, v, 0);
            if (slot_is_block(slot))
                break;
            /* A node of an occupancy octree has no children or all eight (allocateChildren,
             * deleteChildren), so the descent always ends at a block or a childless node. */
            if (slot < 0)
                return;
            o.allocate_children(slot);
        }
        const int bi = slot_block(slot);
        OccBlock& b = o.blocks[(size_t) bi];
        const int last_scale = b.min_scale == -1 ? 0 : b.current_scale;
        const V3 c_W = occ_voxel_to_point(m, b.coord, 8);
        const V3 c_S = apply(T_SW, c_W);
        int scale = leica_integration_scale(L, c_S, m.res, last_scale, b.min_scale, kOccMaxScale);
        const int fs = m.cfg.fs_integr_scale;
        if (state == RayState::FreeSpace && scale < fs)
            scale = b.min_scale == -1 ? fs : std::min(fs, b.current_scale);
        update_block(bi, v, scale, norm(r_S));
        computed_scale = scale;
        if (updated_set.count(bi) == 0) {
            updated_set.insert(bi);
            updated_blocks.push_back(bi);
        }
        if (updated_octants)
            updated_octants->insert(OctKey{b.coord[0], b.coord[1], b.coord[2], 8});
    }

    /* operator()() (ray_integrator_impl.hpp:82-129) */
    void run()
    {
        m.octree.allocate_children(0);
        if (ray_dist < L.near_plane)
            return;
        const V3 dir = normalized(ray);
        const float max_dist = std::min(ray_dist + tau, L.far_plane);
        V3 r = L.near_plane * dir;
        const Tf T_WS = inverse_iso(T_SW);
        while (norm(r) < max_dist) {
            const RayState state = variance(norm(r));
            const V3 r_W = apply(T_WS, r);
            const V3 p_M = apply(m.T_MW, r_W);
            if (!(p_M.x >= 0.0f && p_M.x < m.dim && p_M.y >= 0.0f && p_M.y < m.dim && p_M.z >= 0.0f && p_M.z < m.dim))
                break;
            const V3 vf = p_M / m.res;
            const int32_t v[3] = {(int32_t) vf.x, (int32_t) vf.y, (int32_t) vf.z};
            if (v[0] != last_voxel[0] || v[1] != last_voxel[1] || v[2] != last_voxel[2]) {
                last_voxel[0] = v[0];
                last_voxel[1] = v[1];
                last_voxel[2] = v[2];
                sample(r, v, state);
            }
            const float step = (float) (0.5 * (double) m.res * (double) (1 << computed_scale));
            r = r + step * dir;
        }
    }

    /* propagateBlocksToCoarsestScale (ray_integrator_impl.hpp:124-132) */
    void propagate_blocks()
    {
        for (int bi : updated_blocks) {
            OccBlock& b = m.octree.blocks[(size_t) bi];
            if (b.current_scale != kOccMaxScale)
                ri_propagate_to_scale(b, kOccMaxScale);
        }
    }

    /* propagateToRoot (ray_integrator_impl.hpp:304-354) */
    void propagate_to_root()
    {
        OccOctree& o = m.octree;
        const int bd = o.block_depth();
        std::vector<std::set<int>> node_set((size_t) std::max(bd, 1));
        for (int bi : updated_blocks)
            if (o.blocks[(size_t) bi].parent >= 0)
                node_set[(size_t) bd - 1].insert(o.blocks[(size_t) bi].parent);
        for (int d = bd - 1; d > 0; d--) {
            for (int n : node_set[(size_t) d]) {
                if (o.nodes[(size_t) n].timestamp == timestamp)
                    continue;
                if (o.nodes[(size_t) n].parent < 0)
                    continue;
                const OccData nd = ri_propagate_node(o, n, timestamp);
                node_set[(size_t) d - 1].insert(o.nodes[(size_t) n].parent);
                const OccNode& N = o.nodes[(size_t) n];
                const OctKey key{N.coord[0], N.coord[1], N.coord[2], N.size};
                if (updated_octants)
                    updated_octants->insert(key);
                if (nd.observed && (double) occ_field(nd) <= 0.95 * (double) kMinOccupancy) {
                    if (updated_octants && !N.is_leaf())
                        updated_octants->erase(key);
                    o.delete_children(n);
                }
            }
        }
        ri_propagate_node(o, 0, timestamp);
    }
};

/* An occupancy map seen by the dual marching cubes: BlockMultiRes<Occupancy>::data(voxel, scale)
 * (block_impl.hpp:326-340: the init data below the finest allocated scale), get_field =
 * occupancy * weight (data.hpp:123-127), is_valid = weight != 0 (data_field_impl.hpp:12-15),
 * is_inside = field > 0 (data.hpp:139-143); fetcher::block by descent from the root. */
struct OccView {
    const OccOctree& o;
    int size() const { return o.size; }
    int num_blocks() const { return (int) o.blocks.size(); }
    bool live(int b) const { return o.block_live[(size_t) b] != 0; }
    const int32_t* coord(int b) const { return o.blocks[(size_t) b].coord; }
    int current_scale(int b) const { return o.blocks[(size_t) b].current_scale; }
    int block_at(const int32_t c[3]) const
    {
        const int s = o.leaf(c);
        return (s != -1 && slot_is_block(s)) ? slot_block(s) : -1;
    }
    bool data(int b, const int32_t c[3], int scale, float& field) const
    {
        const OccBlock& B = o.blocks[(size_t) b];
        const OccData& d = scale < B.finest ? B.init_data : B.mean[kOccScaleOffset[scale] + B.voxel_idx(c, scale)];
        field = occ_field(d);
        return occ_valid(d);
    }
    bool inside(float field) const { return field > 0.0f; }
};

} // namespace

extern "C" {

so_occ_map* so_occ_map_create(const float dim[3], float res, const float* T_MW)
{
    so_occ_map* m = new so_occ_map();
    const float dmax = std::max(std::max(dim[0], dim[1]), dim[2]);
    const int requested = (int) std::ceil(dmax / res);
    int sz = 1;
    while (sz < std::max(requested, 16))
        sz <<= 1;
    m->octree.init(sz);
    m->res = res;
    m->dim = (float) sz * res;
    if (T_MW) {
        m->T_MW = tf_from16(T_MW);
    }
    else {
        m->T_MW = tf_identity();
        m->T_MW.t[0] = dim[0] / 2.0f;
        m->T_MW.t[1] = dim[1] / 2.0f;
        m->T_MW.t[2] = dim[2] / 2.0f;
    }
    m->T_WM = inverse_iso(m->T_MW);
    m->cfg = default_occ_config();
    return m;
}

so_occ_map* so_occ_map_create_cfg(const float dim[3], float res, const float* T_MW, const float cfg[9])
{
    so_occ_map* m = so_occ_map_create(dim, res, T_MW);
    if (cfg) {
        m->cfg.k_sigma = cfg[0];
        m->cfg.sigma_min_factor = cfg[1];
        m->cfg.sigma_max_factor = cfg[2];
        m->cfg.k_tau = cfg[3];
        m->cfg.tau_min_factor = cfg[4];
        m->cfg.tau_max_factor = cfg[5];
        m->cfg.log_odd_min = cfg[6];
        m->cfg.log_odd_max = cfg[7];
        m->cfg.fs_integr_scale = (int) cfg[8];
    }
    return m;
}

void so_occ_map_destroy(so_occ_map* m) { delete m; }

/* Map::getData(point) (Safe::Off): the leaf's data, a block's at its current scale. */
void so_occ_get_data(const so_occ_map* mp, const float p[3], float out[3])
{
    const OccData d = occ_get_data(*mp, v3(p[0], p[1], p[2]));
    out[0] = d.occ;
    out[1] = d.weight;
    out[2] = d.observed ? 1.0f : 0.0f;
}

/* Map::getFieldInterp(point) (Safe::Off). Returns 0 for nullopt. */
int so_occ_get_field_interp(const so_occ_map* mp, const float p[3], float* value, int* scale)
{
    const V3 pm = apply(mp->T_MW, v3(p[0], p[1], p[2]));
    int sc = 0;
    float v = 0.0f;
    if (!occ_interp(*mp, pm / mp->res, 0, v, &sc))
        return 0;
    *value = v;
    if (scale)
        *scale = sc;
    return 1;
}

/* Map::getFieldGrad(point) (Safe::Off, map_impl.hpp:238-265): the multi-res gradient at the point's
 * voxel coordinates, divided by the resolution. Returns 0 for nullopt. */
int so_occ_get_field_grad(const so_occ_map* mp, const float p[3], float g[3])
{
    const V3 pm = apply(mp->T_MW, v3(p[0], p[1], p[2]));
    V3 gv;
    if (!occ_grad(*mp, pm / mp->res, gv))
        return 0;
    g[0] = gv.x / mp->res;
    g[1] = gv.y / mp->res;
    g[2] = gv.z / mp->res;
    return 1;
}

/* MapIntegrator<OccupancyMap<Res::Multi>>::integrateDepth after the sensor-specific frame set-up:
 * sigma image, pooling images, VolumeCarver, Updater (map_integrator_impl.hpp:96-125). */
static void occ_integrate_frame(so_occ_map& m, Frame& f, const float* depth, const float T_WC[16], float far_plane,
                                int timestamp, so_occ_stats* stats)
{
    OccOctree& oct = m.octree;
    f.m = &m;
    f.T_WS = tf_from16(T_WC);
    f.T_SW = inverse_iso(f.T_WS);
    f.depth = depth;
    const int npx = f.w * f.h;
    f.sigma.resize((size_t) npx);
    depth_sigma(depth, npx, m.res, m.cfg, f.sigma.data());
    f.sigma_min = m.cfg.sigma_min_factor * m.res;
    f.sigma_max = m.cfg.sigma_max_factor * m.res;
    f.tau_min = m.cfg.tau_min_factor * m.res;
    f.tau_max = m.cfg.tau_max_factor * m.res;
    f.depth_pool.build(depth, f.w, f.h, f.lidar);
    f.sigma_pool.build(f.sigma.data(), f.w, f.h, f.lidar);
    f.max_depth_value = std::min(far_plane, f.depth_pool.max_value + f.tau_max);

    /* VolumeCarver::operator()(), volume_carver_impl.hpp:46-70 */
    Allocation alloc;
    oct.allocate_children(0);
    const int csize = oct.size / 2;
    for (int i = 0; i < 8; ++i) {
        int32_t cc[3];
        for (int a = 0; a < 3; ++a)
            cc[a] = csize * ((i >> a) & 1);
        if (f.lidar)
            carve_lidar(m, f, cc, csize, 1, oct.nodes[0].child[i], alloc);
        else
            carve(m, f, cc, csize, 1, oct.nodes[0].child[i], alloc);
    }
    for (int n : alloc.node_list)
        if (oct.nodes[n].is_leaf())
            oct.aabb_extend(oct.nodes[n].coord, oct.nodes[n].size);

    /* Updater::operator(), multires_ofusion_updater_impl.hpp:59-125 */
    UpdaterState st;
    st.node_set.assign((size_t) std::max(oct.block_depth(), 1), std::set<int>());
    for (int n : alloc.node_list) {
        const int depth = (int) std::lround(std::log2((double) oct.size)) - (int) std::lround(std::log2((double) oct.nodes[n].size));
        free_node_recurse(m, f, n, depth, st);
    }
#pragma omp parallel for
    for (long long i = 0; i < (long long) alloc.block_list.size(); ++i)
        update_block(m, f, oct.blocks[alloc.block_list[i]], alloc.var_list[i] == VarState::Constant,
                     alloc.inside_list[i] != 0);
#pragma omp parallel for
    for (long long i = 0; i < (long long) alloc.block_list.size(); ++i)
        propagate_block(oct.blocks[alloc.block_list[i]]);
#pragma omp parallel for
    for (long long i = 0; i < (long long) st.freed_blocks.size(); ++i)
        propagate_block(oct.blocks[st.freed_blocks[i]]);

    /* Updater::propagateToRoot, multires_ofusion_updater_impl.hpp:129-164 */
    const int bd = oct.block_depth();
    long long n_pruned = 0;
    for (int b : alloc.block_list)
        if (oct.blocks[b].parent >= 0)
            st.node_set[bd - 1].insert(oct.blocks[b].parent);
    for (int d = bd - 1; d > 0; d--) {
        for (int n : st.node_set[d]) {
            if (oct.nodes[n].timestamp == timestamp)
                continue;
            if (oct.nodes[n].parent >= 0) {
                const OccData nd = propagate_to_parent_node(oct, n, timestamp);
                st.node_set[d - 1].insert(oct.nodes[n].parent);
                if (nd.observed && (double) occ_field(nd) <= 0.95 * (double) kMinOccupancy) {
                    oct.delete_children(n);
                    ++n_pruned;
                }
            }
        }
    }
    propagate_to_parent_node(oct, 0, timestamp);
    if (stats) {
        stats->n_blocks_listed = (long long) alloc.block_list.size();
        stats->n_nodes_listed = (long long) alloc.node_list.size();
        stats->n_blocks_freed = (long long) st.freed_blocks.size();
        stats->n_nodes_pruned = n_pruned;
    }
}

void so_occ_integrate_depth(so_occ_map* mp, const float* depth, const so_pinhole* sensor, const float T_WC[16],
                            int timestamp, so_occ_stats* stats)
{
    Frame f;
    f.s = make_pinhole(sensor);
    f.w = sensor->width;
    f.h = sensor->height;
    occ_integrate_frame(*mp, f, depth, T_WC, f.s.far_plane, timestamp, stats);
}

void so_occ_integrate_lidar(so_occ_map* mp, const float* range, const so_lidar* sensor, const float T_WS[16],
                            int timestamp, so_occ_stats* stats)
{
    Frame f;
    f.lidar = true;
    f.L = make_lidar(sensor);
    f.w = sensor->width;
    f.h = sensor->height;
    occ_integrate_frame(*mp, f, range, T_WS, f.L.far_plane, timestamp, stats);
}

int so_lidar_project(const so_lidar* sensor, const float p_S[3], float uv[2])
{
    const Lidar L = make_lidar(sensor);
    return lidar_project(L, v3(p_S[0], p_S[1], p_S[2]), uv[0], uv[1]) ? 1 : 0;
}

float so_atan2(float y, float x) { return atan2_as(y, x); }

float so_lidar_tan_half_min_angle(const so_lidar* sensor) { return make_lidar(sensor).tan_half_min_angle; }

int so_occ_lidar_integration_scale(const so_lidar* sensor, const float c_S[3], float res, int last_scale,
                                   int min_scale)
{
    const Lidar L = make_lidar(sensor);
    return lidar_integration_scale(L, v3(c_S[0], c_S[1], c_S[2]), res, last_scale, min_scale, kOccMaxScale);
}

/* DensePoolingImage<OusterLidar>: the same layout as so_occ_pooling_image */
int so_occ_pooling_image_lidar(const float* depth, int w, int h, float* out, float* max_value)
{
    PoolingImage P;
    P.build(depth, w, h, true);
    if (out)
        for (int l = 0; l <= P.max_level; ++l)
            for (int i = 0; i < w * h; ++i) {
                const PPixel& p = P.img[(size_t) l][(size_t) i];
                float* o = out + 4 * ((size_t) l * w * h + i);
                o[0] = p.min;
                o[1] = p.max;
                o[2] = (float) p.crossing;
                o[3] = (float) p.known;
            }
    if (max_value)
        *max_value = P.max_value;
    return P.max_level;
}

/* MapIntegrator::integrateRayBatch for a multi-res occupancy map and a LeicaLidar
 * (map_integrator_impl.hpp:137-176): rays[3 i] (sensor frame) with poses[16 i] (T_WS, row-major),
 * in order; writes up to capacity updated octants (x, y, z, size) and returns their number. */
long long so_occ_integrate_ray_batch(so_occ_map* mp, const so_leica* sensor, const float* poses, const float* rays,
                                     long long n, int timestamp, int32_t* octants, long long capacity)
{
    const Leica L = make_leica(sensor);
    std::set<OctKey> updated;
    RayIntegrator ri(*mp, L, timestamp, &updated);
    for (long long i = 0; i < n; ++i) {
        ri.reset(v3(rays[3 * i], rays[3 * i + 1], rays[3 * i + 2]), tf_from16(poses + 16 * i));
        ri.run();
    }
    ri.propagate_blocks();
    ri.propagate_to_root();
    long long k = 0;
    for (const OctKey& key : updated) {
        if (octants && k < capacity)
            for (int a = 0; a < 4; ++a)
                octants[4 * k + a] = key[(size_t) a];
        ++k;
    }
    return k;
}

/* LeicaLidar::computeIntegrationScale for a block centre in the sensor frame. */
int so_leica_integration_scale(const so_leica* sensor, const float c_S[3], float res, int last_scale, int min_scale)
{
    const Leica L = make_leica(sensor);
    return leica_integration_scale(L, v3(c_S[0], c_S[1], c_S[2]), res, last_scale, min_scale, kOccMaxScale);
}

/* Block timestamps of the live blocks in allocation order (Octant::timestamp). */
void so_occ_block_timestamps(const so_occ_map* mp, int32_t* ts)
{
    long long k = 0;
    for (size_t i = 0; i < mp->octree.blocks.size(); ++i)
        if (mp->octree.block_live[i])
            ts[k++] = mp->octree.blocks[i].timestamp;
}

long long so_occ_num_blocks(const so_occ_map* m)
{
    long long n = 0;
    for (char l : m->octree.block_live)
        n += l ? 1 : 0;
    return n;
}

long long so_occ_num_nodes(const so_occ_map* m) { return (long long) m->octree.nodes.size(); }

/* Test set-up: allocates the path to the block holding voxel c (Octree::allocateChildren at
 * every level, as integration does) and sets the block's current and minimum scale and its mean
 * pyramid (585 x (occupancy, weight, observed)), the finest scale taken as 0. */
void so_occ_set_block(so_occ_map* mp, const int32_t c[3], int current_scale, int min_scale, const float* mean585)
{
    OccOctree& o = mp->octree;
    int n = 0;
    int slot = -1;
    for (int cs = o.size >> 1; cs >= 8; cs >>= 1) {
        const int idx = ((c[0] & cs) > 0) + 2 * ((c[1] & cs) > 0) + 4 * ((c[2] & cs) > 0);
        if (o.nodes[(size_t) n].child[idx] == -1)
            o.allocate_children(n);
        slot = o.nodes[(size_t) n].child[idx];
        if (slot_is_block(slot))
            break;
        n = slot;
    }
    if (slot == -1 || !slot_is_block(slot))
        return;
    OccBlock& b = o.blocks[(size_t) slot_block(slot)];
    for (int i = 0; i < 585; ++i) {
        b.mean[i].occ = mean585[3 * i];
        b.mean[i].weight = mean585[3 * i + 1];
        b.mean[i].observed = mean585[3 * i + 2] != 0.0f;
    }
    b.finest = 0;
    b.current_scale = current_scale;
    b.min_scale = min_scale;
}

/* Dual marching cubes of an occupancy map (algorithms::marching_cube for Res::Multi,
 * marching_cube_impl.hpp:895-975, 1175-1201): faces (9 floats each, voxel units) between
 * occupied and free space and the integration scale of each face; returns the face count. */
long long so_occ_dual_marching_cubes(const so_occ_map* m, int min_desired_scale, float* faces, int8_t* scales,
                                     long long capacity)
{
    std::vector<int32_t> ntri(256), tri(256 * 24);
    so_mc_table(ntri.data(), tri.data());
    return dual_mc::dual_marching_cubes(OccView{m->octree}, min_desired_scale, ntri.data(), tri.data(), 24, faces,
                                        scales, capacity);
}

/* Live blocks in allocation order: coords (3), scales (current, min, buffer), counters
 * (curr_integr, curr_obs, buffer_integr, buffer_obs), init data, and the 585-entry mean / min /
 * max pyramids as (occupancy, weight, observed) with min / max at the finest scale taken from
 * the mean data; entries below the finest allocated scale are reported as the init data. */
void so_occ_blocks(const so_occ_map* mp, int32_t* coords, int32_t* scales, int64_t* counts, float* mean, float* minv,
                   float* maxv)
{
    so_occ_map& m = *const_cast<so_occ_map*>(mp);
    long long k = 0;
    for (size_t i = 0; i < m.octree.blocks.size(); ++i) {
        if (!m.octree.block_live[i])
            continue;
        OccBlock& b = m.octree.blocks[i];
        if (coords)
            for (int a = 0; a < 3; ++a)
                coords[3 * k + a] = b.coord[a];
        if (scales) {
            scales[3 * k] = b.current_scale;
            scales[3 * k + 1] = b.min_scale;
            scales[3 * k + 2] = b.buffer_scale;
        }
        if (counts) {
            counts[4 * k] = (int64_t) b.curr_integr;
            counts[4 * k + 1] = (int64_t) b.curr_obs;
            counts[4 * k + 2] = (int64_t) b.buf_integr;
            counts[4 * k + 3] = (int64_t) b.buf_obs;
        }
        for (int s = 0; s <= kOccMaxScale; ++s) {
            const int nv = cube(8 >> s);
            for (int v = 0; v < nv; ++v) {
                const size_t o = ((size_t) k * 585 + kOccScaleOffset[s] + v) * 3;
                const OccData e = s < b.finest ? b.init_data : b.mean_at(s)[v];
                const OccData mn = s < b.finest ? b.init_data : b.min_at(s)[v];
                const OccData mx = s < b.finest ? b.init_data : b.max_at(s)[v];
                if (mean) {
                    mean[o] = e.occ;
                    mean[o + 1] = e.weight;
                    mean[o + 2] = e.observed ? 1.0f : 0.0f;
                }
                if (minv) {
                    minv[o] = mn.occ;
                    minv[o + 1] = mn.weight;
                    minv[o + 2] = mn.observed ? 1.0f : 0.0f;
                }
                if (maxv) {
                    maxv[o] = mx.occ;
                    maxv[o + 1] = mx.weight;
                    maxv[o + 2] = mx.observed ? 1.0f : 0.0f;
                }
            }
        }
        ++k;
    }
}

/* Nodes reachable from the root, depth-first in child order: coord (3) + size, and the
 * min / max data as (occupancy, weight, observed); leaf flag. */
long long so_occ_nodes(const so_occ_map* mp, int32_t* coords, float* min_data, float* max_data, int32_t* leaf)
{
    const OccOctree& oct = mp->octree;
    std::vector<int> stack{0};
    long long k = 0;
    while (!stack.empty()) {
        const int n = stack.back();
        stack.pop_back();
        const OccNode& nd = oct.nodes[n];
        if (coords) {
            for (int a = 0; a < 3; ++a)
                coords[4 * k + a] = nd.coord[a];
            coords[4 * k + 3] = nd.size;
        }
        if (min_data) {
            min_data[3 * k] = nd.min_data.occ;
            min_data[3 * k + 1] = nd.min_data.weight;
            min_data[3 * k + 2] = nd.min_data.observed ? 1.0f : 0.0f;
        }
        if (max_data) {
            max_data[3 * k] = nd.max_data.occ;
            max_data[3 * k + 1] = nd.max_data.weight;
            max_data[3 * k + 2] = nd.max_data.observed ? 1.0f : 0.0f;
        }
        if (leaf)
            leaf[k] = nd.is_leaf() ? 1 : 0;
        ++k;
        for (int i = 7; i >= 0; --i)
            if (nd.child[i] >= 0)
                stack.push_back(nd.child[i]);
    }
    return k;
}

int so_occ_map_size(const so_occ_map* m) { return m->octree.size; }

/* raycaster::raycast_volume for occupancy maps (raycaster_impl.hpp:537-627): normals are the
 * negated normalised field gradient (normals_along_gradient is false for occupancy). */
void so_occ_raycast_volume(const so_occ_map* mp, const so_pinhole* sensor_c, const float T_WS_m[16], float* pts_W,
                           float* nrm_W, int8_t* scale)
{
    const so_occ_map& m = *mp;
    const Pinhole s = make_pinhole(sensor_c);
    const Tf T_WS = tf_from16(T_WS_m);
    const V3 origin = v3(T_WS.t[0], T_WS.t[1], T_WS.t[2]);
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < s.h; y++) {
        for (int x = 0; x < s.w; x++) {
            const size_t idx = (size_t) x + (size_t) y * (size_t) s.w;
            const V3 ray_S = back_project(s, (float) x, (float) y);
            const V3 dir_W = rot(T_WS, normalized(ray_S));
            V3 hit;
            int sc = 0;
            V3 p = v3(0.0f, 0.0f, 0.0f), n = v3(0.0f, 0.0f, 0.0f);
            if (raycast_occ(m, origin, dir_W, far_dist(s, ray_S), hit, sc)) {
                p = hit;
                V3 g;
                if (occ_grad(m, apply(m.T_MW, hit) / m.res, g)) {
                    g = g / m.res;
                    const float nn = norm(g);
                    if (nn > 0.0f)
                        n = v3(-(g.x / nn), -(g.y / nn), -(g.z / nn));
                    else
                        n = v3(-g.x, -g.y, -g.z);
                }
            }
            else {
                sc = 0;
            }
            scale[idx] = (int8_t) sc;
            pts_W[3 * idx + 0] = p.x;
            pts_W[3 * idx + 1] = p.y;
            pts_W[3 * idx + 2] = p.z;
            nrm_W[3 * idx + 0] = n.x;
            nrm_W[3 * idx + 1] = n.y;
            nrm_W[3 * idx + 2] = n.z;
        }
    }
}

int so_occ_aabb(const so_occ_map* m, int32_t mn[3], int32_t mx[3])
{
    if (m->octree.aabb_empty)
        return 0;
    for (int i = 0; i < 3; ++i) {
        mn[i] = m->octree.aabb_min[i];
        mx[i] = m->octree.aabb_max[i];
    }
    return 1;
}

void so_occ_depth_sigma(const float* depth, int n, float res, float* sigma)
{
    depth_sigma(depth, n, res, default_occ_config(), sigma);
}

/* The pooling image of a depth image: per level (max_level + 1 of them) w*h pixels of
 * (min, max, crossing, known); returns max_level and writes the max value. */
int so_occ_pooling_image(const float* depth, int w, int h, float* out, float* max_value)
{
    PoolingImage p;
    p.build(depth, w, h);
    if (out) {
        for (int l = 0; l <= p.max_level; ++l)
            for (size_t i = 0; i < (size_t) w * h; ++i) {
                const PPixel& q = p.img[l][i];
                float* o = out + ((size_t) l * w * h + i) * 4;
                o[0] = q.min;
                o[1] = q.max;
                o[2] = (float) q.crossing;
                o[3] = (float) q.known;
            }
    }
    if (max_value)
        *max_value = p.max_value;
    return p.max_level;
}

} // extern "C"
