// voxelize.cu -- strand-density voxelizer (vertex-count and segment modes).
//
// Bit-exact restatement of vkhr::HairStyle::voxelize_vertices / _segments
// (src/vkhr/scene_graph/hair_style.cc:257-342) for GB300:
//
//   1. count    one thread per vertex / index pair: the reference's FP32
//               coordinate and stepping arithmetic (no contraction, IEEE
//               division), red.global.add into uint32 counts;
//   2. ranges   each voxel with visits gets a contiguous slice of a visit
//               list (block-wide scan, one atomic per 4096 voxels);
//   3. fill     the same visits again, each appends its serial key (vertex
//               index, or index-pair number) to its voxel's slice;
//   4. resolve  per voxel: u8 density = min(count, 255); the keys are sorted
//               (register sorting network, or a shared-memory bitonic sort
//               for crowded voxels), the first min(count, 255) tangents are
//               summed in that order in FP32 and quantised.  This reproduces
//               the reference's serial loop, its stop-at-255 rule and its
//               float summation order exactly, so the int8 tangents are
//               bit-identical too, independent of atomic ordering.
#include "common.cuh"

#include <algorithm>
#include <cmath>

namespace {

constexpr int kSmallSort = 16;     // voxels with <= this many visits resolve in the main pass
constexpr int kMediumSort = 64;    // <= this many: one thread per voxel, 64-key register network
constexpr int kHeavyTile = 2048;   // shared-memory sort tile of the heavy resolve
constexpr int kKeep = 256;         // smallest keys carried between heavy tiles (>= 255)
constexpr int kRangeThreads = 256;
constexpr int kRangeItems = 16;

struct Grid {
    float org[3];
    float vs[3];   // voxel size, bounds.size / resolution (IEEE division)
    float rm1[3];  // resolution - 1.0f
    float fw, fh;  // (float)width, (float)height
    float fn;      // (float)(width * height * depth)
    uint32_t w, h, n;
    int mode;
};

__device__ __forceinline__ bool linear_index(const Grid& g, float vx, float vy, float vz, uint32_t& out)
{
    if (g.mode == VKHR_INDEX_REF_FP32) {
        // voxel.x + voxel.y*width + voxel.z*width*height in FP32 (hair_style.cc:276, :321)
        float a = __fmul_rn(vy, g.fw);
        float b = __fmul_rn(__fmul_rn(vz, g.fw), g.fh);
        float fi = __fadd_rn(__fadd_rn(vx, a), b);
        if (!(fi >= 0.0f) || !(fi < g.fn)) return false;
        out = (uint32_t)fi;
        return out < g.n;
    }
    if (!(vx >= 0.0f) || !(vy >= 0.0f) || !(vz >= 0.0f)) return false;
    out = (uint32_t)vx + g.w * ((uint32_t)vy + g.h * (uint32_t)vz);
    return true;
}

// hair_style.cc:274-276: voxel = min(floor((vertex - origin) / voxel_size), resolution - 1)
__device__ __forceinline__ bool vertex_voxel(const Grid& g, const float* __restrict__ v, uint32_t i, uint32_t& out)
{
    float c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
        c[a] = glm_min(floorf(__fdiv_rn(__fsub_rn(__ldg(v + 3 * (size_t)i + a), g.org[a]), g.vs[a])), g.rm1[a]);
    return linear_index(g, c[0], c[1], c[2], out);
}

// hair_style.cc:311-329 for one index pair; calls f(voxel) per visit in serial order.
template <class F>
__device__ __forceinline__ void segment_visits(const Grid& g, const float* __restrict__ v, uint32_t i0, uint32_t i1,
                                               unsigned& status, F&& f)
{
    float root[3], dir[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        root[a] = __fdiv_rn(__fsub_rn(__ldg(v + 3 * (size_t)i0 + a), g.org[a]), g.vs[a]);
        float tip = __fdiv_rn(__fsub_rn(__ldg(v + 3 * (size_t)i1 + a), g.org[a]), g.vs[a]);
        dir[a] = __fsub_rn(tip, root[a]);
    }
    float steps = glm_max(glm_max(fabsf(dir[0]), fabsf(dir[1])), fabsf(dir[2])); // compMax(abs(direction))
#pragma unroll
    for (int a = 0; a < 3; ++a) dir[a] = __fdiv_rn(dir[a], steps);
    if (!(steps > 0.0f)) return;  // `while (steps-- > 0.0f)` never runs (0 or NaN)
    if (steps > 16777216.0f) {    // the FP32 decrement no longer terminates reliably
        status |= VKHR_DEV_STEPS_OVERFLOW;
        return;
    }
    // Below 2^24 every `steps - 1.0f` is exact, so the loop runs ceil(steps) times.
    const uint32_t n = (uint32_t)ceilf(steps);
    for (uint32_t k = 0; k < n; ++k) {
        uint32_t vox;
        if (linear_index(g, glm_min(floorf(root[0]), g.rm1[0]), glm_min(floorf(root[1]), g.rm1[1]),
                         glm_min(floorf(root[2]), g.rm1[2]), vox))
            f(vox);
#pragma unroll
        for (int a = 0; a < 3; ++a) root[a] = __fadd_rn(root[a], dir[a]);
    }
}

__device__ __forceinline__ void warp_add_total(unsigned long long local, unsigned long long* total)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(total, local);
}

__global__ void count_vertices_kernel(Grid g, const float* __restrict__ v, uint32_t n_vertices, uint32_t* counts,
                                      unsigned long long* words)
{
    unsigned long long local = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_vertices; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t vox;
        if (vertex_voxel(g, v, i, vox)) {
            atomicAdd(counts + vox, 1u);
            ++local;
        }
    }
    warp_add_total(local, words + WORD_TOTAL_VISITS);
}

__global__ void count_segments_kernel(Grid g, const float* __restrict__ v, const uint2* __restrict__ pairs_idx,
                                      uint32_t n_pairs, uint32_t* counts, unsigned long long* words)
{
    unsigned long long local = 0;
    unsigned status = 0;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n_pairs; p += (uint64_t)gridDim.x * blockDim.x) {
        uint2 ij = __ldg(pairs_idx + p);
        segment_visits(g, v, ij.x, ij.y, status, [&](uint32_t vox) {
            atomicAdd(counts + vox, 1u);
            ++local;
        });
    }
    warp_add_total(local, words + WORD_TOTAL_VISITS);
    if (status) atomicOr(words + WORD_STATUS, (unsigned long long)status);
}

// Gives each voxel with visits a contiguous slice [cursor, cursor + count) of
// the visit list.  Voxels are read warp-striped (coalesced); slices are
// handed out per thread in the same order; one atomic per block.
__global__ void __launch_bounds__(kRangeThreads) alloc_ranges_kernel(const uint32_t* __restrict__ counts, uint32_t n,
                                                                   uint32_t* cursor, unsigned long long* words)
{
    __shared__ uint32_t warp_sums[kRangeThreads / 32];
    __shared__ uint32_t block_base;
    const uint32_t tile = kRangeThreads * kRangeItems;
    for (uint64_t base = (uint64_t)blockIdx.x * tile; base < n; base += (uint64_t)gridDim.x * tile) {
        uint32_t c[kRangeItems];
        uint32_t sum = 0;
#pragma unroll
        for (int j = 0; j < kRangeItems; ++j) {
            uint64_t i = base + (uint64_t)j * kRangeThreads + threadIdx.x;
            c[j] = i < n ? __ldg(counts + i) : 0u;
            sum += c[j];
        }
        // block-wide exclusive scan of the per-thread sums
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (int w = 0; w < kRangeThreads / 32; ++w) {
                uint32_t t = warp_sums[w];
                warp_sums[w] = run;
                run += t;
            }
            block_base = run ? (uint32_t)atomicAdd(words + WORD_LIST_CURSOR, (unsigned long long)run) : 0u;
        }
        __syncthreads();
        uint32_t start = block_base + warp_sums[warp] + (incl - sum);
#pragma unroll
        for (int j = 0; j < kRangeItems; ++j) {
            uint64_t i = base + (uint64_t)j * kRangeThreads + threadIdx.x;
            if (i < n) cursor[i] = start;
            start += c[j];
        }
        __syncthreads();
    }
}

__global__ void fill_vertices_kernel(Grid g, const float* __restrict__ v, uint32_t n_vertices, uint32_t* cursor,
                                     uint32_t* list, size_t list_cap, unsigned long long* words)
{
    unsigned status = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_vertices; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t vox;
        if (vertex_voxel(g, v, i, vox)) {
            uint32_t slot = atomicAdd(cursor + vox, 1u);
            if (slot < list_cap) list[slot] = (uint32_t)i;
            else status |= VKHR_DEV_LIST_OVERFLOW;
        }
    }
    if (status) atomicOr(words + WORD_STATUS, (unsigned long long)status);
}

__global__ void fill_segments_kernel(Grid g, const float* __restrict__ v, const uint2* __restrict__ pairs_idx,
                                     uint32_t n_pairs, uint32_t* cursor, uint32_t* list, size_t list_cap,
                                     unsigned long long* words)
{
    unsigned status = 0;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n_pairs; p += (uint64_t)gridDim.x * blockDim.x) {
        uint2 ij = __ldg(pairs_idx + p);
        segment_visits(g, v, ij.x, ij.y, status, [&](uint32_t vox) {
            uint32_t slot = atomicAdd(cursor + vox, 1u);
            if (slot < list_cap) list[slot] = (uint32_t)p;
            else status |= VKHR_DEV_LIST_OVERFLOW;
        });
    }
    if (status) atomicOr(words + WORD_STATUS, (unsigned long long)status);
}

// Tangent of a visit key: the vertex's own (voxelize_vertices) or the pair's
// first vertex's (voxelize_segments, `tangents[indices[i]]`).
__device__ __forceinline__ uint32_t key_vertex(uint32_t key, const uint2* __restrict__ pairs_idx)
{
    return pairs_idx ? __ldg(pairs_idx + key).x : key;
}

// i8vec3(sum / float(density) * 127.0f), truncating; NaN gives 0.
__device__ __forceinline__ int quantize1(float s, float m)
{
    float q = __fmul_rn(__fdiv_rn(s, m), 127.0f);
    return (q == q) ? __float2int_rz(q) : 0;
}

__device__ __forceinline__ uint32_t pack_tangent(float sx, float sy, float sz, uint32_t m)
{
    const float fm = (float)m;
    int x = quantize1(sx, fm), y = quantize1(sy, fm), z = quantize1(sz, fm);
    return ((uint32_t)(x & 0xff)) | ((uint32_t)(y & 0xff) << 8) | ((uint32_t)(z & 0xff) << 16);
}

template <int N, int CAP>
__device__ __forceinline__ void sort_network(uint32_t (&x)[CAP])
{
#pragma unroll
    for (int k = 2; k <= N; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    uint32_t a = x[i], b = x[l];
                    if ((a > b) == up) { x[i] = b; x[l] = a; }
                }
            }
}

template <int N>
__device__ __forceinline__ uint32_t resolve_small(uint32_t c, const uint32_t* __restrict__ list, uint32_t start,
                                                  const float* __restrict__ tan, const uint2* __restrict__ pairs_idx)
{
    uint32_t k[kSmallSort];
#pragma unroll
    for (int i = 0; i < kSmallSort; ++i) k[i] = (i < N && (uint32_t)i < c) ? __ldg(list + start + i) : 0xffffffffu;
    if (N > 2) sort_network<N, kSmallSort>(k);
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
#pragma unroll
    for (int i = 0; i < N; ++i)
        if ((uint32_t)i < c) {
            const float* t = tan + 3 * (size_t)key_vertex(k[i], pairs_idx);
            sx = __fadd_rn(sx, __ldg(t + 0));
            sy = __fadd_rn(sy, __ldg(t + 1));
            sz = __fadd_rn(sz, __ldg(t + 2));
        }
    return pack_tangent(sx, sy, sz, c);
}

__global__ void resolve_kernel(uint32_t n, const uint32_t* __restrict__ counts, const uint32_t* __restrict__ cursor,
                               const uint32_t* __restrict__ list, const float* __restrict__ tan,
                               const uint2* __restrict__ pairs_idx, uint8_t* dens, uint32_t* tq, uint32_t* heavy,
                               size_t heavy_cap, unsigned long long* words)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = __ldg(counts + v);
        if (dens) dens[v] = (uint8_t)(c < 255u ? c : 255u);
        if (!tq) continue;
        if (c == 0) { tq[v] = 0u; continue; }
        const uint32_t start = __ldg(cursor + v) - c;
        uint32_t packed;
        if (c <= 2) packed = resolve_small<2>(c, list, start, tan, pairs_idx);      // order-free
        else if (c <= 4) packed = resolve_small<4>(c, list, start, tan, pairs_idx);
        else if (c <= 8) packed = resolve_small<8>(c, list, start, tan, pairs_idx);
        else if (c <= kSmallSort) packed = resolve_small<kSmallSort>(c, list, start, tan, pairs_idx);
        else {
            // crowded voxels: medium ones to a register-network pass, the
            // rest to one block each; both lists share the heavy buffer
            // (medium from the front, crowded from the back)
            const bool medium = c <= kMediumSort;
            unsigned long long slot = atomicAdd(words + (medium ? WORD_MEDIUM_COUNT : WORD_HEAVY_COUNT), 1ull);
            const unsigned long long at = medium ? slot : heavy_cap - 1 - slot;
            if (slot < heavy_cap / 2) heavy[at] = (uint32_t)v;
            else atomicOr(words + WORD_STATUS, (unsigned long long)VKHR_DEV_LIST_OVERFLOW);
            continue;
        }
        tq[v] = packed;
    }
}

// Voxels with kSmallSort < count <= kMediumSort: one thread each, keys sorted
// by a 64-wide register network (SIMT across voxels beats cooperation within one).
__global__ void __launch_bounds__(128) resolve_medium_kernel(const uint32_t* __restrict__ counts,
                                                             const uint32_t* __restrict__ cursor,
                                                             const uint32_t* __restrict__ list,
                                                             const float* __restrict__ tan,
                                                             const uint2* __restrict__ pairs_idx,
                                                             const uint32_t* __restrict__ medium, size_t heavy_cap,
                                                             uint32_t* tq, const unsigned long long* words)
{
    unsigned long long nm = words[WORD_MEDIUM_COUNT];
    if (nm > heavy_cap / 2) nm = heavy_cap / 2;
    for (unsigned long long h = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; h < nm;
         h += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t v = medium[h];
        const uint32_t c = counts[v];
        const uint32_t start = cursor[v] - c;
        uint32_t k[kMediumSort];
#pragma unroll
        for (int i = 0; i < kMediumSort; ++i) k[i] = (uint32_t)i < c ? __ldg(list + start + i) : 0xffffffffu;
        sort_network<kMediumSort, kMediumSort>(k);
        float sx = 0.0f, sy = 0.0f, sz = 0.0f;
#pragma unroll
        for (int i = 0; i < kMediumSort; ++i)
            if ((uint32_t)i < c) {
                const float* t = tan + 3 * (size_t)key_vertex(k[i], pairs_idx);
                sx = __fadd_rn(sx, __ldg(t + 0));
                sy = __fadd_rn(sy, __ldg(t + 1));
                sz = __fadd_rn(sz, __ldg(t + 2));
            }
        tq[v] = pack_tangent(sx, sy, sz, c);
    }
}

__device__ void block_bitonic_sort(uint32_t* s, int n)
{
    for (int k = 2; k <= n; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    uint32_t a = s[i], b = s[l];
                    if ((a > b) == up) { s[i] = b; s[l] = a; }
                }
            }
            __syncthreads();
        }
}

// One block per crowded voxel: the first min(count, 255) keys in serial order
// by repeated tile sorts that carry the smallest kKeep keys forward.
__global__ void __launch_bounds__(256) resolve_heavy_kernel(const uint32_t* __restrict__ counts,
                                                            const uint32_t* __restrict__ cursor,
                                                            const uint32_t* __restrict__ list,
                                                            const float* __restrict__ tan,
                                                            const uint2* __restrict__ pairs_idx,
                                                            const uint32_t* __restrict__ heavy, size_t heavy_cap,
                                                            uint32_t* tq, const unsigned long long* words)
{
    __shared__ uint32_t keys[kHeavyTile];
    __shared__ float tv[3][kKeep];
    unsigned long long nh = words[WORD_HEAVY_COUNT];
    if (nh > heavy_cap / 2) nh = heavy_cap / 2;
    for (unsigned long long h = blockIdx.x; h < nh; h += gridDim.x) {
        const uint32_t v = heavy[heavy_cap - 1 - h];
        const uint32_t c = counts[v];
        const uint32_t start = cursor[v] - c;
        const uint32_t m = c < 255u ? c : 255u;
        uint32_t done = 0;
        int first = 0; // slots already holding carried keys
        while (done < c) {
            const uint32_t take = min((uint32_t)(kHeavyTile - first), c - done);
            for (int i = threadIdx.x; i < kHeavyTile - first; i += blockDim.x)
                keys[first + i] = (uint32_t)i < take ? list[start + done + i] : 0xffffffffu;
            __syncthreads();
            block_bitonic_sort(keys, kHeavyTile);
            done += take;
            first = kKeep;
        }
        for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
            const float* t = tan + 3 * (size_t)key_vertex(keys[i], pairs_idx);
            tv[0][i] = t[0];
            tv[1][i] = t[1];
            tv[2][i] = t[2];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            float sx = 0.0f, sy = 0.0f, sz = 0.0f;
            for (uint32_t i = 0; i < m; ++i) {
                sx = __fadd_rn(sx, tv[0][i]);
                sy = __fadd_rn(sy, tv[1][i]);
                sz = __fadd_rn(sz, tv[2][i]);
            }
            tq[v] = pack_tangent(sx, sy, sz, m);
        }
        __syncthreads();
    }
}

__global__ void init_minmax_kernel(unsigned long long* words)
{
    if (threadIdx.x == 0) {
        words[WORD_AABB + 0] = 255ull;
        words[WORD_AABB + 1] = 0ull;
    }
}

__global__ void minmax_u8_kernel(const uint8_t* __restrict__ d, uint64_t n, unsigned long long* words)
{
    uint32_t lo = 255, hi = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = d[i];
        lo = min(lo, x);
        hi = max(hi, x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_down_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_down_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(words + WORD_AABB + 0, (unsigned long long)lo);
        atomicMax(words + WORD_AABB + 1, (unsigned long long)hi);
    }
}

// hair_style.cc:344-357: d = u8((d - min) * (255.0f / (max - min))), truncating.
__global__ void rescale_u8_kernel(uint8_t* d, uint64_t n, const unsigned long long* words)
{
    const uint32_t lo = (uint32_t)words[WORD_AABB + 0], hi = (uint32_t)words[WORD_AABB + 1];
    const float scaling = hi > lo ? __fdiv_rn(255.0f, (float)(int)(hi - lo)) : 0.0f;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = (uint32_t)d[i] - lo;
        d[i] = hi > lo ? (uint8_t)__float2uint_rz(__fmul_rn((float)x, scaling)) : (uint8_t)0;
    }
}

vkhr_status make_grid(vkhr_ctx* ctx, const vkhr_aabb* b, int32_t w, int32_t h, int32_t d, int32_t mode, Grid& g)
{
    if (!b) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "bounds is NULL");
    if (w <= 0 || h <= 0 || d <= 0) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "resolution must be positive");
    const uint64_t n = (uint64_t)w * (uint64_t)h * (uint64_t)d;
    if (n >= (1ull << 32)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "more than 2^32 - 1 voxels");
    if (mode != VKHR_INDEX_REF_FP32 && mode != VKHR_INDEX_EXACT)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "unknown index_mode");
    const float res[3] = {(float)w, (float)h, (float)d};
    for (int a = 0; a < 3; ++a) {
        if (!(b->size[a] > 0.0f) || !std::isfinite(b->size[a]) || !std::isfinite(b->origin[a]))
            return vkhr_fail(ctx, VKHR_ERR_DEGENERATE_AABB, "every AABB extent must be finite and > 0");
        g.org[a] = b->origin[a];
        volatile float q = b->size[a] / res[a]; // one IEEE division, as glm's vec3 / vec3
        g.vs[a] = q;
        g.rm1[a] = res[a] - 1.0f;
    }
    g.fw = res[0];
    g.fh = res[1];
    g.fn = (float)n;
    g.w = (uint32_t)w;
    g.h = (uint32_t)h;
    g.n = (uint32_t)n;
    g.mode = mode;
    return VKHR_OK;
}

vkhr_status check_device_status(vkhr_ctx* ctx)
{
    const unsigned long long s = ctx->h_words[WORD_STATUS];
    if (s & VKHR_DEV_STEPS_OVERFLOW)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG,
                         "a segment spans more than 2^24 voxels (vertices far outside the bounds)");
    if (s & VKHR_DEV_LIST_OVERFLOW) return vkhr_fail(ctx, VKHR_ERR_CAPACITY, "visit list overflow");
    return VKHR_OK;
}

vkhr_status voxelize_impl(vkhr_ctx* ctx, bool segments, const float* v, const float* tan_in, const uint32_t* idx,
                          uint64_t n_items, const vkhr_aabb* bounds, int32_t w, int32_t h, int32_t d, int32_t mode,
                          uint32_t* counts, uint8_t* dens, int8_t* tq, cudaStream_t st)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    Grid g;
    vkhr_status s = make_grid(ctx, bounds, w, h, d, mode, g);
    if (s != VKHR_OK) return s;
    if (!counts) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_counts is NULL");
    if (n_items >= (1ull << 32)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "more than 2^32 - 1 vertices or pairs");
    const uint32_t n_in = (uint32_t)n_items; // vertices, or index pairs
    if (tq && !tan_in && n_in) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_tangents requested without d_tangent_in");
    if (n_in && !v) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_vertices is NULL");
    if (segments && n_in && !idx) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_indices is NULL");
    if (segments && idx && (reinterpret_cast<uintptr_t>(idx) & 7u))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_indices must be 8-byte aligned");
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const uint2* pairs = reinterpret_cast<const uint2*>(idx);

    if (tq) {
        s = vkhr_reserve(ctx, (void**)&ctx->cursor, &ctx->cursor_cap, g.n, sizeof(uint32_t));
        if (s != VKHR_OK) return s;
    }
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_words, 0, 5 * sizeof(unsigned long long), st));
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(counts, 0, (size_t)g.n * sizeof(uint32_t), st));
    const unsigned threads = 256;
    const unsigned max_blocks = (unsigned)ctx->sm_count * 16;
    const unsigned blocks = std::min(vkhr_blocks(n_in, threads), max_blocks);
    if (n_in) {
        if (segments) VKHR_LAUNCH(ctx, count_segments_kernel, blocks, threads, 0, st, g, v, pairs, n_in, counts, ctx->d_words);
        else VKHR_LAUNCH(ctx, count_vertices_kernel, blocks, threads, 0, st, g, v, n_in, counts, ctx->d_words);
        VKHR_CUDA_TRY(ctx, cudaGetLastError());
    }
    const unsigned vblocks = std::min(vkhr_blocks(g.n, threads), (unsigned)ctx->sm_count * 32);
    if (!tq) {
        if (dens) {
            VKHR_LAUNCH(ctx, resolve_kernel, vblocks, threads, 0, st, g.n, counts, nullptr, nullptr, nullptr, nullptr, dens, nullptr,
                                                        nullptr, 0, ctx->d_words);
            VKHR_CUDA_TRY(ctx, cudaGetLastError());
        }
        if (segments) {
            VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->h_words, ctx->d_words, 4 * sizeof(unsigned long long),
                                               cudaMemcpyDeviceToHost, st));
            VKHR_CUDA_TRY(ctx, cudaStreamSynchronize(st));
            return check_device_status(ctx);
        }
        return VKHR_OK;
    }

    // The visit total sizes the list.  Vertex mode: bounded by the vertex
    // count, no round trip.  Segment mode: read it back while the GPU
    // allocates ranges.
    VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->h_words, ctx->d_words, 4 * sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, st));
    VKHR_CUDA_TRY(ctx, cudaEventRecord(ctx->ev, st));
    const unsigned rblocks = std::min(vkhr_blocks(g.n, kRangeThreads * kRangeItems), (unsigned)ctx->sm_count * 8);
    VKHR_LAUNCH(ctx, alloc_ranges_kernel, rblocks, kRangeThreads, 0, st, counts, g.n, ctx->cursor, ctx->d_words);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    uint64_t total = n_in;
    if (segments) {
        VKHR_CUDA_TRY(ctx, cudaEventSynchronize(ctx->ev));
        s = check_device_status(ctx);
        if (s != VKHR_OK) return s;
        total = ctx->h_words[WORD_TOTAL_VISITS];
        if (total >= (1ull << 32))
            return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "more than 2^32 - 1 voxel visits in one call");
    }
    s = vkhr_reserve(ctx, (void**)&ctx->list, &ctx->list_cap, total ? total : 1, sizeof(uint32_t));
    if (s != VKHR_OK) return s;
    // medium voxels (> kSmallSort visits each) fill the buffer from the front,
    // crowded ones (> kMediumSort) from the back: each list fits its half.
    s = vkhr_reserve(ctx, (void**)&ctx->heavy, &ctx->heavy_cap, 2 * (total / (kSmallSort + 1) + 1),
                     sizeof(uint32_t));
    if (s != VKHR_OK) return s;
    if (n_in) {
        if (segments)
            VKHR_LAUNCH(ctx, fill_segments_kernel, blocks, threads, 0, st, g, v, pairs, n_in, ctx->cursor, ctx->list, ctx->list_cap,
                                                             ctx->d_words);
        else
            VKHR_LAUNCH(ctx, fill_vertices_kernel, blocks, threads, 0, st, g, v, n_in, ctx->cursor, ctx->list, ctx->list_cap,
                                                             ctx->d_words);
        VKHR_CUDA_TRY(ctx, cudaGetLastError());
    }
    uint32_t* tq32 = reinterpret_cast<uint32_t*>(tq);
    VKHR_LAUNCH(ctx, resolve_kernel, vblocks, threads, 0, st, g.n, counts, ctx->cursor, ctx->list, tan_in,
                                                segments ? pairs : nullptr, dens, tq32, ctx->heavy, ctx->heavy_cap,
                                                ctx->d_words);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    VKHR_LAUNCH(ctx, resolve_medium_kernel, (unsigned)ctx->sm_count * 8, 128, 0, st, counts, ctx->cursor, ctx->list,
                tan_in, segments ? pairs : nullptr, ctx->heavy, ctx->heavy_cap, tq32, ctx->d_words);
    VKHR_LAUNCH(ctx, resolve_heavy_kernel, (unsigned)ctx->sm_count * 2, 256, 0, st, counts, ctx->cursor, ctx->list,
                tan_in, segments ? pairs : nullptr, ctx->heavy, ctx->heavy_cap, tq32, ctx->d_words);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

} // namespace

extern "C" {

vkhr_status vkhr_voxelize_vertices(vkhr_ctx* ctx, const float* d_vertices, const float* d_tangent_in,
                                   uint32_t vertex_count, const vkhr_aabb* bounds, int32_t width, int32_t height,
                                   int32_t depth, int32_t index_mode, uint32_t* d_counts, uint8_t* d_densities,
                                   int8_t* d_tangents, void* stream)
{
    return voxelize_impl(ctx, false, d_vertices, d_tangent_in, nullptr, vertex_count, bounds, width, height, depth,
                         index_mode, d_counts, d_densities, d_tangents, (cudaStream_t)stream);
}

vkhr_status vkhr_voxelize_segments(vkhr_ctx* ctx, const float* d_vertices, const float* d_tangent_in,
                                   const uint32_t* d_indices, uint64_t index_count, const vkhr_aabb* bounds,
                                   int32_t width, int32_t height, int32_t depth, int32_t index_mode,
                                   uint32_t* d_counts, uint8_t* d_densities, int8_t* d_tangents, void* stream)
{
    // for (i = 0; i < indices.size() - 1; i += 2): floor(n / 2) pairs
    return voxelize_impl(ctx, true, d_vertices, d_tangent_in, d_indices, index_count / 2, bounds, width, height,
                         depth, index_mode, d_counts, d_densities, d_tangents, (cudaStream_t)stream);
}

vkhr_status vkhr_normalize_densities(vkhr_ctx* ctx, uint8_t* d, uint64_t n, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (n == 0) return VKHR_OK;
    if (!d) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_densities is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    VKHR_LAUNCH(ctx, init_minmax_kernel, 1, 32, 0, st, ctx->d_words);
    const unsigned blocks = std::min(vkhr_blocks(n, 256), (unsigned)ctx->sm_count * 8);
    VKHR_LAUNCH(ctx, minmax_u8_kernel, blocks, 256, 0, st, d, n, ctx->d_words);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    VKHR_LAUNCH(ctx, rescale_u8_kernel, blocks, 256, 0, st, d, n, ctx->d_words);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

} // extern "C"
