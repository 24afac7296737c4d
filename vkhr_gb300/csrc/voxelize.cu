// voxelize.cu -- strand-density voxelizer (vertex-count and segment modes).
//
// Bit-exact restatement of vkhr::HairStyle::voxelize_vertices / _segments
// (src/vkhr/scene_graph/hair_style.cc:257-342) for GB300.  Every visit is
// computed with the reference's FP32 operation sequence (IEEE division, no
// FMA contraction, glm's min/max), so counts are exact; the int8 tangents
// are bit-identical too because each voxel's tangents are summed in the
// reference's serial order (ascending vertex index / index-pair number) and
// only the first 255 visits count, as `if (densities[pos] != 255)` does.
//
// Brick path (every voxel whose 8^3 brick receives <= kBrickCap visits):
//   1. bin (count)  one thread per vertex / index pair walks its visits and
//                   splits them into runs of consecutive visits inside one
//                   brick; one reduction per run counts visits per brick
//                   (32K bricks at 256^3, hot in L2).  A pair's set-up (its
//                   root, direction and step count: nine IEEE divisions) and
//                   its first vertex's tangent are stored once;
//   2. bin ranges   each brick gets a slice of the visit list; occupied
//                   bricks are listed; empty bricks are zeroed by a streaming
//                   kernel;
//   3. bin (fill)   the same walk again reserves one slice range per run and
//                   writes (serial key, local voxel) entries into it;
//   4. brick        one CTA per occupied brick reads its entries twice: counts
//                   per voxel in shared memory, then the keys bucketed per
//                   voxel; each voxel's keys are sorted (up to 16 in the
//                   voxel's thread's registers by a bitonic network, up to 64
//                   by a warp) and its tangents summed in that order; the brick's 512
//                   counts, u8 densities and int8x4 tangents are written once;
//   5. crowded      voxels with 65..256 visits: one warp each sorts its keys
//                   in registers; above 256 visits one CTA each selects the
//                   256 smallest keys in shared-memory tiles.
// Bricks above kBrickCap visits take the same brick kernel (a separate
// launch) with their keys bucketed into a slice of a global scratch instead
// of shared memory.
// One-walk calls (segment mode without a visit budget, once the context has
// seen a call's largest brick): step 1 also writes every run into a fixed
// slice of its brick (capacity: the largest brick seen + 25%) and step 3 is
// skipped; a brick past its slice shows in the visit read-back the call
// makes anyway, and that call runs step 3 in the compact layout.
#include "common.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace {

constexpr int kBrickThreads = 512;     // one thread per voxel of an 8^3 brick
constexpr int kBrickCap = 22528;       // visits a brick resolves in shared memory
constexpr int kLightBrick = 512;       // <= this many visits: the brick is resolved by one warp
constexpr int kLightWarps = 4;         // warps per CTA of light_brick_kernel (24 KB of shared memory)
constexpr int kBrickSmall = 64;        // <= this many visits: resolved by the voxel's own thread in the brick kernels
constexpr int kCrowdWarpMax = 256;     // crowded voxels up to this many visits: one warp each
constexpr int kGather = 4;             // tangent loads in flight per voxel thread (64 registers at 2 CTAs / SM)
constexpr int kHeavyTile = 2048;       // crowded voxels: shared-memory sort tile
constexpr int kKeep = 256;             // crowded voxels: tangents summed (>= 255)
constexpr int kRangeThreads = 256;
constexpr int kRangeItems = 2;   // bricks per thread of the range passes (short atomic chains)
constexpr uint32_t kNoBrick = 0xffffffffu;

struct Grid {
    float org[3];
    float vs[3];   // voxel size, bounds.size / resolution (IEEE division)
    float rm1[3];  // resolution - 1.0f
    float fw, fh;  // (float)width, (float)height
    float fn;      // (float)(width * height * depth)
    uint32_t w, h, d, n, wh;
    uint32_t nbx, nby, nbz, nb; // bricks
    int mode;
    int exact_coords; // the linear index always equals the clamped coordinates' exact index
};

struct Visit {
    uint32_t lin;   // linear voxel index
    uint32_t brick;
    uint32_t local; // (x & 7) | (y & 7) << 3 | (z & 7) << 6
};

// One style of a batch.  Items (index pairs, or vertices) and bricks of all
// styles share one global index space; a style owns [item_base, +n_in) and
// [brick_base, +g.nb).  Keys stay style-local (pair / vertex numbers).
constexpr int kMaxJobs = 256;

struct VoxJob {
    Grid g;
    const float* v;
    const float* tan;   // tangent input (NULL: counts only)
    const uint2* pairs; // NULL in vertex mode
    uint32_t* counts;
    uint8_t* dens;
    uint32_t* tq;
    uint32_t item_base;
    uint32_t n_in;
    uint32_t brick_base;
    uint32_t zero_base; // first 4-voxel group of the style (empty-brick zeroing)
};

static_assert(sizeof(VoxJob) * kMaxJobs <= kJobTableBytes, "job table staging too small");
static_assert(sizeof(VoxJob) % 4 == 0 && (sizeof(VoxJob) + 4) * kMaxJobs <= 48 * 1024, "bin kernels keep the table in shared memory");

// Largest j with base[j] <= x (base ascending, base[0] = 0).
__device__ __forceinline__ int find_job(const uint32_t* base, int nj, uint32_t x)
{
    int lo = 0, hi = nj - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (base[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void load_bases(const VoxJob* jobs, int nj, uint32_t* item_base, uint32_t* brick_base)
{
    for (int j = threadIdx.x; j < nj; j += blockDim.x) {
        if (item_base) item_base[j] = jobs[j].item_base;
        if (brick_base) brick_base[j] = jobs[j].brick_base;
    }
    __syncthreads();
}

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

// Visit of the clamped voxel coordinate (vx, vy, vz): its linear index as the
// reference forms it, and the brick/local position of that index.
__device__ __forceinline__ bool locate(const Grid& g, float vx, float vy, float vz, Visit& o)
{
    uint32_t x, y, z;
    if (g.exact_coords && vx >= 0.0f && vy >= 0.0f && vz >= 0.0f) {
        // coordinates in [0, res-1] (clamped above): the FP32 index of the
        // reference is exact below 2^24 voxels, so it is this voxel's index
        x = (uint32_t)vx;
        y = (uint32_t)vy;
        z = (uint32_t)vz;
        o.lin = x + g.w * (y + g.h * z);
    } else { // the FP32 index may have wrapped or rounded: decompose it
        if (!linear_index(g, vx, vy, vz, o.lin)) return false;
        z = o.lin / g.wh;
        const uint32_t r = o.lin - z * g.wh;
        y = r / g.w;
        x = r - y * g.w;
    }
    o.brick = (x >> 3) + g.nbx * ((y >> 3) + g.nby * (z >> 3));
    o.local = (x & 7u) | ((y & 7u) << 3) | ((z & 7u) << 6);
    return true;
}

// hair_style.cc:274-276: voxel = min(floor((vertex - origin) / voxel_size), resolution - 1)
__device__ __forceinline__ bool vertex_visit(const Grid& g, const float* __restrict__ v, uint32_t i, Visit& o)
{
    float c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
        c[a] = glm_min(floorf(__fdiv_rn(__fsub_rn(__ldg(v + 3 * (size_t)i + a), g.org[a]), g.vs[a])), g.rm1[a]);
    return locate(g, c[0], c[1], c[2], o);
}

// One index pair of voxelize_segments (hair_style.cc:311-329).
struct Seg {
    float root[3], dir[3];
    uint32_t n; // iterations of `while (steps-- > 0.0f)`
};

__device__ __forceinline__ bool seg_setup(const Grid& g, const float* __restrict__ v, uint2 ij, Seg& s,
                                          unsigned& status)
{
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        s.root[a] = __fdiv_rn(__fsub_rn(__ldg(v + 3 * (size_t)ij.x + a), g.org[a]), g.vs[a]);
        const float tip = __fdiv_rn(__fsub_rn(__ldg(v + 3 * (size_t)ij.y + a), g.org[a]), g.vs[a]);
        s.dir[a] = __fsub_rn(tip, s.root[a]);
    }
    const float steps = glm_max(glm_max(fabsf(s.dir[0]), fabsf(s.dir[1])), fabsf(s.dir[2])); // compMax(abs(dir))
#pragma unroll
    for (int a = 0; a < 3; ++a) s.dir[a] = __fdiv_rn(s.dir[a], steps);
    s.n = 0;
    if (!(steps > 0.0f)) return false;  // 0 or NaN: the loop never runs
    if (steps > 16777216.0f) {          // the FP32 decrement no longer terminates reliably
        status |= VKHR_DEV_STEPS_OVERFLOW;
        return false;
    }
    // Below 2^24 every `steps - 1.0f` is exact, so the loop runs ceil(steps) times.
    s.n = (uint32_t)ceilf(steps);
    return true;
}

__device__ __forceinline__ bool seg_visit(const Grid& g, const Seg& s, Visit& o)
{
    return locate(g, glm_min(floorf(s.root[0]), g.rm1[0]), glm_min(floorf(s.root[1]), g.rm1[1]),
                  glm_min(floorf(s.root[2]), g.rm1[2]), o);
}

__device__ __forceinline__ void seg_advance(Seg& s)
{
#pragma unroll
    for (int a = 0; a < 3; ++a) s.root[a] = __fadd_rn(s.root[a], s.dir[a]); // root += direction
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// ---- brick path -----------------------------------------------------------------

// A visit entry of the brick path: the visit's serial key (pair or vertex
// number within its style) and its local voxel in the brick.  PACK = true
// packs both into 32 bits (key < 2^23), otherwise a uint2.
template <bool PACK>
struct Entry;
template <>
struct Entry<true> {
    typedef uint32_t T;
    static __device__ __forceinline__ T make(uint32_t key, uint32_t local) { return (key << 9) | local; }
    static __device__ __forceinline__ uint32_t key(T e) { return e >> 9; }
    static __device__ __forceinline__ uint32_t local(T e) { return e & 511u; }
};
template <>
struct Entry<false> {
    typedef uint2 T;
    static __device__ __forceinline__ T make(uint32_t key, uint32_t local) { return make_uint2(key, local); }
    static __device__ __forceinline__ uint32_t key(T e) { return e.x; }
    static __device__ __forceinline__ uint32_t local(T e) { return e.y & 511u; }
};
constexpr uint32_t kPackedKeyLimit = 1u << 23;
constexpr uint64_t kDirectBytes = 8ull << 30; // fixed per-brick slices of a one-walk call: at most 8 GB

// The local voxels (9 bits each) of a run of up to kMaxRun visits: 7 per word.
constexpr uint32_t kMaxRun = 14;
struct Locals {
    uint64_t lo, hi;
    __device__ __forceinline__ void start(uint32_t l)
    {
        lo = l;
        hi = 0;
    }
    __device__ __forceinline__ void put(uint32_t j, uint32_t l)
    {
        if (j < 7) lo |= (uint64_t)l << (9 * j);
        else hi |= (uint64_t)l << (9 * (j - 7));
    }
    __device__ __forceinline__ uint32_t get(uint32_t j) const
    {
        return (uint32_t)((j < 7 ? lo >> (9 * j) : hi >> (9 * (j - 7)))) & 511u;
    }
    static __device__ __forceinline__ Locals one(uint32_t l)
    {
        Locals r;
        r.start(l);
        return r;
    }
};

// A run of `len` (<= kMaxRun) consecutive visits of one pair / vertex inside brick b,
// their local voxels packed 9 bits each (Locals): counted per brick (FILL = false),
// or written as (key, local voxel) entries into the brick's slice of the
// visit list.
// DIRECT (a counting walk that also fills): the brick's count is its cursor
// and the entries go to the brick's fixed slice -- [b * entries_cap, + entries_cap)
// or, with a learned layout, {first slot, capacity} = layout[b]; a run past
// the slice is counted but not written, and raises the call's overflow word
// (the fill pass then lays the call out compactly from the exact counts).
template <bool FILL, bool PACK, bool DIRECT = false>
__device__ __forceinline__ void emit_run(uint32_t b, uint32_t key, Locals locals, uint32_t len, uint32_t* visits,
                                         uint32_t* cursor, typename Entry<PACK>::T* entries, size_t entries_cap,
                                         const uint2* __restrict__ layout, unsigned long long* words, unsigned& status)
{
    if (DIRECT) {
        const uint32_t at = atomicAdd(visits + b, len); // the run's range in the brick's slice
        uint64_t first = (uint64_t)b * entries_cap, cap = entries_cap;
        if (layout) {
            const uint2 sl = __ldg(layout + b);
            first = sl.x;
            cap = sl.y;
        }
        if ((uint64_t)at + len <= cap) {
            typename Entry<PACK>::T* e = entries + first + at;
            for (uint32_t j = 0; j < len; ++j) e[j] = Entry<PACK>::make(key, locals.get(j));
        } else {
            *reinterpret_cast<volatile unsigned long long*>(words + WORD_DIRECT_OVERFLOW) = 1ull;
        }
    } else if (!FILL) {
        atomicAdd(visits + b, len); // fire-and-forget reduction
    } else {
        const uint32_t base = atomicAdd(cursor + b, len);
        if ((uint64_t)base + len <= entries_cap) {
            for (uint32_t j = 0; j < len; ++j)
                entries[base + j] = Entry<PACK>::make(key, locals.get(j));
        } else {
            status |= VKHR_DEV_LIST_OVERFLOW;
        }
    }
}

// The visits of pair p (set up in s) in order, emitted as runs of up to
// kMaxRun consecutive visits inside one brick.
template <bool FILL, bool PACK, bool DIRECT>
__device__ __forceinline__ void walk_pair(const VoxJob& J, uint32_t p, Seg& s, uint32_t* visits, uint32_t* cursor,
                                          typename Entry<PACK>::T* entries, size_t entries_cap,
                                          const uint2* __restrict__ layout, unsigned long long* words,
                                          unsigned& status)
{
    const Grid& g = J.g;
    uint32_t cur = kNoBrick, len = 0;
    Locals locals;
    for (uint32_t k = 0; k < s.n; ++k) {
        Visit o;
        const bool ok = seg_visit(g, s, o);
        if (ok && o.brick == cur && len < kMaxRun) {
            locals.put(len, o.local);
            ++len;
        } else {
            if (len)
                emit_run<FILL, PACK, DIRECT>(J.brick_base + cur, p, locals, len, visits, cursor, entries, entries_cap,
                                             layout, words, status);
            cur = ok ? o.brick : kNoBrick;
            len = ok ? 1u : 0u;
            locals.start(ok ? o.local : 0u);
        }
        seg_advance(s);
    }
    if (len)
        emit_run<FILL, PACK, DIRECT>(J.brick_base + cur, p, locals, len, visits, cursor, entries, entries_cap, layout,
                                     words, status);
}

constexpr int kWalkThreads = 256; // threads per block of the bin kernels
constexpr int kWalkBuckets = 64;  // walk lengths a block groups its pairs by (the last: 63 visits or more)
constexpr size_t kWalkStaticSmem = (8 * kWalkThreads + kWalkBuckets) * sizeof(uint32_t); // balanced_walk's arrays

// The one walk (counts and entries in one pass) of a one-style call, in
// rounds of 256 pairs per block, its warps' lanes matched by walk length:
// each thread sets up the pair of its own index (coalesced index and vertex
// loads, the pair-tangent store), the block ranks the 256 pairs by visit
// count (a counting sort over kWalkBuckets lengths in shared memory), and
// thread t walks the pair of rank t.  A warp then runs about as many steps
// as its lanes' walks take, where 32 consecutive pairs (1 to about 40 visits
// each) run as long as their longest (production style: one walk 0.273 ->
// 0.262 ms).  A batch's grid-stride rounds keep the consecutive pairs: a
// barrier per round measured slower.
template <bool PACK, bool SINGLE>
__device__ __forceinline__ void balanced_walk(const VoxJob& job0, const VoxJob* s_jobs, const uint32_t* s_item_base,
                                              int nj, uint32_t total_items, float4* pair_tan, uint32_t* visits,
                                              typename Entry<PACK>::T* entries, size_t entries_cap,
                                              const uint2* __restrict__ layout, unsigned long long* words,
                                              unsigned& status)
{
    __shared__ uint32_t s_walk[8][kWalkThreads]; // root x y z, direction x y z, visits, pair (by rank)
    __shared__ uint32_t s_rank[kWalkBuckets];
    const uint32_t t = threadIdx.x;
    for (uint64_t base = (uint64_t)blockIdx.x * kWalkThreads; base < total_items;
         base += (uint64_t)gridDim.x * kWalkThreads) {
        const uint64_t q = base + t;
        Seg s = {};
        if (q < total_items) {
            const VoxJob& J = SINGLE ? job0 : s_jobs[find_job(s_item_base, nj, (uint32_t)q)];
            const uint2 ij = __ldg(J.pairs + ((uint32_t)q - J.item_base));
            seg_setup(J.g, J.v, ij, s, status);
            if (J.tan) // tangents[indices[i]]: every visit of the pair adds this one
                pair_tan[q] = make_float4(__ldg(J.tan + 3 * (size_t)ij.x), __ldg(J.tan + 3 * (size_t)ij.x + 1),
                                          __ldg(J.tan + 3 * (size_t)ij.x + 2), 0.0f);
        }
        if (t < (uint32_t)kWalkBuckets) s_rank[t] = 0u;
        __syncthreads();
        const uint32_t bucket = s.n < (uint32_t)kWalkBuckets ? s.n : (uint32_t)kWalkBuckets - 1;
        const uint32_t r = atomicAdd(s_rank + bucket, 1u);
        __syncthreads();
        if (t < 32) { // exclusive scan of the bucket sizes, two per lane
            const uint32_t a = s_rank[2 * t], b = s_rank[2 * t + 1];
            uint32_t incl = a + b;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (t >= (uint32_t)o) incl += y;
            }
            s_rank[2 * t] = incl - a - b;
            s_rank[2 * t + 1] = incl - b;
        }
        __syncthreads();
        const uint32_t at = s_rank[bucket] + r;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            s_walk[a][at] = __float_as_uint(s.root[a]);
            s_walk[3 + a][at] = __float_as_uint(s.dir[a]);
        }
        s_walk[6][at] = s.n;
        s_walk[7][at] = (uint32_t)q;
        __syncthreads();
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            s.root[a] = __uint_as_float(s_walk[a][t]);
            s.dir[a] = __uint_as_float(s_walk[3 + a][t]);
        }
        s.n = s_walk[6][t];
        const uint32_t wq = s_walk[7][t];
        if (s.n) {
            const VoxJob& J = SINGLE ? job0 : s_jobs[find_job(s_item_base, nj, wq)];
            walk_pair<false, PACK, true>(J, wq - J.item_base, s, visits, nullptr, entries, entries_cap, layout, words,
                                         status);
        }
        // the next round writes the shared arrays only after its first barrier, which every
        // thread reaches after its reads of this round
    }
}

// SINGLE = true: a one-style call; the style comes as the kernel parameter
// job0 (constant bank, free to read in the visit loop).  Otherwise the job
// table is copied into shared memory and each item looks its style up.
// DIRECT (with FILL = false): the counting walk also writes the entries
// into fixed per-brick slices (see emit_run).
template <bool FILL, bool SEG, bool PACK, bool SINGLE, bool SPREAD = false, bool DIRECT = false>
__global__ void bin_kernel(const __grid_constant__ VoxJob job0, const VoxJob* __restrict__ jobs, int nj,
                           uint32_t total_items, float4* pair_tan, uint32_t* visits,
                           uint32_t* cursor, void* entries_raw, size_t entries_cap, const uint2* __restrict__ layout,
                           unsigned long long* words, int fallback)
{
    // a budgeted one-walk call's fill (fallback != 0): needed only when a
    // brick outgrew its fixed slice
    if (FILL && fallback && !words[WORD_DIRECT_OVERFLOW]) return;
    typename Entry<PACK>::T* entries = reinterpret_cast<typename Entry<PACK>::T*>(entries_raw);
    // the job table in shared memory (nj * (sizeof(VoxJob) + 4) bytes of dynamic shared memory)
    extern __shared__ __align__(16) unsigned char bin_smem[];
    VoxJob* s_jobs = reinterpret_cast<VoxJob*>(bin_smem);
    uint32_t* s_item_base = reinterpret_cast<uint32_t*>(s_jobs + nj);
    if (!SINGLE) {
        for (int i = threadIdx.x; i < nj * (int)(sizeof(VoxJob) / 4); i += blockDim.x)
            reinterpret_cast<uint32_t*>(s_jobs)[i] = __ldg(reinterpret_cast<const uint32_t*>(jobs) + i);
        load_bases(jobs, nj, s_item_base, nullptr);
    }
    unsigned status = 0;
    // Fill pass of one style whose visit list is near the L2 size (SPREAD):
    // lane l of global warp w takes item l * cols + w, so a warp's 32 walks
    // come from distant strands and its slice reservations spread over many
    // bricks instead of queueing on one brick's counter.  The scattered entry
    // stores merge in L2 there; a much larger list would reach DRAM as
    // partial sectors, so it keeps consecutive items per warp, as do the
    // counting and one-walk passes (coalesced index, vertex and pair-tangent
    // accesses) and a batch.
    if constexpr (SEG && DIRECT && !FILL && SINGLE) { // a batch keeps its grid-stride rounds barrier-free
        balanced_walk<PACK, SINGLE>(job0, s_jobs, s_item_base, nj, total_items, pair_tan, visits, entries,
                                    entries_cap, layout, words, status);
        if (status) atomicOr(words + WORD_STATUS, (unsigned long long)status);
        return;
    }
    constexpr bool sp = FILL && SINGLE && SEG && SPREAD;
    const uint64_t cols = (total_items + 31) / 32;
    const uint64_t span = sp ? cols * 32 : total_items;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < span;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t q = sp ? (i & 31) * cols + (i >> 5) : i;
        if (q >= total_items) continue;
        const VoxJob& J = SINGLE ? job0 : s_jobs[find_job(s_item_base, nj, (uint32_t)q)];
        const Grid& g = J.g;
        const uint32_t p = (uint32_t)q - J.item_base;
        if (SEG) {
            // the pair's set-up (the fill pass recomputes it: the same bytes as a stored record, no store)
            Seg s;
            const uint2 ij = __ldg(J.pairs + p);
            seg_setup(g, J.v, ij, s, status);
            if (!FILL && J.tan) // tangents[indices[i]]: every visit of the pair adds this one
                pair_tan[q] = make_float4(__ldg(J.tan + 3 * (size_t)ij.x), __ldg(J.tan + 3 * (size_t)ij.x + 1),
                                          __ldg(J.tan + 3 * (size_t)ij.x + 2), 0.0f);
            walk_pair<FILL, PACK, DIRECT>(J, p, s, visits, cursor, entries, entries_cap, layout, words, status);
        } else {
            Visit o;
            if (vertex_visit(g, J.v, p, o))
                emit_run<FILL, PACK>(J.brick_base + o.brick, p, Locals::one(o.local), 1u, visits, cursor, entries, entries_cap,
                                     layout, words, status);
        }
    }
    if (status) atomicOr(words + WORD_STATUS, (unsigned long long)status);
}

// Slices of the visit list per brick (one atomic per 512 bricks), the
// visit total, the largest brick, and the lists of visited bricks by size.
// Two bricks per thread: each list append is a warp's returning atomic, so
// a thread's bricks form a chain of them (16 per thread: 0.014 ms for the
// 32,768 bricks of a 256^3 grid; 2 per thread: 0.008 ms).
__global__ void __launch_bounds__(kRangeThreads) bin_ranges_kernel(const uint32_t* __restrict__ visits, uint32_t nb,
                                                                 uint32_t* cursor, uint32_t* list,
                                                                 unsigned long long* words)
{
    __shared__ uint32_t warp_sums[kRangeThreads / 32];
    __shared__ uint32_t block_base;
    const uint32_t tile = kRangeThreads * kRangeItems;
    for (uint64_t base = (uint64_t)blockIdx.x * tile; base < nb; base += (uint64_t)gridDim.x * tile) {
        uint32_t c[kRangeItems];
        uint32_t sum = 0, vmax = 0;
        unsigned long long vsum = 0;
#pragma unroll
        for (int j = 0; j < kRangeItems; ++j) {
            const uint64_t i = base + (uint64_t)j * kRangeThreads + threadIdx.x;
            c[j] = i < nb ? __ldg(visits + i) : 0u;
            sum += c[j];
            vsum += c[j];
            vmax = max(vmax, c[j]);
        }
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            vsum += __shfl_down_sync(0xffffffffu, vsum, o);
            vmax = max(vmax, __shfl_down_sync(0xffffffffu, vmax, o));
        }
        if (lane == 0) {
            if (vsum) atomicAdd(words + WORD_TOTAL_VISITS, vsum);
            atomicMax(words + WORD_MAX_BRICK_VISITS, (unsigned long long)vmax);
        }
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (int w = 0; w < kRangeThreads / 32; ++w) {
                const uint32_t t = warp_sums[w];
                warp_sums[w] = run;
                run += t;
            }
            block_base = run ? (uint32_t)atomicAdd(words + WORD_BRICK_CURSOR, (unsigned long long)run) : 0u;
        }
        __syncthreads();
        uint32_t start = block_base + warp_sums[warp] + (incl - sum);
#pragma unroll
        for (int j = 0; j < kRangeItems; ++j) {
            const uint64_t i = base + (uint64_t)j * kRangeThreads + threadIdx.x;
            if (i < nb) cursor[i] = start;
            start += c[j];
            // visited bricks: up to kLightBrick visits listed in list[nb, 2 nb) (a warp each), up to
            // kBrickCap from the front of list[0, nb), more from its back
            const bool light = c[j] > 0u && c[j] <= (uint32_t)kLightBrick;
            const bool small = c[j] > (uint32_t)kLightBrick && c[j] <= (uint32_t)kBrickCap, big = c[j] > (uint32_t)kBrickCap;
            const unsigned ml = __ballot_sync(0xffffffffu, light);
            const unsigned m = __ballot_sync(0xffffffffu, small), mb = __ballot_sync(0xffffffffu, big);
            uint32_t at = 0, atb = 0, atl = 0;
            if (lane == 0 && ml) atl = (uint32_t)atomicAdd(words + WORD_LIGHT_LIST, (unsigned long long)__popc(ml));
            if (lane == 0 && m) at = (uint32_t)atomicAdd(words + WORD_BRICK_LIST, (unsigned long long)__popc(m));
            if (lane == 0 && mb) atb = (uint32_t)atomicAdd(words + WORD_BIG_LIST, (unsigned long long)__popc(mb));
            atl = __shfl_sync(0xffffffffu, atl, 0);
            at = __shfl_sync(0xffffffffu, at, 0);
            atb = __shfl_sync(0xffffffffu, atb, 0);
            const unsigned below = (1u << lane) - 1u;
            if (light) list[nb + atl + __popc(ml & below)] = (uint32_t)i;
            if (small) list[at + __popc(m & below)] = (uint32_t)i;
            if (big) list[nb - 1u - (atb + __popc(mb & below))] = (uint32_t)i;
        }
        __syncthreads();
    }
}

// Slice capacity a learned batch layout gives a brick the counted call saw
// `v` visits in: v + 25% + 32, rounded up to 8 entries (unvisited: none).
__host__ __device__ __forceinline__ uint32_t layout_slice(uint32_t v)
{
    return v ? (v + (v >> 2) + 32u + 7u) & ~7u : 0u;
}

// The learned layout of a batch's one-walk calls from a counted call's
// per-brick visits: {first slot, capacity} per brick, the slices disjoint
// (tiles of kRangeThreads * kRangeItems bricks take their ranges with one
// atomic each, so the slices of a tile are contiguous, the tiles in any
// order).  The next calls with the same bricks walk once, each brick's
// entries going to its slice.
__global__ void __launch_bounds__(kRangeThreads) layout_kernel(const uint32_t* __restrict__ visits, uint32_t nb,
                                                             uint2* __restrict__ layout, unsigned long long* words)
{
    __shared__ uint32_t warp_sums[kRangeThreads / 32];
    __shared__ uint32_t block_base;
    const uint32_t tile = kRangeThreads * kRangeItems;
    for (uint64_t base = (uint64_t)blockIdx.x * tile; base < nb; base += (uint64_t)gridDim.x * tile) {
        uint32_t c[kRangeItems];
        uint32_t sum = 0;
#pragma unroll
        for (int j = 0; j < kRangeItems; ++j) {
            const uint64_t i = base + (uint64_t)j * kRangeThreads + threadIdx.x;
            c[j] = i < nb ? layout_slice(__ldg(visits + i)) : 0u;
            sum += c[j];
        }
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (int w = 0; w < kRangeThreads / 32; ++w) {
                const uint32_t t = warp_sums[w];
                warp_sums[w] = run;
                run += t;
            }
            block_base = run ? (uint32_t)atomicAdd(words + WORD_LAYOUT_CURSOR, (unsigned long long)run) : 0u;
        }
        __syncthreads();
        uint32_t start = block_base + warp_sums[warp] + (incl - sum);
#pragma unroll
        for (int j = 0; j < kRangeItems; ++j) {
            const uint64_t i = base + (uint64_t)j * kRangeThreads + threadIdx.x;
            if (i < nb) layout[i] = make_uint2(start, c[j]);
            start += c[j];
        }
        __syncthreads();
    }
}

// Zeroes every voxel of the bricks no visit reached (visited bricks are
// written by the brick kernel).  A streaming pass in the volumes' own order:
// one thread per group of 4 voxels along x (16-byte stores of counts and
// tangents, 4-byte stores of densities when aligned), so that a warp writes
// contiguous memory wherever neighbouring bricks are empty.
__global__ void zero_empty_kernel(const VoxJob* __restrict__ jobs, int nj, uint32_t total_groups,
                                  const uint32_t* __restrict__ visits)
{
    __shared__ uint32_t s_base[kMaxJobs];
    for (int j = threadIdx.x; j < nj; j += blockDim.x) s_base[j] = jobs[j].zero_base;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total_groups; i += gridDim.x * blockDim.x) {
        const VoxJob& J = jobs[find_job(s_base, nj, i)];
        const Grid& g = J.g;
        const uint32_t li = i - J.zero_base, gw = (g.w + 3) / 4;
        const uint32_t row = li / gw, x0 = 4 * (li - row * gw);
        const uint32_t z = row / g.h, y = row - z * g.h;
        if (__ldg(visits + J.brick_base + (x0 >> 3) + g.nbx * ((y >> 3) + g.nby * (z >> 3)))) continue;
        const size_t vi = x0 + (size_t)g.w * (y + (size_t)g.h * z);
        uint32_t* c = J.counts + vi;
        uint32_t* t = J.tq ? J.tq + vi : nullptr;
        uint8_t* d = J.dens ? J.dens + vi : nullptr;
        const uint32_t n = min(4u, g.w - x0);
        if (n == 4 && !(reinterpret_cast<uintptr_t>(c) & 15u) && (!t || !(reinterpret_cast<uintptr_t>(t) & 15u)) &&
            (!d || !(reinterpret_cast<uintptr_t>(d) & 3u))) {
            *reinterpret_cast<uint4*>(c) = make_uint4(0u, 0u, 0u, 0u);
            if (t) *reinterpret_cast<uint4*>(t) = make_uint4(0u, 0u, 0u, 0u);
            if (d) *reinterpret_cast<uint32_t*>(d) = 0u;
        } else {
            for (uint32_t k = 0; k < n; ++k) {
                c[k] = 0u;
                if (t) t[k] = 0u;
                if (d) d[k] = 0;
            }
        }
    }
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
    const float q = __fmul_rn(__fdiv_rn(s, m), 127.0f);
    return (q == q) ? __float2int_rz(q) : 0;
}

__device__ __forceinline__ uint32_t pack_tangent(float sx, float sy, float sz, uint32_t m)
{
    const float fm = (float)m;
    const int x = quantize1(sx, fm), y = quantize1(sy, fm), z = quantize1(sz, fm);
    return ((uint32_t)(x & 0xff)) | ((uint32_t)(y & 0xff) << 8) | ((uint32_t)(z & 0xff) << 16);
}

// Exclusive scan of 512 values, one per thread; `warp_sums` holds 16 words.
__device__ __forceinline__ uint32_t block_exclusive_scan_512(uint32_t x, uint32_t* warp_sums)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t s = lane < kBrickThreads / 32 ? warp_sums[lane] : 0u;
        uint32_t si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += y;
        }
        if (lane < kBrickThreads / 32) warp_sums[lane] = si - s;
    }
    __syncthreads();
    return warp_sums[warp] + incl - x;
}

template <bool SEG>
__device__ __forceinline__ float4 visit_tangent(const float4* __restrict__ pair_tan, const float* __restrict__ tan,
                                                uint32_t key)
{
    if (SEG) return __ldg(pair_tan + key);
    const float* t = tan + 3 * (size_t)key;
    return make_float4(__ldg(t), __ldg(t + 1), __ldg(t + 2), 0.0f);
}

// The reference's tangent of a voxel with c <= 255 visits is
// trunc(fl(fl(S / c) * 127)) per component, S the serial FP32 sum of its
// visits' tangents in key order (hair_style.cc:311-335).  That map is
// monotone in S, and any other order of the same additions gives a sum F with
// |S - F| <= 2 gamma(c - 1) sum |t_i| (recursive summation, N. J. Higham,
// "Accuracy and Stability of Numerical Algorithms", 2nd ed., 4.2).  So when
// the map agrees at both ends of [F - B, F + B] (B that bound, with the ends
// rounded outward), it is the reference's value, whatever S is; only the
// voxels where it does not are sorted and summed in key order.  c <= 2: every
// order gives the same sum.
__device__ __forceinline__ bool certify(float f, float a, float bound_scale, float m, int& q)
{
    if (!(a < INFINITY)) return false;                 // inf or NaN tangents: the ordered sum decides
    const float b = __fmul_ru(a, bound_scale);
    const int lo = quantize1(__fsub_rd(f, b), m), hi = quantize1(__fadd_ru(f, b), m);
    q = lo;
    return lo == hi;
}

// Per-voxel results of one brick whose visit keys are grouped by local voxel
// at `keys` (shared memory, or the global scratch for bricks above
// kBrickCap): counts and u8 densities, and the tangents.  Every voxel's thread
// of up to kBrickSmall visits adds its tangents in the order its keys were
// grouped and certifies the quantized result (certify).  The voxels it cannot
// certify, and those of more than kBrickSmall visits, go to the crowded
// kernels through a descriptor (their keys copied to the global scratch),
// which sort the keys and add the tangents in key order; should the
// descriptor list be full, an uncertified voxel's thread sorts its keys in
// place (insertion sort) and adds them in order itself.  Block-wide.
template <bool SEG, bool TANG>
__device__ __forceinline__ void resolve_brick(const VoxJob& J, const Grid& g, uint32_t b, const float4* pair_tan,
                                              const uint32_t* cnt, const uint32_t* off, uint32_t* keys,
                                              bool keys_global, uint32_t keys_at,
                                              uint4* hdesc, size_t hdesc_cap, size_t uncert_cap, uint32_t* hkeys,
                                              size_t hkeys_cap, uint32_t job, unsigned long long* words, unsigned& status)
{
    const int tid = threadIdx.x;
    const float* tan = J.tan;
    uint32_t* tq = J.tq;
    const uint32_t bx = b % g.nbx, by = (b / g.nbx) % g.nby, bz = b / (g.nbx * g.nby);
    const uint32_t x = bx * 8 + (tid & 7), y = by * 8 + ((tid >> 3) & 7), z = bz * 8 + (tid >> 6);
    const bool inside = x < g.w && y < g.h && z < g.d;
    const uint32_t c = cnt[tid];
    const uint32_t vi = x + g.w * (y + g.h * z);
    uint32_t* k = keys + (off[tid] - c);
    if (inside) {
        J.counts[vi] = c;
        if (J.dens) J.dens[vi] = (uint8_t)(c < 255u ? c : 255u);
    }
    if (!TANG) return;
    // ---- every voxel of up to kBrickSmall visits: its sum in grouped order, certified
    bool sorted_needed = false;
    if (inside && c <= (uint32_t)kBrickSmall) {
        if (c == 0) {
            tq[vi] = 0u;
        } else {
            float sx = 0.0f, sy = 0.0f, sz = 0.0f, am = 0.0f; // am: sum of max |t_i| over the components
            for (uint32_t i0 = 0; i0 < c; i0 += kGather) {
                float4 tv[kGather];
#pragma unroll
                for (int j = 0; j < kGather; ++j)
                    if (i0 + j < c) tv[j] = visit_tangent<SEG>(pair_tan, tan, k[i0 + j]);
#pragma unroll
                for (int j = 0; j < kGather; ++j)
                    if (i0 + j < c) {
                        sx = __fadd_rn(sx, tv[j].x);
                        sy = __fadd_rn(sy, tv[j].y);
                        sz = __fadd_rn(sz, tv[j].z);
                        am = __fadd_ru(am, fmaxf(fmaxf(fabsf(tv[j].x), fabsf(tv[j].y)), fabsf(tv[j].z)));
                    }
            }
            if (c <= 2u) { // one addition at most: the same sum in every order
                tq[vi] = pack_tangent(sx, sy, sz, c);
            } else {
                // B = 2 gamma(c - 1) sum |t| per component, gamma(n) = n u / (1 - n u) <= 1.01 n u for
                // n < 256 (u = 2^-24); am (rounded up) bounds every component's sum |t|; 2.05 covers both
                const float scale = __fmul_ru((float)(c - 1), 2.05f * 5.9604645e-8f);
                const float fm = (float)c;
                int qx, qy, qz;
                if (certify(sx, am, scale, fm, qx) && certify(sy, am, scale, fm, qy) && certify(sz, am, scale, fm, qz))
                    tq[vi] = ((uint32_t)(qx & 0xff)) | ((uint32_t)(qy & 0xff) << 8) | ((uint32_t)(qz & 0xff) << 16);
                else
                    sorted_needed = true;
            }
        }
    }
    if (inside && (c > (uint32_t)kBrickSmall || sorted_needed)) {
        // crowded: the crowded kernels sort the keys (a warp up to kCrowdWarpMax visits,
        // descriptors from the front of the crowded list; a CTA above, from its back);
        // uncertified: a warp of the crowded-warp kernel, from the list behind it
        unsigned long long hd;
        size_t at;
        bool slot;
        if (sorted_needed) {
            hd = atomicAdd(words + WORD_UNCERT_COUNT, 1ull);
            at = hdesc_cap + (size_t)hd;
            slot = hd < uncert_cap;
        } else {
            const bool by_warp = c <= (uint32_t)kCrowdWarpMax;
            hd = atomicAdd(words + (by_warp ? WORD_BHEAVY_COUNT : WORD_BHEAVY_BIG), 1ull);
            at = by_warp ? (size_t)hd : hdesc_cap - 1 - (size_t)hd;
            slot = hd < hdesc_cap;
        }
        bool listed = false;
        if (slot && keys_global) { // already in the scratch
            hdesc[at] = make_uint4(vi, keys_at + off[tid] - c, c, job);
            listed = true;
        } else if (slot) {
            const unsigned long long hb = atomicAdd(words + WORD_HKEYS_CURSOR, (unsigned long long)c);
            listed = hb + c <= hkeys_cap;
            if (listed)
                for (uint32_t i = 0; i < c; ++i) hkeys[hb + i] = k[i];
            // every slot below the count is written: count 0 marks one the crowded kernels skip
            hdesc[at] = listed ? make_uint4(vi, (uint32_t)hb, c, job) : make_uint4(0u, 0u, 0u, 0u);
        }
        if (!listed && sorted_needed) { // the list is full: this thread sorts the keys in place
            for (uint32_t i = 1; i < c; ++i) {
                const uint32_t key = k[i];
                uint32_t j = i;
                while (j > 0 && k[j - 1] > key) {
                    k[j] = k[j - 1];
                    --j;
                }
                k[j] = key;
            }
            float sx = 0.0f, sy = 0.0f, sz = 0.0f;
            for (uint32_t i = 0; i < c; ++i) {
                const float4 t = visit_tangent<SEG>(pair_tan, tan, k[i]);
                sx = __fadd_rn(sx, t.x);
                sy = __fadd_rn(sy, t.y);
                sz = __fadd_rn(sz, t.z);
            }
            tq[vi] = pack_tangent(sx, sy, sz, c);
        } else if (!listed) {
            status |= VKHR_DEV_LIST_OVERFLOW;
        }
    }
}

// One CTA per visited brick (a device queue over a list of bricks): counts
// per local voxel from the brick's visit entries, then, with tangents, a
// counting sort of the keys by voxel and the per-voxel resolve.  BIG = false
// takes the bricks of up to kBrickCap visits (keys sorted in shared memory,
// list from the front); BIG = true the others (keys sorted into a slice of
// the global key scratch, list from the back).  A brick's entries are the
// slice its fill reserved (compact layout), or the fixed slice of a one-walk
// call: [brick * direct_cap, + count), or with a learned layout
// [layout[brick].x, + count).  The next brick's queue slot
// and bounds are fetched while the current one is processed, and the entry
// passes keep kBrickUnroll loads in flight per thread.  Descriptors for the
// crowded kernels: crowded voxels in hdesc[0, hdesc_cap) (from the front and
// the back), uncertified ones in hdesc[hdesc_cap, + uncert_cap).
constexpr int kBrickUnroll = 4;

template <bool SEG, bool TANG, bool BIG, bool PACK>
__global__ void __launch_bounds__(kBrickThreads, 2)
brick_kernel(const VoxJob* __restrict__ jobs, int nj, const float4* __restrict__ pair_tan_all,
             const uint32_t* __restrict__ visits, const uint32_t* __restrict__ cursor, const uint32_t* __restrict__ list,
             uint32_t list_n, const void* __restrict__ entries_raw, size_t entries_cap,
             const void* __restrict__ slots_raw, size_t slots_n, uint32_t direct_cap, const uint2* __restrict__ layout,
             int speculative, uint4* hdesc, size_t hdesc_cap, size_t uncert_cap, uint32_t* hkeys,
             size_t hkeys_cap, unsigned long long* words)
{
    typedef Entry<PACK> E;
    typedef typename E::T ET;
    // The layout, chosen once into shared memory (kept out of registers).
    // speculative: a budgeted one-walk call, whose overflow only the device
    // knows -- the fixed slices hold every brick's entries when none outgrew
    // its slice, else the fill pass has laid them out compactly.
    __shared__ const ET* s_entries;
    __shared__ const uint2* s_layout;
    __shared__ unsigned long long s_entries_cap;
    __shared__ uint32_t s_dcap;
    if (threadIdx.x == 0) {
        const bool direct = (direct_cap || layout) && !(speculative && words[WORD_DIRECT_OVERFLOW]);
        s_dcap = direct && !layout ? direct_cap : 0u;
        s_layout = direct ? layout : nullptr;
        s_entries = reinterpret_cast<const ET*>(direct ? slots_raw : entries_raw);
        s_entries_cap = direct ? (unsigned long long)slots_n : (unsigned long long)entries_cap;
    }
    extern __shared__ uint32_t sm[];
    uint32_t* cnt = sm;                       // visits per local voxel
    uint32_t* off = sm + kBrickThreads;       // slice cursor per local voxel
    uint32_t* warp_sums = sm + 2 * kBrickThreads;
    uint32_t* keys = sm + 2 * kBrickThreads + 32;              // (BIG = false only)
    __shared__ uint32_t s_gb, s_nv, s_start, s_cap, s_job, s_hb;
    __shared__ uint32_t s_brick_base[kMaxJobs];
    load_bases(jobs, nj, nullptr, s_brick_base);
    const int tid = threadIdx.x;
    unsigned status = 0;
    const uint32_t listed = (uint32_t)words[BIG ? WORD_BIG_LIST : WORD_BRICK_LIST];
    unsigned long long* queue = words + (BIG ? WORD_BIG_QUEUE : WORD_BRICK_QUEUE);
    // thread 0 holds the next brick: its queue slot, then its id and bounds
    uint32_t nq = 0, ngb = 0, nnv = 0, nstart = 0, ncap = 0;
    // a brick's entries: its first one and the capacity of its slice
    auto bounds = [&](uint32_t b, uint32_t nv) {
        if (s_layout) {
            const uint2 sl = s_layout[b];
            nstart = sl.x;
            ncap = sl.y;
        } else if (s_dcap) {
            nstart = b * s_dcap;
            ncap = s_dcap;
        } else {
            nstart = cursor[b] - nv;
            ncap = 0xffffffffu;
        }
    };
    if (tid == 0) {
        nq = (uint32_t)atomicAdd(queue, 1ull);
        if (nq < listed) {
            ngb = BIG ? list[list_n - 1 - nq] : list[nq];
            nnv = visits[ngb];
            bounds(ngb, nnv);
        }
    }
    for (;;) {
        if (tid == 0) {
            s_gb = nq < listed ? ngb : 0xffffffffu;
            s_nv = nnv;
            s_start = nstart;
            s_cap = ncap;
            if (nq < listed) {
                s_job = (uint32_t)find_job(s_brick_base, nj, ngb);
                s_hb = (TANG && BIG) ? (uint32_t)atomicAdd(words + WORD_HKEYS_CURSOR, (unsigned long long)nnv) : 0u;
                nq = (uint32_t)atomicAdd(queue, 1ull); // the brick after: arrives while this one is processed
            }
        }
        cnt[tid] = 0;
        __syncthreads();
        const uint32_t gb = s_gb, nv = s_nv, start = s_start;
        if (gb == 0xffffffffu) break;
        const bool skip = (uint64_t)start + nv > s_entries_cap ||               // visit budget exceeded
                          nv > s_cap ||                                         // past its fixed slice
                          (TANG && BIG && (uint64_t)s_hb + nv > hkeys_cap);     // key scratch exhausted
        if (skip) {
            status |= VKHR_DEV_LIST_OVERFLOW;
            if (tid == 0 && nq < listed) {
                ngb = BIG ? list[list_n - 1 - nq] : list[nq];
                nnv = visits[ngb];
                bounds(ngb, nnv);
            }
        } else {
            const VoxJob& J = jobs[s_job];
            const Grid& g = J.g;
            const uint32_t b = gb - J.brick_base;   // brick within the style's grid
            const float4* pair_tan = pair_tan_all + J.item_base;
            uint32_t* kbase = BIG ? hkeys + s_hb : keys;
            const ET* src = s_entries + start;
            for (uint32_t i0 = tid; i0 < nv; i0 += kBrickThreads * kBrickUnroll) {
                ET e[kBrickUnroll];
#pragma unroll
                for (int j = 0; j < kBrickUnroll; ++j)
                    if (i0 + j * kBrickThreads < nv) e[j] = __ldg(src + i0 + j * kBrickThreads);
#pragma unroll
                for (int j = 0; j < kBrickUnroll; ++j)
                    if (i0 + j * kBrickThreads < nv) atomicAdd(cnt + E::local(e[j]), 1u);
            }
            if (tid == 0 && nq < listed) { // the next brick's bounds, while this one's passes run
                ngb = BIG ? list[list_n - 1 - nq] : list[nq];
                nnv = visits[ngb];
                bounds(ngb, nnv);
            }
            __syncthreads();
            if (TANG) {
                off[tid] = block_exclusive_scan_512(cnt[tid], warp_sums);
                __syncthreads();
                for (uint32_t i0 = tid; i0 < nv; i0 += kBrickThreads * kBrickUnroll) {
                    ET e[kBrickUnroll];
#pragma unroll
                    for (int j = 0; j < kBrickUnroll; ++j)
                        if (i0 + j * kBrickThreads < nv) e[j] = __ldg(src + i0 + j * kBrickThreads);
#pragma unroll
                    for (int j = 0; j < kBrickUnroll; ++j)
                        if (i0 + j * kBrickThreads < nv) kbase[atomicAdd(off + E::local(e[j]), 1u)] = E::key(e[j]);
                }
                __syncthreads(); // also orders the scratch writes before the block's reads
            }
            resolve_brick<SEG, TANG>(J, g, b, pair_tan, cnt, off, kbase, BIG, s_hb, hdesc, hdesc_cap, uncert_cap,
                                     hkeys, hkeys_cap, s_job, words, status);
        }
        __syncthreads();
    }
    if (status) atomicOr(words + WORD_STATUS, (unsigned long long)status);
}

// Bricks of up to kLightBrick visits, one warp each from a device queue over
// list[nb, 2 nb): the same results as brick_kernel with a warp's resources
// instead of a 512-thread CTA's.  31% of the production style's visited
// bricks are this light, with 1.2% of its visits; a CTA's phases and
// barriers cost them as much as a full brick.  The warp counts its brick's
// visits per local voxel, groups the keys by voxel (counting sort in its
// shared memory), then lane l resolves the voxels l, l + 32, ...: counts and
// u8, and the tangent from an any-order sum when certify settles it, else
// from the keys sorted in place (insertion sort, up to kBrickSmall visits)
// or, above that, by the crowded kernels through a descriptor.
template <bool SEG, bool TANG, bool PACK>
__global__ void __launch_bounds__(32 * kLightWarps)
light_brick_kernel(const VoxJob* __restrict__ jobs, int nj, const float4* __restrict__ pair_tan_all,
                   const uint32_t* __restrict__ visits, const uint32_t* __restrict__ cursor,
                   const uint32_t* __restrict__ list, uint32_t list_n, const void* __restrict__ entries_raw,
                   size_t entries_cap, const void* __restrict__ slots_raw, size_t slots_n, uint32_t direct_cap,
                   const uint2* __restrict__ layout, int speculative, uint4* hdesc, size_t hdesc_cap, uint32_t* hkeys,
                   size_t hkeys_cap, unsigned long long* words)
{
    typedef Entry<PACK> E;
    typedef typename E::T ET;
    __shared__ uint32_t s_cnt[kLightWarps][kBrickThreads]; // visits per local voxel
    __shared__ uint32_t s_off[kLightWarps][kBrickThreads]; // each voxel's key range (end after the grouping)
    __shared__ uint32_t s_keys[kLightWarps][kLightBrick];  // the keys grouped by voxel
    __shared__ uint32_t s_brick_base[kMaxJobs];
    load_bases(jobs, nj, nullptr, s_brick_base);
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    uint32_t* cnt = s_cnt[warp];
    uint32_t* off = s_off[warp];
    uint32_t* keys = s_keys[warp];
    // the layout (as brick_kernel chooses it)
    const bool direct = (direct_cap || layout) && !(speculative && words[WORD_DIRECT_OVERFLOW]);
    const ET* ent = reinterpret_cast<const ET*>(direct ? slots_raw : entries_raw);
    const unsigned long long ent_cap = direct ? (unsigned long long)slots_n : (unsigned long long)entries_cap;
    const uint32_t listed = (uint32_t)words[WORD_LIGHT_LIST];
    unsigned status = 0;
    for (;;) {
        uint32_t qi = 0;
        if (lane == 0) qi = (uint32_t)atomicAdd(words + WORD_LIGHT_QUEUE, 1ull);
        qi = __shfl_sync(0xffffffffu, qi, 0);
        if (qi >= listed) break;
        const uint32_t gb = list[list_n + qi];
        const uint32_t nv = visits[gb];
        uint32_t start, cap;
        if (direct && layout) {
            const uint2 sl = layout[gb];
            start = sl.x;
            cap = sl.y;
        } else if (direct) {
            start = gb * direct_cap;
            cap = direct_cap;
        } else {
            start = cursor[gb] - nv;
            cap = 0xffffffffu;
        }
        if ((uint64_t)start + nv > ent_cap || nv > cap || nv > (uint32_t)kLightBrick) {
            status |= VKHR_DEV_LIST_OVERFLOW;
            continue;
        }
        const uint32_t job = (uint32_t)find_job(s_brick_base, nj, gb);
        const VoxJob& J = jobs[job];
        const Grid& g = J.g;
        const uint32_t b = gb - J.brick_base;
        const float4* pair_tan = pair_tan_all + J.item_base;
        const ET* src = ent + start;
        for (uint32_t v = lane; v < (uint32_t)kBrickThreads; v += 32) cnt[v] = 0u;
        __syncwarp();
        for (uint32_t i = lane; i < nv; i += 32) atomicAdd(cnt + E::local(__ldg(src + i)), 1u);
        __syncwarp();
        if (TANG) { // counting sort of the keys by voxel: lane l owns the counters [16 l, 16 l + 16)
            uint32_t run = 0;
#pragma unroll
            for (int j = 0; j < 16; ++j) run += cnt[16 * lane + j];
            uint32_t incl = run;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (unsigned)o) incl += y;
            }
            run = incl - run;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                off[16 * lane + j] = run;
                run += cnt[16 * lane + j];
            }
            __syncwarp();
            for (uint32_t i = lane; i < nv; i += 32) {
                const ET e = __ldg(src + i);
                keys[atomicAdd(off + E::local(e), 1u)] = E::key(e);
            }
            __syncwarp();
        }
        const uint32_t bx = b % g.nbx, by = (b / g.nbx) % g.nby, bz = b / (g.nbx * g.nby);
        for (uint32_t v = lane; v < (uint32_t)kBrickThreads; v += 32) {
            const uint32_t x = bx * 8 + (v & 7), y = by * 8 + ((v >> 3) & 7), z = bz * 8 + (v >> 6);
            if (!(x < g.w && y < g.h && z < g.d)) continue;
            const uint32_t c = cnt[v];
            const uint32_t vi = x + g.w * (y + g.h * z);
            J.counts[vi] = c;
            if (J.dens) J.dens[vi] = (uint8_t)(c < 255u ? c : 255u);
            if (!TANG) continue;
            if (c == 0u) {
                J.tq[vi] = 0u;
                continue;
            }
            uint32_t* k = keys + (off[v] - c);
            if (c <= 255u) { // any-order sum, certified (c <= 2: every order gives the serial sum)
                float sx = 0.0f, sy = 0.0f, sz = 0.0f, am = 0.0f;
                for (uint32_t i0 = 0; i0 < c; i0 += kGather) {
                    float4 tv[kGather];
#pragma unroll
                    for (int j = 0; j < kGather; ++j)
                        if (i0 + j < c) tv[j] = visit_tangent<SEG>(pair_tan, J.tan, k[i0 + j]);
#pragma unroll
                    for (int j = 0; j < kGather; ++j)
                        if (i0 + j < c) {
                            sx = __fadd_rn(sx, tv[j].x);
                            sy = __fadd_rn(sy, tv[j].y);
                            sz = __fadd_rn(sz, tv[j].z);
                            am = __fadd_ru(am, fmaxf(fmaxf(fabsf(tv[j].x), fabsf(tv[j].y)), fabsf(tv[j].z)));
                        }
                }
                if (c <= 2u) {
                    J.tq[vi] = pack_tangent(sx, sy, sz, c);
                    continue;
                }
                const float scale = __fmul_ru((float)(c - 1), 2.05f * 5.9604645e-8f), fm = (float)c;
                int qx, qy, qz;
                if (certify(sx, am, scale, fm, qx) && certify(sy, am, scale, fm, qy) && certify(sz, am, scale, fm, qz)) {
                    J.tq[vi] = ((uint32_t)(qx & 0xff)) | ((uint32_t)(qy & 0xff) << 8) | ((uint32_t)(qz & 0xff) << 16);
                    continue;
                }
            }
            if (c <= (uint32_t)kBrickSmall) { // uncertified: the keys in order (insertion sort), added in that order
                for (uint32_t i = 1; i < c; ++i) {
                    const uint32_t key = k[i];
                    uint32_t j = i;
                    while (j > 0 && k[j - 1] > key) {
                        k[j] = k[j - 1];
                        --j;
                    }
                    k[j] = key;
                }
                float sx = 0.0f, sy = 0.0f, sz = 0.0f;
                for (uint32_t i = 0; i < c; ++i) {
                    const float4 t = visit_tangent<SEG>(pair_tan, J.tan, k[i]);
                    sx = __fadd_rn(sx, t.x);
                    sy = __fadd_rn(sy, t.y);
                    sz = __fadd_rn(sz, t.z);
                }
                J.tq[vi] = pack_tangent(sx, sy, sz, c);
                continue;
            }
            // crowded: the keys to the global scratch and a descriptor for the crowded kernels
            const bool by_warp = c <= (uint32_t)kCrowdWarpMax;
            const unsigned long long hd = atomicAdd(words + (by_warp ? WORD_BHEAVY_COUNT : WORD_BHEAVY_BIG), 1ull);
            if (hd < hdesc_cap) {
                const unsigned long long hb = atomicAdd(words + WORD_HKEYS_CURSOR, (unsigned long long)c);
                const bool fits = hb + c <= hkeys_cap;
                if (fits)
                    for (uint32_t i = 0; i < c; ++i) hkeys[hb + i] = k[i];
                // every slot below the count is written: count 0 marks one the crowded kernels skip
                hdesc[by_warp ? (size_t)hd : hdesc_cap - 1 - (size_t)hd] =
                    fits ? make_uint4(vi, (uint32_t)hb, c, job) : make_uint4(0u, 0u, 0u, 0u);
                if (!fits) status |= VKHR_DEV_LIST_OVERFLOW;
            } else {
                status |= VKHR_DEV_LIST_OVERFLOW;
            }
        }
        __syncwarp(); // the warp's arrays are reused by its next brick
    }
    if (status) atomicOr(words + WORD_STATUS, (unsigned long long)status);
}

__device__ void block_bitonic_sort(uint32_t* s, int n)
{
    for (int k = 2; k <= n; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    const uint32_t a = s[i], bb = s[l];
                    if ((a > bb) == up) { s[i] = bb; s[l] = a; }
                }
            }
            __syncthreads();
        }
}

// Ascending sort of the first `have` keys of s (padded with 0xffffffff to
// the next power of two, at most kHeavyTile).  Block-wide.
__device__ __forceinline__ void sort_prefix(uint32_t* s, uint32_t have)
{
    int n = 2;
    while (n < (int)have) n <<= 1;
    for (int i = (int)have + threadIdx.x; i < n; i += blockDim.x) s[i] = 0xffffffffu;
    __syncthreads();
    block_bitonic_sort(s, n);
}

// Tangent of a crowded voxel from its c keys at src: the smallest min(c, 255)
// keys in ascending (serial) order, then a sequential FP32 sum.  The keys
// stream through in chunks of kCrowdThreads * kCrowdPer; only keys below
// the current 255th-smallest key (thr) are kept, and the buffer is sorted
// and cut back to 255 keys when a chunk would overflow it.  A key equal to
// thr can be dropped: the multiset of the 255 smallest values is unchanged
// (equal keys carry equal tangents).  Block-wide, kCrowdThreads threads.
constexpr int kCrowdThreads = 256;
constexpr int kCrowdPer = 4;
static_assert(kKeep - 1 + kCrowdThreads * kCrowdPer <= kHeavyTile, "a chunk must fit after a cut");

__device__ void resolve_crowded(const uint32_t* src, uint32_t c, const float* __restrict__ tan,
                                const uint2* __restrict__ pairs, uint32_t* keys, float (*tv)[kKeep], uint32_t* out)
{
    __shared__ uint32_t warp_tot[kCrowdThreads / 32];
    __shared__ uint32_t s_thr;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t m = c < 255u ? c : 255u;
    uint32_t have = 0, thr = 0xffffffffu;
    for (uint32_t base = 0; base < c; base += kCrowdThreads * kCrowdPer) {
        uint32_t k[kCrowdPer];
#pragma unroll
        for (int j = 0; j < kCrowdPer; ++j) {
            const uint32_t i = base + j * kCrowdThreads + threadIdx.x;
            k[j] = i < c ? __ldg(src + i) : 0xffffffffu;
        }
        for (int pass = 0; pass < 2; ++pass) {
            uint32_t a = 0;
#pragma unroll
            for (int j = 0; j < kCrowdPer; ++j) a += k[j] < thr ? 1u : 0u;
            if (!__syncthreads_or(a != 0)) break; // nothing below the threshold
            // block exclusive scan of the accepted counts
            uint32_t incl = a;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            if (lane == 31) warp_tot[warp] = incl;
            __syncthreads();
            uint32_t before = 0, total = 0;
#pragma unroll
            for (int w = 0; w < kCrowdThreads / 32; ++w) {
                const uint32_t t = warp_tot[w];
                before += w < warp ? t : 0u;
                total += t;
            }
            __syncthreads(); // warp_tot is rewritten by the next scan
            if (have + total > (uint32_t)kHeavyTile) { // cut back to the 255 smallest, raise the threshold
                sort_prefix(keys, have);
                have = 255u;
                if (threadIdx.x == 0) s_thr = keys[254];
                __syncthreads();
                thr = s_thr;
                continue; // filter the chunk again (it fits now)
            }
            uint32_t at = have + before + incl - a;
#pragma unroll
            for (int j = 0; j < kCrowdPer; ++j)
                if (k[j] < thr) keys[at++] = k[j];
            have += total;
            __syncthreads();
            break;
        }
    }
    sort_prefix(keys, have);
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const float* t = tan + 3 * (size_t)key_vertex(keys[i], pairs);
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
        *out = pack_tangent(sx, sy, sz, m);
    }
    __syncthreads();
}

// Tangent input of a visit key: the pair's stored tangent (segments) or the
// vertex's own (vertices).
__device__ __forceinline__ void key_tangent(const VoxJob& J, const float4* __restrict__ pair_tan_all, uint32_t key,
                                            float& x, float& y, float& z)
{
    if (J.pairs) {
        const float4 t = __ldg(pair_tan_all + J.item_base + key);
        x = t.x;
        y = t.y;
        z = t.z;
    } else {
        const float* t = J.tan + 3 * (size_t)key;
        x = __ldg(t);
        y = __ldg(t + 1);
        z = __ldg(t + 2);
    }
}

// Ascending bitonic sort of 32 * R keys held R per lane; after it the key at
// (lane, r) has rank lane * R + r.  Exchanges with partners less than R
// apart stay in registers, the others go through shuffles.
template <int R>
__device__ __forceinline__ void warp_sort(uint32_t (&v)[R])
{
    const unsigned lane = lane_id();
#pragma unroll
    for (int k = 2; k <= 32 * R; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j < R) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int pr = r ^ j;
                    if (pr > r) {
                        const bool up = ((lane * R + r) & k) == 0;
                        const uint32_t a = v[r], b = v[pr];
                        if ((a > b) == up) {
                            v[r] = b;
                            v[pr] = a;
                        }
                    }
                }
            } else {
                const int lj = j / R;
                const bool lower = (lane & lj) == 0;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const uint32_t o = __shfl_xor_sync(0xffffffffu, v[r], lj);
                    const bool up = ((lane * R + r) & k) == 0;
                    v[r] = (lower == up) ? min(v[r], o) : max(v[r], o);
                }
            }
        }
    }
}

// One crowded voxel (c <= 32 * R keys at src) by one warp.  Up to 255
// visits (every tangent is summed): the warp adds them in any order and
// certifies the quantized result as resolve_brick does (the bound holds for
// any order of the c - 1 additions); otherwise -- or past 255 visits, where
// the 255 smallest keys are the ones summed -- sort, gather the first
// min(c, 255) tangents into shared memory in parallel, then lanes 0..2 add
// the x, y and z components in key order.
template <int R>
__device__ __forceinline__ void resolve_warp(const VoxJob& J, const float4* __restrict__ pair_tan_all,
                                             const uint32_t* __restrict__ src, uint32_t c, float (*wt)[kKeep],
                                             uint32_t* out)
{
    const unsigned lane = lane_id();
    uint32_t v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) { // coalesced load; a sorting network takes any input order
        const uint32_t i = (uint32_t)r * 32u + lane;
        v[r] = i < c ? __ldg(src + i) : 0xffffffffu;
    }
    if (c <= 255u) {
        float sx = 0.0f, sy = 0.0f, sz = 0.0f, am = 0.0f;
#pragma unroll
        for (int r = 0; r < R; ++r)
            if ((uint32_t)r * 32u + lane < c) {
                float x, y, z;
                key_tangent(J, pair_tan_all, v[r], x, y, z);
                sx = __fadd_rn(sx, x);
                sy = __fadd_rn(sy, y);
                sz = __fadd_rn(sz, z);
                am = __fadd_ru(am, fmaxf(fmaxf(fabsf(x), fabsf(y)), fabsf(z)));
            }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) { // every lane ends with the same sums
            sx = __fadd_rn(sx, __shfl_xor_sync(0xffffffffu, sx, o));
            sy = __fadd_rn(sy, __shfl_xor_sync(0xffffffffu, sy, o));
            sz = __fadd_rn(sz, __shfl_xor_sync(0xffffffffu, sz, o));
            am = __fadd_ru(am, __shfl_xor_sync(0xffffffffu, am, o));
        }
        const float scale = __fmul_ru((float)(c - 1), 2.05f * 5.9604645e-8f), fm = (float)c;
        int qx, qy, qz;
        if (certify(sx, am, scale, fm, qx) && certify(sy, am, scale, fm, qy) && certify(sz, am, scale, fm, qz)) {
            if (lane == 0) *out = ((uint32_t)(qx & 0xff)) | ((uint32_t)(qy & 0xff) << 8) | ((uint32_t)(qz & 0xff) << 16);
            return;
        }
    }
    warp_sort<R>(v);
    const uint32_t m = c < 255u ? c : 255u;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t p = lane * R + r;
        if (p < m) key_tangent(J, pair_tan_all, v[r], wt[0][p], wt[1][p], wt[2][p]);
    }
    __syncwarp();
    float sum = 0.0f;
    if (lane < 3)
        for (uint32_t i = 0; i < m; ++i) sum = __fadd_rn(sum, wt[lane][i]);
    const float sx = __shfl_sync(0xffffffffu, sum, 0), sy = __shfl_sync(0xffffffffu, sum, 1),
                sz = __shfl_sync(0xffffffffu, sum, 2);
    if (lane == 0) *out = pack_tangent(sx, sy, sz, m);
    __syncwarp();
}

constexpr int kCrowdWarps = 8; // warps per CTA of crowded_warp_kernel

// Crowded voxels of up to kCrowdWarpMax visits, one warp each (descriptors
// from the front of the list: voxel, key offset, count, style).
__global__ void __launch_bounds__(32 * kCrowdWarps) crowded_warp_kernel(const VoxJob* __restrict__ jobs,
                                                                        const float4* __restrict__ pair_tan_all,
                                                                        const uint4* __restrict__ hdesc,
                                                                        size_t hdesc_cap, size_t uncert_cap,
                                                                        const uint32_t* __restrict__ hkeys,
                                                                        const unsigned long long* words)
{
    __shared__ float wt[kCrowdWarps][3][kKeep];
    unsigned long long nh = words[WORD_BHEAVY_COUNT], nu = words[WORD_UNCERT_COUNT];
    if (nh > hdesc_cap) nh = hdesc_cap;
    if (nu > uncert_cap) nu = uncert_cap;
    const unsigned warp = threadIdx.x >> 5;
    for (unsigned long long h = (unsigned long long)blockIdx.x * kCrowdWarps + warp; h < nh + nu;
         h += (unsigned long long)gridDim.x * kCrowdWarps) {
        const uint4 d = hdesc[h < nh ? h : hdesc_cap + (h - nh)];
        if (d.z == 0u) continue; // a slot whose keys did not fit the scratch
        const VoxJob& J = jobs[d.w];
        if (d.z <= 128u) resolve_warp<4>(J, pair_tan_all, hkeys + d.y, d.z, wt[warp], J.tq + d.x);
        else resolve_warp<8>(J, pair_tan_all, hkeys + d.y, d.z, wt[warp], J.tq + d.x);
    }
}

// Crowded voxels above kCrowdWarpMax visits, one CTA each (descriptors from
// the back of the list).
__global__ void __launch_bounds__(kCrowdThreads) crowded_kernel(const VoxJob* __restrict__ jobs,
                                                                const uint4* __restrict__ hdesc, size_t hdesc_cap,
                                                                const uint32_t* __restrict__ hkeys,
                                                                const unsigned long long* words)
{
    __shared__ uint32_t keys[kHeavyTile];
    __shared__ float tv[3][kKeep];
    unsigned long long nh = words[WORD_BHEAVY_BIG];
    if (nh > hdesc_cap) nh = hdesc_cap;
    for (unsigned long long h = blockIdx.x; h < nh; h += gridDim.x) {
        const uint4 d = hdesc[hdesc_cap - 1 - h];
        if (d.z == 0u) continue; // a slot whose keys did not fit the scratch
        const VoxJob& J = jobs[d.w];
        resolve_crowded(hkeys + d.y, d.z, J.tan, J.pairs, keys, tv, J.tq + d.x);
    }
}

// ---- Volume::normalize ------------------------------------------------------------------

__global__ void init_minmax_kernel(unsigned long long* words)
{
    if (threadIdx.x == 0) {
        words[WORD_NORM + 0] = 255ull;
        words[WORD_NORM + 1] = 0ull;
    }
}

__global__ void minmax_u8_kernel(const uint8_t* __restrict__ d, uint64_t n, unsigned long long* words)
{
    __shared__ uint32_t s_lo, s_hi;
    if (threadIdx.x == 0) {
        s_lo = 255u;
        s_hi = 0u;
    }
    __syncthreads();
    uint32_t lo = 255, hi = 0;
    const uint64_t n16 = n / 16;
    const uint4* d16 = reinterpret_cast<const uint4*>(d);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n16; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 q = __ldg(d16 + i);
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int s = 0; s < 32; s += 8) {
                const uint32_t x = (w[k] >> s) & 0xffu;
                lo = min(lo, x);
                hi = max(hi, x);
            }
    }
    for (uint64_t i = n16 * 16 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        lo = min(lo, (uint32_t)d[i]);
        hi = max(hi, (uint32_t)d[i]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_down_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_down_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&s_lo, lo);
        atomicMax(&s_hi, hi);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicMin(words + WORD_NORM + 0, (unsigned long long)s_lo);
        atomicMax(words + WORD_NORM + 1, (unsigned long long)s_hi);
    }
}

// hair_style.cc:344-357: d = u8((d - min) * (255.0f / (max - min))), truncating.
__device__ __forceinline__ uint32_t rescale1(uint32_t x, uint32_t lo, uint32_t hi, float scaling)
{
    return hi > lo ? (__float2uint_rz(__fmul_rn((float)(x - lo), scaling)) & 0xffu) : 0u;
}

__global__ void rescale_u8_kernel(uint8_t* d, uint64_t n, const unsigned long long* words)
{
    const uint32_t lo = (uint32_t)words[WORD_NORM + 0], hi = (uint32_t)words[WORD_NORM + 1];
    const float scaling = hi > lo ? __fdiv_rn(255.0f, (float)(int)(hi - lo)) : 0.0f;
    auto word = [&](uint32_t q) {
        return rescale1(q & 0xffu, lo, hi, scaling) | (rescale1((q >> 8) & 0xffu, lo, hi, scaling) << 8) |
               (rescale1((q >> 16) & 0xffu, lo, hi, scaling) << 16) | (rescale1(q >> 24, lo, hi, scaling) << 24);
    };
    const uint64_t n16 = n / 16; // 16 texels (one 16-byte load and store) per item
    uint4* d16 = reinterpret_cast<uint4*>(d);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n16; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 q = d16[i];
        d16[i] = make_uint4(word(q.x), word(q.y), word(q.z), word(q.w));
    }
    for (uint64_t i = n16 * 16 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        d[i] = (uint8_t)rescale1(d[i], lo, hi, scaling);
}

// ---- Volume::downsample ----------------------------------------------------------------

// One output voxel per thread: the 2x2x2 neighbourhood of the input in the
// reference's order (x fastest), reduced by the filter.
__global__ void downsample_kernel(const uint8_t* __restrict__ in, uint32_t w, uint32_t h, uint32_t d, int filter,
                                  uint8_t* __restrict__ out)
{
    const uint32_t ow = w / 2, oh = h / 2, od = d / 2;
    const uint64_t n = (uint64_t)ow * oh * od;
    for (uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; o < n; o += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(o % ow), j = (uint32_t)((o / ow) % oh), k = (uint32_t)(o / ((uint64_t)ow * oh));
        uint32_t mx = 0, mn = 255, sum = 0;
#pragma unroll
        for (int z = 0; z < 2; ++z)
#pragma unroll
            for (int y = 0; y < 2; ++y)
#pragma unroll
                for (int x = 0; x < 2; ++x) {
                    const uint32_t v =
                        __ldg(in + (2 * i + x) + (size_t)w * ((2 * j + y) + (size_t)h * (2 * k + z)));
                    mx = max(mx, v);
                    mn = min(mn, v);
                    sum += v;
                }
        out[o] = (uint8_t)(filter == VKHR_FILTER_MAX ? mx
                           : filter == VKHR_FILTER_MIN ? mn
                           : filter == VKHR_FILTER_MEAN ? sum / 8u
                                                        : min(sum, 255u));
    }
}

// ---- host ----------------------------------------------------------------------------------

vkhr_status make_grid(vkhr_ctx* ctx, const vkhr_aabb* b, int32_t w, int32_t h, int32_t d, int32_t mode, Grid& g)
{
    if (!b) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "bounds is NULL");
    if (w <= 0 || h <= 0 || d <= 0) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "resolution must be positive");
    if (h > 65535 || d > 65535) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "height and depth must be <= 65535");
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
    g.d = (uint32_t)d;
    g.n = (uint32_t)n;
    g.wh = (uint32_t)w * (uint32_t)h;
    g.nbx = (g.w + 7) / 8;
    g.nby = (g.h + 7) / 8;
    g.nbz = (g.d + 7) / 8;
    g.nb = g.nbx * g.nby * g.nbz;
    g.mode = mode;
    g.exact_coords = (mode == VKHR_INDEX_EXACT || n <= (1ull << 24)) ? 1 : 0;
    return VKHR_OK;
}

vkhr_status check_device_status(vkhr_ctx* ctx, unsigned long long s)
{
    if (s & VKHR_DEV_STEPS_OVERFLOW)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG,
                         "a segment spans more than 2^24 voxels (vertices far outside the bounds)");
    if (s & VKHR_DEV_LIST_OVERFLOW) return vkhr_fail(ctx, VKHR_ERR_CAPACITY, "visit list overflow");
    if (s & VKHR_DEV_REPLAY_MISMATCH) return vkhr_fail(ctx, VKHR_ERR_CUDA, "brick replay disagreed with binning");
    if (s & VKHR_DEV_TIMEOUT) return vkhr_fail(ctx, VKHR_ERR_TIMEOUT, "a bounded device wait ran out (a brick load never landed)");
    if (s & VKHR_DEV_BAD_INDEX)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "a fragment's pixel or a PPLL node link is out of range");
    return VKHR_OK;
}

// Reports (and clears) the device status bits; a visit-list overflow also
// forgets the learned visit totals, so the next unbudgeted call at each size
// counts its visits again.
vkhr_status report_status(vkhr_ctx* ctx, unsigned long long status, cudaStream_t st)
{
    if (!status) return VKHR_OK;
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_words + WORD_STATUS, 0, sizeof(unsigned long long), st));
    if (status & VKHR_DEV_LIST_OVERFLOW)
        for (int i = 0; i < kLearnedSizes; ++i) ctx->learned[i].visits = 0;
    return check_device_status(ctx, status);
}

bool same_size(const vkhr_learned_visits& l, const vkhr_voxel_job& j, bool tang)
{
    return l.visits && l.items == j.item_count && l.w == j.width && l.h == j.height && l.d == j.depth &&
           l.mode == (j.index_mode | (tang ? 2 : 0));
}

// Visit total of the last counted call at this size (0: none).
uint64_t learned_visits(const vkhr_ctx* ctx, const vkhr_voxel_job& j, bool tang)
{
    for (int i = 0; i < kLearnedSizes; ++i)
        if (same_size(ctx->learned[i], j, tang)) return ctx->learned[i].visits;
    return 0;
}

void learn_visits(vkhr_ctx* ctx, const vkhr_voxel_job& j, bool tang, uint64_t visits)
{
    int at = -1;
    for (int i = 0; i < kLearnedSizes && at < 0; ++i)
        if (same_size(ctx->learned[i], j, tang)) at = i;
    if (at < 0) {
        at = ctx->learned_next;
        ctx->learned_next = (ctx->learned_next + 1) % kLearnedSizes;
    }
    ctx->learned[at] = vkhr_learned_visits{j.item_count, j.width, j.height, j.depth, j.index_mode | (tang ? 2 : 0),
                                           visits ? visits : 1};
}

template <bool SEG, bool TANG, bool PACK>
vkhr_status launch_brick(vkhr_ctx* ctx, const VoxJob* d_jobs, int nj, uint32_t total_bricks, cudaStream_t st,
                         unsigned blocks, size_t entries_cap, size_t keys_cap, uint32_t direct_cap,
                         const uint2* layout, size_t slots_n, bool speculative, size_t crowd_cap, size_t uncert_cap)
{
    const int spec = speculative ? 1 : 0;
    // bricks above kBrickCap (their keys go to the global scratch) on the side
    // stream, alongside the rest on st; the caller joins the side stream
    const size_t small = (size_t)(2 * kBrickThreads + 32) * sizeof(uint32_t); // counters, cursors, warp sums
    const size_t smem = small + (TANG ? (size_t)kBrickCap * sizeof(uint32_t) : 0);
    vkhr_status s = vkhr_fork_side(ctx, st); // after the fill
    if (s != VKHR_OK) return s;
    VKHR_LAUNCH(ctx, (brick_kernel<SEG, TANG, true, PACK>), (unsigned)ctx->sm_count * 2, kBrickThreads, small, ctx->side,
                d_jobs, nj, ctx->pair_tan, ctx->brick_visits, ctx->brick_cursor, ctx->brick_list, total_bricks,
                ctx->items, entries_cap, ctx->slots, slots_n, direct_cap, layout, spec, ctx->hdesc, crowd_cap,
                uncert_cap, ctx->hkeys, keys_cap, ctx->d_words);
    // bricks of up to kLightBrick visits, a warp each, also on the side stream (launched before the
    // shared-memory bricks' persistent CTAs take the SMs)
    VKHR_LAUNCH(ctx, (light_brick_kernel<SEG, TANG, PACK>), (unsigned)ctx->sm_count * 8, 32 * kLightWarps, 0, ctx->side,
                d_jobs, nj, ctx->pair_tan, ctx->brick_visits, ctx->brick_cursor, ctx->brick_list, total_bricks,
                ctx->items, entries_cap, ctx->slots, slots_n, direct_cap, layout, spec, ctx->hdesc, crowd_cap,
                ctx->hkeys, keys_cap, ctx->d_words);
    VKHR_CUDA_TRY(ctx, cudaFuncSetAttribute(brick_kernel<SEG, TANG, false, PACK>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    VKHR_LAUNCH(ctx, (brick_kernel<SEG, TANG, false, PACK>), blocks, kBrickThreads, smem, st, d_jobs, nj,
                ctx->pair_tan, ctx->brick_visits, ctx->brick_cursor, ctx->brick_list, total_bricks, ctx->items,
                entries_cap, ctx->slots, slots_n, direct_cap, layout, spec, ctx->hdesc, crowd_cap, uncert_cap, ctx->hkeys,
                keys_cap, ctx->d_words);
    return VKHR_OK;
}

// Validates one job and fills its device description.
vkhr_status make_job(vkhr_ctx* ctx, bool segments, const vkhr_voxel_job& in, VoxJob& out)
{
    vkhr_status s = make_grid(ctx, &in.bounds, in.width, in.height, in.depth, in.index_mode, out.g);
    if (s != VKHR_OK) return s;
    const uint64_t n_items = segments ? in.item_count / 2 : in.item_count; // floor(n / 2) index pairs
    if (n_items >= (1ull << 32)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "more than 2^32 - 1 vertices or pairs");
    const uint32_t n_in = (uint32_t)n_items;
    if (!in.d_counts) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_counts is NULL");
    if (in.d_tangents && !in.d_tangent_in && n_in)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_tangents requested without d_tangent_in");
    if (n_in && !in.d_vertices) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_vertices is NULL");
    if (segments && n_in && !in.d_indices) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_indices is NULL");
    if (segments && in.d_indices && (reinterpret_cast<uintptr_t>(in.d_indices) & 7u))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_indices must be 8-byte aligned");
    if (in.d_tangents && (reinterpret_cast<uintptr_t>(in.d_tangents) & 3u))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_tangents must be 4-byte aligned");
    out.v = in.d_vertices;
    out.tan = in.d_tangents ? in.d_tangent_in : nullptr;
    out.pairs = segments ? reinterpret_cast<const uint2*>(in.d_indices) : nullptr;
    out.counts = in.d_counts;
    out.dens = in.d_densities;
    out.tq = reinterpret_cast<uint32_t*>(in.d_tangents);
    out.n_in = n_in;
    out.zero_base = 0;
    return VKHR_OK;
}

// Dynamic shared memory of a launch that keeps at most k of its CTAs
// resident per SM (k CTAs of it fit in an SM's shared memory, k + 1 do
// not), at least `base` bytes, next to the kernel's `static_bytes` of static
// shared memory; k <= 0 or k >= 8 (the register limit of the walk kernels):
// base.
size_t residency_smem(const vkhr_ctx* ctx, int k, size_t base, size_t static_bytes)
{
    if (k <= 0 || k >= 8 || ctx->smem_per_sm <= 0) return base;
    const size_t per_block = (size_t)ctx->smem_per_sm / (size_t)k;
    const size_t fixed = (size_t)ctx->smem_reserved + static_bytes;
    const size_t s = per_block > fixed ? per_block - fixed : 0;
    return std::max(s, base);
}

// The shape a learned batch layout is kept for: the styles' grids and pair
// counts, tangents requested, entry size.
uint64_t batch_shape(const VoxJob* jobs, int nj, bool tang, bool pack)
{
    uint64_t h = 1469598103934665603ull; // FNV-1a over the fields
    auto mix = [&h](uint64_t x) { h = (h ^ x) * 1099511628211ull; };
    mix((uint64_t)nj);
    mix(tang ? 1 : 0);
    mix(pack ? 1 : 0);
    for (int j = 0; j < nj; ++j) {
        mix(jobs[j].g.w);
        mix(jobs[j].g.h);
        mix(jobs[j].g.d);
        mix(jobs[j].n_in);
    }
    return h | 1u; // 0 means "no layout"
}

// Learns a batch's one-walk layout from the exact per-brick visits of this
// call's counting walk (queued after it on st): each visited brick gets a
// slice of layout_slice(visits) entries.  The slices span at most
// visits + visits / 4 + 39 per visited brick; a batch whose span would pass
// kDirectBytes (or 2^32 entries), or a context with live frame graphs, keeps
// two walks.
vkhr_status learn_layout(vkhr_ctx* ctx, uint64_t shape, uint32_t nb, uint64_t visits, uint64_t visited,
                         size_t entry_bytes, cudaStream_t st)
{
    ctx->layout_shape = 0;
    const uint64_t slots = visits + visits / 4 + 39 * visited + 8;
    if (slots >= (1ull << 32) || slots * entry_bytes > kDirectBytes || ctx->live_graphs) return VKHR_OK;
    vkhr_status s = vkhr_reserve(ctx, (void**)&ctx->layout, &ctx->layout_cap, nb ? nb : 1, sizeof(uint2));
    if (s != VKHR_OK) return s;
    s = vkhr_reserve(ctx, (void**)&ctx->slots, &ctx->slots_cap, (slots * entry_bytes + 7) / 8, sizeof(uint2));
    if (s != VKHR_OK) return s;
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_words + WORD_LAYOUT_CURSOR, 0, sizeof(unsigned long long), st));
    const unsigned blocks = std::min(vkhr_blocks(nb, kRangeThreads * kRangeItems), (unsigned)ctx->sm_count * 8);
    VKHR_LAUNCH(ctx, layout_kernel, blocks, kRangeThreads, 0, st, ctx->brick_visits, nb, ctx->layout, ctx->d_words);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    ctx->layout_shape = shape;
    ctx->layout_bricks = nb;
    ctx->layout_slots = slots;
    return VKHR_OK;
}

// count_visits: a segment call without a budget reads its visit total back
// even when an earlier call at its size taught the context one.
vkhr_status voxelize_batch(vkhr_ctx* ctx, bool segments, const vkhr_voxel_job* jobs_in, int nj, cudaStream_t st,
                           bool count_visits = false)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (nj <= 0 || nj > kMaxJobs || !jobs_in) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "job count must be in [1, 256]");
    VoxJob jobs[kMaxJobs];
    uint64_t items = 0, bricks = 0, groups = 0;
    const bool tang = jobs_in[0].d_tangents != nullptr;
    for (int j = 0; j < nj; ++j) {
        vkhr_status s = make_job(ctx, segments, jobs_in[j], jobs[j]);
        if (s != VKHR_OK) return s;
        if ((jobs_in[j].d_tangents != nullptr) != tang)
            return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "every job of a batch requests tangents, or none does");
        jobs[j].item_base = (uint32_t)items;
        jobs[j].brick_base = (uint32_t)bricks;
        jobs[j].zero_base = (uint32_t)groups;
        items += jobs[j].n_in;
        bricks += jobs[j].g.nb;
        groups += (uint64_t)((jobs[j].g.w + 3) / 4) * jobs[j].g.h * jobs[j].g.d;
        if (items >= (1ull << 32) || bricks >= (1ull << 32) || groups >= (1ull << 32))
            return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "batch too large (2^32 items, bricks or 4-voxel groups)");
    }
    const uint32_t total_items = (uint32_t)items, total_bricks = (uint32_t)bricks, total_groups = (uint32_t)groups;
    // 4-byte visit entries when every key fits in 23 bits (or keys are not needed)
    bool pack = true;
    for (int j = 0; j < nj; ++j) pack = pack && (!tang || jobs[j].n_in <= kPackedKeyLimit);
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));

    // job table: pinned staging (reused once the previous upload has run) -> device
    vkhr_status s = vkhr_reserve(ctx, (void**)&ctx->d_jobs, &ctx->jobs_cap, (size_t)nj * sizeof(VoxJob), 1);
    if (s != VKHR_OK) return s;
    // A captured call leaves the copy in the graph, which reads the staging
    // again at each replay: the staging then keeps this table until the
    // context's next voxelization.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    VKHR_CUDA_TRY(ctx, cudaStreamIsCapturing(st, &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    if (!capturing) VKHR_CUDA_TRY(ctx, cudaEventSynchronize(ctx->jobs_ev));
    std::memcpy(ctx->h_jobs, jobs, (size_t)nj * sizeof(VoxJob));
    VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_jobs, ctx->h_jobs, (size_t)nj * sizeof(VoxJob), cudaMemcpyHostToDevice, st));
    if (!capturing) VKHR_CUDA_TRY(ctx, cudaEventRecord(ctx->jobs_ev, st));
    const VoxJob* d_jobs = reinterpret_cast<const VoxJob*>(ctx->d_jobs);

    // per-brick bookkeeping: visits and visit-list cursor
    s = vkhr_reserve(ctx, (void**)&ctx->brick_runs, &ctx->brick_cap, 2ull * total_bricks + 1, sizeof(uint32_t));
    if (s != VKHR_OK) return s;
    ctx->brick_visits = ctx->brick_runs;
    ctx->brick_cursor = ctx->brick_runs + total_bricks;
    // visited bricks: [0, nb) the shared-memory and global-scratch bricks, [nb, 2 nb) the light ones
    s = vkhr_reserve(ctx, (void**)&ctx->brick_list, &ctx->brick_list_cap, 2ull * total_bricks + 1ull, sizeof(uint32_t));
    if (s != VKHR_OK) return s;
    if (segments && total_items) {
        if (tang) {
            s = vkhr_reserve(ctx, (void**)&ctx->pair_tan, &ctx->pair_tan_cap, total_items, sizeof(float4));
            if (s != VKHR_OK) return s;
        }
    }
    // Capacities that do not depend on the data: vertex mode is bounded by
    // the vertex count; segment mode by the visit budget when one is set,
    // and a one-style call without a budget, at a size the context counted
    // before, by twice that count (a call above it records a list overflow).
    // Only the first call at a size reads its visit total back.
    uint64_t learned = 0;
    if (segments && !ctx->visit_budget && nj == 1 && ctx->direct_cap && total_items && !count_visits)
        learned = learned_visits(ctx, jobs_in[0], tang);
    const bool bounded = !segments || ctx->visit_budget > 0 || learned > 0;
    uint64_t visits_total = 0; // unbounded: the count read back below
    if (!segments) visits_total = total_items;
    else if (ctx->visit_budget) visits_total = ctx->visit_budget;
    else if (learned) visits_total = std::min<uint64_t>(2 * learned + 4096, (1ull << 32) - 1);
    if (bounded) {
        s = vkhr_reserve(ctx, (void**)&ctx->items, &ctx->items_cap, visits_total ? visits_total : 1, sizeof(uint2));
        if (s != VKHR_OK) return s;
    }
    // One walk instead of two: when the context knows a slice per brick and
    // the slices fit in memory, the counting walk also writes every run into
    // its brick's slice of a separate buffer.  One style: the slices are
    // [brick * capacity, + capacity), the capacity learned from earlier
    // calls' largest brick.  A batch: the layout learned from the last
    // counted call of the same shape (each visited brick its count + 25%).
    // A brick past its slice is counted but not written and raises the
    // call's overflow word.  Without a budget the read-back shows it and the
    // call fills again compactly; with a budget (no read-back, the call may
    // be captured) the device decides: the fill pass runs only after an
    // overflow, and the brick kernel reads whichever layout holds the entries.
    const size_t entry_bytes = pack ? sizeof(uint32_t) : sizeof(uint2);
    const uint64_t shape = (segments && nj > 1) ? batch_shape(jobs, nj, tang, pack) : 0;
    uint32_t direct_cap = 0;
    size_t slots_n = 0;
    bool use_layout = shape && total_items && ctx->layout && ctx->layout_shape == shape &&
                      ctx->layout_bricks == total_bricks;
    if (use_layout) {
        s = vkhr_reserve(ctx, (void**)&ctx->slots, &ctx->slots_cap, (ctx->layout_slots * entry_bytes + 7) / 8,
                         sizeof(uint2));
        if (s != VKHR_OK) return s;
        slots_n = ctx->layout_slots;
    } else if (segments && total_items && ctx->direct_cap && nj == 1) {
        const uint64_t slots = (uint64_t)total_bricks * ctx->direct_cap;
        if (slots < (1ull << 32) && slots * entry_bytes <= kDirectBytes) {
            s = vkhr_reserve(ctx, (void**)&ctx->slots, &ctx->slots_cap, (slots * entry_bytes + 7) / 8, sizeof(uint2));
            if (s != VKHR_OK) return s;
            direct_cap = ctx->direct_cap;
            slots_n = slots;
        }
    }
    const bool one_walk = direct_cap != 0 || use_layout;
    const bool speculative = bounded && one_walk; // the device picks the layout
    // per-call words; the status bits stay until a check reports them
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_words, 0, WORD_STATUS * sizeof(unsigned long long), st));
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_words + WORD_STATUS + 1, 0,
                                       (WORD_NORM - WORD_STATUS - 1) * sizeof(unsigned long long), st));
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(ctx->brick_visits, 0, (size_t)total_bricks * sizeof(uint32_t), st));
    const unsigned threads = kWalkThreads;
    // one style: one item per thread (blocks retire and start staggered, so
    // their set-up loads overlap other blocks' walks); a batch caps the grid,
    // as every block copies the job table into shared memory
    const unsigned in_blocks = nj == 1 ? vkhr_blocks(total_items, threads)
                                       : std::min(vkhr_blocks(total_items, threads), (unsigned)ctx->sm_count * 16);
    const size_t bin_smem_bytes = (size_t)nj * (sizeof(VoxJob) + sizeof(uint32_t));
    const bool single = nj == 1;
    const uint2* layout = use_layout ? ctx->layout : nullptr;
    // the one walk's dynamic shared memory, sized to keep walk_ctas CTAs resident per SM
    const size_t walk_smem = residency_smem(ctx, ctx->walk_ctas[single ? 0 : 1], single ? 0 : bin_smem_bytes,
                                           single ? kWalkStaticSmem : 0);
#define VKHR_DIRECT(PACK_)                                                                                        \
    do {                                                                                                         \
        if (single) {                                                                                            \
            VKHR_CUDA_TRY(ctx, cudaFuncSetAttribute(bin_kernel<false, true, PACK_, true, false, true>,            \
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)walk_smem)); \
            VKHR_LAUNCH(ctx, (bin_kernel<false, true, PACK_, true, false, true>), in_blocks, threads, walk_smem,   \
                        st, jobs[0], d_jobs, nj, total_items, ctx->pair_tan, ctx->brick_visits,                  \
                        ctx->brick_cursor, ctx->slots, (size_t)direct_cap, layout, ctx->d_words, 0);              \
        } else {                                                                                                 \
            VKHR_CUDA_TRY(ctx, cudaFuncSetAttribute(bin_kernel<false, true, PACK_, false, false, true>,           \
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)walk_smem)); \
            VKHR_LAUNCH(ctx, (bin_kernel<false, true, PACK_, false, false, true>), in_blocks, threads, walk_smem,  \
                        st, jobs[0], d_jobs, nj, total_items, ctx->pair_tan, ctx->brick_visits,                  \
                        ctx->brick_cursor, ctx->slots, (size_t)direct_cap, layout, ctx->d_words, 0);              \
        }                                                                                                        \
    } while (0)
    if (total_items && one_walk) {
        if (pack) VKHR_DIRECT(true);
        else VKHR_DIRECT(false);
    } else if (total_items) {
        if (segments && single)
            VKHR_LAUNCH(ctx, (bin_kernel<false, true, false, true>), in_blocks, threads, 0, st, jobs[0], d_jobs, nj,
                        total_items, ctx->pair_tan, ctx->brick_visits, ctx->brick_cursor, nullptr,
                        (size_t)0, nullptr, ctx->d_words, 0);
        else if (segments)
            VKHR_LAUNCH(ctx, (bin_kernel<false, true, false, false>), in_blocks, threads, bin_smem_bytes, st, jobs[0],
                        d_jobs, nj, total_items, ctx->pair_tan, ctx->brick_visits, ctx->brick_cursor,
                        nullptr, (size_t)0, nullptr, ctx->d_words, 0);
        else if (single)
            VKHR_LAUNCH(ctx, (bin_kernel<false, false, false, true>), in_blocks, threads, 0, st, jobs[0], d_jobs, nj,
                        total_items, ctx->pair_tan, ctx->brick_visits, ctx->brick_cursor, nullptr,
                        (size_t)0, nullptr, ctx->d_words, 0);
        else
            VKHR_LAUNCH(ctx, (bin_kernel<false, false, false, false>), in_blocks, threads, bin_smem_bytes, st, jobs[0],
                        d_jobs, nj, total_items, ctx->pair_tan, ctx->brick_visits, ctx->brick_cursor,
                        nullptr, (size_t)0, nullptr, ctx->d_words, 0);
    }
#undef VKHR_DIRECT
    const unsigned rblocks = std::min(vkhr_blocks(total_bricks, kRangeThreads * kRangeItems), (unsigned)ctx->sm_count * 8);
    VKHR_LAUNCH(ctx, bin_ranges_kernel, rblocks, kRangeThreads, 0, st, ctx->brick_visits, total_bricks,
                ctx->brick_cursor, ctx->brick_list, ctx->d_words);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());

    if (!bounded) {          // segment mode without a budget: read the visit total back
        if (capturing)
            return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG,
                             "segment voxelization under stream capture needs a visit budget (vkhr_set_visit_budget)");
        VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->h_words, ctx->d_words, WORD_NORM * sizeof(unsigned long long),
                                           cudaMemcpyDeviceToHost, st));
        VKHR_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        s = report_status(ctx, ctx->h_words[WORD_STATUS], st); // this call's, or earlier unreported errors
        if (s != VKHR_OK) return s;
        visits_total = ctx->h_words[WORD_TOTAL_VISITS];
        if (visits_total >= (1ull << 32))
            return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "more than 2^32 - 1 voxel visits in one call");
        if (nj == 1) learn_visits(ctx, jobs_in[0], tang, visits_total);
        // the next calls' per-brick capacity: this call's largest brick + 25%, grow-only
        const uint64_t largest = ctx->h_words[WORD_MAX_BRICK_VISITS];
        const uint64_t want = (largest + largest / 4 + 63) / 64 * 64;
        if (want > ctx->direct_cap && want < (1ull << 31)) ctx->direct_cap = (uint32_t)want;
        if (one_walk && ctx->h_words[WORD_DIRECT_OVERFLOW]) { // a brick outgrew its slice: fill compactly
            direct_cap = 0;
            use_layout = false;
        }
        if (!direct_cap && !use_layout) {
            s = vkhr_reserve(ctx, (void**)&ctx->items, &ctx->items_cap, visits_total ? visits_total : 1, sizeof(uint2));
            if (s != VKHR_OK) return s;
            // a batch learns (again) the layout its next calls walk once into
            if (shape) {
                s = learn_layout(ctx, shape, total_bricks, visits_total,
                                 ctx->h_words[WORD_LIGHT_LIST] + ctx->h_words[WORD_BRICK_LIST] +
                                     ctx->h_words[WORD_BIG_LIST],
                                 entry_bytes, st);
                if (s != VKHR_OK) return s;
            }
        }
    }
    // capacities the kernels check against (the budget, not the grown scratch)
    const size_t cap_visits = visits_total ? (size_t)visits_total : 1;
    const size_t crowd_cap = (size_t)(visits_total / (kBrickSmall + 1)) + 1;
    if (tang) {
        s = vkhr_reserve(ctx, (void**)&ctx->hkeys, &ctx->hkeys_cap, visits_total ? visits_total : 1, sizeof(uint32_t));
        if (s != VKHR_OK) return s;
        // crowded voxels (above kBrickSmall visits: at most crowd_cap of them), then as many
        // uncertified ones at least (past the list's end their own threads sort their keys)
        s = vkhr_reserve(ctx, (void**)&ctx->hdesc, &ctx->hdesc_cap, 2 * crowd_cap, sizeof(uint4));
        if (s != VKHR_OK) return s;
    }
    const size_t uncert_cap = tang ? ctx->hdesc_cap - crowd_cap : 0;
    // Unvisited bricks are zeroed on the side stream, alongside the fill and
    // the brick kernel (disjoint voxels); every return below joins it.
    s = vkhr_fork_side(ctx, st);
    if (s != VKHR_OK) return s;
    VKHR_LAUNCH(ctx, zero_empty_kernel, std::min(vkhr_blocks(total_groups, 256), (unsigned)ctx->sm_count * 16), 256, 0,
                ctx->side, d_jobs, nj, total_groups, ctx->brick_visits);
    if (total_items && (!(direct_cap || use_layout) || speculative)) {
        void* ent = ctx->items;
        const int fallback = speculative ? 1 : 0; // the fill runs only after an overflow
        // as a fallback its blocks mostly return at once: a grid of 8 per SM (grid-stride)
        const unsigned fill_blocks = speculative ? std::min(in_blocks, (unsigned)ctx->sm_count * 8) : in_blocks;
        // spread a one-style fill's warps over distant strands when its visit
        // list is within twice the L2 size: most scattered entry stores still
        // merge in L2 (measured: a 123 MB list gains, a 1.8 GB list loses)
        const bool spread = single && segments && (uint64_t)cap_visits * (pack ? sizeof(uint32_t) : sizeof(uint2)) <=
                                                      2ull * (uint64_t)ctx->l2_bytes;
#define VKHR_FILL(SEG_, PACK_)                                                                                    \
    do {                                                                                                         \
        if (single && SEG_ && spread)                                                                            \
            VKHR_LAUNCH(ctx, (bin_kernel<true, SEG_, PACK_, true, true>), fill_blocks, threads, 0, st, jobs[0],      \
                        d_jobs, nj, total_items, ctx->pair_tan, ctx->brick_visits,                 \
                        ctx->brick_cursor, ent, cap_visits, nullptr, ctx->d_words, fallback);                          \
        else if (single)                                                                                         \
            VKHR_LAUNCH(ctx, (bin_kernel<true, SEG_, PACK_, true>), fill_blocks, threads, 0, st, jobs[0], d_jobs, nj,  \
                        total_items, ctx->pair_tan, ctx->brick_visits, ctx->brick_cursor, ent,     \
                        cap_visits, nullptr, ctx->d_words, fallback);                                                  \
        else                                                                                                     \
            VKHR_LAUNCH(ctx, (bin_kernel<true, SEG_, PACK_, false>), fill_blocks, threads, bin_smem_bytes, st,       \
                        jobs[0], d_jobs, nj, total_items, ctx->pair_tan, ctx->brick_visits,        \
                        ctx->brick_cursor, ent, cap_visits, nullptr, ctx->d_words, fallback);                          \
    } while (0)
        if (segments && pack) VKHR_FILL(true, true);
        else if (segments) VKHR_FILL(true, false);
        else if (pack) VKHR_FILL(false, true);
        else VKHR_FILL(false, false);
#undef VKHR_FILL
    }
    const unsigned bblocks = std::min(total_bricks, (unsigned)ctx->sm_count * 2);
#define VKHR_BRICK(SEG_, TANG_, PACK_)                                                                            \
    launch_brick<SEG_, TANG_, PACK_>(ctx, d_jobs, nj, total_bricks, st, bblocks, cap_visits, cap_visits, direct_cap,     \
                                     use_layout ? ctx->layout : nullptr, slots_n, speculative, crowd_cap, uncert_cap)
    if (segments) {
        if (!tang) s = VKHR_BRICK(true, false, true);
        else if (pack) s = VKHR_BRICK(true, true, true);
        else s = VKHR_BRICK(true, true, false);
    } else {
        if (!tang) s = VKHR_BRICK(false, false, true);
        else if (pack) s = VKHR_BRICK(false, true, true);
        else s = VKHR_BRICK(false, true, false);
    }
#undef VKHR_BRICK
    const vkhr_status joined = vkhr_join_side(ctx, st); // zeroing and big bricks done before the crowded voxels
    if (s != VKHR_OK) return s;
    if (joined != VKHR_OK) return joined;
    if (tang) { // crowded voxels of up to / above kCrowdWarpMax visits: independent descriptor lists
        s = vkhr_fork_side(ctx, st);
        if (s != VKHR_OK) return s;
        VKHR_LAUNCH(ctx, crowded_kernel, (unsigned)ctx->sm_count * 6, kCrowdThreads, 0, ctx->side, d_jobs, ctx->hdesc,
                    crowd_cap, ctx->hkeys, ctx->d_words);
        VKHR_LAUNCH(ctx, crowded_warp_kernel, (unsigned)ctx->sm_count * 8, 32 * kCrowdWarps, 0, st, d_jobs,
                    ctx->pair_tan, ctx->hdesc, crowd_cap, uncert_cap, ctx->hkeys, ctx->d_words);
        s = vkhr_join_side(ctx, st);
        if (s != VKHR_OK) return s;
    }
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
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!bounds) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "bounds is NULL");
    vkhr_voxel_job j = {d_vertices, d_tangent_in, nullptr, vertex_count, *bounds, width, height, depth, index_mode,
                        d_counts, d_densities, d_tangents};
    return voxelize_batch(ctx, false, &j, 1, (cudaStream_t)stream);
}

vkhr_status vkhr_voxelize_segments(vkhr_ctx* ctx, const float* d_vertices, const float* d_tangent_in,
                                   const uint32_t* d_indices, uint64_t index_count, const vkhr_aabb* bounds,
                                   int32_t width, int32_t height, int32_t depth, int32_t index_mode,
                                   uint32_t* d_counts, uint8_t* d_densities, int8_t* d_tangents, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!bounds) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "bounds is NULL");
    vkhr_voxel_job j = {d_vertices, d_tangent_in, d_indices, index_count, *bounds, width, height, depth, index_mode,
                        d_counts, d_densities, d_tangents};
    return voxelize_batch(ctx, true, &j, 1, (cudaStream_t)stream);
}

vkhr_status vkhr_voxelize_batched(vkhr_ctx* ctx, int32_t segments, const vkhr_voxel_job* jobs, int32_t job_count,
                                  void* stream)
{
    return voxelize_batch(ctx, segments != 0, jobs, job_count, (cudaStream_t)stream);
}

} // extern "C"

vkhr_status vkhr_voxelize_counted(vkhr_ctx* ctx, const vkhr_voxel_job* job, void* stream, uint64_t* visits)
{
    const uint64_t keep = ctx->visit_budget;
    ctx->visit_budget = 0;
    const vkhr_status s = voxelize_batch(ctx, true, job, 1, (cudaStream_t)stream, true);
    ctx->visit_budget = keep;
    if (s == VKHR_OK) *visits = ctx->h_words[WORD_TOTAL_VISITS];
    return s;
}

extern "C" {

vkhr_status vkhr_set_visit_budget(vkhr_ctx* ctx, uint64_t max_visits)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (max_visits >= (1ull << 32)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "budget must be below 2^32 visits");
    ctx->visit_budget = max_visits;
    return VKHR_OK;
}

vkhr_status vkhr_set_voxelize_walk(vkhr_ctx* ctx, int32_t which, int32_t ctas_per_sm)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (which != 0 && which != 1) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "which must be 0 (one style) or 1 (batch)");
    if (ctas_per_sm < 0 || ctas_per_sm > 8) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "ctas_per_sm must be in [0, 8]");
    ctx->walk_ctas[which] = ctas_per_sm;
    return VKHR_OK;
}

vkhr_status vkhr_autotune_voxelize(vkhr_ctx* ctx, const vkhr_voxel_job* jobs, int32_t job_count, int32_t* chosen,
                                   float* ms_out, void* stream)
{
    static const int kChoices[VKHR_WALK_CHOICES] = {0, 2, 3, 4, 5, 6};
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!chosen) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "chosen is required");
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    const int which = job_count == 1 ? 0 : 1;
    // counted once, without a budget: the sizes, the one-walk capacity or
    // layout, and the visits; then timed under the budget
    const uint64_t saved_budget = ctx->visit_budget;
    ctx->visit_budget = 0;
    vkhr_status s = voxelize_batch(ctx, true, jobs, job_count, st, true);
    if (s != VKHR_OK) {
        ctx->visit_budget = saved_budget;
        return s;
    }
    const uint64_t v = ctx->h_words[WORD_TOTAL_VISITS];
    ctx->visit_budget = saved_budget ? saved_budget : std::min<uint64_t>(v + v / 4 + 4096, (1ull << 32) - 1);
    cudaEvent_t e[2];
    VKHR_CUDA_TRY(ctx, cudaEventCreate(&e[0]));
    if (cudaEventCreate(&e[1]) != cudaSuccess) {
        cudaEventDestroy(e[0]);
        ctx->visit_budget = saved_budget;
        return vkhr_fail(ctx, VKHR_ERR_CUDA, "cudaEventCreate failed");
    }
    const int previous = ctx->walk_ctas[which];
    float ms[VKHR_WALK_CHOICES] = {0.0f};
    int best = 0;
    for (int c = 0; c < VKHR_WALK_CHOICES && s == VKHR_OK; ++c) {
        ctx->walk_ctas[which] = kChoices[c];
        float t[3] = {0.0f, 0.0f, 0.0f};
        for (int r = -1; r < 3 && s == VKHR_OK; ++r) { // one warm-up, three timed runs
            if (cudaEventRecord(e[0], st) != cudaSuccess) s = vkhr_fail(ctx, VKHR_ERR_CUDA, "cudaEventRecord failed");
            if (s == VKHR_OK) s = voxelize_batch(ctx, true, jobs, job_count, st);
            if (s == VKHR_OK && (cudaEventRecord(e[1], st) != cudaSuccess || cudaEventSynchronize(e[1]) != cudaSuccess))
                s = vkhr_fail(ctx, VKHR_ERR_CUDA, "timing the autotune runs failed");
            if (s == VKHR_OK && r >= 0 && cudaEventElapsedTime(&t[r], e[0], e[1]) != cudaSuccess)
                s = vkhr_fail(ctx, VKHR_ERR_CUDA, "cudaEventElapsedTime failed");
        }
        std::sort(t, t + 3);
        ms[c] = t[1];
        if (c > 0 && ms[c] < ms[best]) best = c;
    }
    cudaEventDestroy(e[0]);
    cudaEventDestroy(e[1]);
    ctx->visit_budget = saved_budget;
    if (s == VKHR_OK) s = vkhr_check_status(ctx, stream); // a run that overflowed its budget
    if (s != VKHR_OK) {
        ctx->walk_ctas[which] = previous;
        return s;
    }
    ctx->walk_ctas[which] = kChoices[best];
    *chosen = kChoices[best];
    if (ms_out)
        for (int c = 0; c < VKHR_WALK_CHOICES; ++c) ms_out[c] = ms[c];
    return VKHR_OK;
}

vkhr_status vkhr_downsample_densities(vkhr_ctx* ctx, const uint8_t* d_in, int32_t width, int32_t height,
                                      int32_t depth, int32_t filter, uint8_t* d_out, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!d_in || !d_out) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_in and d_out are required");
    if (width <= 0 || height <= 0 || depth <= 0 || (width | height | depth) & 1)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "dimensions must be positive and even");
    if (filter < VKHR_FILTER_MAX || filter > VKHR_FILTER_SUM)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "unknown filter");
    if ((uint64_t)width * height * depth >= (1ull << 32))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "more than 2^32 - 1 voxels");
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const uint64_t n = (uint64_t)(width / 2) * (height / 2) * (depth / 2);
    VKHR_LAUNCH(ctx, downsample_kernel, std::min(vkhr_blocks(n, 256), (unsigned)ctx->sm_count * 32), 256, 0,
                (cudaStream_t)stream, d_in, (uint32_t)width, (uint32_t)height, (uint32_t)depth, filter, d_out);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

vkhr_status vkhr_check_status(vkhr_ctx* ctx, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->h_words, ctx->d_words, WORD_NORM * sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    VKHR_CUDA_TRY(ctx, cudaStreamSynchronize((cudaStream_t)stream));
    return report_status(ctx, ctx->h_words[WORD_STATUS], (cudaStream_t)stream); // reported once

}

vkhr_status vkhr_normalize_densities(vkhr_ctx* ctx, uint8_t* d, uint64_t n, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (n == 0) return VKHR_OK;
    if (!d) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_densities is NULL");
    if (reinterpret_cast<uintptr_t>(d) & 15u)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_densities must be 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    VKHR_LAUNCH(ctx, init_minmax_kernel, 1, 32, 0, st, ctx->d_words);
    const unsigned blocks = std::min(vkhr_blocks(n / 16 + 1, 256), (unsigned)ctx->sm_count * 4);
    VKHR_LAUNCH(ctx, minmax_u8_kernel, blocks, 256, 0, st, d, n, ctx->d_words);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    const unsigned rb = std::min(vkhr_blocks(n / 16 + 1, 256), (unsigned)ctx->sm_count * 16);
    VKHR_LAUNCH(ctx, rescale_u8_kernel, rb, 256, 0, st, d, n, ctx->d_words);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

} // extern "C"
