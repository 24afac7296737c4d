// composite.cu -- the hybrid level-of-detail compositing step: the reference's
// per-pixel linked-list resolve (share/shaders/transparency/resolve.comp:15-101
// over ppll.glsl's nodes) and a PPLL-free form of the same step.
//
// vkhr_resolve_ppll walks the reference's lists as they are: one thread per
// pixel, the k-buffer in registers.
//
// vkhr_composite needs no list.  Each pixel resolves the list a PPLL would
// hold had the strand fragments been linked in buffer order and the volume
// fragment after them: the volume fragment first, then the strand fragments
// newest first.  The fragments are put in pixel order by a stable LSD radix
// sort (digits of at most 10 bits: two passes below 2^20 pixels), which keeps
// buffer order within each pixel, so every pixel's list is its slice of the
// sorted payloads read backwards:
//   radix pass (x2)  -- per tile of 4096 fragments a digit histogram, an
//                       exclusive scan over (digit, tile), and a scatter that
//                       ranks equal digits in buffer order (warp-private
//                       counters, __match_any_sync within a round of 32);
//   slice bounds     -- the first sorted entry of every pixel (binary search);
//   resolve          -- one thread per pixel runs resolve.comp's k-buffer over
//                       its volume fragment and the last 1040 entries of its
//                       slice, loaded 8 at a time.
// The payload that moves is 8 bytes (colour | depth bits << 32) with a 4-byte
// key; fragments whose pixel is outside the image sort past the last pixel.
#include "common.cuh"

#include <algorithm>

namespace {

constexpr int kK = VKHR_K_BUFFER_SIZE;     // 16
constexpr int kTail = VKHR_MAX_FRAGMENTS;  // 1024
constexpr uint32_t kList = kK + kTail;     // nodes one pixel can resolve
constexpr uint32_t kNull = VKHR_PPLL_NULL;

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4 * kScanThreads;  // values per scan block

constexpr int kTileWarps = 8;
constexpr int kTileThreads = 32 * kTileWarps;
constexpr int kRounds = 16;                   // rounds of 32 fragments per warp
constexpr int kTile = kTileThreads * kRounds; // 4096 fragments per tile
constexpr int kMaxDigitBits = 10;

static_assert(sizeof(vkhr_fragment) == 12 && sizeof(vkhr_ppll_node) == 12, "12-byte nodes and fragments");

// ---- colour arithmetic (unpackUnorm4x8, mix, packUnorm4x8) --------------------
struct Frag {
    uint32_t c;
    float d;
};

__device__ __forceinline__ Frag unpack_payload(unsigned long long x)
{
    return Frag{(uint32_t)x, __uint_as_float((uint32_t)(x >> 32))};
}

// tab[i] = i / 255 (IEEE division), one copy per block in shared memory
__device__ __forceinline__ void fill_unorm_table(float* tab)
{
    for (int i = threadIdx.x; i < 256; i += blockDim.x) tab[i] = __fdiv_rn((float)i, 255.0f);
    __syncthreads();
}

__device__ __forceinline__ float4 unpack(const float* tab, uint32_t c)
{
    return make_float4(tab[c & 0xffu], tab[(c >> 8) & 0xffu], tab[(c >> 16) & 0xffu], tab[c >> 24]);
}

// resolved = mix(resolved, c, c.a) (resolve.comp:72-73, :97-98)
__device__ __forceinline__ void blend(float4& r, const float* tab, uint32_t c)
{
    const float4 f = unpack(tab, c);
    const float t = __fsub_rn(1.0f, f.w);
    r.x = __fadd_rn(__fmul_rn(r.x, t), __fmul_rn(f.x, f.w));
    r.y = __fadd_rn(__fmul_rn(r.y, t), __fmul_rn(f.y, f.w));
    r.z = __fadd_rn(__fmul_rn(r.z, t), __fmul_rn(f.z, f.w));
    r.w = __fadd_rn(__fmul_rn(r.w, t), __fmul_rn(f.w, f.w));
}

// float -> UNORM8: clamp to [0, 1] (NaN to 0), times 255, nearest, ties to even
__device__ __forceinline__ uint32_t unorm8(float x) { return __float2uint_rn(__fmul_rn(__saturatef(x), 255.0f)); }
__device__ __forceinline__ uint32_t pack(float4 v)
{
    return unorm8(v.x) | unorm8(v.y) << 8 | unorm8(v.z) << 16 | unorm8(v.w) << 24;
}

// ---- exclusive scan of n words (3 kernels) --------------------------------------
// Exclusive scan of one value per thread over a block of kScanThreads;
// `total` receives the block's sum.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t* warp_sums, uint32_t& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) warp_sums[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = warp_sums[lane];
        uint32_t s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_sums[lane] = s - w; // exclusive over warps
        if (lane == 31) warp_sums[32] = s;
    }
    __syncthreads();
    const uint32_t r = warp_sums[warp] + v - x;
    total = warp_sums[32];
    __syncthreads(); // warp_sums is reused by the next call
    return r;
}

// The 4 values at base (values past n count 0); `in` is 16-byte aligned.
__device__ __forceinline__ uint4 load4(const uint32_t* __restrict__ in, uint32_t n, uint32_t base)
{
    if (base + 4 <= n) return *reinterpret_cast<const uint4*>(in + base);
    uint4 c = make_uint4(0, 0, 0, 0);
    if (base + 0 < n) c.x = in[base + 0];
    if (base + 1 < n) c.y = in[base + 1];
    if (base + 2 < n) c.z = in[base + 2];
    if (base + 3 < n) c.w = in[base + 3];
    return c;
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const uint32_t* __restrict__ in, uint32_t n,
                                                                   uint32_t* __restrict__ partials)
{
    __shared__ uint32_t warp_sums[33];
    const uint4 c = load4(in, n, blockIdx.x * kScanItems + 4 * threadIdx.x);
    uint32_t total;
    block_exclusive_scan(c.x + c.y + c.z + c.w, warp_sums, total);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

// One block: partials[b] becomes the exclusive prefix of the block sums.
__global__ void __launch_bounds__(kScanThreads) scan_partials_kernel(uint32_t* __restrict__ partials, uint32_t nb)
{
    __shared__ uint32_t warp_sums[33];
    uint32_t carry = 0;
    for (uint32_t c0 = 0; c0 < nb; c0 += kScanThreads) {
        const uint32_t i = c0 + threadIdx.x;
        const uint32_t x = i < nb ? partials[i] : 0u;
        uint32_t total;
        const uint32_t e = block_exclusive_scan(x, warp_sums, total);
        if (i < nb) partials[i] = carry + e;
        carry += total;
    }
}

// out[i] = exclusive prefix of in (out may be in).
__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const uint32_t* in, uint32_t n,
                                                                  const uint32_t* __restrict__ partials, uint32_t* out)
{
    __shared__ uint32_t warp_sums[33];
    const uint32_t base = blockIdx.x * kScanItems + 4 * threadIdx.x;
    const uint4 c = load4(in, n, base);
    uint32_t total;
    uint32_t s = block_exclusive_scan(c.x + c.y + c.z + c.w, warp_sums, total) + partials[blockIdx.x];
    const uint32_t cv[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) out[base + k] = s;
        s += cv[k];
    }
}

// ---- stable LSD radix sort of the fragments by pixel ---------------------------
// Keys are pixels (npix for a fragment outside the image); a pass orders by
// the digit (key >> shift) & (2^bits - 1).  The histograms are stored
// digit-major, hist[digit * tiles + tile], so that their exclusive scan gives
// every (digit, tile) its first output slot.
template <bool FIRST>
__global__ void __launch_bounds__(kTileThreads) radix_hist_kernel(const vkhr_fragment* __restrict__ f,
                                                                  const uint32_t* __restrict__ keys, uint32_t n,
                                                                  uint32_t npix, int shift, int bits, uint32_t tiles,
                                                                  uint32_t* __restrict__ hist,
                                                                  unsigned long long* words)
{
    __shared__ uint32_t h[1 << kMaxDigitBits];
    const uint32_t radix = 1u << bits, mask = radix - 1u;
    for (uint32_t d = threadIdx.x; d < radix; d += kTileThreads) h[d] = 0u;
    __syncthreads();
    bool bad = false;
    const uint32_t base = blockIdx.x * kTile;
    for (uint32_t k = threadIdx.x; k < (uint32_t)kTile; k += kTileThreads) {
        const uint32_t i = base + k;
        if (i >= n) break;
        uint32_t key;
        if (FIRST) {
            key = __ldg(&f[i].pixel);
            if (key >= npix) {
                key = npix;
                bad = true;
            }
        } else {
            key = keys[i];
        }
        atomicAdd(&h[(key >> shift) & mask], 1u);
    }
    if (FIRST && bad) atomicOr(&words[WORD_STATUS], (unsigned long long)VKHR_DEV_BAD_INDEX);
    __syncthreads();
    for (uint32_t d = threadIdx.x; d < radix; d += kTileThreads) hist[d * tiles + blockIdx.x] = h[d];
}

// Warp w of a tile owns its fragments [w * 512, (w + 1) * 512) in rounds of
// 32 (buffer order: round-major, lane-minor).  Pass 1 counts every digit per
// warp; the counts become slots (the tile's scanned offset, then the warps in
// order); pass 2 hands them out round by round, lanes with equal digits in
// lane order.  So equal digits keep buffer order: the sort is stable.
template <bool FIRST>
__global__ void __launch_bounds__(kTileThreads) radix_scatter_kernel(
    const vkhr_fragment* __restrict__ f, const uint32_t* __restrict__ keys_in,
    const unsigned long long* __restrict__ vals_in, uint32_t n, uint32_t npix, int shift, int bits, uint32_t tiles,
    const uint32_t* __restrict__ offsets, uint32_t* __restrict__ keys_out, unsigned long long* __restrict__ vals_out)
{
    __shared__ uint32_t wh[kTileWarps << kMaxDigitBits];
    const uint32_t radix = 1u << bits, mask = radix - 1u;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    for (uint32_t i = threadIdx.x; i < (uint32_t)kTileWarps * radix; i += kTileThreads) wh[i] = 0u;
    __syncthreads();
    uint32_t* my = wh + warp * radix;
    const uint32_t base = blockIdx.x * kTile + warp * (kRounds * 32);
    uint32_t key[kRounds];
    unsigned long long val[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const uint32_t i = base + r * 32 + lane;
        const bool ok = i < n;
        key[r] = 0xffffffffu;
        val[r] = 0ull;
        if (ok) {
            if (FIRST) {
                const uint32_t p = __ldg(&f[i].pixel);
                key[r] = p < npix ? p : npix;
                val[r] = (unsigned long long)__ldg(&f[i].color) |
                         (unsigned long long)__float_as_uint(__ldg(&f[i].depth)) << 32;
            } else {
                key[r] = keys_in[i];
                val[r] = vals_in[i];
            }
        }
        const uint32_t d = ok ? (key[r] >> shift) & mask : 0xffffffffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        if (ok && lane == __ffs(peers) - 1) my[d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (uint32_t d = threadIdx.x; d < radix; d += kTileThreads) {
        uint32_t run = offsets[d * tiles + blockIdx.x];
        for (int w = 0; w < kTileWarps; ++w) {
            const uint32_t c = wh[w * radix + d];
            wh[w * radix + d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const uint32_t i = base + r * 32 + lane;
        const bool ok = i < n;
        const uint32_t d = ok ? (key[r] >> shift) & mask : 0xffffffffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t pos = ok ? my[d] + __popc(peers & lt) : 0u;
        __syncwarp();
        if (ok && lane == __ffs(peers) - 1) my[d] += __popc(peers);
        __syncwarp();
        if (ok) {
            keys_out[pos] = key[r];
            vals_out[pos] = val[r];
        }
    }
}

// start[p] = the first sorted entry whose pixel is >= p, for p in [0, npix];
// start[npix] counts the fragments inside the image.
__global__ void __launch_bounds__(256) slice_bounds_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                                           uint32_t npix, uint32_t* __restrict__ start)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > npix) return;
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (__ldg(&keys[mid]) < p) lo = mid + 1;
        else hi = mid;
    }
    start[p] = lo;
}

// ---- resolve --------------------------------------------------------------------------
// resolve.comp:15-101 for one pixel.  The k-buffer lives in shared memory,
// slot k of thread t at [k * kResolveThreads + t]: a lane's dynamic slot always
// falls in its own bank, and a swap is three accesses.  Empty slots (depth
// 3e38, colour 0) blend as no-ops, so the back-to-front pass runs once per
// filled slot only: the filled slots keep their order among themselves, and
// once no depth above 0 is left the shader blends slot 0 again, as here.
// During the tail the furthest slot is a function of the k-buffer alone, so
// it is searched again only after a swap changed the k-buffer.
constexpr int kResolveThreads = 256;

struct KBuffer {
    float* kd;     // this thread's slot 0 (stride kResolveThreads)
    uint32_t* kc;
    int m;         // filled slots
    float fd;      // furthest depth and slot (valid unless stale)
    int fi;
    bool stale;
    float4 r;      // the blended colour

    __device__ __forceinline__ float& d(int k) { return kd[k * kResolveThreads]; }
    __device__ __forceinline__ uint32_t& c(int k) { return kc[k * kResolveThreads]; }

    __device__ __forceinline__ void init(float* sd, uint32_t* sc, uint32_t background, const float* tab)
    {
        kd = sd + threadIdx.x;
        kc = sc + threadIdx.x;
        m = 0;
        fd = 0.0f;
        fi = 0;
        stale = true;
        r = unpack(tab, background);
    }

    __device__ __forceinline__ void put(int k, Frag f)
    {
        d(k) = f.d;
        c(k) = f.c;
    }

    // later nodes: blended as they come, each swapped first with the
    // k-buffer's furthest node when nearer (resolve.comp:44-76)
    __device__ __forceinline__ void tail(Frag f, const float* tab)
    {
        if (stale) {
            fd = 0.0f;
            fi = 0;
#pragma unroll
            for (int k = 0; k < kK; ++k) {
                const float x = d(k);
                if (x > fd) {
                    fd = x;
                    fi = k;
                }
            }
            stale = false;
        }
        uint32_t bc = f.c;
        if (f.d < fd) {
            bc = c(fi);
            c(fi) = f.c;
            d(fi) = f.d;
            stale = true;
        }
        blend(r, tab, bc);
    }

    // the k-buffer, furthest first (resolve.comp:80-99)
    __device__ __forceinline__ uint32_t finish(const float* tab)
    {
        for (int it = 0; it < m; ++it) {
            float x = 0.0f;
            int i = 0;
#pragma unroll
            for (int k = 0; k < kK; ++k)
                if (k < m) {
                    const float y = d(k);
                    if (y > x) {
                        x = y;
                        i = k;
                    }
                }
            d(i) = 0.0f;
            blend(r, tab, c(i));
        }
        return pack(r);
    }
};

// ---- work list: pixels with fragments, longest lists first -----------------------
// Lists longer than kList resolve kList nodes; lengths are bucketed by 65
// (kList / 16) so that the lanes of a resolve warp run about as long.
constexpr int kBuckets = 16;
__device__ __forceinline__ uint32_t list_length(const uint32_t* start, const float* vol_depth, uint32_t p)
{
    uint32_t n = start ? start[p + 1] - start[p] : 0u;
    if (vol_depth && vol_depth[p] < 1.0f) ++n;
    return min(n, kList);
}
__device__ __forceinline__ int bucket_of(uint32_t len) { return kBuckets - 1 - min(kBuckets - 1, (int)((len - 1) / 65u)); }

// words[0..15]: pixels per bucket; words[16..31]: fill cursors; words[32]: total
__global__ void __launch_bounds__(256) worklist_count_kernel(const uint32_t* __restrict__ start,
                                                             const float* __restrict__ vol_depth, uint32_t npix,
                                                             uint32_t* __restrict__ words)
{
    __shared__ uint32_t h[kBuckets];
    if (threadIdx.x < kBuckets) h[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < npix) {
        const uint32_t len = list_length(start, vol_depth, p);
        if (len) atomicAdd(&h[bucket_of(len)], 1u);
    }
    __syncthreads();
    if (threadIdx.x < kBuckets && h[threadIdx.x]) atomicAdd(&words[threadIdx.x], h[threadIdx.x]);
}

__global__ void __launch_bounds__(256) worklist_fill_kernel(const uint32_t* __restrict__ start,
                                                            const float* __restrict__ vol_depth, uint32_t npix,
                                                            uint32_t* __restrict__ words, uint32_t* __restrict__ list)
{
    __shared__ uint32_t h[kBuckets], base[kBuckets];
    if (threadIdx.x < kBuckets) h[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    int b = -1;
    uint32_t rank = 0;
    if (p < npix) {
        const uint32_t len = list_length(start, vol_depth, p);
        if (len) {
            b = bucket_of(len);
            rank = atomicAdd(&h[b], 1u);
        }
    }
    __syncthreads();
    if (threadIdx.x < kBuckets) {
        uint32_t off = 0;
        for (int k = 0; k < (int)threadIdx.x; ++k) off += words[k];
        base[threadIdx.x] = h[threadIdx.x] ? off + atomicAdd(&words[kBuckets + threadIdx.x], h[threadIdx.x]) : 0u;
        if (threadIdx.x == kBuckets - 1 && blockIdx.x == 0) words[2 * kBuckets] = off + words[kBuckets - 1];
    }
    __syncthreads();
    if (b >= 0) list[base[b] + rank] = p;
}

// A pixel's list without links: its volume fragment (when it has one), then
// its slice of the pixel-sorted payloads from the last entry back.
template <bool VOL>
__global__ void __launch_bounds__(kResolveThreads) composite_resolve_kernel(
    const uint32_t* __restrict__ list, const uint32_t* __restrict__ list_words, const uint32_t* __restrict__ start,
    const unsigned long long* __restrict__ vals, const float4* __restrict__ vol_rgba,
    const float* __restrict__ vol_depth, uint32_t* __restrict__ color)
{
    __shared__ float tab[256];
    __shared__ float sd[kK * kResolveThreads];
    __shared__ uint32_t sc[kK * kResolveThreads];
    fill_unorm_table(tab);
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= list_words[2 * kBuckets]) return;
    const uint32_t p = list[t];
    const uint32_t lo = start ? start[p] : 0u;
    const uint32_t hi = start ? start[p + 1] : 0u;
    int v = 0;
    Frag vf{0u, 0.0f};
    if (VOL) {
        const float dv = vol_depth[p];
        if (dv < 1.0f) {
            v = 1;
            vf = Frag{pack(vol_rgba[p]), dv};
        }
    }
    const uint32_t total = min(hi - lo + (uint32_t)v, kList);
    KBuffer kb;
    kb.init(sd, sc, color[p], tab);
    // list entry e >= v is the slice's entry top - e, top = hi - 1 + v (>= lo)
    const uint32_t top = hi - 1u + (uint32_t)v;
    kb.m = (int)min(total, (uint32_t)kK);
#pragma unroll
    for (int k = 0; k < kK; ++k)
        if (k < kb.m) kb.put(k, (VOL && k == 0 && v) ? vf : unpack_payload(__ldg(vals + (top - k))));
    // the tail in batches of 8, the next batch loading while one blends
    constexpr int kBatch = 8;
    unsigned long long cur[kBatch], nxt[kBatch];
#pragma unroll
    for (int j = 0; j < kBatch; ++j) cur[j] = kK + j < total ? __ldg(vals + (top - (kK + j))) : 0ull;
    for (uint32_t e = kK; e < total; e += kBatch) {
#pragma unroll
        for (int j = 0; j < kBatch; ++j)
            nxt[j] = e + kBatch + j < total ? __ldg(vals + (top - (e + kBatch + j))) : 0ull;
#pragma unroll
        for (int j = 0; j < kBatch; ++j)
            if (e + j < total) kb.tail(unpack_payload(cur[j]), tab);
#pragma unroll
        for (int j = 0; j < kBatch; ++j) cur[j] = nxt[j];
    }
    color[p] = kb.finish(tab);
}

// A PPLL list; a link outside the node array ends it and is recorded.
__global__ void __launch_bounds__(kResolveThreads) ppll_resolve_kernel(const uint32_t* __restrict__ heads,
                                                                       const vkhr_ppll_node* __restrict__ nodes,
                                                                       uint32_t count, uint32_t npix,
                                                                       uint32_t* __restrict__ color,
                                                                       unsigned long long* words)
{
    __shared__ float tab[256];
    __shared__ float sd[kK * kResolveThreads];
    __shared__ uint32_t sc[kK * kResolveThreads];
    fill_unorm_table(tab);
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    uint32_t node = heads[p];
    if (node == kNull) return; // resolve.comp:19-20
    bool bad = false;
    KBuffer kb;
    kb.init(sd, sc, color[p], tab);
    for (int k = 0; k < kK && node != kNull; ++k) { // resolve.comp:31-36
        if (node >= count) {
            bad = true;
            break;
        }
        const vkhr_ppll_node* nd = nodes + node;
        kb.put(k, Frag{__ldg(&nd->color), __ldg(&nd->depth)});
        node = __ldg(&nd->prev);
        kb.m = k + 1;
    }
    for (int t = 0; t < kTail && node != kNull && !bad; ++t) {
        if (node >= count) {
            bad = true;
            break;
        }
        const vkhr_ppll_node* nd = nodes + node;
        const Frag f{__ldg(&nd->color), __ldg(&nd->depth)};
        node = __ldg(&nd->prev);
        kb.tail(f, tab);
    }
    if (bad) atomicOr(&words[WORD_STATUS], (unsigned long long)VKHR_DEV_BAD_INDEX);
    color[p] = kb.finish(tab);
}

bool misaligned(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) != 0; }

vkhr_status check_image(vkhr_ctx* ctx, int32_t width, int32_t height, const uint32_t* d_color, uint32_t* npix)
{
    if (width <= 0 || height <= 0) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "width and height must be positive");
    const uint64_t n = (uint64_t)width * (uint64_t)height;
    if (n >= 0x80000000ull) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "2^31 pixels or more");
    if (!d_color) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_color is NULL");
    if (misaligned(d_color, 4)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_color must be 4-byte aligned");
    *npix = (uint32_t)n;
    return VKHR_OK;
}

} // namespace

extern "C" {

vkhr_status vkhr_resolve_ppll(vkhr_ctx* ctx, const uint32_t* d_heads, const vkhr_ppll_node* d_nodes,
                              uint32_t node_count, int32_t width, int32_t height, uint32_t* d_color, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    uint32_t npix = 0;
    vkhr_status s = check_image(ctx, width, height, d_color, &npix);
    if (s != VKHR_OK) return s;
    if (!d_heads || misaligned(d_heads, 4)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_heads is NULL or misaligned");
    if (node_count && (!d_nodes || misaligned(d_nodes, 4)))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_nodes is NULL or misaligned");
    cudaStream_t st = (cudaStream_t)stream;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    VKHR_LAUNCH(ctx, ppll_resolve_kernel, vkhr_blocks(npix, kResolveThreads), kResolveThreads, 0, st, d_heads, d_nodes,
                node_count, npix, d_color, ctx->d_words);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

vkhr_status vkhr_composite(vkhr_ctx* ctx, const vkhr_fragment* d_fragments, uint32_t fragment_count,
                           const float* d_volume_rgba, const float* d_volume_depth, int32_t width, int32_t height,
                           uint32_t* d_color, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    uint32_t npix = 0;
    vkhr_status s = check_image(ctx, width, height, d_color, &npix);
    if (s != VKHR_OK) return s;
    if (fragment_count >= 0x80000000u) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "2^31 fragments or more");
    if (fragment_count && (!d_fragments || misaligned(d_fragments, 4)))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_fragments is NULL or misaligned");
    if ((d_volume_rgba == nullptr) != (d_volume_depth == nullptr))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "give both d_volume_rgba and d_volume_depth, or neither");
    if (d_volume_rgba && (misaligned(d_volume_rgba, 16) || misaligned(d_volume_depth, 4)))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_volume_rgba must be 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));

    const uint32_t* start = nullptr;
    const unsigned long long* vals = nullptr;
    // work list: 64 words (bucket counts, cursors, total) and one entry a pixel
    const size_t list_words_at = 0, list_at = 64;
    const size_t list_need = list_at + ((size_t)npix + 3) / 4 * 4;
    if (fragment_count) {
        const uint32_t F = fragment_count;
        const uint32_t tiles = (F + kTile - 1) / kTile;
        // keys run to npix (fragments outside the image): its bit length
        int key_bits = 0;
        while (key_bits < 32 && (npix >> key_bits) != 0u) ++key_bits;
        const int passes = (key_bits + kMaxDigitBits - 1) / kMaxDigitBits;
        const int digit = (key_bits + passes - 1) / passes;
        const size_t hist_n = ((size_t)1 << digit) * tiles;
        const uint32_t nb = (uint32_t)((hist_n + kScanItems - 1) / kScanItems);
        auto round4 = [](size_t x) { return (x + 3) / 4 * 4; };
        // scratch (32-bit words, 16-byte aligned pieces):
        //   hist | partials | start | keys x2 | payloads x2
        const size_t partials_at = list_need + round4(hist_n);
        const size_t start_at = partials_at + round4(nb);
        const size_t keys_at = start_at + round4((size_t)npix + 1);
        const size_t vals_at = keys_at + 2 * round4(F);
        const size_t need = vals_at + 4 * (size_t)F;
        s = vkhr_reserve(ctx, (void**)&ctx->comp, &ctx->comp_cap, need, sizeof(uint32_t));
        if (s != VKHR_OK) return s;
        uint32_t* w = ctx->comp;
        uint32_t* d_hist = w + list_need;
        uint32_t* d_partials = w + partials_at;
        uint32_t* d_start = w + start_at;
        uint32_t* d_keys[2] = {w + keys_at, w + keys_at + round4(F)};
        unsigned long long* d_vals[2] = {reinterpret_cast<unsigned long long*>(w + vals_at),
                                         reinterpret_cast<unsigned long long*>(w + vals_at + 2 * (size_t)F)};
        for (int pass = 0; pass < passes; ++pass) {
            const int shift = pass * digit;
            const int bits = std::min(digit, key_bits - shift);
            const int src = (pass + 1) & 1, dst = pass & 1;
            if (pass == 0)
                VKHR_LAUNCH(ctx, radix_hist_kernel<true>, tiles, kTileThreads, 0, st, d_fragments, nullptr, F, npix,
                            shift, bits, tiles, d_hist, ctx->d_words);
            else
                VKHR_LAUNCH(ctx, radix_hist_kernel<false>, tiles, kTileThreads, 0, st, nullptr, d_keys[src], F, npix,
                            shift, bits, tiles, d_hist, ctx->d_words);
            const uint32_t hn = (uint32_t)(((size_t)1 << bits) * tiles);
            const uint32_t hb = (hn + kScanItems - 1) / kScanItems;
            VKHR_LAUNCH(ctx, scan_reduce_kernel, hb, kScanThreads, 0, st, d_hist, hn, d_partials);
            VKHR_LAUNCH(ctx, scan_partials_kernel, 1, kScanThreads, 0, st, d_partials, hb);
            VKHR_LAUNCH(ctx, scan_apply_kernel, hb, kScanThreads, 0, st, d_hist, hn, d_partials, d_hist);
            if (pass == 0)
                VKHR_LAUNCH(ctx, radix_scatter_kernel<true>, tiles, kTileThreads, 0, st, d_fragments, nullptr, nullptr,
                            F, npix, shift, bits, tiles, d_hist, d_keys[dst], d_vals[dst]);
            else
                VKHR_LAUNCH(ctx, radix_scatter_kernel<false>, tiles, kTileThreads, 0, st, nullptr, d_keys[src],
                            d_vals[src], F, npix, shift, bits, tiles, d_hist, d_keys[dst], d_vals[dst]);
        }
        const int last = (passes - 1) & 1;
        VKHR_LAUNCH(ctx, slice_bounds_kernel, vkhr_blocks((size_t)npix + 1, 256), 256, 0, st, d_keys[last], F, npix,
                    d_start);
        start = d_start;
        vals = d_vals[last];
    } else {
        s = vkhr_reserve(ctx, (void**)&ctx->comp, &ctx->comp_cap, list_need, sizeof(uint32_t));
        if (s != VKHR_OK) return s;
    }
    uint32_t* d_list_words = ctx->comp + list_words_at;
    uint32_t* d_list = ctx->comp + list_at;
    VKHR_CUDA_TRY(ctx, cudaMemsetAsync(d_list_words, 0, 64 * sizeof(uint32_t), st));
    const unsigned pb = vkhr_blocks(npix, 256);
    VKHR_LAUNCH(ctx, worklist_count_kernel, pb, 256, 0, st, start, d_volume_depth, npix, d_list_words);
    VKHR_LAUNCH(ctx, worklist_fill_kernel, pb, 256, 0, st, start, d_volume_depth, npix, d_list_words, d_list);
    const unsigned rb = vkhr_blocks(npix, kResolveThreads);
    if (d_volume_rgba)
        VKHR_LAUNCH(ctx, composite_resolve_kernel<true>, rb, kResolveThreads, 0, st, d_list, d_list_words, start, vals,
                    reinterpret_cast<const float4*>(d_volume_rgba), d_volume_depth, d_color);
    else
        VKHR_LAUNCH(ctx, composite_resolve_kernel<false>, rb, kResolveThreads, 0, st, d_list, d_list_words, start,
                    vals, nullptr, nullptr, d_color);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    return VKHR_OK;
}

// glm::smoothstep (rasterizer.cc:165-167)
float vkhr_level_of_detail(float magnified_distance, float minified_distance, float distance)
{
    float t = (distance - magnified_distance) / (minified_distance - magnified_distance);
    t = t > 0.0f ? (t < 1.0f ? t : 1.0f) : 0.0f;
    const float t2 = t * t;
    const float h = 3.0f - 2.0f * t;
    return t2 * h;
}

// scheme.glsl:7-11
float vkhr_lod(int32_t renderer, float magnified_distance, float minified_distance, float distance)
{
    if (renderer == VKHR_RENDERER_RASTERIZER) return 0.0f;
    if (renderer == VKHR_RENDERER_RAYMARCHER) return 1.0f;
    return vkhr_level_of_detail(magnified_distance, minified_distance, distance);
}

// interface.cc:534-540
int32_t vkhr_rasterizer_enabled(int32_t renderer, float level_of_detail)
{
    return renderer == VKHR_RENDERER_RASTERIZER || (renderer == VKHR_RENDERER_HYBRID_LOD && level_of_detail != 1.0f);
}

int32_t vkhr_raymarcher_enabled(int32_t renderer, float level_of_detail)
{
    return renderer == VKHR_RENDERER_RAYMARCHER || (renderer == VKHR_RENDERER_HYBRID_LOD && level_of_detail != 0.0f);
}

} // extern "C"
