// prepare.cu -- strand data preparation on the device: the bounding box,
// per-vertex tangents and segment index pairs of vkhr::HairStyle
// (src/vkhr/scene_graph/hair_style.cc:171-255), all bit-exact in FP32.
#include "common.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace {

// Order-preserving int encoding of floats, so that integer min/max atomics
// give float min/max (-0 sorts below +0).
__device__ __forceinline__ int ordered(float f)
{
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float unordered(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__global__ void aabb_init_kernel(int* mm)
{
    if (threadIdx.x < 3) {
        mm[threadIdx.x] = ordered(0.0f);      // generate_bounding_box starts at (0,0,0)
        mm[3 + threadIdx.x] = ordered(0.0f);
    }
    if (threadIdx.x == 0) mm[6] = 0;           // non-finite coordinate count
}

__global__ void aabb_reduce_kernel(const float* __restrict__ v, uint64_t n_floats, int* mm)
{
    float lo[3] = {0.0f, 0.0f, 0.0f}, hi[3] = {0.0f, 0.0f, 0.0f};
    int bad = 0;
    // thread t covers floats t, t + stride, ...: component = index % 3
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * 3;
    for (uint64_t base = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) * 3; base < n_floats; base += stride) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float x = __ldg(v + base + a);
            if (!isfinite(x)) { ++bad; continue; }
            lo[a] = glm_min(x, lo[a]);
            hi[a] = glm_max(x, hi[a]);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int l = ordered(lo[a]), h = ordered(hi[a]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            l = min(l, __shfl_down_sync(0xffffffffu, l, o));
            h = max(h, __shfl_down_sync(0xffffffffu, h, o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(mm + a, l);
            atomicMax(mm + 3 + a, h);
        }
    }
    if (bad) atomicAdd(mm + 6, bad);
}

// get_bounding_box (hair_style.cc:236-255): size = max - min, radius =
// sqrt((x*x + y*y) + z*z), volume = (x*y)*z, all FP32.
__global__ void aabb_finish_kernel(const int* mm, vkhr_aabb* out)
{
    if (threadIdx.x != 0) return;
    float s[3];
    for (int a = 0; a < 3; ++a) {
        float lo = unordered(mm[a]), hi = unordered(mm[3 + a]);
        out->origin[a] = lo;
        s[a] = __fsub_rn(hi, lo);
        out->size[a] = s[a];
    }
    float dot = __fadd_rn(__fadd_rn(__fmul_rn(s[0], s[0]), __fmul_rn(s[1], s[1])), __fmul_rn(s[2], s[2]));
    out->radius = __fsqrt_rn(dot);
    out->volume = __fmul_rn(__fmul_rn(s[0], s[1]), s[2]);
}

// generate_tangents (hair_style.cc:171-194), pass 1: one thread per strand
// writes its segment tangents d * (1 / sqrt(dot(d, d))) (glm::normalize).
__global__ void tangents_kernel(const float* __restrict__ v, const uint32_t* __restrict__ first_vertex,
                                const uint16_t* __restrict__ segs, uint32_t strands, float* t)
{
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < strands; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t v0 = first_vertex[s];
        const uint32_t n = segs[s];
        for (uint32_t k = 0; k < n; ++k) {
            float d[3];
            for (int a = 0; a < 3; ++a) d[a] = __fsub_rn(v[3 * (v0 + k + 1) + a], v[3 * (v0 + k) + a]);
            float dot = __fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2]));
            float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot));
            for (int a = 0; a < 3; ++a) t[3 * (v0 + k) + a] = __fmul_rn(d[a], inv);
        }
    }
}

// Pass 2: a strand's last vertex repeats tangents.back(), the tangent of the
// vertex before it: its own last segment's, or, for a strand without
// segments, the previous strand's last vertex (followed back across
// consecutive segment-less strands; 0 before the first segment).
__global__ void tangents_last_kernel(const uint32_t* __restrict__ first_vertex, const uint16_t* __restrict__ segs,
                                     uint32_t strands, float* t)
{
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < strands; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t last = (uint64_t)first_vertex[s] + segs[s];
        int64_t src = -1;
        for (int64_t q = (int64_t)s; q >= 0; --q)
            if (segs[q] > 0) {
                src = (int64_t)first_vertex[q] + segs[q] - 1;
                break;
            }
        for (int a = 0; a < 3; ++a) t[3 * last + a] = src >= 0 ? t[3 * src + a] : 0.0f;
    }
}

// generate_indices (hair_style.cc:196-213).
__global__ void indices_kernel(const uint32_t* __restrict__ first_vertex, const uint16_t* __restrict__ segs,
                               uint32_t strands, uint32_t* idx)
{
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < strands; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v0 = first_vertex[s];
        const uint32_t n = segs[s];
        const uint64_t o = 2ull * ((uint64_t)v0 - s); // segments before strand s
        for (uint32_t k = 0; k < n; ++k) {
            idx[o + 2 * k] = v0 + k;
            idx[o + 2 * k + 1] = v0 + k + 1;
        }
    }
}

// Uploads the per-strand segment counts and first-vertex offsets; the
// staging copies complete before this returns.
vkhr_status upload_strands(vkhr_ctx* ctx, const uint16_t* h_segments, uint32_t strands, cudaStream_t st,
                           uint16_t** d_segs, uint32_t** d_first, uint64_t* vertex_total)
{
    std::vector<uint32_t> first(strands);
    uint64_t acc = 0;
    for (uint32_t s = 0; s < strands; ++s) {
        first[s] = (uint32_t)acc;
        acc += (uint64_t)h_segments[s] + 1;
    }
    if (acc >= (1ull << 32)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "more than 2^32 - 1 vertices");
    *vertex_total = acc;
    VKHR_CUDA_TRY(ctx, cudaMallocAsync((void**)d_segs, std::max<size_t>(strands, 1) * sizeof(uint16_t), st));
    VKHR_CUDA_TRY(ctx, cudaMallocAsync((void**)d_first, std::max<size_t>(strands, 1) * sizeof(uint32_t), st));
    VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(*d_segs, h_segments, strands * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
    VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(*d_first, first.data(), strands * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    VKHR_CUDA_TRY(ctx, cudaStreamSynchronize(st)); // `first` goes out of scope
    return VKHR_OK;
}

} // namespace

extern "C" {

vkhr_status vkhr_bounding_box(vkhr_ctx* ctx, const float* d_vertices, uint32_t vertex_count, vkhr_aabb* out,
                              void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!out) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "out_bounds is NULL");
    if (vertex_count && !d_vertices) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_vertices is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    int* mm = reinterpret_cast<int*>(ctx->d_words + WORD_AABB);
    vkhr_aabb* d_out = reinterpret_cast<vkhr_aabb*>(ctx->d_words + WORD_AABB + 4);
    VKHR_LAUNCH(ctx, aabb_init_kernel, 1, 32, 0, st, mm);
    if (vertex_count) {
        const unsigned blocks = std::min(vkhr_blocks(vertex_count, 256), (unsigned)ctx->sm_count * 8);
        VKHR_LAUNCH(ctx, aabb_reduce_kernel, blocks, 256, 0, st, d_vertices, 3ull * vertex_count, mm);
    }
    VKHR_LAUNCH(ctx, aabb_finish_kernel, 1, 32, 0, st, mm, d_out);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->h_words, ctx->d_words + WORD_AABB, 8 * sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, st));
    VKHR_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    int bad;
    std::memcpy(&bad, reinterpret_cast<const int*>(ctx->h_words) + 6, sizeof(int));
    if (bad) return vkhr_fail(ctx, VKHR_ERR_NAN_INPUT, "vertices contain NaN or Inf coordinates");
    std::memcpy(out, ctx->h_words + 4, sizeof(vkhr_aabb));
    return VKHR_OK;
}

vkhr_status vkhr_generate_tangents(vkhr_ctx* ctx, const float* d_vertices, const uint16_t* h_segments,
                                   uint32_t strand_count, float* d_tangents, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (strand_count == 0) return VKHR_OK;
    if (!d_vertices || !h_segments || !d_tangents) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "NULL argument");
    cudaStream_t st = (cudaStream_t)stream;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    uint16_t* segs = nullptr;
    uint32_t* first = nullptr;
    uint64_t verts = 0;
    vkhr_status s = upload_strands(ctx, h_segments, strand_count, st, &segs, &first, &verts);
    if (s == VKHR_OK) {
        const unsigned blocks = std::min(vkhr_blocks(strand_count, 128), (unsigned)ctx->sm_count * 16);
        VKHR_LAUNCH(ctx, tangents_kernel, blocks, 128, 0, st, d_vertices, first, segs, strand_count, d_tangents);
        VKHR_LAUNCH(ctx, tangents_last_kernel, blocks, 128, 0, st, first, segs, strand_count, d_tangents);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) s = vkhr_fail_cuda(ctx, e, "tangents_kernel", __FILE__, __LINE__);
    }
    if (segs) cudaFreeAsync(segs, st);
    if (first) cudaFreeAsync(first, st);
    return s;
}

vkhr_status vkhr_generate_indices(vkhr_ctx* ctx, const uint16_t* h_segments, uint32_t strand_count,
                                  uint32_t* d_indices, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (strand_count == 0) return VKHR_OK;
    if (!h_segments || !d_indices) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "NULL argument");
    cudaStream_t st = (cudaStream_t)stream;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    uint16_t* segs = nullptr;
    uint32_t* first = nullptr;
    uint64_t verts = 0;
    vkhr_status s = upload_strands(ctx, h_segments, strand_count, st, &segs, &first, &verts);
    if (s == VKHR_OK) {
        VKHR_LAUNCH(ctx, indices_kernel, std::min(vkhr_blocks(strand_count, 128), (unsigned)ctx->sm_count * 16),
                    128, 0, st, first, segs, strand_count, d_indices);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) s = vkhr_fail_cuda(ctx, e, "indices_kernel", __FILE__, __LINE__);
    }
    if (segs) cudaFreeAsync(segs, st);
    if (first) cudaFreeAsync(first, st);
    return s;
}

} // extern "C"
