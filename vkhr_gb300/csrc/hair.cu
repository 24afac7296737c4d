// hair.cu -- `.hair` files into device memory, and strand reduction.
//
// vkhr_hair_load restates HairStyle::load (src/vkhr/scene_graph/hair_style.cc:
// 24-45, field readers :576-623) for a GPU consumer: the arrays stream from
// the file through two alternating pinned chunks with asynchronous copies,
// so reading the next chunk overlaps the copy of the last.  vkhr_reduce_strands
// restates HairStyle::reduce (:375-449): the strand choice is the reference's
// sequential xorshift64 walk, made on the host; a kernel gathers the kept
// strands' vertices and tangents on the device.
#include "common.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#include <sys/types.h>

static_assert(sizeof(vkhr_hair_header) == 128, "the .hair header is 128 bytes");

namespace {

struct FileCloser {
    FILE* f;
    ~FileCloser()
    {
        if (f) fclose(f);
    }
};

constexpr size_t kChunk = 8u << 20; // bytes per pinned staging chunk (two of them)

// The reference's error state names (HairStyle::Error).
vkhr_status hair_error(vkhr_ctx* ctx, const char* what)
{
    return ctx ? vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, what) : VKHR_ERR_INVALID_ARG;
}

vkhr_status read_header(vkhr_ctx* ctx, FILE* f, vkhr_hair_header* h)
{
    if (fread(h, 1, sizeof(*h), f) != sizeof(*h)) return hair_error(ctx, "ReadingFileHeader");
    if (std::memcmp(h->signature, "HAIR", 4) != 0) return hair_error(ctx, "InvalidSignature");
    return VKHR_OK;
}

bool skip(FILE* f, uint64_t bytes) { return fseeko(f, (off_t)bytes, SEEK_CUR) == 0; }

// `bytes` of the file from its current position to device memory `dst`
// (NULL: skipped), through the two pinned chunks; chunk k's next read waits
// for its previous copy only.
vkhr_status to_device(vkhr_ctx* ctx, FILE* f, uint64_t bytes, void* dst, unsigned char* stage[2], cudaEvent_t ev[2],
                      cudaStream_t st, const char* what)
{
    if (!dst) return skip(f, bytes) ? VKHR_OK : hair_error(ctx, what);
    uint64_t done = 0;
    int k = 0;
    while (done < bytes) {
        const size_t n = (size_t)std::min<uint64_t>(kChunk, bytes - done);
        VKHR_CUDA_TRY(ctx, cudaEventSynchronize(ev[k]));
        if (fread(stage[k], 1, n, f) != n) return hair_error(ctx, what);
        VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(static_cast<unsigned char*>(dst) + done, stage[k], n, cudaMemcpyHostToDevice,
                                           st));
        VKHR_CUDA_TRY(ctx, cudaEventRecord(ev[k], st));
        done += n;
        k ^= 1;
    }
    return VKHR_OK;
}

// hair_style.cc:679-685
uint64_t xorshift64(uint64_t x)
{
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return x;
}

// One warp per kept strand: (source vertex, destination vertex, vertices)
// per entry; the lanes copy the strand's floats coalesced.
__global__ void gather_strands_kernel(const uint4* __restrict__ table, uint32_t n, const float* __restrict__ v_in,
                                      const float* __restrict__ t_in, float* __restrict__ v_out,
                                      float* __restrict__ t_out)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < n; s += warps) {
        const uint4 e = __ldg(table + s);
        const uint32_t nf = 3u * e.z;
        const float* vs = v_in + 3ull * e.x;
        float* vd = v_out + 3ull * e.y;
        for (uint32_t i = lane; i < nf; i += 32) vd[i] = __ldg(vs + i);
        if (t_in) {
            const float* ts = t_in + 3ull * e.x;
            float* td = t_out + 3ull * e.y;
            for (uint32_t i = lane; i < nf; i += 32) td[i] = __ldg(ts + i);
        }
    }
}

} // namespace

extern "C" {

vkhr_status vkhr_hair_read_header(const char* path, vkhr_hair_header* header)
{
    if (!path || !header) return VKHR_ERR_INVALID_ARG;
    FileCloser fc{fopen(path, "rb")};
    if (!fc.f) return VKHR_ERR_INVALID_ARG;
    return read_header(nullptr, fc.f, header);
}

vkhr_status vkhr_hair_load(vkhr_ctx* ctx, const char* path, vkhr_hair_header* header, uint16_t* h_segments,
                           float* d_vertices, float* d_tangents, uint32_t* d_indices, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!path || !header) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "path and header are required");
    FileCloser fc{fopen(path, "rb")};
    if (!fc.f) return hair_error(ctx, "OpeningFile");
    vkhr_status s = read_header(ctx, fc.f, header);
    if (s != VKHR_OK) return s;
    const uint64_t nstr = header->strand_count, nv = header->vertex_count;
    const uint32_t bits = header->fields;
    if ((bits & VKHR_HAIR_INDICES) && nv < nstr) return hair_error(ctx, "ReadingIndices");
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char* stage[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaMallocHost((void**)&stage[0], 2 * kChunk);
    if (e == cudaSuccess) stage[1] = stage[0] + kChunk;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    if (e == cudaSuccess) {
        // the fields in the file's order (hair_style.cc:33-39)
        if (bits & VKHR_HAIR_SEGMENTS) {
            if (h_segments ? fread(h_segments, 2, nstr, fc.f) != nstr : !skip(fc.f, 2 * nstr))
                s = hair_error(ctx, "ReadingSegments");
        }
        if (s == VKHR_OK && (bits & VKHR_HAIR_VERTICES))
            s = to_device(ctx, fc.f, 12 * nv, d_vertices, stage, ev, st, "ReadingVertices");
        if (s == VKHR_OK && (bits & VKHR_HAIR_THICKNESS) && !skip(fc.f, 4 * nv)) s = hair_error(ctx, "ReadingThickness");
        if (s == VKHR_OK && (bits & VKHR_HAIR_TRANSPARENCY) && !skip(fc.f, 4 * nv))
            s = hair_error(ctx, "ReadingTransparency");
        if (s == VKHR_OK && (bits & VKHR_HAIR_COLOR) && !skip(fc.f, 12 * nv)) s = hair_error(ctx, "ReadingColor");
        if (s == VKHR_OK && (bits & VKHR_HAIR_TANGENTS))
            s = to_device(ctx, fc.f, 12 * nv, d_tangents, stage, ev, st, "ReadingTangents");
        if (s == VKHR_OK && (bits & VKHR_HAIR_INDICES))
            s = to_device(ctx, fc.f, 8 * (nv - nstr), d_indices, stage, ev, st, "ReadingIndices");
        if (s == VKHR_OK && !(bits & VKHR_HAIR_VERTICES)) s = hair_error(ctx, "InvalidFormat");
        const cudaError_t done = cudaStreamSynchronize(st); // the staging is freed below
        if (s == VKHR_OK && done != cudaSuccess) s = vkhr_fail_cuda(ctx, done, "cudaStreamSynchronize", __FILE__, __LINE__);
    } else {
        s = vkhr_fail_cuda(ctx, e, "pinned staging", __FILE__, __LINE__);
    }
    for (int k = 0; k < 2; ++k)
        if (ev[k]) cudaEventDestroy(ev[k]);
    if (stage[0]) cudaFreeHost(stage[0]);
    return s;
}

vkhr_status vkhr_reduce_strands(vkhr_ctx* ctx, float ratio, uint64_t* seed, const uint16_t* h_segments,
                                uint32_t strand_count, uint32_t default_segment_count, const float* d_vertices,
                                const float* d_tangents, uint16_t* h_segments_out, uint32_t* strands_out,
                                uint32_t* vertices_out, float* d_vertices_out, float* d_tangents_out, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!seed || !strands_out || !vertices_out || !h_segments_out)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "seed, h_segments_out and the counts are required");
    if (!(ratio >= 0.0f && ratio <= 1.0f)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "ratio must be in [0, 1]");
    if (strand_count && (!d_vertices || !d_vertices_out))
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_vertices and d_vertices_out are required");
    if (d_tangents && !d_tangents_out) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "d_tangents_out is required");
    // The reference's arithmetic, in its types: an FP32 product and ceil, the
    // FP32 difference converted to unsigned, and an unsigned pre-decrement
    // (0 wraps, so every strand is kept: ratio 1 is HairStyle::shuffle).
    const float prod = (float)strand_count * ratio;
    const float left = (float)strand_count - std::ceil(prod);
    uint32_t strands_left = (uint32_t)left;
    std::vector<uint64_t> offset(strand_count);
    std::vector<uint32_t> segs(strand_count);
    uint64_t acc = 0;
    for (uint32_t i = 0; i < strand_count; ++i) {
        segs[i] = h_segments ? h_segments[i] : default_segment_count;
        offset[i] = acc;
        acc += (uint64_t)segs[i] + 1;
    }
    if (acc >= (1ull << 32)) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "more than 2^32 - 1 vertices");
    std::vector<uint4> table;
    table.reserve(strand_count);
    uint64_t state = *seed;
    uint32_t dst = 0;
    while (--strands_left && !offset.empty()) {
        state = xorshift64(state);
        const double r = (double)state / (double)std::numeric_limits<uint64_t>::max();
        size_t k = (size_t)(r * (double)offset.size());
        if (k >= offset.size()) k = offset.size() - 1; // r = 1 exactly: the reference would index past the end
        const uint32_t sc = segs[k];
        h_segments_out[table.size()] = (uint16_t)sc;
        table.push_back(make_uint4((uint32_t)offset[k], dst, sc + 1, 0u));
        dst += sc + 1;
        std::swap(segs[k], segs.back());
        segs.pop_back();
        std::swap(offset[k], offset.back());
        offset.pop_back();
    }
    *seed = state;
    *strands_out = (uint32_t)table.size();
    *vertices_out = dst;
    if (table.empty()) return VKHR_OK;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    vkhr_status s = vkhr_reserve(ctx, (void**)&ctx->d_gather, &ctx->d_gather_cap, table.size(), sizeof(uint4));
    if (s != VKHR_OK) return s;
    VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_gather, table.data(), table.size() * sizeof(uint4),
                                       cudaMemcpyHostToDevice, st));
    const unsigned blocks = std::min(vkhr_blocks((uint64_t)table.size() * 32, 256), (unsigned)ctx->sm_count * 8);
    VKHR_LAUNCH(ctx, gather_strands_kernel, blocks, 256, 0, st, ctx->d_gather, (uint32_t)table.size(), d_vertices,
                d_tangents, d_vertices_out, d_tangents_out);
    VKHR_CUDA_TRY(ctx, cudaGetLastError());
    VKHR_CUDA_TRY(ctx, cudaStreamSynchronize(st)); // the table is pageable host memory
    return VKHR_OK;
}

} // extern "C"
