// context.cu -- library context, scratch management and error reporting.
#include "common.cuh"

#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <new>

vkhr_status vkhr_fail(vkhr_ctx* ctx, vkhr_status s, const char* msg)
{
    if (ctx) std::snprintf(ctx->last_error, sizeof(ctx->last_error), "%s: %s", vkhr_status_string(s), msg);
    return s;
}

vkhr_status vkhr_fail_cuda(vkhr_ctx* ctx, cudaError_t e, const char* what, const char* file, int line)
{
    if (ctx)
        std::snprintf(ctx->last_error, sizeof(ctx->last_error), "VKHR_ERR_CUDA: %s failed with %s (%s) at %s:%d",
                      what, cudaGetErrorName(e), cudaGetErrorString(e), file, line);
    return e == cudaErrorMemoryAllocation ? VKHR_ERR_OOM : VKHR_ERR_CUDA;
}

vkhr_status vkhr_reserve(vkhr_ctx* ctx, void** ptr, size_t* cap_elems, size_t need_elems, size_t elem_bytes)
{
    if (need_elems <= *cap_elems && *ptr) return VKHR_OK;
    if (*ptr && ctx->live_graphs > 0)
        return vkhr_fail(ctx, VKHR_ERR_CAPACITY,
                         "scratch would have to grow while a frame graph holds it: destroy the graph first");
    size_t grow = need_elems + need_elems / 8 + 1024; // headroom against creeping sizes
    if (*ptr) {
        // the old buffer may still be read by work queued on any stream
        VKHR_CUDA_TRY(ctx, cudaDeviceSynchronize());
        cudaFree(*ptr);
        *ptr = nullptr;
        *cap_elems = 0;
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, grow * elem_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return vkhr_fail_cuda(ctx, e, "cudaMalloc(scratch)", __FILE__, __LINE__);
    }
    *ptr = p;
    *cap_elems = grow;
    return VKHR_OK;
}

void vkhr_prof_begin(vkhr_ctx* ctx, const char* name, cudaStream_t st)
{
    if (ctx->prof_n >= kProfileMax) return;
    ctx->prof_name[ctx->prof_n] = name;
    cudaEventRecord(ctx->prof_ev[2 * ctx->prof_n], st);
}

void vkhr_prof_end(vkhr_ctx* ctx, cudaStream_t st)
{
    if (ctx->prof_n >= kProfileMax) return;
    cudaEventRecord(ctx->prof_ev[2 * ctx->prof_n + 1], st);
    ++ctx->prof_n;
}

vkhr_status vkhr_fork_side(vkhr_ctx* ctx, cudaStream_t st)
{
    VKHR_CUDA_TRY(ctx, cudaEventRecord(ctx->fork_ev, st));
    VKHR_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->side, ctx->fork_ev, 0));
    return VKHR_OK;
}

vkhr_status vkhr_join_side(vkhr_ctx* ctx, cudaStream_t st)
{
    VKHR_CUDA_TRY(ctx, cudaEventRecord(ctx->join_ev, ctx->side));
    VKHR_CUDA_TRY(ctx, cudaStreamWaitEvent(st, ctx->join_ev, 0));
    return VKHR_OK;
}

extern "C" {

int vkhr_abi_version(void) { return VKHR_CUDA_ABI_VERSION; }

vkhr_status vkhr_set_profiling(vkhr_ctx* ctx, int enable)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    if (enable && !ctx->prof_ev) {
        ctx->prof_ev = new (std::nothrow) cudaEvent_t[2 * kProfileMax];
        ctx->prof_name = new (std::nothrow) const char*[kProfileMax];
        if (!ctx->prof_ev || !ctx->prof_name) return vkhr_fail(ctx, VKHR_ERR_OOM, "profiling tables");
        for (int i = 0; i < 2 * kProfileMax; ++i) VKHR_CUDA_TRY(ctx, cudaEventCreate(&ctx->prof_ev[i]));
    }
    ctx->profiling = enable ? 1 : 0;
    ctx->prof_n = 0;
    return VKHR_OK;
}

vkhr_status vkhr_profile_read(vkhr_ctx* ctx, int index, const char** name, float* ms)
{
    if (!ctx || !name || !ms) return VKHR_ERR_INVALID_ARG;
    if (index < 0 || index >= ctx->prof_n) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "profile index out of range");
    VKHR_CUDA_TRY(ctx, cudaEventSynchronize(ctx->prof_ev[2 * index + 1]));
    VKHR_CUDA_TRY(ctx, cudaEventElapsedTime(ms, ctx->prof_ev[2 * index], ctx->prof_ev[2 * index + 1]));
    *name = ctx->prof_name[index];
    return VKHR_OK;
}

int vkhr_profile_count(const vkhr_ctx* ctx) { return ctx ? ctx->prof_n : 0; }

const char* vkhr_status_string(vkhr_status s)
{
    switch (s) {
    case VKHR_OK: return "VKHR_OK";
    case VKHR_ERR_INVALID_ARG: return "VKHR_ERR_INVALID_ARG";
    case VKHR_ERR_DEGENERATE_AABB: return "VKHR_ERR_DEGENERATE_AABB";
    case VKHR_ERR_OOM: return "VKHR_ERR_OOM";
    case VKHR_ERR_CUDA: return "VKHR_ERR_CUDA";
    case VKHR_ERR_TIMEOUT: return "VKHR_ERR_TIMEOUT";
    case VKHR_ERR_NAN_INPUT: return "VKHR_ERR_NAN_INPUT";
    case VKHR_ERR_CAPACITY: return "VKHR_ERR_CAPACITY";
    case VKHR_ERR_NOT_SUPPORTED: return "VKHR_ERR_NOT_SUPPORTED";
    }
    return "VKHR_ERR_UNKNOWN";
}

const char* vkhr_last_error(const vkhr_ctx* ctx) { return ctx ? ctx->last_error : "no context"; }

vkhr_status vkhr_create(int device, vkhr_ctx** out)
{
    if (!out) return VKHR_ERR_INVALID_ARG;
    *out = nullptr;
    vkhr_ctx* ctx = new (std::nothrow) vkhr_ctx();
    if (!ctx) return VKHR_ERR_OOM;
    std::memset(ctx, 0, sizeof(*ctx));
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->l2_bytes, cudaDevAttrL2CacheSize, device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&ctx->smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&ctx->smem_reserved, cudaDevAttrReservedSharedMemoryPerBlock, device);
    ctx->walk_ctas[0] = 0; // no residency limit for the one walk: measured fastest on both workloads
    ctx->walk_ctas[1] = 0; // (vkhr_autotune_voxelize retunes per workload)
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_words, WORD_COUNT * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_words, 0, WORD_COUNT * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_words, WORD_COUNT * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->join_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->jobs_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_jobs, kJobTableBytes);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->rjobs_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_rjobs, kRayTableBytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        vkhr_destroy(ctx);
        return e == cudaErrorMemoryAllocation ? VKHR_ERR_OOM : VKHR_ERR_CUDA;
    }
    *out = ctx;
    return VKHR_OK;
}

vkhr_status vkhr_destroy(vkhr_ctx* ctx)
{
    if (!ctx) return VKHR_OK;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    void* bufs[] = {ctx->brick_runs, ctx->items, ctx->brick_list, ctx->pair_tan, ctx->hkeys, ctx->hdesc,
                    ctx->d_jobs, ctx->d_rjobs, ctx->g_acc, ctx->slots, ctx->layout, ctx->d_gather, ctx->comp};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (ctx->occ) cudaFree(ctx->occ);
    if (ctx->tex_obj) cudaDestroyTextureObject(ctx->tex_obj);
    if (ctx->tex_array) cudaFreeArray(ctx->tex_array);
    if (ctx->gat_obj) cudaDestroyTextureObject(ctx->gat_obj);
    if (ctx->gat_surf) cudaDestroySurfaceObject(ctx->gat_surf);
    if (ctx->gat_array) cudaFreeArray(ctx->gat_array);
    if (ctx->gat_stage) cudaFree(ctx->gat_stage);
    if (ctx->d_words) cudaFree(ctx->d_words);
    if (ctx->h_words) cudaFreeHost(ctx->h_words);
    if (ctx->ev) cudaEventDestroy(ctx->ev);
    if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
    if (ctx->join_ev) cudaEventDestroy(ctx->join_ev);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->jobs_ev) cudaEventDestroy(ctx->jobs_ev);
    if (ctx->h_jobs) cudaFreeHost(ctx->h_jobs);
    if (ctx->rjobs_ev) cudaEventDestroy(ctx->rjobs_ev);
    if (ctx->h_rjobs) cudaFreeHost(ctx->h_rjobs);
    if (ctx->prof_ev) {
        for (int i = 0; i < 2 * kProfileMax; ++i) cudaEventDestroy(ctx->prof_ev[i]);
        delete[] ctx->prof_ev;
    }
    delete[] ctx->prof_name;
    delete ctx;
    return VKHR_OK;
}

vkhr_status vkhr_malloc(vkhr_ctx* ctx, size_t bytes, void** out)
{
    if (!ctx || !out) return VKHR_ERR_INVALID_ARG;
    *out = nullptr;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    VKHR_CUDA_TRY(ctx, cudaMalloc(out, bytes ? bytes : 1));
    return VKHR_OK;
}

vkhr_status vkhr_free(vkhr_ctx* ctx, void* p)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!p) return VKHR_OK;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    VKHR_CUDA_TRY(ctx, cudaFree(p));
    return VKHR_OK;
}

vkhr_status vkhr_upload(vkhr_ctx* ctx, void* dst, const void* src, size_t bytes, void* stream)
{
    if (!ctx || (bytes && (!dst || !src))) return VKHR_ERR_INVALID_ARG;
    if (!bytes) return VKHR_OK;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    return VKHR_OK;
}

vkhr_status vkhr_download(vkhr_ctx* ctx, void* dst, const void* src, size_t bytes, void* stream)
{
    if (!ctx || (bytes && (!dst || !src))) return VKHR_ERR_INVALID_ARG;
    if (!bytes) return VKHR_OK;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    VKHR_CUDA_TRY(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    return VKHR_OK;
}

vkhr_status vkhr_sync(vkhr_ctx* ctx, void* stream)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    VKHR_CUDA_TRY(ctx, cudaStreamSynchronize((cudaStream_t)stream));
    return VKHR_OK;
}

uint64_t vkhr_launch_count(const vkhr_ctx* ctx) { return ctx ? ctx->launches : 0; }

size_t vkhr_sizeof_aabb(void) { return sizeof(vkhr_aabb); }
size_t vkhr_sizeof_voxel_job(void) { return sizeof(vkhr_voxel_job); }
size_t vkhr_sizeof_raymarch_job(void) { return sizeof(vkhr_raymarch_job); }
size_t vkhr_sizeof_raymarch_params(void) { return sizeof(vkhr_raymarch_params); }

} // extern "C"
