// frame.cu -- per-frame voxelization feeding the raymarcher as one CUDA graph.
//
// The paper's per-frame path (rasterizer.cc:216-230 voxelizes each frame for
// simulated hair, then volume.cc:104-112 raymarches the volume) without a
// host round trip: one style's voxelization under a fixed visit budget,
// Volume::normalize (hair_style.cc:344-357), the occupancy pass and the
// raymarch of one view, captured once and replayed per frame.  Every piece
// is the context's own entry point; capture only removes the per-call host
// work and the launch gaps between them.
#include "common.cuh"

#include <new>

struct vkhr_frame_graph {
    vkhr_ctx* ctx;   // launches report errors here (the context must outlive launches)
    int device;      // destroy needs no context
    cudaGraph_t graph;
    cudaGraphExec_t exec;
};

namespace {

// The frame's calls, in order, on `stream` (captured or not).
vkhr_status frame_calls(vkhr_ctx* ctx, int32_t segments, const vkhr_voxel_job* job, int32_t normalize,
                        const vkhr_raymarch_params* p, const float* d_depth_in, float* d_rgba, float* d_depth_out,
                        void* stream)
{
    vkhr_status s = vkhr_voxelize_batched(ctx, segments, job, 1, stream);
    if (s != VKHR_OK) return s;
    if (normalize) {
        s = vkhr_normalize_densities(ctx, job->d_densities, (uint64_t)job->width * job->height * job->depth, stream);
        if (s != VKHR_OK) return s;
    }
    const void* density = p->density_format == VKHR_DENSITY_U8_UNORM ? (const void*)job->d_densities
                                                                      : (const void*)job->d_counts;
    return vkhr_raymarch(ctx, p, density, job->d_tangents, d_depth_in, d_rgba, d_depth_out, stream);
}

} // namespace

extern "C" {

vkhr_status vkhr_frame_graph_create(vkhr_ctx* ctx, int32_t segments, const vkhr_voxel_job* job, int32_t normalize,
                                    uint64_t visit_budget, const vkhr_raymarch_params* params, const float* d_depth_in,
                                    float* d_rgba, float* d_depth_out, void* stream, vkhr_frame_graph** out)
{
    if (!ctx) return VKHR_ERR_INVALID_ARG;
    if (!job || !params || !out) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "job, params and out are required");
    *out = nullptr;
    // the volume the raymarch reads is the job's own output
    if (params->density_format == VKHR_DENSITY_F32)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "a frame graph raymarches the voxelizer's u8 or u32 volume");
    if (params->density_format == VKHR_DENSITY_U8_UNORM && !job->d_densities)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "u8 densities need the job's d_densities");
    if (params->tangent_format != VKHR_TANGENT_I8_SNORM || !job->d_tangents)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "the raymarch reads the job's int8x4 d_tangents");
    if (normalize && !job->d_densities) return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "normalize needs d_densities");
    if (params->volume_resolution[0] != job->width || params->volume_resolution[1] != job->height ||
        params->volume_resolution[2] != job->depth)
        return vkhr_fail(ctx, VKHR_ERR_INVALID_ARG, "the view's volume_resolution must be the job's grid");
    VKHR_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    vkhr_status s = VKHR_OK;
    if (segments) { // a capacity for every frame: no visit total is read back inside the graph
        uint64_t budget = visit_budget;
        if (!budget) { // count this frame's visits once
            uint64_t v = 0;
            s = vkhr_voxelize_counted(ctx, job, stream, &v);
            if (s != VKHR_OK) return s;
            budget = v + v / 4 + 4096;
        }
        s = vkhr_set_visit_budget(ctx, budget);
        if (s != VKHR_OK) return s;
    }
    // one uncaptured frame: every scratch buffer reaches its size
    s = frame_calls(ctx, segments, job, normalize, params, d_depth_in, d_rgba, d_depth_out, stream);
    if (s != VKHR_OK) return s;
    VKHR_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    s = vkhr_check_status(ctx, stream);
    if (s != VKHR_OK) return s;

    // captured on a private stream (the caller's may be the legacy default
    // stream, which cannot be captured); the graph launches on any stream
    cudaStream_t cap = nullptr;
    VKHR_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    const cudaError_t began = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (began != cudaSuccess) {
        cudaStreamDestroy(cap);
        return vkhr_fail_cuda(ctx, began, "cudaStreamBeginCapture", __FILE__, __LINE__);
    }
    s = frame_calls(ctx, segments, job, normalize, params, d_depth_in, d_rgba, d_depth_out, cap);
    const cudaError_t ended = cudaStreamEndCapture(cap, &graph); // always ends the capture
    cudaStreamDestroy(cap);
    if (s != VKHR_OK) {
        if (ended == cudaSuccess && graph) cudaGraphDestroy(graph);
        return s;
    }
    if (ended != cudaSuccess) return vkhr_fail_cuda(ctx, ended, "cudaStreamEndCapture", __FILE__, __LINE__);
    cudaGraphExec_t exec = nullptr;
    const cudaError_t inst = cudaGraphInstantiate(&exec, graph, 0);
    if (inst != cudaSuccess) {
        cudaGraphDestroy(graph);
        return vkhr_fail_cuda(ctx, inst, "cudaGraphInstantiate", __FILE__, __LINE__);
    }
    vkhr_frame_graph* fg = new (std::nothrow) vkhr_frame_graph{ctx, ctx->device, graph, exec};
    if (!fg) {
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        return vkhr_fail(ctx, VKHR_ERR_OOM, "frame graph");
    }
    ++ctx->live_graphs; // the context's scratch may no longer move
    *out = fg;
    return VKHR_OK;
}

vkhr_status vkhr_frame_graph_launch(vkhr_frame_graph* fg, void* stream)
{
    if (!fg) return VKHR_ERR_INVALID_ARG;
    VKHR_CUDA_TRY(fg->ctx, cudaSetDevice(fg->ctx->device));
    VKHR_CUDA_TRY(fg->ctx, cudaGraphLaunch(fg->exec, (cudaStream_t)stream));
    return VKHR_OK;
}

vkhr_status vkhr_frame_graph_destroy(vkhr_frame_graph* fg)
{
    if (!fg) return VKHR_OK;
    cudaSetDevice(fg->device);
    if (fg->ctx && fg->ctx->live_graphs > 0) --fg->ctx->live_graphs;
    if (fg->exec) cudaGraphExecDestroy(fg->exec);
    if (fg->graph) cudaGraphDestroy(fg->graph);
    delete fg;
    return VKHR_OK;
}

} // extern "C"
