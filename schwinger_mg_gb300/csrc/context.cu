// Context lifetime, error reporting and per-context scratch.
#include "smg_internal.h"

#include <cstring>

smg_status smg_fail(smg_context* ctx, smg_status s, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return s;
}

smg_status smg_reduce_reserve(smg_context* ctx, size_t doubles) {
    if (ctx->red.capacity >= doubles) return SMG_OK;
    // kernels already queued (or captured in a graph) may still use the old
    // buffer, so it is retired rather than freed
    if (ctx->red.partials) ctx->retired.push_back(ctx->red.partials);
    ctx->red.partials = nullptr;
    ctx->red.capacity = 0;
    size_t cap = doubles < (1u << 16) ? (1u << 16) : doubles;
    SMG_CUDA(ctx, cudaMalloc(&ctx->red.partials, cap * sizeof(double)));
    ctx->red.capacity = cap;
    return SMG_OK;
}

smg_status smg_host_stage_reserve(smg_context* ctx, size_t bytes) {
    if (ctx->host_stage_bytes >= bytes) return SMG_OK;
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->host_stage) cudaFreeHost(ctx->host_stage);
    ctx->host_stage = nullptr;
    ctx->host_stage_bytes = 0;
    size_t cap = bytes < 4096 ? 4096 : bytes;
    SMG_CUDA(ctx, cudaHostAlloc((void**)&ctx->host_stage, cap, cudaHostAllocDefault));
    ctx->host_stage_bytes = cap;
    return SMG_OK;
}

extern "C" {

SMG_API const char* smg_version(void) { return "smg-gb300 0.1 sm_103a"; }

SMG_API const char* smg_status_string(smg_status s) {
    switch (s) {
        case SMG_OK: return "ok";
        case SMG_NOT_CONVERGED: return "not converged";
        case SMG_BREAKDOWN: return "breakdown";
        case SMG_NONFINITE: return "non-finite value";
        case SMG_BAD_ARG: return "bad argument";
        case SMG_DEVICE_ERROR: return "device error";
        case SMG_TIMEOUT: return "device wait timed out";
        case SMG_NO_MEMORY: return "out of device memory";
        case SMG_UNSUPPORTED: return "unsupported";
        case SMG_IO_ERROR: return "file input/output error";
    }
    return "unknown status";
}

SMG_API smg_status smg_context_create(int device, void* stream, smg_context** out) {
    if (!out) return SMG_BAD_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SMG_DEVICE_ERROR;
    if (device < 0 || device >= ndev) return SMG_BAD_ARG;
    smg_context* ctx = new smg_context();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete ctx; return SMG_DEVICE_ERROR; }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete ctx;
            return SMG_DEVICE_ERROR;
        }
        ctx->own_stream = true;
    }
    if (cudaMalloc(&ctx->red.tickets, kMaxTickets * sizeof(unsigned int)) != cudaSuccess ||
        cudaMemset(ctx->red.tickets, 0, kMaxTickets * sizeof(unsigned int)) != cudaSuccess) {
        if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return SMG_NO_MEMORY;
    }
    if (smg_reduce_reserve(ctx, 1u << 16) != SMG_OK || smg_host_stage_reserve(ctx, 1 << 16) != SMG_OK) {
        cudaFree(ctx->red.tickets);
        if (ctx->red.partials) cudaFree(ctx->red.partials);
        if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return SMG_NO_MEMORY;
    }
    *out = ctx;
    return SMG_OK;
}

SMG_API smg_status smg_context_destroy(smg_context* ctx) {
    if (!ctx) return SMG_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (smg_field* f : ctx->field_pool) smg_field_destroy(f);
    for (auto& b : ctx->buf_pool) cudaFree(b.second);
    if (ctx->red.partials) cudaFree(ctx->red.partials);
    for (double* p : ctx->retired) cudaFree(p);
    if (ctx->red.tickets) cudaFree(ctx->red.tickets);
    if (ctx->host_stage) cudaFreeHost(ctx->host_stage);
    if (ctx->ev_begin) cudaEventDestroy(ctx->ev_begin);
    if (ctx->ev_end) cudaEventDestroy(ctx->ev_end);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SMG_OK;
}

SMG_API smg_status smg_timer_begin(smg_context* ctx) {
    if (!ctx) return SMG_BAD_ARG;
    if (!ctx->ev_begin) SMG_CUDA(ctx, cudaEventCreate(&ctx->ev_begin));
    if (!ctx->ev_end) SMG_CUDA(ctx, cudaEventCreate(&ctx->ev_end));
    SMG_CUDA(ctx, cudaEventRecord(ctx->ev_begin, ctx->stream));
    return SMG_OK;
}

SMG_API smg_status smg_timer_end(smg_context* ctx, double* ms) {
    if (!ctx || !ms || !ctx->ev_begin) return SMG_BAD_ARG;
    SMG_CUDA(ctx, cudaEventRecord(ctx->ev_end, ctx->stream));
    SMG_CUDA(ctx, cudaEventSynchronize(ctx->ev_end));
    float f = 0.f;
    SMG_CUDA(ctx, cudaEventElapsedTime(&f, ctx->ev_begin, ctx->ev_end));
    *ms = (double)f;
    return SMG_OK;
}

SMG_API smg_status smg_context_synchronize(smg_context* ctx) {
    if (!ctx) return SMG_BAD_ARG;
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

SMG_API smg_status smg_context_set_stream(smg_context* ctx, void* stream) {
    if (!ctx || !stream) return SMG_BAD_ARG;
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    ctx->own_stream = false;
    ctx->stream = (cudaStream_t)stream;
    return SMG_OK;
}

SMG_API void* smg_context_stream(smg_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

SMG_API const char* smg_last_error(smg_context* ctx) {
    return ctx ? ctx->last_error.c_str() : "null context";
}

SMG_API uint64_t smg_context_kernel_launches(smg_context* ctx) { return ctx ? ctx->launches : 0; }

}  // extern "C"
