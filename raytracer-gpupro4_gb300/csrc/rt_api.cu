// rt_api.cu -- context, error reporting and version entry points of the C ABI.
//
// An rt_ctx stands in for the reference's D3D11 device + immediate context
// (RayTracerCS/RayTracerCS.cpp:67-83, DeviceCore/DX11/DeviceDX11.inl:80-119):
// one CUDA device and one stream on which every call is queued.
#include <cstdarg>
#include <cstdio>

#include "rt_internal.cuh"

rt_status rt_fail(rt_ctx* ctx, rt_status s, const char* fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return s;
}

extern "C" int rt_api_version(void) { return RT_API_VERSION; }

extern "C" const char* rt_status_string(rt_status s) {
    switch (s) {
        case RT_OK: return "RT_OK";
        case RT_ERR_INVALID: return "RT_ERR_INVALID";
        case RT_ERR_CAPACITY: return "RT_ERR_CAPACITY";
        case RT_ERR_CUDA: return "RT_ERR_CUDA";
        case RT_ERR_TIMEOUT: return "RT_ERR_TIMEOUT";
        case RT_ERR_NONFINITE: return "RT_ERR_NONFINITE";
    }
    return "RT_ERR_UNKNOWN";
}

extern "C" rt_status rt_ctx_create(int device, void* stream, rt_ctx** out) {
    if (!out) return RT_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return RT_ERR_CUDA;
    if (cudaSetDevice(device) != cudaSuccess) return RT_ERR_CUDA;
    rt_ctx* c = new rt_ctx();
    c->device = device;
    c->stream = static_cast<cudaStream_t>(stream);
    if (cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaMalloc((void**)&c->d_words, 64 * sizeof(uint32_t)) != cudaSuccess ||
        cudaMemset(c->d_words, 0, 64 * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc((void**)&c->d_spill, sizeof(uint32_t) * kSpillCap) != cudaSuccess ||
        cudaMalloc((void**)&c->d_order, sizeof(uint32_t) * kOrderKinds * kOrderWords) != cudaSuccess ||
        cudaMemset(c->d_order, 0, sizeof(uint32_t) * kOrderKinds * kOrderWords) != cudaSuccess) {
        if (c->d_words) cudaFree(c->d_words);
        if (c->d_spill) cudaFree(c->d_spill);
        if (c->d_order) cudaFree(c->d_order);
        delete c;
        return RT_ERR_CUDA;
    }
    c->d_err = c->d_words;
    c->d_work = c->d_words + 16;
    c->d_spill_count = c->d_words + 32;
    *out = c;
    return RT_OK;
}

extern "C" rt_status rt_ctx_destroy(rt_ctx* ctx) {
    if (!ctx) return RT_OK;
    if (ctx->d_words) cudaFree(ctx->d_words);
    if (ctx->d_spill) cudaFree(ctx->d_spill);
    if (ctx->d_order) cudaFree(ctx->d_order);
    delete ctx;
    return RT_OK;
}

extern "C" rt_status rt_ctx_set_stream(rt_ctx* ctx, void* stream) {
    if (!ctx) return RT_ERR_INVALID;
    ctx->stream = static_cast<cudaStream_t>(stream);
    return RT_OK;
}

extern "C" rt_status rt_ctx_set_trace_budget(rt_ctx* ctx, uint32_t budget) {
    if (!ctx) return RT_ERR_INVALID;
    for (uint32_t& b : ctx->trace_budget) b = budget;
    return RT_OK;
}

extern "C" rt_status rt_ctx_set_trace_budget_kind(rt_ctx* ctx, uint32_t kind, uint32_t budget) {
    if (!ctx) return RT_ERR_INVALID;
    if (kind > 2u) return rt_fail(ctx, RT_ERR_INVALID, "rt_ctx_set_trace_budget_kind: kind is 0, 1 or 2");
    ctx->trace_budget[kind] = budget;
    return RT_OK;
}

extern "C" rt_status rt_ctx_set_heavy_block(rt_ctx* ctx, uint32_t kinds) {
    if (!ctx) return RT_ERR_INVALID;
    if (kinds > 7u) return rt_fail(ctx, RT_ERR_INVALID, "rt_ctx_set_heavy_block: kinds is a 3-bit mask");
    ctx->heavy_team = kinds;
    return RT_OK;
}

extern "C" rt_status rt_ctx_set_tile_order(rt_ctx* ctx, uint32_t kinds) {
    if (!ctx) return RT_ERR_INVALID;
    if (kinds > 7u) return rt_fail(ctx, RT_ERR_INVALID, "rt_ctx_set_tile_order: kinds is a 3-bit mask");
    ctx->tile_order = kinds;
    return RT_OK;
}

extern "C" rt_status rt_ctx_sync(rt_ctx* ctx) {
    if (!ctx) return RT_ERR_INVALID;
    RT_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RT_OK;
}

extern "C" rt_status rt_ctx_check(rt_ctx* ctx) {
    if (!ctx) return RT_ERR_INVALID;
    RT_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    uint32_t e = 0;
    RT_CHECK_CUDA(ctx, cudaMemcpy(&e, ctx->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (e) RT_CHECK_CUDA(ctx, cudaMemset(ctx->d_err, 0, sizeof(uint32_t)));
    if (e & RT_DEVERR_TIMEOUT) return rt_fail(ctx, RT_ERR_TIMEOUT, "a bounded device-side wait gave up");
    if (e & RT_DEVERR_BOUNDS) return rt_fail(ctx, RT_ERR_INVALID, "a device-side bounds check rejected an index");
    if (e & RT_DEVERR_NONFINITE) return rt_fail(ctx, RT_ERR_NONFINITE, "the triangle soup holds NaN or Inf coordinates");
    return RT_OK;
}

extern "C" const char* rt_last_error(const rt_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }
