// rt_graph.cu -- one frame of the dynamic path captured as a CUDA graph.
//
// RayTracerCS::Render with dynamic = 1 (RayTracerCS.cpp:258-295) issues the
// rebuild (2*depth + 46 dispatches in the reference) and the trace stages
// every frame.  Here the 10 build kernels, the two work-counter resets and
// the two trace kernels of one frame are captured once and replayed with a
// single cudaGraphLaunch, so the frame carries no per-kernel launch cost.
// Every kernel parameter (soup pointer, camera, output buffers) is fixed at
// capture time; a caller that streams new vertex data writes it into the
// captured soup buffer, or captures one frame object per buffer.
#include "rt_internal.cuh"

struct rt_frame {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint32_t nodes = 0;
    rt_lbvh* lbvh = nullptr;    // the structure whose buffers the graph points into (a reference)
    rt_batch* batch = nullptr;
};

// The frame keeps l's (b's) buffers alive and at their size until it is destroyed.
static void hold(rt_frame* f, rt_lbvh* l) {
    f->lbvh = l;
    ++l->graph_refs;
}
static void hold(rt_frame* f, rt_batch* b) {
    f->batch = b;
    ++b->graph_refs;
}

// Records what `record` issues on the context stream into a graph: the
// context stream is swapped for a private non-blocking stream (the legacy
// default stream cannot be captured) for the duration of the capture.
template <typename F>
static rt_status capture_frame(rt_ctx* ctx, const char* who, F record, rt_frame** out) {
    *out = nullptr;
    cudaStream_t cs = nullptr;
    RT_CHECK_CUDA(ctx, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    // the context stream's pending work must finish before the private stream
    // records the frame (the frame reads buffers that work may still write)
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cudaStreamDestroy(cs);
        return rt_fail(ctx, RT_ERR_CUDA, "%s: %s", who, cudaGetErrorString(e));
    }
    cudaStream_t saved = ctx->stream;
    ctx->stream = cs;
    rt_status s = RT_OK;
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        s = record();
        e = cudaStreamEndCapture(cs, &graph);
    }
    ctx->stream = saved;
    cudaStreamDestroy(cs);
    if (s != RT_OK) {
        if (graph) cudaGraphDestroy(graph);
        return s;
    }
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return rt_fail(ctx, RT_ERR_CUDA, "%s: stream capture failed: %s", who, cudaGetErrorString(e));
    }
    rt_frame* f = new rt_frame();
    f->graph = graph;
    e = cudaGraphInstantiate(&f->exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        delete f;
        return rt_fail(ctx, RT_ERR_CUDA, "%s: cudaGraphInstantiate failed: %s", who, cudaGetErrorString(e));
    }
    size_t count = 0;
    if (cudaGraphGetNodes(graph, nullptr, &count) == cudaSuccess) f->nodes = (uint32_t)count;
    *out = f;
    return RT_OK;
}

extern "C" rt_status rt_frame_capture(rt_ctx* ctx, rt_lbvh* l, const float* d_tris, uint32_t n, uint32_t flags,
                                      const rt_camera* cam, const float light[3], rt_hit* d_primary, uint8_t* d_vis,
                                      rt_hit* d_mirror, rt_frame** out) {
    if (!ctx) return RT_ERR_INVALID;
    if (!l || !d_tris || !cam || !light || !d_primary || !out)
        return rt_fail(ctx, RT_ERR_INVALID, "rt_frame_capture: null argument");
    // buffers the frame's calls would otherwise allocate inside the capture
    if ((d_vis || d_mirror) && cam->width && cam->height) {
        const rt_status es = ensure_shade_lists(ctx, l, (size_t)cam->width * cam->height);
        if (es != RT_OK) return es;
    }
    const rt_status s = capture_frame(
        ctx, "rt_frame_capture",
        [&]() {
            rt_status s = rt_lbvh_build(ctx, l, d_tris, n, flags);
            if (s == RT_OK) s = trace_frame(ctx, l, cam, light, d_primary, d_vis, d_mirror, "rt_frame_capture");
            return s;
        },
        out);
    if (s == RT_OK) hold(*out, l);
    return s;
}

// A host buffer a captured copy may use: page-locked (cudaHostAlloc /
// cudaHostRegister) or managed.
static bool pinned(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged;
}

extern "C" rt_status rt_frame_capture_host(rt_ctx* ctx, rt_lbvh* l, const float* h_tris, uint32_t n, uint32_t flags,
                                           const rt_camera* cam, const float light[3], rt_hit* h_primary,
                                           uint8_t* h_vis, rt_hit* h_mirror, rt_frame** out) {
    if (!ctx) return RT_ERR_INVALID;
    if (!l || !h_tris || !cam || !light || !out) return rt_fail(ctx, RT_ERR_INVALID, "rt_frame_capture_host: null argument");
    if (n == 0 || n > l->cap) return rt_fail(ctx, RT_ERR_CAPACITY, "rt_frame_capture_host: n=%u (capacity %u)", n, l->cap);
    const size_t px = (size_t)cam->width * cam->height;
    if (px == 0 || px > (1ull << 31)) return rt_fail(ctx, RT_ERR_INVALID, "rt_frame_capture_host: bad image size");
    const void* host[] = {h_tris, h_primary, h_vis, h_mirror};
    for (const void* h : host)
        if (h && !pinned(h))
            return rt_fail(ctx, RT_ERR_INVALID, "rt_frame_capture_host: host buffers must be page-locked");
    // buffers the frame's calls would otherwise allocate inside the capture
    rt_status es = ensure_frame_buffers(ctx, l, px);
    if (es == RT_OK && (h_vis || h_mirror)) es = ensure_shade_lists(ctx, l, px);
    if (es != RT_OK) return es;
    const rt_status cs = capture_frame(
        ctx, "rt_frame_capture_host",
        [&]() {
            cudaStream_t st = ctx->stream;
            RT_CHECK_CUDA(ctx, cudaMemcpyAsync(l->tris, h_tris, sizeof(float) * 9 * (size_t)n, cudaMemcpyHostToDevice, st));
            rt_status s = rt_lbvh_build(ctx, l, l->tris, n, flags);
            if (s == RT_OK)
                s = trace_frame(ctx, l, cam, light, l->f_primary, h_vis ? l->f_vis : nullptr,
                                h_mirror ? l->f_mirror : nullptr, "rt_frame_capture_host");
            if (s != RT_OK) return s;
            if (h_primary)
                RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_primary, l->f_primary, sizeof(rt_hit) * px, cudaMemcpyDeviceToHost, st));
            if (h_vis) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_vis, l->f_vis, px, cudaMemcpyDeviceToHost, st));
            if (h_mirror)
                RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_mirror, l->f_mirror, sizeof(rt_hit) * px, cudaMemcpyDeviceToHost, st));
            return RT_OK;
        },
        out);
    if (cs == RT_OK) hold(*out, l);
    return cs;
}

extern "C" rt_status rt_batch_frame_capture(rt_ctx* ctx, rt_batch* b, const float* d_tris, uint32_t flags,
                                            rt_hit* d_hits, uint8_t* d_vis, rt_frame** out) {
    if (!ctx) return RT_ERR_INVALID;
    if (!b || !d_tris || !d_hits || !out) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_frame_capture: null argument");
    if (b->width == 0) return rt_fail(ctx, RT_ERR_INVALID, "rt_batch_frame_capture: no views set (rt_batch_set_views)");
    const rt_status cs = capture_frame(
        ctx, "rt_batch_frame_capture",
        [&]() {
            rt_status s = rt_batch_build(ctx, b, d_tris, flags);
            if (s == RT_OK) s = rt_batch_trace(ctx, b, d_hits, d_vis);
            return s;
        },
        out);
    if (cs == RT_OK) hold(*out, b);
    return cs;
}

extern "C" rt_status rt_frame_launch(rt_ctx* ctx, rt_frame* f) {
    if (!ctx) return RT_ERR_INVALID;
    if (!f || !f->exec) return rt_fail(ctx, RT_ERR_INVALID, "rt_frame_launch: null frame");
    RT_CHECK_CUDA(ctx, cudaGraphLaunch(f->exec, ctx->stream));
    return RT_OK;
}

extern "C" uint32_t rt_frame_node_count(const rt_frame* f) { return f ? f->nodes : 0u; }

extern "C" rt_status rt_frame_destroy(rt_frame* f) {
    if (!f) return RT_OK;
    if (f->exec) cudaGraphExecDestroy(f->exec);
    if (f->graph) cudaGraphDestroy(f->graph);
    if (rt_lbvh* l = f->lbvh) {
        if (--l->graph_refs == 0 && l->destroy_pending) free_lbvh(l);
    }
    if (rt_batch* b = f->batch) {
        if (--b->graph_refs == 0 && b->destroy_pending) free_batch(b);
    }
    delete f;
    return RT_OK;
}
