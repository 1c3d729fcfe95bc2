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

// ---------------------------------------------------------------------------
// Double-buffered host frames (rt_pipe_*).  Frame k uses slot s = k mod 2:
//   upload stream:  wait for the kernels of frame k-2 (they read soup[s]),
//                   copy the host soup into soup[s]                  -> ev_in[s]
//   context stream: wait ev_in[s] and the read-back of frame k-2 (it reads
//                   the results of slot s), the captured frame of slot s -> ev_comp[s]
//   read-back stream: wait ev_comp[s], copy the results to the host  -> ev_out[s]
// The kernels of consecutive frames are ordered by the context stream, so
// only copies overlap kernels.
struct rt_pipe {
    rt_ctx* ctx = nullptr;
    rt_lbvh* lbvh = nullptr;
    uint32_t n = 0;
    size_t px = 0;
    bool vis = false, mirror = false;
    float* soup[2] = {nullptr, nullptr};
    rt_hit* prim[2] = {nullptr, nullptr};
    uint8_t* vbuf[2] = {nullptr, nullptr};
    rt_hit* mbuf[2] = {nullptr, nullptr};
    rt_frame* frame[2] = {nullptr, nullptr};
    cudaStream_t up = nullptr, down = nullptr;
    cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_comp[2] = {nullptr, nullptr}, ev_out[2] = {nullptr, nullptr};
    uint64_t next = 0;
};

static void free_pipe(rt_pipe* p) {
    for (int s = 0; s < 2; ++s) {
        if (p->frame[s]) rt_frame_destroy(p->frame[s]);
        for (void* q : {(void*)p->soup[s], (void*)p->prim[s], (void*)p->vbuf[s], (void*)p->mbuf[s]})
            if (q) cudaFree(q);
        for (cudaEvent_t e : {p->ev_in[s], p->ev_comp[s], p->ev_out[s]})
            if (e) cudaEventDestroy(e);
    }
    if (p->up) cudaStreamDestroy(p->up);
    if (p->down) cudaStreamDestroy(p->down);
    delete p;
}

extern "C" rt_status rt_pipe_create(rt_ctx* ctx, rt_lbvh* l, uint32_t n, uint32_t flags, const rt_camera* cam,
                                    const float light[3], int want_vis, int want_mirror, rt_pipe** out) {
    if (!ctx) return RT_ERR_INVALID;
    if (!l || !cam || !light || !out) return rt_fail(ctx, RT_ERR_INVALID, "rt_pipe_create: null argument");
    *out = nullptr;
    if (n == 0 || n > l->cap) return rt_fail(ctx, RT_ERR_CAPACITY, "rt_pipe_create: n=%u (capacity %u)", n, l->cap);
    const size_t px = (size_t)cam->width * cam->height;
    if (px == 0 || px > (1ull << 31)) return rt_fail(ctx, RT_ERR_INVALID, "rt_pipe_create: bad image size");
    RT_CHECK_CUDA(ctx, cudaSetDevice(ctx->device));
    rt_pipe* p = new rt_pipe();
    p->ctx = ctx;
    p->n = n;
    p->px = px;
    p->vis = want_vis != 0;
    p->mirror = want_mirror != 0;
    cudaError_t e = cudaSuccess;
    auto ok = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
        return e == cudaSuccess;
    };
    for (int s = 0; s < 2; ++s) {
        ok(cudaMalloc((void**)&p->soup[s], sizeof(float) * 9 * (size_t)n));
        ok(cudaMalloc((void**)&p->prim[s], sizeof(rt_hit) * px));
        if (p->vis) ok(cudaMalloc((void**)&p->vbuf[s], px));
        if (p->mirror) ok(cudaMalloc((void**)&p->mbuf[s], sizeof(rt_hit) * px));
        ok(cudaEventCreateWithFlags(&p->ev_in[s], cudaEventDisableTiming));
        ok(cudaEventCreateWithFlags(&p->ev_comp[s], cudaEventDisableTiming));
        ok(cudaEventCreateWithFlags(&p->ev_out[s], cudaEventDisableTiming));
    }
    ok(cudaStreamCreateWithFlags(&p->up, cudaStreamNonBlocking));
    ok(cudaStreamCreateWithFlags(&p->down, cudaStreamNonBlocking));
    // the captured frames read an uninitialised soup only if submitted
    // without an upload, which rt_pipe_submit never does
    if (e != cudaSuccess) {
        free_pipe(p);
        return rt_fail(ctx, RT_ERR_CUDA, "rt_pipe_create: %s", cudaGetErrorString(e));
    }
    for (int s = 0; s < 2; ++s) {
        const rt_status cs = rt_frame_capture(ctx, l, p->soup[s], n, flags, cam, light, p->prim[s], p->vbuf[s],
                                              p->mbuf[s], &p->frame[s]);
        if (cs != RT_OK) {
            free_pipe(p);
            return cs;
        }
    }
    p->lbvh = l;
    *out = p;
    return RT_OK;
}

extern "C" rt_status rt_pipe_submit(rt_pipe* p, const float* h_tris, rt_hit* h_primary, uint8_t* h_vis,
                                    rt_hit* h_mirror, uint64_t* ticket) {
    if (!p) return RT_ERR_INVALID;
    rt_ctx* ctx = p->ctx;
    if (!h_tris) return rt_fail(ctx, RT_ERR_INVALID, "rt_pipe_submit: null soup");
    if ((h_vis && !p->vis) || (h_mirror && !p->mirror))
        return rt_fail(ctx, RT_ERR_INVALID, "rt_pipe_submit: the pipe was created without that output");
    const void* host[] = {h_tris, h_primary, h_vis, h_mirror};
    for (const void* h : host)
        if (h && !pinned(h)) return rt_fail(ctx, RT_ERR_INVALID, "rt_pipe_submit: host buffers must be page-locked");
    const uint64_t k = p->next;
    const int s = (int)(k & 1u);
    cudaStream_t cs = ctx->stream;
    if (k >= 2) RT_CHECK_CUDA(ctx, cudaStreamWaitEvent(p->up, p->ev_comp[s], 0));
    RT_CHECK_CUDA(ctx, cudaMemcpyAsync(p->soup[s], h_tris, sizeof(float) * 9 * (size_t)p->n, cudaMemcpyHostToDevice, p->up));
    RT_CHECK_CUDA(ctx, cudaEventRecord(p->ev_in[s], p->up));
    RT_CHECK_CUDA(ctx, cudaStreamWaitEvent(cs, p->ev_in[s], 0));
    if (k >= 2) RT_CHECK_CUDA(ctx, cudaStreamWaitEvent(cs, p->ev_out[s], 0));
    RT_CHECK_CUDA(ctx, cudaGraphLaunch(p->frame[s]->exec, cs));
    RT_CHECK_CUDA(ctx, cudaEventRecord(p->ev_comp[s], cs));
    RT_CHECK_CUDA(ctx, cudaStreamWaitEvent(p->down, p->ev_comp[s], 0));
    if (h_primary)
        RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_primary, p->prim[s], sizeof(rt_hit) * p->px, cudaMemcpyDeviceToHost, p->down));
    if (h_vis) RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_vis, p->vbuf[s], p->px, cudaMemcpyDeviceToHost, p->down));
    if (h_mirror)
        RT_CHECK_CUDA(ctx, cudaMemcpyAsync(h_mirror, p->mbuf[s], sizeof(rt_hit) * p->px, cudaMemcpyDeviceToHost, p->down));
    RT_CHECK_CUDA(ctx, cudaEventRecord(p->ev_out[s], p->down));
    p->next = k + 1;
    if (ticket) *ticket = k;
    return RT_OK;
}

extern "C" rt_status rt_pipe_wait(rt_pipe* p, uint64_t ticket) {
    if (!p) return RT_ERR_INVALID;
    if (ticket >= p->next) return rt_fail(p->ctx, RT_ERR_INVALID, "rt_pipe_wait: frame %llu was not submitted",
                                          (unsigned long long)ticket);
    RT_CHECK_CUDA(p->ctx, cudaEventSynchronize(p->ev_out[ticket & 1u]));
    return RT_OK;
}

extern "C" rt_status rt_pipe_destroy(rt_pipe* p) {
    if (!p) return RT_OK;
    cudaStreamSynchronize(p->up);
    cudaStreamSynchronize(p->ctx->stream);
    cudaStreamSynchronize(p->down);
    free_pipe(p);
    return RT_OK;
}
