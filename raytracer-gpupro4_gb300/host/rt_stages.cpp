// rt_stages.cpp -- implementation of the C++ stage classes over the C ABI.
#include "rt_stages.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

namespace rtgb {

void check(rt_status s, const rt_ctx* ctx, const char* what) {
    if (s == RT_OK) return;
    std::string msg = std::string(what) + ": " + rt_status_string(s);
    if (ctx) msg += std::string(": ") + rt_last_error(ctx);
    throw Error(s, msg);
}

static void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Error(RT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------
Context::Context(int device, void* stream) { check(rt_ctx_create(device, stream, &ctx_), nullptr, "rt_ctx_create"); }
Context::~Context() { rt_ctx_destroy(ctx_); }
void Context::Sync() { check(rt_ctx_sync(ctx_), ctx_, "rt_ctx_sync"); }
void Context::Check() { check(rt_ctx_check(ctx_), ctx_, "rt_ctx_check"); }

// ---------------------------------------------------------------------------
Model::Model(const std::string& sFileName) : m_sName(sFileName.substr(0, sFileName.find('.'))) {
    char err[512] = {0};
    const rt_status s = rt_model_load(sFileName.c_str(), &m_model, err, sizeof(err));
    if (s != RT_OK) throw Error(s, std::string("rt_model_load: ") + err);
}
Model::~Model() { rt_model_free(m_model); }
const rt_material& Model::GetMaterial(unsigned int i) const {
    const rt_material* m = rt_model_material(m_model, i);
    if (!m) throw Error(RT_ERR_INVALID, "Model::GetMaterial: index out of range");
    return *m;
}

// ---------------------------------------------------------------------------
DeviceBuffer::DeviceBuffer(size_t bytes) { resize(bytes); }
DeviceBuffer::~DeviceBuffer() {
    if (p_) cudaFree(p_);
}
DeviceBuffer::DeviceBuffer(DeviceBuffer&& o) noexcept : p_(o.p_), bytes_(o.bytes_) {
    o.p_ = nullptr;
    o.bytes_ = 0;
}
DeviceBuffer& DeviceBuffer::operator=(DeviceBuffer&& o) noexcept {
    if (this != &o) {
        if (p_) cudaFree(p_);
        p_ = o.p_;
        bytes_ = o.bytes_;
        o.p_ = nullptr;
        o.bytes_ = 0;
    }
    return *this;
}
void DeviceBuffer::resize(size_t bytes) {
    if (bytes <= bytes_) return;
    if (p_) cudaFree(p_);
    p_ = nullptr;
    bytes_ = 0;
    cuda_check(cudaMalloc(&p_, bytes), "cudaMalloc");
    bytes_ = bytes;
}
void DeviceBuffer::upload(const void* h, size_t bytes, void* stream) {
    resize(bytes);
    cuda_check(cudaMemcpyAsync(p_, h, bytes, cudaMemcpyHostToDevice, static_cast<cudaStream_t>(stream)),
               "cudaMemcpyAsync H2D");
}
void DeviceBuffer::download(void* h, size_t bytes, void* stream) const {
    cuda_check(cudaMemcpyAsync(h, p_, bytes, cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream)),
               "cudaMemcpyAsync D2H");
    cuda_check(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "cudaStreamSynchronize");
}

// ---------------------------------------------------------------------------
static unsigned int depth_of(int n) {
    unsigned int d = 0;
    while ((1u << (d + 1)) <= (unsigned)n) ++d;
    return d;
}

LBVHGpu::LBVHGpu(Context& ctx, const float* soup, unsigned int numPrimitives, int n, bool soupOnDevice)
    : m_ctx(ctx), m_soup(soup), m_soupOnDevice(soupOnDevice), m_depth(depth_of(n)) {
    m_sName = "LBVH";
    m_uiNumPrimitives = numPrimitives;
    check(rt_lbvh_create(ctx.get(), numPrimitives ? numPrimitives : 1, m_depth, &m_lbvh), ctx.get(), "rt_lbvh_create");
}

LBVHGpu::~LBVHGpu() { rt_lbvh_destroy(m_lbvh); }

void LBVHGpu::SetSoup(const float* soup, unsigned int numPrimitives, bool soupOnDevice) {
    m_soup = soup;
    m_uiNumPrimitives = numPrimitives;
    m_soupOnDevice = soupOnDevice;
}

void LBVHGpu::Build() {
    if (m_soupOnDevice)
        check(rt_lbvh_build(m_ctx.get(), m_lbvh, m_soup, m_uiNumPrimitives, 0), m_ctx.get(), "rt_lbvh_build");
    else
        check(rt_lbvh_build_host(m_ctx.get(), m_lbvh, m_soup, m_uiNumPrimitives, 0), m_ctx.get(),
              "rt_lbvh_build_host");
    m_mirrorValid = false;
}

void LBVHGpu::IntersectP(const Ray* rays, size_t count, TIntersection* out) {
    if (count == 0) return;
    std::vector<rt_ray> r(count);
    for (size_t k = 0; k < count; ++k) {
        r[k].o[0] = rays[k].o.x; r[k].o[1] = rays[k].o.y; r[k].o[2] = rays[k].o.z;
        r[k].d[0] = rays[k].d.x; r[k].d[1] = rays[k].d.y; r[k].d[2] = rays[k].d.z;
        r[k].exclude_id = rays[k].TriangleID;
        r[k].tmax = rays[k].maxt;
    }
    void* st = nullptr;  // the context's stream is used by every C-ABI call
    m_rays.upload(r.data(), sizeof(rt_ray) * count, st);
    m_hits.resize(sizeof(rt_hit) * count);
    check(rt_trace_rays(m_ctx.get(), m_lbvh, static_cast<const rt_ray*>(m_rays.data()), (uint32_t)count, 0,
                        static_cast<rt_hit*>(m_hits.data()), nullptr),
          m_ctx.get(), "rt_trace_rays");
    m_ctx.Sync();
    std::vector<rt_hit> h(count);
    m_hits.download(h.data(), sizeof(rt_hit) * count, st);
    for (size_t k = 0; k < count; ++k) {
        out[k].IDTr = h[k].id;
        out[k].u = h[k].u;
        out[k].v = h[k].v;
        out[k].t = h[k].t;
    }
}

TIntersection LBVHGpu::IntersectP(Ray& a_Ray) {
    TIntersection res;
    IntersectP(&a_Ray, 1, &res);
    return res;
}

void* LBVHGpu::GetPtrToElements() {
    if (!m_mirrorValid) {
        m_hostNodes.resize(GetNumberOfElements());
        m_hostIds.resize(m_uiNumPrimitives);
        check(rt_lbvh_download(m_ctx.get(), m_lbvh, reinterpret_cast<rt_node*>(m_hostNodes.data()), m_hostIds.data(),
                               nullptr),
              m_ctx.get(), "rt_lbvh_download");
        m_mirrorValid = true;
    }
    return m_hostNodes.data();
}

unsigned int* LBVHGpu::GetOrderedElementsIds() {
    GetPtrToElements();
    return m_hostIds.data();
}

BBox LBVHGpu::WorldBound() {
    float b[6];
    check(rt_lbvh_world_bound(m_ctx.get(), m_lbvh, b), m_ctx.get(), "rt_lbvh_world_bound");
    BBox box;
    box.pMin = Vector3{b[0], b[1], b[2]};
    box.pMax = Vector3{b[3], b[4], b[5]};
    return box;
}

void LBVHGpu::PrintOutput(float& totaltime) {
    // occupancy figures of LBVH::PrintOutput (LBVH.cpp:1580-1594)
    const LBVHNode* nodes = static_cast<const LBVHNode*>(GetPtrToElements());
    const unsigned int num = GetNumberOfElements();
    std::vector<char> reach(num, 0);
    unsigned int occupied = 0, leaves = 0;
    if (num > 1) reach[1] = 1;
    for (unsigned int i = 1; i < num; ++i) {
        if (!reach[i]) continue;
        ++occupied;
        if (nodes[i].PrimCount & 4) {
            ++leaves;
        } else if (2 * i + 1 < num) {
            reach[2 * i] = reach[2 * i + 1] = 1;
        }
    }
    std::printf("LBVH: %u Nodes * %zu Bytes per Node = %.2f MB\n", num, sizeof(LBVHNode),
                num * sizeof(LBVHNode) / 1048576.0);
    std::printf("LBVH: Occupied Nodes = %u, Free Nodes = %u\n", occupied, num - occupied);
    std::printf("LBVH: Occupied Leafs = %u, Primitives/Leaf = %.3f, build %.3f ms\n", leaves,
                leaves ? double(m_uiNumPrimitives) / leaves : 0.0, totaltime * 1e3);
}

// ---------------------------------------------------------------------------
StructureConstruction::StructureConstruction(Context& ctx, unsigned int maxPrimitives, unsigned int depth)
    : m_ctx(ctx), m_depth(depth) {
    check(rt_lbvh_create(ctx.get(), maxPrimitives, depth, &m_lbvh), ctx.get(), "rt_lbvh_create");
}

StructureConstruction::~StructureConstruction() { rt_lbvh_destroy(m_lbvh); }

void StructureConstruction::GPUBuildStructure(unsigned int uiDepth, const float* d_soup, unsigned int numPrimitives) {
    if (uiDepth != m_depth) throw Error(RT_ERR_INVALID, "GPUBuildStructure: depth differs from the construction's");
    check(rt_lbvh_build(m_ctx.get(), m_lbvh, d_soup, numPrimitives, 0), m_ctx.get(), "rt_lbvh_build");
}

// ---------------------------------------------------------------------------
RayTracerCS::RayTracerCS(Context& ctx, const Scene& scene, const rt_camera& camera, const float light[3],
                         unsigned int lbvhDepth, bool dynamic)
    : m_ctx(ctx), m_scene(scene), m_camera(camera), m_depth(lbvhDepth), m_dynamic(dynamic),
      m_construction(ctx, scene.numPrimitives, lbvhDepth) {
    std::memcpy(m_light, light, sizeof(m_light));
    const size_t px = (size_t)camera.width * camera.height;
    m_primary.resize(sizeof(rt_hit) * px);
    m_roots.resize(sizeof(uint32_t) * px);
    m_vis.resize(px);
    m_mirror.resize(sizeof(rt_hit) * px);
    UpdateScene(scene.soup);
}

void RayTracerCS::UpdateScene(const float* soup) {
    m_scene.soup = soup;
    m_soup.upload(soup, sizeof(float) * 9 * (size_t)m_scene.numPrimitives, nullptr);
    cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    m_built = false;
}

void RayTracerCS::Render() {
    // Render (RayTracerCS.cpp:258-295): rebuild when dynamic, then primary
    // rays and the colour stage's shadow + mirror rays, which start their
    // walks at the primary hit's leaf (the iRoot the reference keeps in
    // g_uIntersections, CSComputeColorRT.hlsl:160)
    Rebuild();
    rt_lbvh* l = m_construction.lbvh();
    uint32_t* roots = static_cast<uint32_t*>(m_roots.data());
    check(rt_trace_primary_leaves(m_ctx.get(), l, &m_camera, static_cast<rt_hit*>(m_primary.data()), roots, nullptr),
          m_ctx.get(), "rt_trace_primary_leaves");
    check(rt_trace_shadow_mirror_from(m_ctx.get(), l, &m_camera, m_light, static_cast<const rt_hit*>(m_primary.data()),
                                      roots, static_cast<uint8_t*>(m_vis.data()), static_cast<rt_hit*>(m_mirror.data()),
                                      nullptr, nullptr, nullptr),
          m_ctx.get(), "rt_trace_shadow_mirror_from");
    ++m_NumMuestras;
}

void RayTracerCS::Rebuild() {
    if (m_dynamic || !m_built) {
        m_construction.GPUBuildStructure(m_depth, static_cast<const float*>(m_soup.data()), m_scene.numPrimitives);
        m_built = true;
    }
}

void RayTracerCS::RenderColor(const rt_shade_params& params, const rt_material* materials, unsigned int numMaterials,
                              const int32_t* materialIds) {
    if (!materials || numMaterials == 0) throw Error(RT_ERR_INVALID, "RayTracerCS::RenderColor: no materials");
    Rebuild();
    const size_t px = (size_t)m_camera.width * m_camera.height;
    m_materials.upload(materials, sizeof(rt_material) * numMaterials, nullptr);
    if (materialIds) m_materialIds.upload(materialIds, sizeof(int32_t) * m_scene.numPrimitives, nullptr);
    m_accum.resize(sizeof(float) * 4 * px);
    m_result.resize(sizeof(float) * 4 * px);
    cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    check(rt_render_whitted(m_ctx.get(), m_construction.lbvh(), &m_camera, m_light, &params,
                            materialIds ? static_cast<const int32_t*>(m_materialIds.data()) : nullptr,
                            static_cast<const rt_material*>(m_materials.data()), numMaterials, nullptr,
                            static_cast<float*>(m_accum.data()), static_cast<float*>(m_result.data())),
          m_ctx.get(), "rt_render_whitted");
}

std::vector<float> RayTracerCS::DownloadAccumulation() const {
    m_ctx.Sync();
    std::vector<float> v((size_t)m_camera.width * m_camera.height * 4);
    m_accum.download(v.data(), sizeof(float) * v.size(), nullptr);
    return v;
}

std::vector<float> RayTracerCS::DownloadResult() const {
    m_ctx.Sync();
    std::vector<float> v((size_t)m_camera.width * m_camera.height * 4);
    m_result.download(v.data(), sizeof(float) * v.size(), nullptr);
    return v;
}

void RayTracerCS::SetGIMaterials(const float* albedo, const float* emission) {
    if (!albedo || !emission) throw Error(RT_ERR_INVALID, "RayTracerCS::SetGIMaterials: null array");
    m_albedo.upload(albedo, sizeof(float) * 3 * m_scene.numPrimitives, nullptr);
    m_emission.upload(emission, sizeof(float) * 3 * m_scene.numPrimitives, nullptr);
    cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
}

void RayTracerCS::RenderGI(unsigned int spp, unsigned int bounces, uint64_t seed, const float sky[3]) {
    if (!m_albedo.data() || !m_emission.data())
        throw Error(RT_ERR_INVALID, "RayTracerCS::RenderGI: SetGIMaterials first");
    Rebuild();
    m_gi.resize(sizeof(float) * 4 * (size_t)m_camera.width * m_camera.height);
    rt_pt_params p;
    p.spp = spp;
    p.bounces = bounces;
    p.seed = seed;
    for (int c = 0; c < 3; ++c) p.sky[c] = sky[c];
    p.first_sample = m_giSamples;
    check(rt_pathtrace(m_ctx.get(), m_construction.lbvh(), static_cast<const float*>(m_albedo.data()),
                       static_cast<const float*>(m_emission.data()), &m_camera, &p, static_cast<float*>(m_gi.data())),
          m_ctx.get(), "rt_pathtrace");
    m_giSamples += spp;
}

std::vector<float> RayTracerCS::DownloadGI() const {
    m_ctx.Sync();
    std::vector<float> v((size_t)m_camera.width * m_camera.height * 4);
    m_gi.download(v.data(), sizeof(float) * v.size(), nullptr);
    return v;
}

std::vector<rt_hit> RayTracerCS::DownloadPrimary() const {
    m_ctx.Sync();
    std::vector<rt_hit> h((size_t)m_camera.width * m_camera.height);
    m_primary.download(h.data(), sizeof(rt_hit) * h.size(), nullptr);
    return h;
}

std::vector<uint8_t> RayTracerCS::DownloadVisibility() const {
    m_ctx.Sync();
    std::vector<uint8_t> v((size_t)m_camera.width * m_camera.height);
    m_vis.download(v.data(), v.size(), nullptr);
    return v;
}

std::vector<rt_hit> RayTracerCS::DownloadMirror() const {
    m_ctx.Sync();
    std::vector<rt_hit> h((size_t)m_camera.width * m_camera.height);
    m_mirror.download(h.data(), sizeof(rt_hit) * h.size(), nullptr);
    return h;
}

// ---------------------------------------------------------------------------
PinnedBuffer::PinnedBuffer(size_t bytes) {
    cuda_check(cudaHostAlloc(&p_, bytes, cudaHostAllocDefault), "cudaHostAlloc");
    bytes_ = bytes;
}
PinnedBuffer::~PinnedBuffer() {
    if (p_) cudaFreeHost(p_);
}
PinnedBuffer::PinnedBuffer(PinnedBuffer&& o) noexcept : p_(o.p_), bytes_(o.bytes_) {
    o.p_ = nullptr;
    o.bytes_ = 0;
}
PinnedBuffer& PinnedBuffer::operator=(PinnedBuffer&& o) noexcept {
    if (this != &o) {
        if (p_) cudaFreeHost(p_);
        p_ = o.p_;
        bytes_ = o.bytes_;
        o.p_ = nullptr;
        o.bytes_ = 0;
    }
    return *this;
}

// ---------------------------------------------------------------------------
FramePipeline::FramePipeline(Context& ctx, unsigned int numPrimitives, const rt_camera& camera, const float light[3],
                             unsigned int lbvhDepth, bool visibility, bool mirror)
    : m_ctx(ctx) {
    check(rt_lbvh_create(ctx.get(), numPrimitives, lbvhDepth, &m_lbvh), ctx.get(), "rt_lbvh_create");
    const rt_status s = rt_pipe_create(ctx.get(), m_lbvh, numPrimitives, 0, &camera, light, visibility ? 1 : 0,
                                       mirror ? 1 : 0, &m_pipe);
    if (s != RT_OK) {
        rt_lbvh_destroy(m_lbvh);
        check(s, ctx.get(), "rt_pipe_create");
    }
}
FramePipeline::~FramePipeline() {
    rt_pipe_destroy(m_pipe);
    rt_lbvh_destroy(m_lbvh);  // freed with the pipe's last captured frame
}
uint64_t FramePipeline::Submit(const float* h_soup, rt_hit* h_primary, uint8_t* h_vis, rt_hit* h_mirror) {
    uint64_t ticket = 0;
    check(rt_pipe_submit(m_pipe, h_soup, h_primary, h_vis, h_mirror, &ticket), m_ctx.get(), "rt_pipe_submit");
    return ticket;
}
void FramePipeline::Wait(uint64_t ticket) { check(rt_pipe_wait(m_pipe, ticket), m_ctx.get(), "rt_pipe_wait"); }

}  // namespace rtgb
