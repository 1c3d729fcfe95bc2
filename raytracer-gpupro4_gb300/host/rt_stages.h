// rt_stages.h -- C++ drop-in for the reference's LBVH stage classes.
//
// Same class and method names as the reference, implemented over the C ABI
// (include/rt_api.h), so host code written against the reference's
// interfaces keeps its call sequence:
//   AccelerationStructure  AccelerationStructures/AccelerationStructure.h:40-67
//   LBVHGpu                AccelerationStructures/LBVH/LBVH.h:70-118 (LBVH)
//   StructureConstruction  RayTracerCS/StructureConstruction.h:67-91
//   RayTracerCS            RayTracerCS/RayTracerCS.h:64-144 (headless: the
//                          swap chain becomes device hit buffers)
//   Model                  Common/Scenes/Model.h:35-80 (file -> triangle soup
//                          through include/rt_model.h; no Direct3D objects)
// The geometry types mirror Common/Geometry (Vector3, BBox, Ray,
// TIntersection) and the 32-byte LBVHNode (LBVH.h:25-28).
//
// Errors: the reference printed or exit()ed; these classes throw rtgb::Error
// carrying the rt_status and message of the failing C-ABI call.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "rt_api.h"
#include "rt_model.h"

namespace rtgb {

struct Vector3 {
    float x = 0.f, y = 0.f, z = 0.f;
};

// LBVHNode (LBVH.h:25-28): PrimCount = (count << 3) | leaf*4 | axis.
struct LBVHNode {
    Vector3 minCoord, maxCoord;
    int PrimCount, PrimPos;
};
static_assert(sizeof(LBVHNode) == sizeof(rt_node), "LBVHNode must match rt_node");

struct BBox {
    Vector3 pMin, pMax;
};

// Ray (Common/Geometry/Ray.h:22-49, without the shading factor).
struct Ray {
    Vector3 o, d;
    float mint = 0.f, maxt = 1e16f;
    int TriangleID = -1;  // triangle the ray leaves from (ignored by the test)
};

// TIntersection (Geometry.h:116-122).
struct TIntersection {
    int IDTr = -1;
    float u = 0.f, v = 0.f, t = 0.f;
    int tmp[2] = {0, 0};
};

class Error : public std::runtime_error {
   public:
    Error(rt_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    rt_status status;
};

void check(rt_status s, const rt_ctx* ctx, const char* what);

// A CUDA device + stream (replaces the D3D11 device / immediate context).
class Context {
   public:
    explicit Context(int device = 0, void* stream = nullptr);
    ~Context();
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    rt_ctx* get() const { return ctx_; }
    void Sync();
    void Check();  // synchronise and raise on a device-side error flag

   private:
    rt_ctx* ctx_ = nullptr;
};

// Owned device buffer.
class DeviceBuffer {
   public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes);
    ~DeviceBuffer();
    DeviceBuffer(DeviceBuffer&& o) noexcept;
    DeviceBuffer& operator=(DeviceBuffer&& o) noexcept;
    DeviceBuffer(const DeviceBuffer&) = delete;
    void* data() const { return p_; }
    size_t size() const { return bytes_; }
    void resize(size_t bytes);
    void upload(const void* h, size_t bytes, void* stream);
    void download(void* h, size_t bytes, void* stream) const;

   private:
    void* p_ = nullptr;
    size_t bytes_ = 0;
};

// AccelerationStructure (AccelerationStructure.h:40-67).
class AccelerationStructure {
   public:
    virtual ~AccelerationStructure() = default;
    const char* GetName() const { return m_sName; }
    virtual TIntersection IntersectP(Ray& a_Ray) = 0;
    virtual void PrintOutput(float& totaltime) = 0;
    virtual void Build() = 0;
    virtual unsigned int GetNumberOfElements() = 0;
    virtual size_t GetSizeOfElement() = 0;
    virtual void* GetPtrToElements() = 0;
    virtual unsigned int* GetOrderedElementsIds() = 0;
    virtual unsigned int GetKeyboardId() = 0;
    virtual BBox WorldBound() = 0;
    unsigned int GetNumPrimitives() const { return m_uiNumPrimitives; }

   protected:
    const char* m_sName = "";
    unsigned int m_uiNumPrimitives = 0;
};

// LBVH (LBVH.h:70-118) built and traversed on the GPU.  The reference's
// constructor takes Primitive** (borrowed); this one takes a triangle soup
// (n x 9 floats), on the host or on the device, also borrowed until the
// next Build().  n = number of heap slots, as LBVH(prims, N, 1 << depth).
class LBVHGpu : public AccelerationStructure {
   public:
    LBVHGpu(Context& ctx, const float* soup, unsigned int numPrimitives, int n = 1 << 21, bool soupOnDevice = false);
    ~LBVHGpu() override;

    void Build() override;                        // LBVH::Build (LBVH.cpp:488-632)
    TIntersection IntersectP(Ray& a_Ray) override;  // one ray (interface completeness)
    void IntersectP(const Ray* rays, size_t count, TIntersection* out);  // batched
    void PrintOutput(float& totaltime) override;
    unsigned int GetNumberOfElements() override { return 1u << m_depth; }
    size_t GetSizeOfElement() override { return sizeof(LBVHNode); }
    void* GetPtrToElements() override;             // host mirror, downloaded on demand
    unsigned int* GetOrderedElementsIds() override;  // host mirror, downloaded on demand
    unsigned int GetKeyboardId() override { return 9; }
    BBox WorldBound() override;

    void SetSoup(const float* soup, unsigned int numPrimitives, bool soupOnDevice);
    rt_lbvh* handle() const { return m_lbvh; }
    Context& context() const { return m_ctx; }

   private:
    Context& m_ctx;
    rt_lbvh* m_lbvh = nullptr;
    const float* m_soup = nullptr;
    bool m_soupOnDevice = false;
    unsigned int m_depth = 0;
    std::vector<LBVHNode> m_hostNodes;
    std::vector<unsigned int> m_hostIds;
    bool m_mirrorValid = false;
    DeviceBuffer m_rays, m_hits;
};

// StructureConstruction (StructureConstruction.h:67-91): the per-frame GPU
// rebuild.  The reference dispatched PreBuild, a 45-dispatch bitonic sort and
// 2*depth level dispatches; GPUBuildStructure is one rt_lbvh_build.
class StructureConstruction {
   public:
    StructureConstruction(Context& ctx, unsigned int maxPrimitives, unsigned int depth);
    void GPUBuildStructure(unsigned int uiDepth, const float* d_soup, unsigned int numPrimitives);
    rt_lbvh* lbvh() const { return m_lbvh; }
    ~StructureConstruction();

   private:
    Context& m_ctx;
    rt_lbvh* m_lbvh = nullptr;
    unsigned int m_depth;
};

struct Scene {
    const float* soup = nullptr;  // host, n x 9 floats
    unsigned int numPrimitives = 0;
};

// Model (Model.h:35-80): the constructor loads the file (Model::LoadFile,
// .obj or .txt) and applies Model::Scale; the primitives are the triangle
// soup the acceleration structures take.  The path is used as given (the
// reference prefixed "./Models/").
class Model {
   public:
    explicit Model(const std::string& sFileName);
    ~Model();
    Model(const Model&) = delete;
    Model& operator=(const Model&) = delete;
    unsigned int GetNumPrimitives() const { return rt_model_triangle_count(m_model); }
    unsigned int GetNumMaterials() const { return rt_model_material_count(m_model); }
    const float* GetSoup() const { return rt_model_soup(m_model); }  // n x 9 floats
    const int32_t* GetMaterialIds() const { return rt_model_material_ids(m_model); }
    const rt_material& GetMaterial(unsigned int i) const;
    const std::string& GetName() const { return m_sName; }
    Scene GetScene() const { return Scene{GetSoup(), GetNumPrimitives()}; }

   private:
    rt_model* m_model = nullptr;
    std::string m_sName;
};

// RayTracerCS::Render (RayTracerCS.cpp:241-311) without a window: per frame,
// an optional LBVH rebuild (dynamic = 1), primary rays, then the shadow ray
// and one mirror bounce per pixel.  Results stay in device buffers; Download*
// copies them to the host.
class RayTracerCS {
   public:
    RayTracerCS(Context& ctx, const Scene& scene, const rt_camera& camera, const float light[3],
                unsigned int lbvhDepth = 20, bool dynamic = true);
    void Render();
    void UpdateScene(const float* soup);  // new vertex positions for the next frame (same count)
    std::vector<rt_hit> DownloadPrimary() const;
    std::vector<uint8_t> DownloadVisibility() const;
    std::vector<rt_hit> DownloadMirror() const;
    unsigned int GetNumSamples() const { return m_NumMuestras; }
    StructureConstruction& construction() { return m_construction; }

    // The colour stage of Render without global illumination
    // (RayTracerCS.cpp:284-295, CSComputeColorRT.hlsl): primary rays, then
    // params.bounces + 1 intersection + colour stages into the accumulation
    // and result images (g_uAccumulation / g_uResultTexture, w*h float4).
    // materials: numMaterials host rows; materialIds: host, one per
    // triangle, or null (all 0).  Rebuilds first when dynamic.
    void RenderColor(const rt_shade_params& params, const rt_material* materials, unsigned int numMaterials,
                     const int32_t* materialIds = nullptr);
    std::vector<float> DownloadAccumulation() const;
    std::vector<float> DownloadResult() const;

    // Progressive global illumination (CSComputeColorGI.hlsl with the frame
    // counter of RayTracerCS.cpp:306): each call traces spp more samples per
    // pixel and blends them into the GI image; ResetGI() restarts it (the
    // reset on camera motion, RayTracerCS.cpp:246-250).  albedo / emission:
    // host, n x 3 floats indexed by triangle id.  Rebuilds first when dynamic.
    void SetGIMaterials(const float* albedo, const float* emission);
    void RenderGI(unsigned int spp, unsigned int bounces, uint64_t seed, const float sky[3]);
    void ResetGI() { m_giSamples = 0; }
    unsigned int GetGISamples() const { return m_giSamples; }
    std::vector<float> DownloadGI() const;

   private:
    Context& m_ctx;
    Scene m_scene;
    rt_camera m_camera;
    float m_light[3];
    unsigned int m_depth;
    bool m_dynamic;
    bool m_built = false;
    StructureConstruction m_construction;
    DeviceBuffer m_soup, m_primary, m_roots, m_vis, m_mirror;
    DeviceBuffer m_materials, m_materialIds, m_accum, m_result;
    DeviceBuffer m_albedo, m_emission, m_gi;
    unsigned int m_NumMuestras = 0;
    unsigned int m_giSamples = 0;
    void Rebuild();
};

// Page-locked host buffer (cudaHostAlloc): what rt_pipe_submit copies from
// and into.
class PinnedBuffer {
   public:
    PinnedBuffer() = default;
    explicit PinnedBuffer(size_t bytes);
    ~PinnedBuffer();
    PinnedBuffer(PinnedBuffer&& o) noexcept;
    PinnedBuffer& operator=(PinnedBuffer&& o) noexcept;
    PinnedBuffer(const PinnedBuffer&) = delete;
    void* data() const { return p_; }
    size_t size() const { return bytes_; }

   private:
    void* p_ = nullptr;
    size_t bytes_ = 0;
};

// A dynamic model's frame loop with host data (vertex update + Render +
// read-back of the results, RayTracerCS.cpp:241-311) pipelined over
// rt_pipe_*: two frames in flight, uploads and read-backs on copy streams,
// the frames' rebuild + trace in order on the context stream.  Submit
// returns the frame's ticket; after Wait(ticket) its host results are
// complete and its host soup may be rewritten.  Host buffers must be
// page-locked (PinnedBuffer).  Any output may be null when the pipeline was
// created without it.
class FramePipeline {
   public:
    FramePipeline(Context& ctx, unsigned int numPrimitives, const rt_camera& camera, const float light[3],
                  unsigned int lbvhDepth = 20, bool visibility = true, bool mirror = true);
    ~FramePipeline();
    FramePipeline(const FramePipeline&) = delete;
    FramePipeline& operator=(const FramePipeline&) = delete;
    uint64_t Submit(const float* h_soup, rt_hit* h_primary, uint8_t* h_vis = nullptr, rt_hit* h_mirror = nullptr);
    void Wait(uint64_t ticket);

   private:
    Context& m_ctx;
    rt_lbvh* m_lbvh = nullptr;
    rt_pipe* m_pipe = nullptr;
};

}  // namespace rtgb
