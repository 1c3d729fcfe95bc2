// Test-oracle shim around the reference's own CPU acceleration structures.
//
// This file is compiled together with the unmodified reference sources
//   AccelerationStructures/LBVH/LBVH.cpp   (LBVH::Build, LBVH::IntersectP)
//   AccelerationStructures/BVH/bvh.cpp     (PBRT SAH BVH, CPU baseline)
//   AccelerationStructures/AccelerationStructure.cpp
//   Common/Scenes/Primitive.cpp, Common/Memory.cpp
// by oracle/ref/build_ref.sh into oracle/_ref/libref.so.  It only adapts a
// flat triangle soup (n x 9 floats) to the reference's Vertex/Primitive
// objects and exposes plain C entry points for the parity tests and the CPU
// baseline.  Nothing here is used by the GPU product path.
#include <cstdio>
#include <cmath>
#include <algorithm>
#include <cstring>
#include <vector>
#include <chrono>
#include "LBVH.h"
#include "bvh.h"
#include "model_obj.h"
#include "model_scale_stub.h"

namespace {

struct Scene {
    std::vector<Vertex> verts;
    std::vector<Primitive*> prims;
    explicit Scene(const float* soup, int n) : verts(size_t(n) * 3) {
        for (int i = 0; i < n * 3; ++i)
            verts[i] = Vertex(soup[3 * i + 0], soup[3 * i + 1], soup[3 * i + 2]);
        prims.resize(n);
        for (int i = 0; i < n; ++i)
            prims[i] = new Primitive(&verts[3 * i], &verts[3 * i + 1], &verts[3 * i + 2]);
    }
    ~Scene() { for (Primitive* p : prims) delete p; }
};

struct Handle {
    Scene scene;
    AccelerationStructure* as;
    Handle(const float* soup, int n) : scene(soup, n), as(nullptr) {}
    ~Handle() { delete as; }
};

// Silence the reference's progress printf()s while a build runs.
struct QuietStdout {
    FILE* saved = nullptr;
    QuietStdout() { fflush(stdout); saved = stdout; stdout = fopen("/dev/null", "w"); if (!stdout) stdout = saved; }
    ~QuietStdout() { if (stdout != saved) { fclose(stdout); stdout = saved; } }
};

}  // namespace

extern "C" {

// bsf/bsr were MSVC inline assembly in LBVH.cpp:1577-1578; the build recipe
// turns those two definitions into declarations and they are defined here.
}
int bsf(const int x) { return __builtin_ctz((unsigned)x); }
int bsr(const int x) { return 31 - __builtin_clz((unsigned)x); }

extern "C" {

// Reference LBVH (LBVH.cpp:467-632).  depth -> 1<<depth heap slots.
void* ref_lbvh_create(const float* soup, int n, int depth, int quiet, double* build_seconds) {
    Handle* h = new Handle(soup, n);
    LBVH* l = new LBVH(h->scene.prims.data(), (unsigned)n, 1 << depth);
    h->as = l;
    auto t0 = std::chrono::steady_clock::now();
    if (quiet) { QuietStdout q; h->as->Build(); } else { h->as->Build(); }
    auto t1 = std::chrono::steady_clock::now();
    if (build_seconds) *build_seconds = std::chrono::duration<double>(t1 - t0).count();
    return h;
}

// Reference PBRT-derived BVH (bvh.cpp), SAH, maxPrims primitives per leaf.
void* ref_bvh_create(const float* soup, int n, int max_prims, int quiet, double* build_seconds) {
    Handle* h = new Handle(soup, n);
    h->as = new BVH(h->scene.prims.data(), (unsigned)n, (uint32_t)max_prims, "sah");
    auto t0 = std::chrono::steady_clock::now();
    if (quiet) { QuietStdout q; h->as->Build(); } else { h->as->Build(); }
    auto t1 = std::chrono::steady_clock::now();
    if (build_seconds) *build_seconds = std::chrono::duration<double>(t1 - t0).count();
    return h;
}

void ref_destroy(void* hp) { delete static_cast<Handle*>(hp); }

unsigned ref_num_elements(void* hp) { return static_cast<Handle*>(hp)->as->GetNumberOfElements(); }
unsigned ref_element_size(void* hp) { return (unsigned)static_cast<Handle*>(hp)->as->GetSizeOfElement(); }

void ref_copy_elements(void* hp, void* out) {
    Handle* h = static_cast<Handle*>(hp);
    memcpy(out, h->as->GetPtrToElements(), size_t(h->as->GetNumberOfElements()) * h->as->GetSizeOfElement());
}

void ref_copy_ids(void* hp, unsigned* out) {
    Handle* h = static_cast<Handle*>(hp);
    memcpy(out, h->as->GetOrderedElementsIds(), sizeof(unsigned) * h->as->GetNumPrimitives());
}

void ref_world_bound(void* hp, float* out6) {
    BBox b = static_cast<Handle*>(hp)->as->WorldBound();
    out6[0] = b.pMin.x; out6[1] = b.pMin.y; out6[2] = b.pMin.z;
    out6[3] = b.pMax.x; out6[4] = b.pMax.y; out6[5] = b.pMax.z;
}

// Closest hit through the reference's own IntersectP for each ray.
// rays: n x 8 floats {ox,oy,oz, dx,dy,dz, tmax, exclude_id(as float)}.
// Outputs id / t / u / v per ray.  OpenMP over rays (IntersectP only reads
// the tree; each ray is a private Ray object).
void ref_intersect(void* hp, const float* rays, long n, int* id, float* t, float* u, float* v, int nthreads) {
    Handle* h = static_cast<Handle*>(hp);
    AccelerationStructure* as = h->as;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
    for (long i = 0; i < n; ++i) {
        const float* r = rays + 8 * i;
        Ray ray(Point(r[0], r[1], r[2]), Vector(r[3], r[4], r[5]), 0.f, r[6]);
        ray.TriangleID = (int)r[7];
        TIntersection hit = as->IntersectP(ray);
        id[i] = hit.IDTr;
        t[i] = hit.t; u[i] = hit.u; v[i] = hit.v;
    }
}

// Model ingestion: the reference's vendored OBJ loader
// (Common/Scenes/Loaders/model_obj.cpp: ModelOBJ::import + normalize(), as
// Model::LoadFile calls them, Model.cpp:266-274) followed by the reference's
// own Model::Scale (Model.cpp:647-710, compiled against
// shim/model_scale_stub.h) on the loader's vertex buffer.  Output: the
// triangle soup (ntris x 9 floats) in index-buffer order and the material id
// of each triangle (its mesh's material, Model.cpp:355-372).  Two calls:
// ref_obj_load / ref_txt_load return the triangle count (or -1), then
// ref_obj_fetch copies the result.
static std::vector<float> g_obj_soup;
static std::vector<int> g_obj_mat;
static std::vector<float> g_obj_materials;  // 14 floats per material

// Model::Scale on x y z triples, through a Model holding them as Vertex.
static void reference_scale(std::vector<float>& pos) {
    const int nv = int(pos.size() / 3);
    std::vector<Vertex> v(nv);
    for (int i = 0; i < nv; ++i) v[i] = Vertex(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    Model model;
    model.m_pVertices = v.data();
    model.m_uiNumVertices = unsigned(nv);
    model.Scale();
    for (int i = 0; i < nv; ++i) {
        pos[3 * i] = v[i].Pos.x;
        pos[3 * i + 1] = v[i].Pos.y;
        pos[3 * i + 2] = v[i].Pos.z;
    }
}

int ref_obj_load(const char* path) {
    ModelOBJ m;
    if (!m.import(path)) return -1;
    m.normalize();
    const int nv = m.getNumberOfVertices(), nt = m.getNumberOfTriangles();
    std::vector<float> pos(size_t(nv) * 3);
    for (int i = 0; i < nv; ++i)
        for (int c = 0; c < 3; ++c) pos[3 * i + c] = m.getVertexBuffer()[i].position[c];
    reference_scale(pos);
    g_obj_soup.assign(size_t(nt) * 9, 0.0f);
    g_obj_mat.assign(size_t(nt), 0);
    const int* ib = m.getIndexBuffer();
    for (int t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) g_obj_soup[9 * size_t(t) + 3 * k + c] = pos[3 * ib[3 * t + k] + c];
    // the materials as the loader holds them (its default one when the file
    // names none): ambient, diffuse, specular (4 each), shininess, alpha
    const int nm = std::max(1, m.getNumberOfMaterials());
    g_obj_materials.assign(size_t(nm) * 14, 0.0f);
    for (int i = 0; i < nm; ++i) {
        const ModelOBJ::Material& mt = m.getMaterial(i);
        float* o = &g_obj_materials[14 * size_t(i)];
        for (int c = 0; c < 4; ++c) {
            o[c] = mt.ambient[c];
            o[4 + c] = mt.diffuse[c];
            o[8 + c] = mt.specular[c];
        }
        o[12] = mt.shininess;
        o[13] = mt.alpha;
    }
    if (m.getNumberOfMaterials() > 1) {
        for (int i = 0; i < m.getNumberOfMeshes(); ++i) {
            const ModelOBJ::Mesh& mesh = m.getMesh(i);
            const int id = m.getMaterialCache()[mesh.pMaterial->name];
            for (int j = 0; j < mesh.triangleCount; ++j) g_obj_mat[mesh.startIndex / 3 + j] = id;
        }
    }
    return nt;
}

void ref_obj_fetch(float* soup, int* material) {
    memcpy(soup, g_obj_soup.data(), sizeof(float) * g_obj_soup.size());
    memcpy(material, g_obj_mat.data(), sizeof(int) * g_obj_mat.size());
}

// The .txt branch of Model::LoadFile (Model.cpp:215-262) restated for
// positions: vertex count, triangle count, 8 floats per vertex (position,
// normal, u, v), 3 indices per triangle; then the reference's Model::Scale
// over every vertex.
int ref_txt_load(const char* path) {
    FILE* f = fopen(path, "r");
    if (!f) return -1;
    int nv = 0, nt = 0;
    if (fscanf(f, "%d", &nv) != 1 || fscanf(f, "%d", &nt) != 1 || nv <= 0 || nt <= 0) {
        fclose(f);
        return -1;
    }
    std::vector<float> pos(size_t(nv) * 3);
    for (int i = 0; i < nv; ++i) {
        float p[8];
        if (fscanf(f, "%f %f %f %f %f %f %f %f", &p[0], &p[1], &p[2], &p[3], &p[4], &p[5], &p[6], &p[7]) != 8) {
            fclose(f);
            return -1;
        }
        pos[3 * i] = p[0];
        pos[3 * i + 1] = p[1];
        pos[3 * i + 2] = p[2];
    }
    std::vector<int> idx(size_t(nt) * 3);
    for (int t = 0; t < nt; ++t)
        if (fscanf(f, "%d %d %d", &idx[3 * t], &idx[3 * t + 1], &idx[3 * t + 2]) != 3) {
            fclose(f);
            return -1;
        }
    fclose(f);
    for (int k : idx)
        if (k < 0 || k >= nv) return -1;
    reference_scale(pos);
    g_obj_soup.assign(size_t(nt) * 9, 0.0f);
    g_obj_mat.assign(size_t(nt), 0);
    for (int t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) g_obj_soup[9 * size_t(t) + 3 * k + c] = pos[3 * idx[3 * t + k] + c];
    g_obj_materials.assign(14, 0.0f);
    const float dflt[14] = {0.2f, 0.2f, 0.2f, 1.0f, 0.8f, 0.8f, 0.8f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 1.0f};
    memcpy(g_obj_materials.data(), dflt, sizeof(dflt));
    return nt;
}

int ref_obj_material_count() { return int(g_obj_materials.size() / 14); }

void ref_obj_fetch_materials(float* out) {
    memcpy(out, g_obj_materials.data(), sizeof(float) * g_obj_materials.size());
}

}  // extern "C"
