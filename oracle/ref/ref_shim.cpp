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
#include <cstring>
#include <vector>
#include <chrono>
#include "LBVH.h"
#include "bvh.h"

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

}  // extern "C"
