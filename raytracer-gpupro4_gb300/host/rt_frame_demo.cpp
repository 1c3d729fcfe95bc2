// rt_frame_demo -- drives the C++ stage classes the way the reference's main
// loop drives RayTracerCS (App.cpp:64-86): build the scene's LBVH through the
// AccelerationStructure interface, then render frames with the dynamic
// per-frame rebuild.  Used by the GPU tests to check the C++ layer against
// the Python binding of the same C ABI.
//
//   rt_frame_demo <soup.f32> <n> <camera.f32> <width> <height> <lx> <ly> <lz> <depth> <frames> <out_prefix>
//   rt_frame_demo <model.obj|model.txt> 0 <camera.f32> ...
//
// soup.f32: n x 9 float32, or a model file loaded through Model (Model::
// LoadFile + Model::Scale; n is then the model's triangle count);
// camera.f32: eye, right, up, fwd (3 floats each), tan(fovy/2).  Writes
// <out_prefix>.primary / .vis / .mirror (raw rt_hit / uint8 arrays of the
// last frame), the same frames streamed from pinned host memory through
// FramePipeline to <out_prefix>.pipe.primary / .pipe.vis / .pipe.mirror, the
// colour stage's accumulation image to <out_prefix>.color and a progressive
// GI image (4 samples in two calls) to <out_prefix>.gi, and prints one JSON
// summary line.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "rt_stages.h"

static std::vector<float> read_floats(const char* path, size_t count) {
    std::vector<float> v(count);
    FILE* f = std::fopen(path, "rb");
    if (!f || std::fread(v.data(), sizeof(float), count, f) != count) {
        std::fprintf(stderr, "cannot read %zu floats from %s\n", count, path);
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

template <typename T>
static void write_raw(const std::string& path, const std::vector<T>& v) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f || std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size()) {
        std::fprintf(stderr, "cannot write %s\n", path.c_str());
        std::exit(2);
    }
    std::fclose(f);
}

int main(int argc, char** argv) {
    if (argc != 12) {
        std::fprintf(stderr, "usage: %s soup n camera width height lx ly lz depth frames out_prefix\n", argv[0]);
        return 2;
    }
    unsigned n = (unsigned)std::strtoul(argv[2], nullptr, 10);
    std::vector<float> soup;
    const char* src = argv[1];
    if (std::strstr(src, ".obj") || std::strstr(src, ".OBJ") || std::strstr(src, ".txt") || std::strstr(src, ".TXT")) {
        try {
            rtgb::Model model(src);
            n = model.GetNumPrimitives();
            soup.assign(model.GetSoup(), model.GetSoup() + (size_t)n * 9);
        } catch (const rtgb::Error& e) {
            std::fprintf(stderr, "%s\n", e.what());
            return 2;
        }
    } else {
        soup = read_floats(src, (size_t)n * 9);
    }
    std::vector<float> c = read_floats(argv[3], 13);
    rt_camera cam;
    for (int k = 0; k < 3; ++k) {
        cam.eye[k] = c[k];
        cam.right[k] = c[3 + k];
        cam.up[k] = c[6 + k];
        cam.fwd[k] = c[9 + k];
    }
    cam.tan_half_fovy = c[12];
    cam.width = (uint32_t)std::atoi(argv[4]);
    cam.height = (uint32_t)std::atoi(argv[5]);
    const float light[3] = {std::strtof(argv[6], nullptr), std::strtof(argv[7], nullptr), std::strtof(argv[8], nullptr)};
    const unsigned depth = (unsigned)std::atoi(argv[9]);
    const int frames = std::atoi(argv[10]);
    const std::string out = argv[11];
    try {
        rtgb::Context ctx(0);
        // static path: Model::RebuildStructure -> LBVH::Build, then the
        // structure is handed to the renderer (RayTracerCS.cpp:590-624)
        rtgb::LBVHGpu lbvh(ctx, soup.data(), n, 1 << depth);
        auto t0 = std::chrono::steady_clock::now();
        lbvh.Build();
        ctx.Sync();
        float secs = std::chrono::duration<float>(std::chrono::steady_clock::now() - t0).count();
        rtgb::AccelerationStructure* as = &lbvh;
        const rtgb::LBVHNode* nodes = static_cast<const rtgb::LBVHNode*>(as->GetPtrToElements());
        rtgb::BBox wb = as->WorldBound();
        const bool bound_ok = wb.pMin.x == nodes[1].minCoord.x && wb.pMax.z == nodes[1].maxCoord.z;
        // one ray through the single-ray interface, towards the first triangle's centroid
        rtgb::Ray ray;
        ray.o = rtgb::Vector3{cam.eye[0], cam.eye[1], cam.eye[2]};
        const float cx = (soup[0] + soup[3] + soup[6]) / 3.f, cy = (soup[1] + soup[4] + soup[7]) / 3.f,
                    cz = (soup[2] + soup[5] + soup[8]) / 3.f;
        ray.d = rtgb::Vector3{cx - ray.o.x, cy - ray.o.y, cz - ray.o.z};
        rtgb::TIntersection hit = as->IntersectP(ray);

        // dynamic path: RayTracerCS::Render with the per-frame GPU rebuild
        rtgb::Scene scene;
        scene.soup = soup.data();
        scene.numPrimitives = n;
        rtgb::RayTracerCS rt(ctx, scene, cam, light, depth, true);
        auto t1 = std::chrono::steady_clock::now();
        for (int f = 0; f < frames; ++f) rt.Render();
        ctx.Check();
        float fsecs = std::chrono::duration<float>(std::chrono::steady_clock::now() - t1).count();
        std::vector<rt_hit> prim = rt.DownloadPrimary();
        std::vector<uint8_t> vis = rt.DownloadVisibility();
        std::vector<rt_hit> mir = rt.DownloadMirror();
        write_raw(out + ".primary", prim);
        write_raw(out + ".vis", vis);
        write_raw(out + ".mirror", mir);
        // the same frames with host data, pipelined (rt_pipe_*: two frames
        // in flight, host result buffers alternating); the last frame's
        // results go to <out_prefix>.pipe.primary / .pipe.vis / .pipe.mirror
        {
            const size_t px = (size_t)cam.width * cam.height;
            rtgb::FramePipeline pipe(ctx, n, cam, light, depth);
            rtgb::PinnedBuffer hsoup(sizeof(float) * 9 * (size_t)n);
            std::memcpy(hsoup.data(), soup.data(), sizeof(float) * 9 * (size_t)n);
            rtgb::PinnedBuffer hp[2] = {rtgb::PinnedBuffer(sizeof(rt_hit) * px), rtgb::PinnedBuffer(sizeof(rt_hit) * px)};
            rtgb::PinnedBuffer hv[2] = {rtgb::PinnedBuffer(px), rtgb::PinnedBuffer(px)};
            rtgb::PinnedBuffer hm[2] = {rtgb::PinnedBuffer(sizeof(rt_hit) * px), rtgb::PinnedBuffer(sizeof(rt_hit) * px)};
            uint64_t last = 0;
            for (int f = 0; f < frames; ++f) {
                if (f >= 2) pipe.Wait((uint64_t)(f - 2));
                last = pipe.Submit(static_cast<const float*>(hsoup.data()), static_cast<rt_hit*>(hp[f & 1].data()),
                                   static_cast<uint8_t*>(hv[f & 1].data()), static_cast<rt_hit*>(hm[f & 1].data()));
            }
            pipe.Wait(last);
            ctx.Check();
            const int q = (int)(last & 1u);
            const rt_hit* pp = static_cast<const rt_hit*>(hp[q].data());
            const uint8_t* pv = static_cast<const uint8_t*>(hv[q].data());
            const rt_hit* pm = static_cast<const rt_hit*>(hm[q].data());
            write_raw(out + ".pipe.primary", std::vector<rt_hit>(pp, pp + px));
            write_raw(out + ".pipe.vis", std::vector<uint8_t>(pv, pv + px));
            write_raw(out + ".pipe.mirror", std::vector<rt_hit>(pm, pm + px));
        }
        // the colour stage (one material, one bounce, shadows on) and four
        // progressive GI samples in two calls of two, through RayTracerCS;
        // written to <out_prefix>.color (accumulation) and <out_prefix>.gi
        {
            rt_material mat = {{1.5f, 0.f, 0.f, 0.f}, {0.7f, 0.4f, 0.2f, 1.f}, {0.5f, 0.5f, 0.5f, 1.f}, 0.049f, 0.6f};
            rt_shade_params sp = {1u, 1, 0, 0, -1, {0.2f, 0.3f, 0.4f}, 7u};
            rt.RenderColor(sp, &mat, 1);
            write_raw(out + ".color", rt.DownloadAccumulation());
            std::vector<float> albedo(3 * (size_t)n, 0.6f), emission(3 * (size_t)n, 0.f);
            for (size_t k = 0; k < std::min<size_t>(n, 64) * 3; ++k) emission[k] = 2.f;
            rt.SetGIMaterials(albedo.data(), emission.data());
            const float sky[3] = {1.f, 1.f, 1.f};
            rt.RenderGI(2, 2, 11, sky);
            rt.RenderGI(2, 2, 11, sky);
            ctx.Check();
            write_raw(out + ".gi", rt.DownloadGI());
        }
        size_t hits = 0, lit = 0;
        for (auto& h : prim) hits += h.id >= 0;
        for (auto v : vis) lit += v == 3;
        std::printf("{\"name\": \"%s\", \"n\": %u, \"depth\": %u, \"elements\": %u, \"element_size\": %zu, "
                    "\"build_s\": %.6f, \"world_bound_ok\": %s, \"single_ray_id\": %d, \"single_ray_t\": %.9g, "
                    "\"frames\": %d, \"frames_s\": %.6f, \"primary_hits\": %zu, \"lit\": %zu, \"samples\": %u}\n",
                    as->GetName(), n, depth, as->GetNumberOfElements(), as->GetSizeOfElement(), secs,
                    bound_ok ? "true" : "false", hit.IDTr, hit.t, frames, fsecs, hits, lit, rt.GetNumSamples());
    } catch (const rtgb::Error& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
