// rt_model.cpp -- headless model ingestion (see include/rt_model.h).
//
// The OBJ rules follow the loader the reference uses
// (Common/Scenes/Loaders/model_obj.cpp: importGeometryFirstPass :793-920,
// importGeometrySecondPass :922-1117, importMaterials :1119-1298, bounds
// :77-128, normalize :228-256) as Model::LoadFile drives it
// (Common/Scenes/Model.cpp:266-381), and the scaling follows Model::Scale
// (Model.cpp:647-709).  A model yields the triangle soup the reference's Model
// hands to its acceleration structure bit for bit: the same fp32 operations
// in the same order (the library is compiled with -ffp-contract=off).
//
// Reading is token driven like the reference's loader: a record is chosen by
// the first character of a whitespace-delimited token, and the rest of a
// line is skipped with a 256-byte fgets, so odd files read the same way too.
// Where the reference would index out of range (a face corner that names no
// vertex, a .txt index past the vertex count) this loader reports an error.
#include "rt_model.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

struct rt_model {
    std::vector<float> soup;
    std::vector<int32_t> material_ids;
    std::vector<rt_material> materials;
};

namespace {

constexpr int kLine = 256;  // the reference loader's line / token buffer

struct File {
    FILE* f;
    explicit File(const std::string& path) : f(fopen(path.c_str(), "r")) {}
    ~File() {
        if (f) fclose(f);
    }
    File(const File&) = delete;
    File& operator=(const File&) = delete;
};

bool next_token(FILE* f, char* tok) { return fscanf(f, "%255s", tok) == 1; }

void skip_rest(FILE* f) {
    char line[kLine];
    if (!fgets(line, kLine, f)) return;
}

// Scans with a result the loader ignores: a field that does not parse keeps
// its earlier value.
template <typename... T>
void scan(FILE* f, const char* fmt, T*... out) {
    if (fscanf(f, fmt, out...) < 0) return;
}

// The name argument of mtllib / usemtl / newmtl: the rest of the line is read
// with fgets and scanned as "%s %s" into the buffer it came from, so the
// result is the second word when the line has two, else the first; at end of
// file the buffer still holds the record's own token.
std::string name_arg(FILE* f, const char* tok) {
    char line[kLine];
    if (!fgets(line, kLine, f)) return std::string(tok);
    char w1[kLine] = {0}, w2[kLine] = {0};
    const int got = sscanf(line, "%255s %255s", w1, w2);
    if (got >= 2) return std::string(w2);
    if (got == 1) return std::string(w1);
    return std::string(line);
}

rt_material default_material() {
    rt_material m;
    const float a[4] = {0.2f, 0.2f, 0.2f, 1.0f}, d[4] = {0.8f, 0.8f, 0.8f, 1.0f}, s[4] = {0.0f, 0.0f, 0.0f, 1.0f};
    memcpy(m.ambient, a, sizeof(a));
    memcpy(m.diffuse, d, sizeof(d));
    memcpy(m.specular, s, sizeof(s));
    m.shininess = 0.0f;
    m.alpha = 1.0f;
    return m;
}

struct Materials {
    std::vector<rt_material> mats;
    std::vector<std::string> names;
    std::map<std::string, int> cache;  // name -> index, kept across MTL files
    int count = 0;                     // materials of the last MTL file read
};

// One MTL file (importMaterials): a counting pass over newmtl records, then
// the records themselves, chosen by their first character.  Records before
// the first newmtl are consumed and dropped.
void read_mtl(const std::string& path, Materials& M) {
    File file(path);
    if (!file.f) return;
    FILE* f = file.f;
    char tok[kLine];
    int n = 0;
    while (next_token(f, tok)) {
        if (tok[0] == 'n') ++n;
        skip_rest(f);
    }
    rewind(f);
    M.count = n;
    M.mats.resize(n, rt_material{});
    M.names.resize(n);
    int cur = -1, loaded = 0, illum = 0;
    while (next_token(f, tok)) {
        rt_material* m = cur >= 0 ? &M.mats[cur] : nullptr;
        float scratch[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        switch (tok[0]) {
            case 'N':
                if (tok[1] == 's') {  // Ns in [0, 1000] -> [0, 1]
                    float* dst = m ? &m->shininess : &scratch[0];
                    scan(f, "%f", dst);
                    *dst /= 1000.0f;
                }
                break;
            case 'K': {
                float* dst = nullptr;
                if (tok[1] == 'a') dst = m ? m->ambient : scratch;
                else if (tok[1] == 'd') dst = m ? m->diffuse : scratch;
                else if (tok[1] == 's') dst = m ? m->specular : scratch;
                char line[kLine];
                if (!fgets(line, kLine, f)) snprintf(line, kLine, "%s", tok);
                if (dst && sscanf(line, "%f %f %f %f", &dst[0], &dst[1], &dst[2], &dst[3]) < 4) dst[3] = 1.0f;
                break;
            }
            case 'T':
                if (tok[1] == 'r') {  // transparency
                    float* dst = m ? &m->alpha : &scratch[0];
                    scan(f, "%f", dst);
                    *dst = 1.0f - *dst;
                } else {
                    skip_rest(f);
                }
                break;
            case 'd':
                scan(f, "%f", m ? &m->alpha : &scratch[0]);
                break;
            case 'i':
                scan(f, "%d", &illum);
                if (illum == 1 && m) {  // no specular highlight
                    m->specular[0] = m->specular[1] = m->specular[2] = 0.0f;
                    m->specular[3] = 1.0f;
                }
                break;
            case 'n': {
                const std::string name = name_arg(f, tok);
                if (loaded >= n) break;  // the counting pass saw fewer
                cur = loaded++;
                M.mats[cur] = default_material();
                M.names[cur] = name;
                M.cache[name] = cur;
                break;
            }
            default:  // map_Kd / map_bump (textures are not used) and the rest
                skip_rest(f);
                break;
        }
    }
}

// A face corner in one of the four OBJ forms.
enum class Form { V, VT, VN, VTN };

int read_corner(FILE* f, Form form, int* v) {
    int vt = 0, vn = 0;
    switch (form) {
        case Form::VN: return fscanf(f, "%d//%d", v, &vn);
        case Form::VTN: return fscanf(f, "%d/%d/%d", v, &vt, &vn);
        case Form::VT: return fscanf(f, "%d/%d", v, &vt);
        default: return fscanf(f, "%d", v);
    }
}

Form face_form(const char* first, int* v0) {
    int b = 0, c = 0;
    if (strstr(first, "//")) {
        sscanf(first, "%d//%d", v0, &b);
        return Form::VN;
    }
    if (sscanf(first, "%d/%d/%d", v0, &b, &c) == 3) return Form::VTN;
    if (sscanf(first, "%d/%d", v0, &b) == 2) return Form::VT;
    sscanf(first, "%d", v0);
    return Form::V;
}

// A face corner as the second pass sees it: the vertex index after the
// loader's rule (positive k -> k - 1, negative k -> k + count - 1 with count
// the v records read so far), and whether that record had been read (a later
// one still holds zeros in the loader's coordinate array).
struct Corner {
    int idx;
    bool read;
};

// Reads one face: the fan (v0, v1, v2), (v0, v2, v3), ...  `count` is the
// number of v records before it.  Without `out` the corners are consumed only.
void read_face(FILE* f, int count, std::vector<Corner>* out) {
    char first[kLine];
    if (!next_token(f, first)) return;
    int v[3] = {0, 0, 0};
    const Form form = face_form(first, &v[0]);
    read_corner(f, form, &v[1]);
    read_corner(f, form, &v[2]);
    auto corner = [count](int k) {
        const int idx = k < 0 ? k + count - 1 : k - 1;
        return Corner{idx, idx < count};
    };
    const Corner c0 = corner(v[0]);
    Corner c1 = corner(v[1]), c2 = corner(v[2]);
    for (;;) {
        if (out) {
            out->push_back(c0);
            out->push_back(c1);
            out->push_back(c2);
        }
        int next = 0;
        if (read_corner(f, form, &next) <= 0) break;
        c1 = c2;
        c2 = corner(next);
    }
}

std::string directory_of(const std::string& path) {
    size_t cut = path.find_last_of('\\');
    if (cut == std::string::npos) cut = path.find_last_of('/');
    return cut == std::string::npos ? std::string() : path.substr(0, cut + 1);
}

// Model::Scale's two steps over `verts` (x y z per vertex): shift by the box
// centre and scale by s1 into the 0.9 half-size box, then by s2 into the
// 0.49 sphere.
void scale_params(const float* verts, size_t nv, float shift[3], float* s1, float* s2) {
    float mn[3] = {verts[0], verts[1], verts[2]}, mx[3] = {verts[0], verts[1], verts[2]};
    for (size_t i = 1; i < nv; ++i)
        for (int c = 0; c < 3; ++c) {
            const float x = verts[3 * i + c];
            if (x < mn[c]) mn[c] = x;
            if (x > mx[c]) mx[c] = x;
        }
    for (int c = 0; c < 3; ++c) mx[c] = mx[c] - mn[c];
    *s1 = 1.8f / std::max(mx[0], std::max(mx[1], mx[2]));
    for (int c = 0; c < 3; ++c) shift[c] = mn[c] + 0.5f * mx[c];
    float r2 = 0.0f;
    for (size_t i = 0; i < nv; ++i) {
        const float x = *s1 * (verts[3 * i] - shift[0]);
        const float y = *s1 * (verts[3 * i + 1] - shift[1]);
        const float z = *s1 * (verts[3 * i + 2] - shift[2]);
        const float l = x * x + y * y + z * z;
        if (l > r2) r2 = l;
    }
    *s2 = 0.49f / sqrtf(r2);
}

void apply_scale(std::vector<float>& soup, const float shift[3], float s1, float s2) {
    for (size_t k = 0; k < soup.size(); ++k) {
        const int c = (int)(k % 3);
        soup[k] = (s1 * (soup[k] - shift[c])) * s2;
    }
}

bool load_obj(const std::string& path, rt_model& m, std::string& err) {
    File file(path);
    if (!file.f) {
        err = "cannot open " + path;
        return false;
    }
    FILE* f = file.f;
    const std::string dir = directory_of(path);
    Materials M;
    char tok[kLine];
    int total_v = 0;
    // first pass: MTL files and the number of v records
    while (next_token(f, tok)) {
        switch (tok[0]) {
            case 'f': read_face(f, 0, nullptr); break;
            case 'm': read_mtl(dir + name_arg(f, tok), M); break;
            case 'v':
                if (tok[1] == '\0' || tok[1] == 'n' || tok[1] == 't') skip_rest(f);
                if (tok[1] == '\0') ++total_v;
                break;
            default: skip_rest(f); break;
        }
    }
    if (M.count == 0) {
        M.mats.assign(1, default_material());
        M.names.assign(1, "default");
        M.cache["default"] = 0;
    }
    rewind(f);
    // second pass: coordinates, faces, usemtl
    std::vector<float> coords(size_t(total_v) * 3, 0.0f);
    std::vector<Corner> corners;
    std::vector<int> tri_mat;
    int nread = 0, active = 0;
    while (next_token(f, tok)) {
        switch (tok[0]) {
            case 'f':
                read_face(f, nread, &corners);
                tri_mat.resize(corners.size() / 3, active);
                break;
            case 'u': {
                const auto it = M.cache.find(name_arg(f, tok));
                active = it == M.cache.end() ? 0 : it->second;
                break;
            }
            case 'v':
                if (tok[1] == '\0') {
                    if (nread >= total_v) {
                        err = "vertex records differ between passes in " + path;
                        return false;
                    }
                    float* p = &coords[3 * size_t(nread)];
                    scan(f, "%f %f %f", &p[0], &p[1], &p[2]);
                    ++nread;
                } else if (tok[1] == 'n') {
                    float n3[3];
                    scan(f, "%f %f %f", &n3[0], &n3[1], &n3[2]);
                } else if (tok[1] == 't') {
                    float t2[2];
                    scan(f, "%f %f", &t2[0], &t2[1]);
                }
                break;
            default: skip_rest(f); break;
        }
    }
    if (corners.empty()) {
        err = "no faces in " + path;
        return false;
    }
    for (const Corner& c : corners)
        if (c.idx < 0 || c.idx >= total_v) {
            err = "face corner names no vertex in " + path;
            return false;
        }
    for (int id : tri_mat)
        if (id < 0 || id >= (int)M.mats.size()) {
            err = "material index out of range in " + path;
            return false;
        }
    // corner positions (the loader's vertex buffer holds exactly these values)
    const size_t nc = corners.size();
    std::vector<float> pos(nc * 3);
    for (size_t i = 0; i < nc; ++i)
        for (int c = 0; c < 3; ++c) pos[3 * i + c] = corners[i].read ? coords[3 * size_t(corners[i].idx) + c] : 0.0f;
    // normalize(): bounds (max starting at FLT_MIN, as the loader's does), the
    // centre moved to the origin, the largest extent scaled to 1
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {FLT_MIN, FLT_MIN, FLT_MIN};
    for (size_t i = 0; i < nc; ++i)
        for (int c = 0; c < 3; ++c) {
            const float x = pos[3 * i + c];
            if (x < mn[c]) mn[c] = x;
            if (x > mx[c]) mx[c] = x;
        }
    float offset[3], ext[3];
    for (int c = 0; c < 3; ++c) {
        offset[c] = -((mn[c] + mx[c]) / 2.0f);
        ext[c] = mx[c] - mn[c];
    }
    const float factor = 1.0f / std::max(std::max(ext[0], ext[1]), ext[2]);
    for (size_t k = 0; k < pos.size(); ++k) {
        float x = pos[k];
        x += offset[k % 3];
        x *= factor;
        pos[k] = x;
    }
    // Model::Scale over the same vertices
    float shift[3], s1, s2;
    scale_params(pos.data(), nc, shift, &s1, &s2);
    apply_scale(pos, shift, s1, s2);
    m.soup.swap(pos);
    const size_t nt = nc / 3;
    m.material_ids.assign(nt, 0);
    if (M.count > 1)  // per mesh: the cache's index for the mesh material's name
        for (size_t t = 0; t < nt; ++t) m.material_ids[t] = M.cache[M.names[tri_mat[t]]];
    m.materials = M.mats;
    return true;
}

bool load_txt(const std::string& path, rt_model& m, std::string& err) {
    File file(path);
    if (!file.f) {
        err = "cannot open " + path;
        return false;
    }
    FILE* f = file.f;
    int nv = 0, nt = 0;
    if (fscanf(f, "%d", &nv) != 1 || fscanf(f, "%d", &nt) != 1 || nv <= 0 || nt <= 0) {
        err = "bad header in " + path;
        return false;
    }
    std::vector<float> verts(size_t(nv) * 3);
    for (int i = 0; i < nv; ++i) {
        float p[8];
        if (fscanf(f, "%f %f %f %f %f %f %f %f", &p[0], &p[1], &p[2], &p[3], &p[4], &p[5], &p[6], &p[7]) != 8) {
            err = "bad vertex record in " + path;
            return false;
        }
        verts[3 * size_t(i)] = p[0];
        verts[3 * size_t(i) + 1] = p[1];
        verts[3 * size_t(i) + 2] = p[2];
    }
    m.soup.resize(size_t(nt) * 9);
    for (int t = 0; t < nt; ++t) {
        int idx[3];
        if (fscanf(f, "%d %d %d", &idx[0], &idx[1], &idx[2]) != 3) {
            err = "bad triangle record in " + path;
            return false;
        }
        for (int k = 0; k < 3; ++k) {
            if (idx[k] < 0 || idx[k] >= nv) {
                err = "triangle index out of range in " + path;
                return false;
            }
            for (int c = 0; c < 3; ++c) m.soup[9 * size_t(t) + 3 * k + c] = verts[3 * size_t(idx[k]) + c];
        }
    }
    // Model::Scale over every vertex of the file
    float shift[3], s1, s2;
    scale_params(verts.data(), size_t(nv), shift, &s1, &s2);
    apply_scale(m.soup, shift, s1, s2);
    m.material_ids.assign(size_t(nt), 0);
    m.materials.assign(1, default_material());
    return true;
}

}  // namespace

extern "C" rt_status rt_model_load(const char* path, rt_model** out, char* err, size_t errlen) {
    if (err && errlen) err[0] = '\0';
    if (!path || !out) return RT_ERR_INVALID;
    *out = nullptr;
    rt_model* m = new rt_model();
    std::string e;
    const std::string p(path);
    bool ok = false;
    // Model::LoadFile's format test: ".txt" / ".TXT" anywhere in the name
    // first, then ".obj" / ".OBJ"
    if (strstr(path, ".txt") || strstr(path, ".TXT")) ok = load_txt(p, *m, e);
    else if (strstr(path, ".obj") || strstr(path, ".OBJ")) ok = load_obj(p, *m, e);
    else e = "unknown model format: " + p;
    if (!ok) {
        if (err && errlen) snprintf(err, errlen, "%s", e.c_str());
        delete m;
        return RT_ERR_INVALID;
    }
    *out = m;
    return RT_OK;
}

extern "C" void rt_model_free(rt_model* m) { delete m; }
extern "C" uint32_t rt_model_triangle_count(const rt_model* m) { return m ? (uint32_t)(m->soup.size() / 9) : 0u; }
extern "C" const float* rt_model_soup(const rt_model* m) { return m ? m->soup.data() : nullptr; }
extern "C" const int32_t* rt_model_material_ids(const rt_model* m) { return m ? m->material_ids.data() : nullptr; }
extern "C" uint32_t rt_model_material_count(const rt_model* m) { return m ? (uint32_t)m->materials.size() : 0u; }
extern "C" const rt_material* rt_model_material(const rt_model* m, uint32_t i) {
    return (m && i < m->materials.size()) ? &m->materials[i] : nullptr;
}
