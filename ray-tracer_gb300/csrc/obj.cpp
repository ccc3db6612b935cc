// Wavefront OBJ + MTL scene loading into the engine's scene description (host code, no GPU work).
//
// Reference: OBJ_Reader::loadMesh / loadMaterial (OBJ_Reader.cpp:60-389, 395-470), which reads one "o"
// object at a time: "v", "vn", "vt" records, triangle faces "f a/b/c ..." with 1-based indices into the
// file's running vertex lists, the object's "usemtl" material, and from the MTL file the Kd, Ks and Ns
// of that material over defaults of 0.75 grey and shininess 100. Kept alike: the records read, the
// index base, the defaults. Differences, each for a reason:
//   - faces with more than 3 vertices are triangulated as a fan (the reference reads the first 3 only);
//   - negative (relative) indices are accepted (OBJ allows them; the reference does not);
//   - a face without vertex normals gets its geometric normal on all three vertices (the reference stores
//     zero normals, which the shading stage cannot normalise);
//   - "g" starts a new object like "o"; texture coordinates are parsed and dropped (no textures here).
// Materials get reflectance 0.5 (the MTL format has no mirror weight; the reference halves the colour of
// a reflection, RayTracer.cu:627).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "engine.h"

namespace {

struct ObjOut {
    rsh_obj_data pub;
    std::vector<float> pos, nrm;
    std::vector<uint32_t> mat, obj;
    std::vector<rsh_material> mats;
};

rsh_material default_material() {
    rsh_material m;
    for (int i = 0; i < 3; ++i) {
        m.diffuse[i] = 0.75f;
        m.specular[i] = 0.75f;
    }
    m.diffuse[3] = 0.5f;
    m.specular[3] = 100.0f;
    return m;
}

std::string dir_of(const std::string& path) {
    const size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

// Splits a line into whitespace-separated tokens; '#' starts a comment.
std::vector<std::string> tokens(const std::string& line) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i < line.size()) {
        while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == '\r')) ++i;
        if (i >= line.size() || line[i] == '#') break;
        size_t j = i;
        while (j < line.size() && line[j] != ' ' && line[j] != '\t' && line[j] != '\r') ++j;
        out.push_back(line.substr(i, j - i));
        i = j;
    }
    return out;
}

bool read_lines(const std::string& path, std::vector<std::string>& lines) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::string cur;
    char buf[65536];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) {
        for (size_t i = 0; i < n; ++i) {
            if (buf[i] == '\n') {
                lines.push_back(cur);
                cur.clear();
            } else {
                cur.push_back(buf[i]);
            }
        }
    }
    if (!cur.empty()) lines.push_back(cur);
    std::fclose(f);
    return true;
}

bool parse_float(const std::string& s, float& v) {
    char* end = nullptr;
    v = std::strtof(s.c_str(), &end);
    return end && *end == '\0' && std::isfinite(v);
}

// "Kd r g b" style values; returns false on a malformed record.
bool floats3(const std::vector<std::string>& t, float out[3]) {
    if (t.size() < 4) return false;
    for (int i = 0; i < 3; ++i)
        if (!parse_float(t[1 + i], out[i])) return false;
    return true;
}

// MTL file: newmtl, Kd, Ks, Ns (OBJ_Reader.cpp:395-470); names map to material indices.
bool load_mtl(const std::string& path, std::vector<rsh_material>& mats, std::map<std::string, uint32_t>& names) {
    std::vector<std::string> lines;
    if (!read_lines(path, lines)) return false;
    int cur = -1;
    for (const std::string& ln : lines) {
        const std::vector<std::string> t = tokens(ln);
        if (t.empty()) continue;
        if (t[0] == "newmtl" && t.size() >= 2) {
            auto it = names.find(t[1]);
            if (it == names.end()) {
                names[t[1]] = (uint32_t)mats.size();
                cur = (int)mats.size();
                mats.push_back(default_material());
            } else {
                cur = (int)it->second;
            }
        } else if (cur >= 0) {
            float v[3];
            if (t[0] == "Kd" && floats3(t, v)) {
                for (int i = 0; i < 3; ++i) mats[cur].diffuse[i] = v[i];
            } else if (t[0] == "Ks" && floats3(t, v)) {
                for (int i = 0; i < 3; ++i) mats[cur].specular[i] = v[i];
            } else if (t[0] == "Ns" && t.size() >= 2) {
                float ns;
                if (parse_float(t[1], ns)) mats[cur].specular[3] = ns;
            }
        }
    }
    return true;
}

// One face corner "v", "v/vt", "v//vn" or "v/vt/vn" -> 0-based position and normal indices (-1: none).
bool corner(const std::string& s, size_t nv, size_t nn, long& vi, long& ni) {
    long idx[3] = {0, 0, 0};
    int k = 0;
    size_t i = 0;
    while (k < 3) {
        size_t j = s.find('/', i);
        const std::string part = s.substr(i, j == std::string::npos ? std::string::npos : j - i);
        if (!part.empty()) {
            char* end = nullptr;
            idx[k] = std::strtol(part.c_str(), &end, 10);
            if (!end || *end != '\0' || idx[k] == 0) return false;
        }
        ++k;
        if (j == std::string::npos) break;
        i = j + 1;
    }
    auto resolve = [](long v, size_t n) -> long { return v > 0 ? v - 1 : (long)n + v; };
    vi = resolve(idx[0], nv);
    if (idx[0] == 0 || vi < 0 || (size_t)vi >= nv) return false;
    ni = -1;
    if (idx[2] != 0) {
        ni = resolve(idx[2], nn);
        if (ni < 0 || (size_t)ni >= nn) return false;
    }
    return true;
}

}  // namespace

extern "C" {

rsh_status rsh_obj_load(const char* obj_path, rsh_obj_data** out) {
    if (!obj_path || !out) return RSH_ERR_INVALID;
    *out = nullptr;
    std::vector<std::string> lines;
    if (!read_lines(obj_path, lines)) {
        rsh::set_error(std::string("rsh_obj_load: cannot read ") + obj_path);
        return RSH_ERR_INVALID;
    }
    ObjOut* o = new ObjOut();
    std::map<std::string, uint32_t> names;
    o->mats.push_back(default_material());  // material 0: faces before any known usemtl
    std::vector<float> v, vn;
    uint32_t cur_mat = 0, cur_obj = 0;
    bool any_face_in_obj = false;
    const std::string dir = dir_of(obj_path);
    size_t line_no = 0;
    bool ok = true;
    for (const std::string& ln : lines) {
        ++line_no;
        const std::vector<std::string> t = tokens(ln);
        if (t.empty()) continue;
        float q[3];
        if (t[0] == "v") {
            ok = floats3(t, q);
            if (ok) v.insert(v.end(), q, q + 3);
        } else if (t[0] == "vn") {
            ok = floats3(t, q);
            if (ok) vn.insert(vn.end(), q, q + 3);
        } else if (t[0] == "o" || t[0] == "g") {
            if (any_face_in_obj) ++cur_obj;
            any_face_in_obj = false;
        } else if (t[0] == "mtllib" && t.size() >= 2) {
            for (size_t k = 1; k < t.size(); ++k) load_mtl(dir + t[k], o->mats, names);  // named: 1, 2, ...
        } else if (t[0] == "usemtl" && t.size() >= 2) {
            auto it = names.find(t[1]);
            cur_mat = (it == names.end()) ? 0u : it->second;
        } else if (t[0] == "f") {
            ok = t.size() >= 4;
            std::vector<long> vi(t.size() > 1 ? t.size() - 1 : 0), ni(vi.size());
            for (size_t k = 1; ok && k < t.size(); ++k)
                ok = corner(t[k], v.size() / 3, vn.size() / 3, vi[k - 1], ni[k - 1]);
            for (size_t k = 1; ok && k + 1 < vi.size(); ++k) {  // fan: (0, k, k+1)
                const long c[3] = {vi[0], vi[k], vi[k + 1]};
                const long cn[3] = {ni[0], ni[k], ni[k + 1]};
                float p[3][3];
                for (int a = 0; a < 3; ++a)
                    for (int i = 0; i < 3; ++i) p[a][i] = v[3 * c[a] + i];
                for (int a = 0; a < 3; ++a) o->pos.insert(o->pos.end(), {p[a][0], p[a][1], p[a][2], 1.0f});
                const bool have_n = cn[0] >= 0 && cn[1] >= 0 && cn[2] >= 0;
                float fn[3] = {0.f, 0.f, 0.f};
                if (!have_n) {  // geometric normal (e1 x e2)
                    const float e1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
                    const float e2[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
                    fn[0] = e1[1] * e2[2] - e1[2] * e2[1];
                    fn[1] = e1[2] * e2[0] - e1[0] * e2[2];
                    fn[2] = e1[0] * e2[1] - e1[1] * e2[0];
                }
                for (int a = 0; a < 3; ++a) {
                    if (have_n)
                        o->nrm.insert(o->nrm.end(), {vn[3 * cn[a]], vn[3 * cn[a] + 1], vn[3 * cn[a] + 2], 0.0f});
                    else
                        o->nrm.insert(o->nrm.end(), {fn[0], fn[1], fn[2], 0.0f});
                }
                o->mat.push_back(cur_mat);
                o->obj.push_back(cur_obj);
            }
            any_face_in_obj = true;
        }
        if (!ok) break;
    }
    if (!ok) {
        rsh::set_error("rsh_obj_load: malformed record at " + std::string(obj_path) + ":" + std::to_string(line_no));
        delete o;
        return RSH_ERR_INVALID;
    }
    rsh_obj_data& d = o->pub;
    std::memset(&d, 0, sizeof d);
    d.desc.positions = o->pos.data();
    d.desc.normals = o->nrm.data();
    d.desc.material_ids = o->mat.data();
    d.desc.object_ids = o->obj.data();
    d.desc.materials = o->mats.data();
    d.desc.triangle_count = (uint32_t)o->mat.size();
    d.desc.material_count = (uint32_t)o->mats.size();
    d.object_count = o->obj.empty() ? 0u : o->obj.back() + 1u;
    d.owner = o;
    *out = &d;
    return RSH_OK;
}

void rsh_obj_free(rsh_obj_data* data) {
    if (data) delete static_cast<ObjOut*>(data->owner);
}

}  // extern "C"
