// ObjLoader.cpp — see ObjLoader.hpp.
#include "ObjLoader.hpp"

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>

namespace Foundation {
namespace Renderer {
namespace {

// A malformed or unreadable file: std::runtime_error with the formatted
// message (the exception the reference's constructors throw on failures,
// src/Platform/RHI/Vulkan/Device.cpp:195,203).
[[noreturn]] void IoFail(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw std::runtime_error(buf);
}

std::string DirOf(const std::string& p) {
    const size_t s = p.find_last_of('/');
    return s == std::string::npos ? std::string() : p.substr(0, s + 1);
}

fnd_material DefaultMaterial() {
    fnd_material m{};
    m.type = FND_MAT_LAMBERT;
    m.albedo[0] = m.albedo[1] = m.albedo[2] = 0.8f;
    m.roughness = 1.0f;
    m.light = -1;
    return m;
}

void LoadMtl(const std::string& path, std::map<std::string, uint32_t>& names, std::vector<fnd_material>& mats) {
    std::ifstream in(path);
    if (!in) IoFail("cannot open material library %s", path.c_str());
    std::string line;
    fnd_material* cur = nullptr;
    bool metallic = false;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::string key;
        if (!(ss >> key) || key[0] == '#') continue;
        if (key == "newmtl") {
            std::string name;
            ss >> name;
            names[name] = (uint32_t)mats.size();
            mats.push_back(DefaultMaterial());
            cur = &mats.back();
            metallic = false;
            continue;
        }
        if (!cur) continue;
        if (key == "Kd") {
            ss >> cur->albedo[0] >> cur->albedo[1] >> cur->albedo[2];
        } else if (key == "Ks" && metallic) {
            ss >> cur->albedo[0] >> cur->albedo[1] >> cur->albedo[2];
        } else if (key == "Pm") {
            float m = 0.0f;
            ss >> m;
            metallic = m > 0.0f;
            if (metallic && cur->type != FND_MAT_EMISSIVE) cur->type = FND_MAT_GGX;
        } else if (key == "Pr") {
            ss >> cur->roughness;
        } else if (key == "Ke") {
            ss >> cur->emission[0] >> cur->emission[1] >> cur->emission[2];
            if (cur->emission[0] > 0 || cur->emission[1] > 0 || cur->emission[2] > 0) cur->type = FND_MAT_EMISSIVE;
        }
    }
}

int64_t ParseIndex(const std::string& tok, int64_t nverts) {
    const int64_t v = std::strtoll(tok.c_str(), nullptr, 10);  // stops at the first '/'
    if (v > 0) return v - 1;
    if (v < 0) return nverts + v;
    return -1;
}

}  // namespace

ObjScene LoadObj(const std::string& path) {
    std::ifstream in(path);
    if (!in) IoFail("cannot open %s", path.c_str());
    ObjScene s;
    std::map<std::string, uint32_t> names;
    uint32_t current = 0;
    bool have_default = false;
    std::string line;
    size_t lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        std::istringstream ss(line);
        std::string key;
        if (!(ss >> key)) continue;
        if (key == "#fnd") {
            std::string what;
            ss >> what;
            if (what == "quad_light") {
                fnd_quad_light q{};
                ss >> q.corner[0] >> q.corner[1] >> q.corner[2] >> q.edge_u[0] >> q.edge_u[1] >> q.edge_u[2] >>
                    q.edge_v[0] >> q.edge_v[1] >> q.edge_v[2] >> q.radiance[0] >> q.radiance[1] >> q.radiance[2];
                if (!ss) IoFail("%s:%zu: malformed quad_light", path.c_str(), lineno);
                s.lights.push_back(q);
            }
            continue;
        }
        if (key[0] == '#') continue;
        if (key == "v") {
            float x, y, z;
            if (!(ss >> x >> y >> z)) IoFail("%s:%zu: malformed vertex", path.c_str(), lineno);
            s.verts.insert(s.verts.end(), {x, y, z});
        } else if (key == "f") {
            std::vector<int64_t> poly;
            std::string tok;
            const int64_t nv = (int64_t)(s.verts.size() / 3);
            while (ss >> tok) {
                const int64_t i = ParseIndex(tok, nv);
                if (i < 0 || i >= nv) IoFail("%s:%zu: face index out of range", path.c_str(), lineno);
                poly.push_back(i);
            }
            if (poly.size() < 3) IoFail("%s:%zu: face with fewer than 3 vertices", path.c_str(), lineno);
            if (s.materials.empty()) {
                s.materials.push_back(DefaultMaterial());
                have_default = true;
            }
            for (size_t k = 1; k + 1 < poly.size(); ++k) {
                s.indices.insert(s.indices.end(), {(uint32_t)poly[0], (uint32_t)poly[k], (uint32_t)poly[k + 1]});
                s.tri_material.push_back(current);
            }
        } else if (key == "mtllib") {
            std::string file;
            ss >> file;
            if (s.materials.empty()) {
                LoadMtl(DirOf(path) + file, names, s.materials);
            } else {
                std::vector<fnd_material> more;
                std::map<std::string, uint32_t> more_names;
                LoadMtl(DirOf(path) + file, more_names, more);
                for (auto& [n, i] : more_names) names[n] = i + (uint32_t)s.materials.size();
                s.materials.insert(s.materials.end(), more.begin(), more.end());
            }
        } else if (key == "usemtl") {
            std::string name;
            ss >> name;
            auto it = names.find(name);
            if (it == names.end()) IoFail("%s:%zu: unknown material %s", path.c_str(), lineno, name.c_str());
            current = it->second;
        }
    }
    (void)have_default;
    if (s.materials.empty()) s.materials.push_back(DefaultMaterial());
    // the k-th emissive material is tied to the k-th quad light
    int32_t k = 0;
    for (auto& m : s.materials)
        if (m.type == FND_MAT_EMISSIVE) m.light = k < (int32_t)s.lights.size() ? k++ : -1;
    return s;
}

}  // namespace Renderer
}  // namespace Foundation
