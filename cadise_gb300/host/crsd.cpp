// CRSD scene description loader (host C++17) behind include/cadise_crsd.h.
//
// Format (as the reference reads it, source/file-io/scene-description/):
//   * '#' starts a comment running to the end of the line (sdParser.cpp:37-61);
//   * the text is cut into blocks at every '}' (sdParser.cpp:25-32); a block's
//     class is the word before its '{' (tokenizer.cpp:18-27);
//   * a block holds units "[name type \"value\"]" (tokenizer.cpp:29-114) with
//     types bool, real, int32, rgb, vector3r, string, material, texture,
//     primitive, real-array and vector3r-array ("x y z, x y z, ...");
//   * lookups return the first unit with the name (sdData.h:93-106).
// Objects are assembled in file order like RenderDatabase::setUpData
// (source/core/renderDatabase.cpp:39-76): textures and materials before the
// primitives that use them, lights after their primitive.
#include "../../include/cadise_crsd.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace {

struct Unit {
    std::string name, type, value;
};

struct Block {
    std::string cls;
    std::vector<Unit> units;

    const Unit* find(const std::string& n) const {
        for (const Unit& u : units)
            if (u.name == n) return &u;
        return nullptr;
    }
};

struct LoadError {
    cgpu_status status;
    std::string msg;
};

[[noreturn]] void fail(cgpu_status s, const std::string& m) { throw LoadError{s, m}; }

// std::stold then narrowing, as the reference parses numbers (tokenizer.cpp:139-145)
float to_real(const std::string& s) {
    char* end = nullptr;
    const long double v = std::strtold(s.c_str(), &end);
    if (end == s.c_str()) fail(CGPU_ERR_PARSE, "not a number: '" + s + "'");
    return static_cast<float>(v);
}

std::vector<std::string> split_ws(const std::string& s) {
    std::vector<std::string> out;
    std::istringstream is(s);
    std::string tok;
    while (is >> tok) out.push_back(tok);
    return out;
}

struct V3f {
    float x = 0, y = 0, z = 0;
};

V3f to_vec3(const std::string& s) {
    const auto t = split_ws(s);
    if (t.size() != 3) fail(CGPU_ERR_PARSE, "expected 3 components: '" + s + "'");
    return V3f{to_real(t[0]), to_real(t[1]), to_real(t[2])};
}

// "x y z, x y z, ..." (tokenizer.cpp:204-246); parsed in one pass.
void to_vec3_array(const std::string& s, std::vector<float>* out) {
    const char* p = s.c_str();
    const char* e = p + s.size();
    int k = 0;
    while (p < e) {
        while (p < e && (*p == ' ' || *p == ',' || *p == '\n' || *p == '\t' || *p == '\r')) ++p;
        if (p >= e) break;
        char* end = nullptr;
        const long double v = std::strtold(p, &end);
        if (end == p) fail(CGPU_ERR_PARSE, "bad number in vector3r-array");
        out->push_back(static_cast<float>(v));
        ++k;
        p = end;
    }
    if (k % 3 != 0) fail(CGPU_ERR_PARSE, "vector3r-array length is not a multiple of 3");
}

std::vector<Block> tokenize(const std::string& raw) {
    // strip comments
    std::string text;
    text.reserve(raw.size());
    for (size_t i = 0; i < raw.size(); ++i) {
        if (raw[i] == '#') {
            while (i < raw.size() && raw[i] != '\n') ++i;
            if (i < raw.size()) text.push_back('\n');
        } else {
            text.push_back(raw[i]);
        }
    }
    std::vector<Block> blocks;
    size_t start = 0;
    for (;;) {
        const size_t end = text.find('}', start);
        if (end == std::string::npos) break;
        const std::string chunk = text.substr(start, end - start + 1);
        start = end + 1;
        const size_t brace = chunk.find('{');
        if (brace == std::string::npos) fail(CGPU_ERR_PARSE, "block without '{'");
        // class name: last alphabetic word before '{'
        size_t a = 0;
        while (a < brace && !std::isalpha(static_cast<unsigned char>(chunk[a]))) ++a;
        size_t b = brace;
        while (b > a && !std::isalpha(static_cast<unsigned char>(chunk[b - 1]))) --b;
        Block blk;
        blk.cls = chunk.substr(a, b - a);
        size_t pos = brace;
        for (;;) {
            const size_t ob = chunk.find('[', pos);
            if (ob == std::string::npos) break;
            const size_t cb = chunk.find(']', ob);
            if (cb == std::string::npos) fail(CGPU_ERR_PARSE, "unterminated '[' in block " + blk.cls);
            const std::string body = chunk.substr(ob + 1, cb - ob - 1);
            pos = cb + 1;
            const size_t q0 = body.find('"');
            const size_t q1 = body.rfind('"');
            if (q0 == std::string::npos || q1 == q0) fail(CGPU_ERR_PARSE, "unit without a quoted value in " + blk.cls);
            const auto head = split_ws(body.substr(0, q0));
            if (head.size() != 2) fail(CGPU_ERR_PARSE, "unit needs 'name type': [" + body + "]");
            blk.units.push_back(Unit{head[0], head[1], body.substr(q0 + 1, q1 - q0 - 1)});
        }
        blocks.push_back(std::move(blk));
    }
    return blocks;
}

float find_real(const Block& b, const char* n, float def) {
    const Unit* u = b.find(n);
    return u ? to_real(u->value) : def;
}
int find_int(const Block& b, const char* n, int def) {
    const Unit* u = b.find(n);
    return u ? static_cast<int>(std::stoll(u->value)) : def;
}
bool find_bool(const Block& b, const char* n, bool def) {
    const Unit* u = b.find(n);
    return u ? u->value == "true" : def;
}
std::string find_str(const Block& b, const char* n, const std::string& def) {
    const Unit* u = b.find(n);
    return u ? u->value : def;
}
V3f find_vec3(const Block& b, const char* n, V3f def) {
    const Unit* u = b.find(n);
    return u ? to_vec3(u->value) : def;
}

// Little PFM reader ("PF" colour, scale < 0 little endian, rows bottom to top).
bool read_pfm(const std::string& path, int* w, int* h, std::vector<float>* rgb) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::string magic;
    float scale = 0;
    f >> magic >> *w >> *h >> scale;
    f.get();
    if (magic != "PF" || *w <= 0 || *h <= 0) return false;
    std::vector<float> raw(size_t(*w) * *h * 3);
    f.read(reinterpret_cast<char*>(raw.data()), std::streamsize(raw.size() * 4));
    if (!f) return false;
    // rows in file order: a PFM stores the picture's bottom row first, and
    // row 0 is v = 0, the bottom row, as the reference lays pictures out
    // (file-io/pictureLoader.cpp flips them vertically on load)
    *rgb = std::move(raw);
    return true;
}

}  // namespace

struct cgpu_crsd_scene {
    cgpu_scene_desc desc{};
    cgpu_crsd_settings settings{};
    std::vector<int32_t> kind, material;
    std::vector<float> vertices, normals, uvws;
    bool any_normals = false, any_uvws = false;
    std::vector<cgpu_material> materials;
    std::vector<cgpu_area_light> lights;
    std::vector<cgpu_texture> textures;
    std::vector<std::vector<float>> texels;
    std::map<std::string, int> prim_names, mat_names, spectrum_tex, real_tex;
    std::map<std::string, float> real_const;
    std::string base_dir;

    int default_material() {
        // the reference falls back to LambertianDiffuse() with albedo 0.5 (lambertianDiffuse.cpp:16-18)
        auto it = mat_names.find("<default lambertian>");
        if (it != mat_names.end()) return it->second;
        cgpu_material m{};
        m.type = CGPU_BSDF_LAMBERTIAN;
        m.albedo_texture = -1;
        m.albedo[0] = m.albedo[1] = m.albedo[2] = 0.5f;
        m.ior_outer = 1.0f;
        m.ior_inner = 1.5f;
        materials.push_back(m);
        return mat_names["<default lambertian>"] = int(materials.size()) - 1;
    }

    void add_prim(int k, const float* v9, int mat, const float* n9, const float* uv9) {
        kind.push_back(k);
        material.push_back(mat);
        vertices.insert(vertices.end(), v9, v9 + 9);
        static const float zero9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        static const float uv_default[9] = {0, 0, 0, 1, 0, 0, 0, 1, 0};
        normals.insert(normals.end(), n9 ? n9 : zero9, (n9 ? n9 : zero9) + 9);
        uvws.insert(uvws.end(), uv9 ? uv9 : uv_default, (uv9 ? uv9 : uv_default) + 9);
    }

    void albedo_of(const Block& b, const char* key, cgpu_material* m) {
        const Unit* u = b.find(key);
        m->albedo_texture = -1;
        m->albedo[0] = m->albedo[1] = m->albedo[2] = 0.0f;  // SdData default Spectrum(0)
        if (!u) return;
        if (u->type == "texture") {
            auto it = spectrum_tex.find(u->value);
            if (it == spectrum_tex.end()) fail(CGPU_ERR_NOT_FOUND, "unknown texture '" + u->value + "'");
            const cgpu_texture& t = textures[size_t(it->second)];
            if (t.width == 1 && t.height == 1) {  // constant texture block
                const float* c = texels[size_t(it->second)].data();
                m->albedo[0] = c[0]; m->albedo[1] = c[1]; m->albedo[2] = c[2];
            } else {
                m->albedo_texture = it->second;
            }
        } else {
            const V3f c = to_vec3(u->value);
            m->albedo[0] = c.x; m->albedo[1] = c.y; m->albedo[2] = c.z;
        }
    }

    float roughness_of(const Block& b) {
        const Unit* u = b.find("roughness");
        if (!u) return 0.0f;
        if (u->type == "texture") {
            auto it = real_const.find(u->value);
            if (it == real_const.end()) fail(CGPU_ERR_UNSUPPORTED, "roughness texture '" + u->value + "' is not constant");
            return it->second;
        }
        return to_real(u->value);
    }

    void material_block(const Block& b) {
        const std::string type = find_str(b, "type", "");
        cgpu_material m{};
        m.albedo_texture = -1;
        m.ior_outer = 1.0f;
        m.ior_inner = 1.5f;
        m.f0[0] = m.f0[1] = m.f0[2] = 1.0f;
        if (type == "matte-lambertian") {
            m.type = CGPU_BSDF_LAMBERTIAN;
            albedo_of(b, "albedo", &m);
        } else if (type == "conductor-microfacet") {
            m.type = CGPU_BSDF_CONDUCTOR_GGX;
            const std::string mf = find_str(b, "microfacet-type", "ggx");
            if (mf != "ggx") fail(CGPU_ERR_UNSUPPORTED, "conductor microfacet '" + mf + "' (only ggx)");
            const V3f f0 = find_vec3(b, "f0", V3f{1, 1, 1});
            m.f0[0] = f0.x; m.f0[1] = f0.y; m.f0[2] = f0.z;
            m.roughness = roughness_of(b);
        } else if (type == "glass" || type == "dielectric-microfacet") {
            m.type = type == "glass" ? CGPU_BSDF_GLASS : CGPU_BSDF_DIELECTRIC_GGX;
            albedo_of(b, "albedo", &m);
            m.ior_outer = find_real(b, "ior-outer", 1.0f);
            m.ior_inner = find_real(b, "ior-inner", 1.5f);
            m.roughness = roughness_of(b);
        } else if (type == "absorb") {
            m.type = CGPU_BSDF_ABSORBER;
        } else if (type == "mirror") {  // bsdfInstantiator.cpp:38-64
            m.type = CGPU_BSDF_MIRROR;
            albedo_of(b, "albedo", &m);
            const std::string fr = find_str(b, "fresnel-type", "conductor");
            if (fr == "conductor") {
                m.fresnel = CGPU_FRESNEL_CONDUCTOR;
                const V3f f0 = find_vec3(b, "f0", V3f{1, 1, 1});
                m.f0[0] = f0.x; m.f0[1] = f0.y; m.f0[2] = f0.z;
            } else if (fr == "dielectric") {
                m.fresnel = CGPU_FRESNEL_DIELECTRIC;
                m.ior_outer = find_real(b, "ior-outer", 1.0f);
                m.ior_inner = find_real(b, "ior-inner", 1.5f);
            } else {
                fail(CGPU_ERR_UNSUPPORTED, "mirror fresnel type '" + fr + "'");
            }
        } else if (type == "phong") {  // bsdfInstantiator.cpp:94-102
            m.type = CGPU_BSDF_PHONG;
            m.exponent = find_real(b, "exponent", 32.0f);
        } else if (type == "plastic") {  // bsdfInstantiator.cpp:104-116
            m.type = CGPU_BSDF_PLASTIC;
            albedo_of(b, "diffuse-albedo", &m);
            m.exponent = find_real(b, "specular-exponent", 32.0f);
            m.diffuse_ratio = find_real(b, "diffuse-ratio", 0.7f);
        } else {
            fail(CGPU_ERR_UNSUPPORTED, "material type '" + type + "'");
        }
        materials.push_back(m);
        mat_names.emplace(find_str(b, "name", ""), int(materials.size()) - 1);
    }

    void texture_block(const Block& b, bool spectrum) {
        const std::string type = find_str(b, "type", "");
        const std::string name = find_str(b, "name", "");
        if (!spectrum) {
            if (type != "constant") fail(CGPU_ERR_UNSUPPORTED, "real texture type '" + type + "'");
            real_const.emplace(name, find_real(b, "value", 0.0f));
            return;
        }
        cgpu_texture t{};
        std::vector<float> px;
        if (type == "constant") {
            const V3f c = find_vec3(b, "value", V3f{});
            px = {c.x, c.y, c.z};
            t.width = t.height = 1;
        } else if (type == "image") {
            std::string fn = find_str(b, "filename", "");
            if (!fn.empty() && fn[0] != '/') fn = base_dir + fn;
            if (!read_pfm(fn, &t.width, &t.height, &px))
                fail(CGPU_ERR_UNSUPPORTED, "image texture '" + fn + "' (PFM RGB float images only)");
            const std::string wrap = find_str(b, "wrap-mode", "repeat");
            if (wrap == "clamp") fail(CGPU_ERR_UNSUPPORTED, "clamp wrap mode");
        } else {
            fail(CGPU_ERR_UNSUPPORTED, "spectrum texture type '" + type + "'");
        }
        texels.push_back(std::move(px));
        textures.push_back(t);
        spectrum_tex.emplace(name, int(textures.size()) - 1);
    }

    void read_f32_file(const std::string& name, std::vector<float>* out) {
        const std::string fn = (!name.empty() && name[0] != '/') ? base_dir + name : name;
        std::ifstream f(fn, std::ios::binary | std::ios::ate);
        if (!f) fail(CGPU_ERR_NOT_FOUND, "cannot open mesh sidecar " + fn);
        const std::streamsize n = f.tellg();
        if (n % 36 != 0) fail(CGPU_ERR_PARSE, "mesh sidecar " + fn + " is not whole float32 triangles");
        out->resize(size_t(n) / 4);
        f.seekg(0);
        f.read(reinterpret_cast<char*>(out->data()), n);
        if (!f) fail(CGPU_ERR_PARSE, "short read of mesh sidecar " + fn);
    }

    int material_for(const Block& b, bool required) {
        const std::string n = find_str(b, "bsdf", "");
        auto it = mat_names.find(n);
        if (it != mat_names.end()) return it->second;
        if (required) fail(CGPU_ERR_NOT_FOUND, "unknown material '" + n + "'");
        return default_material();
    }

    void primitive_block(const Block& b) {
        const std::string type = find_str(b, "type", "");
        const std::string name = find_str(b, "name", "");
        const int first = int(kind.size());
        if (type == "triangle" || type == "rectangle") {
            const V3f v1 = find_vec3(b, "v1", V3f{}), v2 = find_vec3(b, "v2", V3f{}), v3 = find_vec3(b, "v3", V3f{});
            const float v[9] = {v1.x, v1.y, v1.z, v2.x, v2.y, v2.z, v3.x, v3.y, v3.z};
            add_prim(type == "triangle" ? CGPU_PRIM_TRIANGLE : CGPU_PRIM_RECTANGLE, v,
                     material_for(b, type == "triangle"), nullptr, nullptr);
        } else if (type == "triangle-mesh") {
            std::vector<float> pos, nrm, uvw;
            if (const Unit* u = b.find("positions")) to_vec3_array(u->value, &pos);
            if (const Unit* u = b.find("normals")) to_vec3_array(u->value, &nrm);
            if (const Unit* u = b.find("uvws")) to_vec3_array(u->value, &uvw);
            // binary sidecars: raw little-endian float32, 3 per vertex, 3 vertices per triangle
            if (const Unit* u = b.find("positions-file")) read_f32_file(u->value, &pos);
            if (const Unit* u = b.find("normals-file")) read_f32_file(u->value, &nrm);
            if (const Unit* u = b.find("uvws-file")) read_f32_file(u->value, &uvw);
            if (pos.size() % 9 != 0) fail(CGPU_ERR_PARSE, "triangle-mesh positions are not whole triangles");
            const size_t nt = pos.size() / 9;
            if (!nrm.empty() && nrm.size() != pos.size()) fail(CGPU_ERR_PARSE, "triangle-mesh normals size");
            if (!uvw.empty() && uvw.size() != pos.size()) fail(CGPU_ERR_PARSE, "triangle-mesh uvws size");
            const int mat = material_for(b, false);
            any_normals |= !nrm.empty();
            any_uvws |= !uvw.empty();
            for (size_t t = 0; t < nt; ++t)
                add_prim(CGPU_PRIM_TRIANGLE, &pos[9 * t], mat, nrm.empty() ? nullptr : &nrm[9 * t],
                         uvw.empty() ? nullptr : &uvw[9 * t]);
        } else if (type == "sphere") {  // primitiveInstantiator.cpp:17-28
            const V3f c = find_vec3(b, "center", V3f{});
            const float v[9] = {c.x, c.y, c.z, find_real(b, "radius", 0.0f), 0, 0, 0, 0, 0};
            add_prim(CGPU_PRIM_SPHERE, v, material_for(b, false), nullptr, nullptr);
        } else {
            fail(CGPU_ERR_UNSUPPORTED, "primitive type '" + type + "'");
        }
        if (int(kind.size()) > first) prim_names.emplace(name, first);  // std::map::insert keeps the first
    }

    int env_texture = 0;

    void light_block(const Block& b) {
        const std::string type = find_str(b, "type", "");
        if (type == "environment") {  // lightInstantiator.cpp:60-82 (PFM images here)
            std::string fn = find_str(b, "hdr-filename", "");
            if (!fn.empty() && fn[0] != '/') fn = base_dir + fn;
            cgpu_texture t{};
            std::vector<float> px;
            if (!read_pfm(fn, &t.width, &t.height, &px))
                fail(CGPU_ERR_UNSUPPORTED, "environment map '" + fn + "' (PFM RGB float images only)");
            texels.push_back(std::move(px));
            textures.push_back(t);
            env_texture = int(textures.size());
            return;
        }
        if (type != "area") fail(CGPU_ERR_UNSUPPORTED, "light type '" + type + "'");
        const std::string pn = find_str(b, "primitive", "");
        auto it = prim_names.find(pn);
        if (it == prim_names.end()) fail(CGPU_ERR_NOT_FOUND, "light on unknown primitive '" + pn + "'");
        cgpu_area_light l{};
        l.primitive = it->second;
        const V3f c = find_vec3(b, "color", V3f{});
        l.color[0] = c.x; l.color[1] = c.y; l.color[2] = c.z;
        l.watt = find_real(b, "watt", 0.0f);
        l.back_face_emit = find_bool(b, "is-back-face-emit", false) ? 1 : 0;
        lights.push_back(l);
    }

    void load(const std::string& text) {
        const std::vector<Block> blocks = tokenize(text);
        const Block *film = nullptr, *camera = nullptr, *renderer = nullptr, *cluster = nullptr, *accel = nullptr;
        for (const Block& b : blocks) {
            if (b.cls == "film") film = &b;
            else if (b.cls == "camera") camera = &b;
            else if (b.cls == "renderer") renderer = &b;
            else if (b.cls == "accelerator") accel = &b;
            else if (b.cls == "light-cluster") cluster = &b;
            else if (b.cls == "texture-real") texture_block(b, false);
            else if (b.cls == "texture-spectrum") texture_block(b, true);
            else if (b.cls == "material") material_block(b);
            else if (b.cls == "primitive") primitive_block(b);
            else if (b.cls == "light") light_block(b);
        }
        if (!film || !camera || !renderer) fail(CGPU_ERR_PARSE, "scene needs film, camera and renderer blocks");
        const std::string cluster_type = cluster ? find_str(*cluster, "type", "uniform") : "uniform";
        if (cluster_type == "power") desc.light_cluster = CGPU_LIGHT_CLUSTER_POWER;
        else if (cluster_type == "uniform") desc.light_cluster = CGPU_LIGHT_CLUSTER_UNIFORM;
        else fail(CGPU_ERR_UNSUPPORTED, "light cluster '" + cluster_type + "' (uniform or power)");
        if (accel) {
            const std::string t = find_str(*accel, "type", "bvh");
            if (t != "bvh" && t != "bruteForce" && t != "kd-tree") fail(CGPU_ERR_UNSUPPORTED, "accelerator '" + t + "'");
        }
        {
            // filterInstantiator.cpp:16-57 (defaults), filmInstantiator.cpp:22-23 (tile size)
            const std::string ft = find_str(*film, "filter", "box");
            cgpu_film_filter& f = desc.filter;
            const float size_default = ft == "box" ? 1.0f : 4.0f;
            if (ft == "box") f.type = CGPU_FILTER_BOX;
            else if (ft == "gaussian") f.type = CGPU_FILTER_GAUSSIAN;
            else if (ft == "mitchell") f.type = CGPU_FILTER_MITCHELL;
            else if (ft == "cone") f.type = CGPU_FILTER_CONE;
            else fail(CGPU_ERR_UNSUPPORTED, "film filter '" + ft + "'");
            f.width = find_real(*film, "filter-width", size_default);
            f.height = find_real(*film, "filter-height", size_default);
            f.sigma_x = find_real(*film, "sigma-x", 0.5f);
            f.sigma_y = find_real(*film, "sigma-y", 0.5f);
            f.amplitude = find_real(*film, "amplitude", 1.0f);
            f.b = find_real(*film, "b", 1.0f / 3.0f);
            f.c = find_real(*film, "c", 1.0f / 3.0f);
            f.tile_width = find_int(*film, "tile-size-x", 16);
            f.tile_height = find_int(*film, "tile-size-y", 16);
        }
        if (find_str(*camera, "type", "") != "perspective-pinhole") fail(CGPU_ERR_UNSUPPORTED, "camera type");
        desc.width = find_int(*film, "image-width", 1024);
        desc.height = find_int(*film, "image-height", 768);
        const V3f p = find_vec3(*camera, "position", V3f{}), d = find_vec3(*camera, "direction", V3f{}),
                  u = find_vec3(*camera, "up", V3f{});
        desc.cam_position[0] = p.x; desc.cam_position[1] = p.y; desc.cam_position[2] = p.z;
        desc.cam_direction[0] = d.x; desc.cam_direction[1] = d.y; desc.cam_direction[2] = d.z;
        desc.cam_up[0] = u.x; desc.cam_up[1] = u.y; desc.cam_up[2] = u.z;
        desc.fov_degrees = find_real(*camera, "fov", 0.0f);
        desc.sensor_width_mm = find_real(*camera, "sensor-width-mm", 36.0f);
        cgpu_crsd_settings& s = settings;
        std::snprintf(s.renderer_type, sizeof(s.renderer_type), "%s", find_str(*renderer, "type", "").c_str());
        std::snprintf(s.estimator, sizeof(s.estimator), "%s", find_str(*renderer, "estimator", "").c_str());
        std::snprintf(s.sampler, sizeof(s.sampler), "%s", find_str(*renderer, "sampler", "").c_str());
        std::snprintf(s.output_filename, sizeof(s.output_filename), "%s",
                      find_str(*film, "output-filename", "cadise.jpg").c_str());
        const std::string rt = s.renderer_type;
        if (rt != "sampling" && rt != "cuda-sampling") fail(CGPU_ERR_UNSUPPORTED, "renderer type '" + rt + "'");
        if (std::string(s.estimator) != "pt") fail(CGPU_ERR_UNSUPPORTED, "estimator '" + std::string(s.estimator) + "'");
        s.spp = find_int(*renderer, "sample-number", 4);
        s.max_depth = find_int(*renderer, "max-depth", 10000);
        const std::string mode = find_str(*renderer, "mode", "wavefront");
        if (mode != "wavefront" && mode != "megakernel") fail(CGPU_ERR_UNSUPPORTED, "mode '" + mode + "'");
        s.mode = mode == "megakernel" ? CGPU_MODE_MEGAKERNEL : CGPU_MODE_WAVEFRONT;
        s.use_graph = find_bool(*renderer, "graph", true) ? 1 : 0;
        s.seed = uint64_t(find_int(*renderer, "seed", 1));
        desc.max_depth = s.max_depth;
        desc.spp = s.spp;
        desc.num_primitives = uint32_t(kind.size());
        desc.prim_kind = kind.data();
        desc.prim_vertices = vertices.data();
        desc.prim_normals = any_normals ? normals.data() : nullptr;
        desc.prim_uvws = any_uvws ? uvws.data() : nullptr;
        desc.prim_material = material.data();
        desc.num_materials = uint32_t(materials.size());
        desc.materials = materials.data();
        for (size_t i = 0; i < textures.size(); ++i) textures[i].texels = texels[i].data();
        desc.num_textures = uint32_t(textures.size());
        desc.textures = textures.data();
        desc.num_lights = uint32_t(lights.size());
        desc.lights = lights.data();
        desc.environment_texture = env_texture;
    }
};

namespace {

cgpu_status load_common(const std::string& text, const std::string& base, cgpu_crsd_scene** out, char* err,
                        size_t err_len) {
    if (!out) return CGPU_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    auto sc = std::make_unique<cgpu_crsd_scene>();
    sc->base_dir = base;
    try {
        sc->load(text);
    } catch (const LoadError& e) {
        if (err && err_len) std::snprintf(err, err_len, "%s", e.msg.c_str());
        return e.status;
    } catch (const std::exception& e) {
        if (err && err_len) std::snprintf(err, err_len, "%s", e.what());
        return CGPU_ERR_PARSE;
    }
    *out = sc.release();
    return CGPU_OK;
}

}  // namespace

extern "C" {

cgpu_status cgpu_crsd_load_file(const char* path, cgpu_crsd_scene** out, char* err, size_t err_len) {
    if (!path) return CGPU_ERR_INVALID_ARGUMENT;
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        if (err && err_len) std::snprintf(err, err_len, "cannot open %s", path);
        return CGPU_ERR_NOT_FOUND;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    std::string p(path);
    const size_t slash = p.find_last_of('/');
    return load_common(ss.str(), slash == std::string::npos ? "" : p.substr(0, slash + 1), out, err, err_len);
}

cgpu_status cgpu_crsd_load_text(const char* text, size_t len, cgpu_crsd_scene** out, char* err, size_t err_len) {
    if (!text) return CGPU_ERR_INVALID_ARGUMENT;
    return load_common(std::string(text, len), "", out, err, err_len);
}

const cgpu_scene_desc* cgpu_crsd_desc(const cgpu_crsd_scene* s) { return s ? &s->desc : nullptr; }

cgpu_status cgpu_crsd_settings_get(const cgpu_crsd_scene* s, cgpu_crsd_settings* out) {
    if (!s || !out) return CGPU_ERR_INVALID_ARGUMENT;
    *out = s->settings;
    return CGPU_OK;
}

int32_t cgpu_crsd_primitive_index(const cgpu_crsd_scene* s, const char* name) {
    if (!s || !name) return -1;
    auto it = s->prim_names.find(name);
    return it == s->prim_names.end() ? -1 : it->second;
}

void cgpu_crsd_free(cgpu_crsd_scene* s) { delete s; }

}  // extern "C"
