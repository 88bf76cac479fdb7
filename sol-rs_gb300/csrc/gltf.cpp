// gltf.cpp — glTF 2.0 scene input (solrt_gltf_*), the host side of
// load_scene (src/scene/mod.rs:138-295) for this path.
//
// A small JSON reader, base64 data URIs, external .bin buffers and .glb
// containers; accessors of float / normalised unsigned byte or short
// components; node matrices or translation-rotation-scale. Output: the same
// arrays solrt_scene_create takes (ModelVertex, u32 indices relative to each
// section, one section and one SceneInstance per primitive, MaterialInfo).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "../../include/solrt.h"

namespace solrt {
void set_error(const char* fmt, ...);
}

namespace {

// ---------------------------------------------------------------------------
// JSON
// ---------------------------------------------------------------------------

struct Json {
    enum Type { Null, Bool, Num, Str, Arr, Obj } type = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    const Json* get(const char* key) const {
        if (type != Obj) return nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    double number(const char* key, double def) const {
        const Json* v = get(key);
        return v && v->type == Num ? v->num : def;
    }
    size_t size() const { return type == Arr ? arr.size() : 0; }
};

struct JsonReader {
    const char* p;
    const char* end;
    bool ok = true;

    void ws() {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
    }
    bool lit(const char* s) {
        const size_t n = std::strlen(s);
        if ((size_t)(end - p) < n || std::strncmp(p, s, n) != 0) return false;
        p += n;
        return true;
    }
    void fail() { ok = false; }
    std::string string() {
        std::string s;
        if (p >= end || *p != '"') { fail(); return s; }
        ++p;
        while (p < end && *p != '"') {
            char c = *p++;
            if (c == '\\' && p < end) {
                const char e = *p++;
                switch (e) {
                    case 'n': s += '\n'; break;
                    case 't': s += '\t'; break;
                    case 'r': s += '\r'; break;
                    case 'b': s += '\b'; break;
                    case 'f': s += '\f'; break;
                    case 'u': {
                        if (end - p < 4) { fail(); return s; }
                        const unsigned cp = (unsigned)std::strtoul(std::string(p, 4).c_str(), nullptr, 16);
                        p += 4;
                        if (cp < 0x80) s += (char)cp;
                        else if (cp < 0x800) { s += (char)(0xC0 | (cp >> 6)); s += (char)(0x80 | (cp & 0x3F)); }
                        else { s += (char)(0xE0 | (cp >> 12)); s += (char)(0x80 | ((cp >> 6) & 0x3F)); s += (char)(0x80 | (cp & 0x3F)); }
                        break;
                    }
                    default: s += e;
                }
            } else {
                s += c;
            }
        }
        if (p >= end) { fail(); return s; }
        ++p;
        return s;
    }
    Json value(int depth = 0) {
        Json v;
        if (depth > 256) { fail(); return v; }
        ws();
        if (p >= end) { fail(); return v; }
        const char c = *p;
        if (c == '{') {
            v.type = Json::Obj;
            ++p;
            ws();
            if (p < end && *p == '}') { ++p; return v; }
            while (ok) {
                ws();
                std::string k = string();
                ws();
                if (p >= end || *p != ':') { fail(); break; }
                ++p;
                v.obj.emplace_back(std::move(k), value(depth + 1));
                ws();
                if (p < end && *p == ',') { ++p; continue; }
                if (p < end && *p == '}') { ++p; break; }
                fail();
            }
        } else if (c == '[') {
            v.type = Json::Arr;
            ++p;
            ws();
            if (p < end && *p == ']') { ++p; return v; }
            while (ok) {
                v.arr.push_back(value(depth + 1));
                ws();
                if (p < end && *p == ',') { ++p; continue; }
                if (p < end && *p == ']') { ++p; break; }
                fail();
            }
        } else if (c == '"') {
            v.type = Json::Str;
            v.str = string();
        } else if (lit("true")) {
            v.type = Json::Bool;
            v.b = true;
        } else if (lit("false")) {
            v.type = Json::Bool;
        } else if (lit("null")) {
            v.type = Json::Null;
        } else {
            char* e = nullptr;
            const std::string tok(p, std::min<size_t>((size_t)(end - p), 64));
            v.num = std::strtod(tok.c_str(), &e);
            if (e == tok.c_str()) { fail(); return v; }
            p += (e - tok.c_str());
            v.type = Json::Num;
        }
        return v;
    }
};

// ---------------------------------------------------------------------------
// buffers
// ---------------------------------------------------------------------------

bool read_file(const std::string& path, std::vector<unsigned char>& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    return true;
}

bool base64_decode(const std::string& s, std::vector<unsigned char>& out) {
    auto val = [](char c) -> int {
        if (c >= 'A' && c <= 'Z') return c - 'A';
        if (c >= 'a' && c <= 'z') return c - 'a' + 26;
        if (c >= '0' && c <= '9') return c - '0' + 52;
        if (c == '+' || c == '-') return 62;
        if (c == '/' || c == '_') return 63;
        return -1;
    };
    out.clear();
    unsigned acc = 0;
    int bits = 0;
    for (char c : s) {
        if (c == '=' || c == '\n' || c == '\r' || c == ' ') continue;
        const int v = val(c);
        if (v < 0) return false;
        acc = (acc << 6) | (unsigned)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((unsigned char)((acc >> bits) & 0xFF));
        }
    }
    return true;
}

std::string dir_of(const std::string& path) {
    const size_t k = path.find_last_of("/\\");
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

// ---------------------------------------------------------------------------
// matrices (column-major, as glTF and glam)
// ---------------------------------------------------------------------------

struct M4 {
    double m[16];
};

M4 identity() {
    M4 r{};
    r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0;
    return r;
}

M4 mul(const M4& a, const M4& b) {
    M4 r{};
    for (int c = 0; c < 4; ++c)
        for (int rr = 0; rr < 4; ++rr) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += a.m[k * 4 + rr] * b.m[c * 4 + k];
            r.m[c * 4 + rr] = s;
        }
    return r;
}

// node.transform().matrix(): the matrix, or T * R * S
M4 node_matrix(const Json& node) {
    if (const Json* mj = node.get("matrix")) {
        M4 r = identity();
        for (size_t i = 0; i < 16 && i < mj->size(); ++i) r.m[i] = mj->arr[i].num;
        return r;
    }
    double t[3] = {0, 0, 0}, q[4] = {0, 0, 0, 1}, s[3] = {1, 1, 1};
    if (const Json* tj = node.get("translation"))
        for (size_t i = 0; i < 3 && i < tj->size(); ++i) t[i] = tj->arr[i].num;
    if (const Json* rj = node.get("rotation"))
        for (size_t i = 0; i < 4 && i < rj->size(); ++i) q[i] = rj->arr[i].num;
    if (const Json* sj = node.get("scale"))
        for (size_t i = 0; i < 3 && i < sj->size(); ++i) s[i] = sj->arr[i].num;
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y + w * z), 2 * (x * z - w * y),
                         2 * (x * y - w * z), 1 - 2 * (x * x + z * z), 2 * (y * z + w * x),
                         2 * (x * z + w * y), 2 * (y * z - w * x), 1 - 2 * (x * x + y * y)};
    M4 r = identity();
    for (int c = 0; c < 3; ++c)
        for (int rr = 0; rr < 3; ++rr) r.m[c * 4 + rr] = R[c * 3 + rr] * s[c];
    r.m[12] = t[0];
    r.m[13] = t[1];
    r.m[14] = t[2];
    return r;
}

bool inverse_transpose(const M4& a, M4& out) {
    const double* m = a.m;
    double inv[16];
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    const double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    if (det == 0.0 || !std::isfinite(det)) return false;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out.m[c * 4 + r] = inv[r * 4 + c] / det;  // transpose of the inverse
    return true;
}

// DFS from `node` for the node holding mesh `mesh`, pushing node matrices;
// restates find_mesh (src/scene/mod.rs:106-122).
bool find_mesh(const Json& nodes, size_t node, size_t mesh, std::vector<M4>& stack, int depth) {
    if (depth > 64 || node >= nodes.size()) return false;
    const Json& n = nodes.arr[node];
    stack.push_back(node_matrix(n));
    const Json* m = n.get("mesh");
    if (m && m->type == Json::Num && (size_t)m->num == mesh) return true;
    if (const Json* ch = n.get("children"))
        for (const Json& c : ch->arr)
            if (c.type == Json::Num && find_mesh(nodes, (size_t)c.num, mesh, stack, depth + 1)) return true;
    stack.pop_back();
    return false;
}

}  // namespace

struct solrt_gltf {
    std::vector<solrt_vertex> vertices;
    std::vector<uint32_t> indices;
    std::vector<solrt_section> sections;
    std::vector<solrt_material> materials;
    std::vector<solrt_instance> instances;
    bool has_camera = false;
    float view[16];
    float yfov = 35.0f, znear = 0.1f, zfar = 100.0f;
};

namespace {

struct Loader {
    Json doc;
    std::vector<std::vector<unsigned char>> buffers;
    std::string err;

    bool fail(const std::string& e) {
        err = e;
        return false;
    }

    // All elements of an accessor as doubles, row-major (count x ncomp).
    // Integer components are scaled to [0, 1] (or [-1, 1]) when the accessor
    // is `normalized` or `to_unit` is set (colours and texture coordinates
    // read as into_rgba_f32 / into_f32); index accessors keep integers.
    bool accessor(size_t index, std::vector<double>& out, int& ncomp, size_t& count, bool to_unit = false) {
        const Json* accs = doc.get("accessors");
        if (!accs || index >= accs->size()) return fail("accessor out of range");
        const Json& a = accs->arr[index];
        if (a.get("sparse")) return fail("sparse accessors are not supported");
        const int ctype = (int)a.number("componentType", 0);
        count = (size_t)a.number("count", 0);
        const Json* tj = a.get("type");
        const std::string type = tj ? tj->str : "";
        ncomp = type == "SCALAR" ? 1 : type == "VEC2" ? 2 : type == "VEC3" ? 3 : type == "VEC4" ? 4 : 0;
        if (ncomp == 0) return fail("unsupported accessor type " + type);
        const Json* nj = a.get("normalized");
        const bool norm = to_unit || (nj && nj->type == Json::Bool && nj->b);
        int csize = 0;
        switch (ctype) {
            case 5120: case 5121: csize = 1; break;
            case 5122: case 5123: csize = 2; break;
            case 5125: case 5126: csize = 4; break;
            default: return fail("unsupported component type");
        }
        out.assign(count * ncomp, 0.0);
        const Json* bvj = a.get("bufferView");
        if (!bvj) return true;  // all zeros
        const Json* views = doc.get("bufferViews");
        const size_t bvi = (size_t)bvj->num;
        if (!views || bvi >= views->size()) return fail("bufferView out of range");
        const Json& bv = views->arr[bvi];
        const size_t bi = (size_t)bv.number("buffer", 0);
        if (bi >= buffers.size()) return fail("buffer out of range");
        const std::vector<unsigned char>& buf = buffers[bi];
        const size_t base = (size_t)bv.number("byteOffset", 0) + (size_t)a.number("byteOffset", 0);
        const size_t stride = bv.get("byteStride") ? (size_t)bv.number("byteStride", 0) : (size_t)(csize * ncomp);
        const size_t view_end = (size_t)bv.number("byteOffset", 0) + (size_t)bv.number("byteLength", 0);
        for (size_t e = 0; e < count; ++e) {
            for (int c = 0; c < ncomp; ++c) {
                const size_t off = base + e * stride + (size_t)c * csize;
                if (off + csize > buf.size() || off + csize > view_end) return fail("accessor reads past its buffer");
                const unsigned char* q = buf.data() + off;
                double v = 0.0;
                switch (ctype) {
                    case 5120: { int8_t x; std::memcpy(&x, q, 1); v = norm ? std::fmax(x / 127.0, -1.0) : x; break; }
                    case 5121: { uint8_t x = q[0]; v = norm ? x / 255.0 : x; break; }
                    case 5122: { int16_t x; std::memcpy(&x, q, 2); v = norm ? std::fmax(x / 32767.0, -1.0) : x; break; }
                    case 5123: { uint16_t x; std::memcpy(&x, q, 2); v = norm ? x / 65535.0 : x; break; }
                    case 5125: { uint32_t x; std::memcpy(&x, q, 4); v = x; break; }
                    case 5126: { float x; std::memcpy(&x, q, 4); v = x; break; }
                }
                out[e * ncomp + c] = v;
            }
        }
        return true;
    }

    bool load(const std::string& path, solrt_gltf& g) {
        std::vector<unsigned char> file;
        if (!read_file(path, file)) return fail("cannot read " + path);
        std::string json;
        std::vector<unsigned char> glb_bin;
        bool glb = file.size() >= 12 && std::memcmp(file.data(), "glTF", 4) == 0;
        if (glb) {
            size_t off = 12;
            while (off + 8 <= file.size()) {
                uint32_t len, type;
                std::memcpy(&len, file.data() + off, 4);
                std::memcpy(&type, file.data() + off + 4, 4);
                if (off + 8 + len > file.size()) return fail("truncated glb chunk");
                if (type == 0x4E4F534Au) json.assign((const char*)file.data() + off + 8, len);
                else if (type == 0x004E4942u) glb_bin.assign(file.data() + off + 8, file.data() + off + 8 + len);
                off += 8 + ((len + 3u) & ~3u);
            }
        } else {
            json.assign(file.begin(), file.end());
        }
        JsonReader rd{json.data(), json.data() + json.size()};
        doc = rd.value();
        if (!rd.ok || doc.type != Json::Obj) return fail("malformed JSON");
        const std::string dir = dir_of(path);
        if (const Json* bufs = doc.get("buffers")) {
            for (size_t i = 0; i < bufs->size(); ++i) {
                const Json* uri = bufs->arr[i].get("uri");
                std::vector<unsigned char> data;
                if (!uri) {
                    data = glb_bin;
                } else if (uri->str.compare(0, 5, "data:") == 0) {
                    const size_t comma = uri->str.find(',');
                    if (comma == std::string::npos || !base64_decode(uri->str.substr(comma + 1), data))
                        return fail("bad data URI");
                } else if (!read_file(dir + uri->str, data)) {
                    return fail("cannot read buffer " + dir + uri->str);
                }
                buffers.push_back(std::move(data));
            }
        }
        // materials (src/scene/mod.rs:144-156)
        if (const Json* mats = doc.get("materials")) {
            for (const Json& m : mats->arr) {
                solrt_material mi{};
                mi.base_color[0] = mi.base_color[1] = mi.base_color[2] = mi.base_color[3] = 1.0f;
                mi.metallic = 1.0f;
                mi.roughness = 1.0f;
                if (const Json* pbr = m.get("pbrMetallicRoughness")) {
                    if (const Json* bc = pbr->get("baseColorFactor"))
                        for (size_t i = 0; i < 4 && i < bc->size(); ++i) mi.base_color[i] = (float)bc->arr[i].num;
                    mi.metallic = (float)pbr->number("metallicFactor", 1.0);
                    mi.roughness = (float)pbr->number("roughnessFactor", 1.0);
                }
                if (const Json* em = m.get("emissiveFactor"))
                    for (size_t i = 0; i < 3 && i < em->size(); ++i) mi.emissive[i] = (float)em->arr[i].num;
                g.materials.push_back(mi);
            }
        }
        uint32_t default_mat = 0xffffffffu;
        const Json* nodes = doc.get("nodes");
        // meshes (src/scene/mod.rs:163-259)
        if (const Json* meshes = doc.get("meshes")) {
            for (size_t mi = 0; mi < meshes->size(); ++mi) {
                // global transform (src/scene/mod.rs:124-136): the first node,
                // in node order, from which a DFS reaches the mesh
                M4 global = identity();
                if (nodes) {
                    for (size_t n = 0; n < nodes->size(); ++n) {
                        std::vector<M4> stack;
                        if (find_mesh(*nodes, n, mi, stack, 0)) {
                            for (const M4& t : stack) global = mul(global, t);
                            break;
                        }
                    }
                }
                M4 git;
                if (!inverse_transpose(global, git)) return fail("singular node transform");
                const Json* prims = meshes->arr[mi].get("primitives");
                if (!prims) continue;
                for (const Json& pr : prims->arr) {
                    const Json* attrs = pr.get("attributes");
                    const Json* pos = attrs ? attrs->get("POSITION") : nullptr;
                    if (!pos) return fail("primitive without POSITION");
                    std::vector<double> P, N, C, T;
                    int np = 0, nn = 0, nc = 0, nt = 0;
                    size_t cp = 0, cn = 0, cc = 0, ct = 0;
                    if (!accessor((size_t)pos->num, P, np, cp) || np != 3) return fail(err.empty() ? "bad POSITION" : err);
                    if (const Json* a = attrs->get("NORMAL"))
                        if (!accessor((size_t)a->num, N, nn, cn)) return false;
                    if (const Json* a = attrs->get("COLOR_0"))
                        if (!accessor((size_t)a->num, C, nc, cc, true)) return false;
                    if (const Json* a = attrs->get("TEXCOORD_0"))
                        if (!accessor((size_t)a->num, T, nt, ct, true)) return false;
                    solrt_section sec{};
                    sec.vertex_offset = (uint32_t)g.vertices.size();
                    sec.vertex_count = (uint32_t)cp;
                    for (size_t v = 0; v < cp; ++v) {  // defaults of src/scene/mod.rs:182-193
                        solrt_vertex vx{};
                        vx.pos[0] = (float)P[3 * v]; vx.pos[1] = (float)P[3 * v + 1]; vx.pos[2] = (float)P[3 * v + 2];
                        vx.pos[3] = 1.0f;
                        if (v < cn && nn >= 3) {
                            vx.normal[0] = (float)N[nn * v]; vx.normal[1] = (float)N[nn * v + 1];
                            vx.normal[2] = (float)N[nn * v + 2];
                        } else {
                            vx.normal[1] = 1.0f;
                        }
                        vx.normal[3] = 1.0f;
                        if (v < cc && nc >= 3) {
                            for (int k = 0; k < 3; ++k) vx.color[k] = (float)C[nc * v + k];
                            vx.color[3] = nc == 4 ? (float)C[nc * v + 3] : 1.0f;
                        } else {
                            vx.color[0] = vx.color[1] = vx.color[2] = vx.color[3] = 1.0f;
                        }
                        if (v < ct && nt >= 2) {
                            vx.uv[0] = (float)T[nt * v];
                            vx.uv[1] = (float)T[nt * v + 1];
                        }
                        g.vertices.push_back(vx);
                    }
                    sec.index_offset = (uint32_t)g.indices.size();
                    if (const Json* ij = pr.get("indices")) {
                        std::vector<double> I;
                        int ni = 0;
                        size_t ci = 0;
                        if (!accessor((size_t)ij->num, I, ni, ci) || ni != 1) return fail(err.empty() ? "bad indices" : err);
                        for (double x : I) g.indices.push_back((uint32_t)x);
                        sec.index_count = (uint32_t)ci;
                    } else {  // non-indexed: consecutive triangles
                        for (size_t v = 0; v < cp; ++v) g.indices.push_back((uint32_t)v);
                        sec.index_count = (uint32_t)cp;
                    }
                    sec.index_count -= sec.index_count % 3;
                    const Json* mode = pr.get("mode");
                    if (mode && (int)mode->num != 4) return fail("only triangle primitives are supported");
                    const Json* mj = pr.get("material");
                    if (mj && (size_t)mj->num < g.materials.size()) {
                        sec.material_index = (uint32_t)mj->num;
                    } else {
                        if (default_mat == 0xffffffffu) {
                            solrt_material d{};
                            d.base_color[0] = d.base_color[1] = d.base_color[2] = d.base_color[3] = 1.0f;
                            d.metallic = 1.0f;
                            d.roughness = 1.0f;
                            default_mat = (uint32_t)g.materials.size();
                            g.materials.push_back(d);
                        }
                        sec.material_index = default_mat;
                    }
                    solrt_instance in{};
                    in.id = (uint32_t)g.sections.size();
                    for (int i = 0; i < 16; ++i) {
                        in.transform[i] = (float)global.m[i];
                        in.transform_it[i] = (float)git.m[i];
                    }
                    g.sections.push_back(sec);
                    g.instances.push_back(in);
                }
            }
        }
        // first camera (src/scene/mod.rs:261-287)
        if (const Json* cams = doc.get("cameras")) {
            if (cams->size() > 0) {
                const Json& c = cams->arr[0];
                const Json* persp = c.get("perspective");
                if (persp && nodes) {
                    for (const Json& n : nodes->arr) {
                        const Json* cj = n.get("camera");
                        if (cj && (size_t)cj->num == 0) {
                            const M4 v = node_matrix(n);
                            for (int i = 0; i < 16; ++i) g.view[i] = (float)v.m[i];
                            g.yfov = (float)persp->number("yfov", 35.0);
                            g.znear = (float)persp->number("znear", 0.1);
                            g.zfar = (float)persp->number("zfar", 100.0);
                            g.has_camera = true;
                            break;
                        }
                    }
                }
            }
        }
        return true;
    }
};

}  // namespace

extern "C" {

solrt_status solrt_gltf_load(const char* path, solrt_gltf** out) {
    if (!path || !out) {
        solrt::set_error("null argument");
        return SOLRT_ERR_INVALID;
    }
    *out = nullptr;
    solrt_gltf* g = new (std::nothrow) solrt_gltf();
    if (!g) return SOLRT_ERR_OOM;
    Loader ld;
    if (!ld.load(path, *g)) {
        solrt::set_error("glTF %s: %s", path, ld.err.c_str());
        delete g;
        return SOLRT_ERR_INVALID;
    }
    *out = g;
    return SOLRT_OK;
}

solrt_status solrt_gltf_scene_desc(const solrt_gltf* g, solrt_scene_desc* d) {
    if (!g || !d) {
        solrt::set_error("null argument");
        return SOLRT_ERR_INVALID;
    }
    d->vertices = g->vertices.data();
    d->vertex_count = (uint32_t)g->vertices.size();
    d->indices = g->indices.data();
    d->index_count = (uint32_t)g->indices.size();
    d->sections = g->sections.data();
    d->section_count = (uint32_t)g->sections.size();
    d->materials = g->materials.data();
    d->material_count = (uint32_t)g->materials.size();
    d->instances = g->instances.data();
    return SOLRT_OK;
}

solrt_status solrt_gltf_camera(const solrt_gltf* g, float aspect, solrt_camera* out) {
    if (!g || !out) {
        solrt::set_error("null argument");
        return SOLRT_ERR_INVALID;
    }
    if (!g->has_camera) {
        solrt::set_error("no perspective camera in the glTF file");
        return SOLRT_ERR_NOT_FOUND;
    }
    return solrt_camera_from_view(g->view, g->yfov, aspect, g->znear, g->zfar, out);
}

solrt_status solrt_gltf_destroy(solrt_gltf* g) {
    delete g;
    return SOLRT_OK;
}

}  // extern "C"
