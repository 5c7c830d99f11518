// gltf.cpp — glTF 2.0 ingest on the host (cp_gltf_*, include/cpq.h).
//
// Reads what the reference's Scene::load / Scene::parse_mesh take from
// tinygltf (src/scene/scene.cpp:48-315, 317-391): triangle geometry
// (POSITION + indices; strips and fans converted as parse_mesh converts
// them), node placement, and for shading the vertex normals, texture
// coordinates and tangents, the material factors and the material's texture
// references with each texture's image (images are not decoded).
// Self-contained: a small JSON
// reader, base64 "data:" URIs, external .bin buffers and .glb containers.
// Everything is bounds-checked against the buffers it indexes; a malformed
// file is an error, never an out-of-range read.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "cpq.h"

namespace cpq {
cp_status set_error(cp_status s, const std::string& msg);
}

namespace {

// ---- JSON ------------------------------------------------------------------

struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;

    const Json* get(const std::string& k) const {
        if (kind != Object) return nullptr;
        auto it = obj.find(k);
        return it == obj.end() ? nullptr : &it->second;
    }
    const Json& at(const std::string& k) const {
        const Json* j = get(k);
        if (!j) throw std::runtime_error("missing \"" + k + "\"");
        return *j;
    }
    double number(const std::string& k, double dflt) const {
        const Json* j = get(k);
        if (!j) return dflt;
        if (j->kind != Number) throw std::runtime_error("\"" + k + "\" is not a number");
        return j->num;
    }
    int64_t integer(const std::string& k, int64_t dflt) const {
        const double v = number(k, (double)dflt);
        if (v != std::floor(v) || std::fabs(v) > 9.0e15) throw std::runtime_error("\"" + k + "\" is not an integer");
        return (int64_t)v;
    }
    const std::vector<Json>& array(const std::string& k) const {
        static const std::vector<Json> empty;
        const Json* j = get(k);
        if (!j) return empty;
        if (j->kind != Array) throw std::runtime_error("\"" + k + "\" is not an array");
        return j->arr;
    }
};

class JsonReader {
public:
    JsonReader(const char* p, size_t n) : p_(p), end_(p + n) {}
    Json parse() {
        Json v = value(0);
        ws();
        if (p_ != end_) fail("trailing characters");
        return v;
    }

private:
    const char* p_;
    const char* end_;
    [[noreturn]] void fail(const char* what) { throw std::runtime_error(std::string("JSON: ") + what); }
    void ws() {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
    }
    bool lit(const char* s) {
        const size_t n = std::strlen(s);
        if ((size_t)(end_ - p_) >= n && std::memcmp(p_, s, n) == 0) {
            p_ += n;
            return true;
        }
        return false;
    }
    Json value(int depth) {
        if (depth > 256) fail("nesting too deep");
        ws();
        if (p_ >= end_) fail("unexpected end");
        Json v;
        const char c = *p_;
        if (c == '{') {
            ++p_;
            v.kind = Json::Object;
            ws();
            if (p_ < end_ && *p_ == '}') {
                ++p_;
                return v;
            }
            for (;;) {
                ws();
                if (p_ >= end_ || *p_ != '"') fail("expected a key");
                std::string k = string();
                ws();
                if (p_ >= end_ || *p_ != ':') fail("expected ':'");
                ++p_;
                v.obj[k] = value(depth + 1);
                ws();
                if (p_ < end_ && *p_ == ',') {
                    ++p_;
                    continue;
                }
                if (p_ < end_ && *p_ == '}') {
                    ++p_;
                    return v;
                }
                fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            ++p_;
            v.kind = Json::Array;
            ws();
            if (p_ < end_ && *p_ == ']') {
                ++p_;
                return v;
            }
            for (;;) {
                v.arr.push_back(value(depth + 1));
                ws();
                if (p_ < end_ && *p_ == ',') {
                    ++p_;
                    continue;
                }
                if (p_ < end_ && *p_ == ']') {
                    ++p_;
                    return v;
                }
                fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.kind = Json::String;
            v.str = string();
            return v;
        }
        if (lit("true")) {
            v.kind = Json::Bool;
            v.b = true;
            return v;
        }
        if (lit("false")) {
            v.kind = Json::Bool;
            return v;
        }
        if (lit("null")) return v;
        v.kind = Json::Number;
        v.num = number();
        return v;
    }
    double number() {
        const char* s = p_;
        if (p_ < end_ && (*p_ == '-' || *p_ == '+')) ++p_;
        while (p_ < end_ && ((*p_ >= '0' && *p_ <= '9') || *p_ == '.' || *p_ == 'e' || *p_ == 'E' ||
                             *p_ == '-' || *p_ == '+'))
            ++p_;
        if (p_ == s) fail("unexpected character");
        const std::string tok(s, p_);
        char* e = nullptr;
        const double d = std::strtod(tok.c_str(), &e);
        if (!e || *e) fail("bad number");
        return d;
    }
    static void utf8(std::string& out, uint32_t cp) {
        if (cp < 0x80) {
            out += (char)cp;
        } else if (cp < 0x800) {
            out += (char)(0xC0 | (cp >> 6));
            out += (char)(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += (char)(0xE0 | (cp >> 12));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
        } else {
            out += (char)(0xF0 | (cp >> 18));
            out += (char)(0x80 | ((cp >> 12) & 0x3F));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
        }
    }
    uint32_t hex4() {
        if (end_ - p_ < 4) fail("bad \\u escape");
        uint32_t v = 0;
        for (int i = 0; i < 4; ++i) {
            const char h = *p_++;
            v <<= 4;
            if (h >= '0' && h <= '9') v |= (uint32_t)(h - '0');
            else if (h >= 'a' && h <= 'f') v |= (uint32_t)(h - 'a' + 10);
            else if (h >= 'A' && h <= 'F') v |= (uint32_t)(h - 'A' + 10);
            else fail("bad \\u escape");
        }
        return v;
    }
    std::string string() {
        ++p_;  // opening quote
        std::string out;
        while (p_ < end_ && *p_ != '"') {
            char c = *p_++;
            if (c != '\\') {
                out += c;
                continue;
            }
            if (p_ >= end_) fail("bad escape");
            c = *p_++;
            switch (c) {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u': {
                    uint32_t cp = hex4();
                    if (cp >= 0xD800 && cp < 0xDC00 && end_ - p_ >= 6 && p_[0] == '\\' && p_[1] == 'u') {
                        p_ += 2;
                        const uint32_t lo = hex4();
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    utf8(out, cp);
                    break;
                }
                default: fail("bad escape");
            }
        }
        if (p_ >= end_) fail("unterminated string");
        ++p_;
        return out;
    }
};

// ---- buffers ---------------------------------------------------------------

std::vector<uint8_t> read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::ostringstream ss;
    ss << f.rdbuf();
    const std::string s = ss.str();
    return std::vector<uint8_t>(s.begin(), s.end());
}

std::vector<uint8_t> base64(const std::string& s) {
    static int8_t tab[256];
    static bool init = false;
    if (!init) {
        std::memset(tab, -1, sizeof tab);
        const char* a = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
        for (int i = 0; i < 64; ++i) tab[(uint8_t)a[i]] = (int8_t)i;
        init = true;
    }
    std::vector<uint8_t> out;
    uint32_t acc = 0;
    int bits = 0;
    for (char c : s) {
        if (c == '=' || c == '\n' || c == '\r' || c == ' ') continue;
        const int v = tab[(uint8_t)c];
        if (v < 0) throw std::runtime_error("bad base64 data");
        acc = (acc << 6) | (uint32_t)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((uint8_t)((acc >> bits) & 0xFF));
        }
    }
    return out;
}

uint32_t rd32(const uint8_t* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

std::string dir_of(const std::string& path) {
    const size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

// Percent-decoding of a relative URI (spaces in file names are %20).
std::string uri_path(const std::string& uri) {
    std::string out;
    for (size_t i = 0; i < uri.size(); ++i) {
        if (uri[i] == '%' && i + 2 < uri.size()) {
            out += (char)std::stoi(uri.substr(i + 1, 2), nullptr, 16);
            i += 2;
        } else {
            out += uri[i];
        }
    }
    return out;
}

// ---- the scene -------------------------------------------------------------

struct Accessor {
    const uint8_t* data = nullptr;
    size_t count = 0, stride = 0;
    int ctype = 0, ncomp = 0;
};

struct Model {
    Json doc;
    std::vector<std::vector<uint8_t>> buffers;

    Accessor accessor(int64_t i) const {
        const auto& acc = doc.array("accessors");
        if (i < 0 || i >= (int64_t)acc.size()) throw std::runtime_error("accessor index out of range");
        const Json& a = acc[(size_t)i];
        if (a.get("sparse")) throw std::runtime_error("sparse accessors are not supported");
        Accessor r;
        r.ctype = (int)a.integer("componentType", 0);
        // sizes and offsets: non-negative, and every bound below is checked
        // without a sum or product that could wrap
        auto size_of = [](const Json& j, const char* k) {
            const int64_t v = j.integer(k, 0);
            if (v < 0) throw std::runtime_error(std::string("negative \"") + k + "\"");
            return (size_t)v;
        };
        r.count = size_of(a, "count");
        const std::string& type = a.at("type").str;
        r.ncomp = type == "SCALAR" ? 1 : type == "VEC2" ? 2 : type == "VEC3" ? 3 : type == "VEC4" ? 4 : 0;
        if (!r.ncomp) throw std::runtime_error("unsupported accessor type " + type);
        size_t csize = 0;
        switch (r.ctype) {
            case 5120: case 5121: csize = 1; break;
            case 5122: case 5123: csize = 2; break;
            case 5125: case 5126: csize = 4; break;
            default: throw std::runtime_error("unsupported componentType " + std::to_string(r.ctype));
        }
        const int64_t bvi = a.integer("bufferView", -1);
        const auto& views = doc.array("bufferViews");
        if (bvi < 0 || bvi >= (int64_t)views.size()) throw std::runtime_error("accessor without a valid bufferView");
        const Json& bv = views[(size_t)bvi];
        const int64_t bi = bv.integer("buffer", -1);
        if (bi < 0 || bi >= (int64_t)buffers.size()) throw std::runtime_error("bufferView buffer out of range");
        const std::vector<uint8_t>& buf = buffers[(size_t)bi];
        const size_t view_off = size_of(bv, "byteOffset");
        const size_t view_len = size_of(bv, "byteLength");
        const size_t off = size_of(a, "byteOffset");
        const size_t elem = csize * (size_t)r.ncomp;
        r.stride = size_of(bv, "byteStride");
        if (r.stride == 0) r.stride = elem;
        if (r.stride < elem) throw std::runtime_error("byteStride smaller than the element");
        if (view_off > buf.size() || view_len > buf.size() - view_off)
            throw std::runtime_error("bufferView past the end of its buffer");
        if (r.count && (off > view_len || elem > view_len - off || (r.count - 1) > (view_len - off - elem) / r.stride))
            throw std::runtime_error("accessor past the end of its bufferView");
        r.data = buf.data() + view_off + off;
        return r;
    }
};

struct Scene {
    std::vector<float> verts;
    std::vector<float> normals;    // per vertex, zeros where the primitive has no NORMAL
    std::vector<float> texcoords;  // per vertex TEXCOORD_0, zeros where absent
    std::vector<float> tangents;   // per vertex TANGENT (xyz, w), zeros where absent
    std::vector<float> materials;  // per primitive: base colour rgb, emission rgb, metalness, roughness
    std::vector<int32_t> prim_tex; // per primitive: base colour, emissive, metal / rough, normal texture or -1
    std::vector<int32_t> tex_image;    // per glTF texture: its image, or -1
    std::vector<std::string> image_uri;  // per image: "uri", or empty
    std::vector<const char*> image_uri_c;
    std::vector<int32_t> image_view;   // per image: "bufferView", or -1
    std::vector<int32_t> tris;
    std::vector<int64_t> voff{0}, toff{0};
    std::vector<int32_t> mesh_first_prim, mesh_num_prim;  // per glTF mesh: its triangle primitives
    std::vector<int32_t> inst_prim;
    std::vector<float> inst_world;
};

uint32_t index_at(const Accessor& a, size_t i) {
    const uint8_t* p = a.data + i * a.stride;
    switch (a.ctype) {
        case 5120: return (uint32_t)(int32_t)(int8_t)p[0];
        case 5121: return p[0];
        case 5122: { int16_t v; std::memcpy(&v, p, 2); return (uint32_t)(int32_t)v; }
        case 5123: { uint16_t v; std::memcpy(&v, p, 2); return v; }
        default: { uint32_t v; std::memcpy(&v, p, 4); return v; }
    }
}

// n numbers of a JSON array member, or the defaults when the member is absent
void numbers(const Json& j, const char* key, size_t n, const float* dflt, float* out) {
    const Json* a = j.get(key);
    if (!a) {
        std::copy(dflt, dflt + n, out);
        return;
    }
    if (a->kind != Json::Array || a->arr.size() < n)
        throw std::runtime_error(std::string("\"") + key + "\" is not an array of " + std::to_string(n) + " numbers");
    for (size_t k = 0; k < n; ++k) {
        if (a->arr[k].kind != Json::Number) throw std::runtime_error(std::string("\"") + key + "\" holds a non-number");
        out[k] = (float)a->arr[k].num;
    }
}

// The factors Scene::parse_mesh copies into its Material (scene.cpp:286-299),
// with glTF's defaults; a primitive without a material gets the default
// material (the reference would index materials[-1]).
void material_factors(const Model& m, const Json& prim, float* out) {
    static const float kOne[4] = {1.0f, 1.0f, 1.0f, 1.0f}, kZero[3] = {0.0f, 0.0f, 0.0f};
    std::copy(kOne, kOne + 3, out);
    std::copy(kZero, kZero + 3, out + 3);
    out[6] = 1.0f;
    out[7] = 1.0f;
    const int64_t mi = prim.integer("material", -1);
    if (mi < 0) return;
    const auto& mats = m.doc.array("materials");
    if (mi >= (int64_t)mats.size()) throw std::runtime_error("material index out of range");
    const Json& mat = mats[(size_t)mi];
    if (const Json* pbr = mat.get("pbrMetallicRoughness")) {
        float rgba[4];
        numbers(*pbr, "baseColorFactor", 4, kOne, rgba);
        std::copy(rgba, rgba + 3, out);
        out[6] = (float)pbr->number("metallicFactor", 1.0);
        out[7] = (float)pbr->number("roughnessFactor", 1.0);
    }
    numbers(mat, "emissiveFactor", 3, kZero, out + 3);
}

// The texture references Scene::parse_mesh copies into its Material
// (scene.cpp:294-302): the "index" of baseColorTexture, emissiveTexture,
// metallicRoughnessTexture and normalTexture, -1 where absent (as tinygltf
// reports it); an index outside the file's textures is refused.
void material_textures(const Model& m, const Json& prim, int32_t* out) {
    for (int k = 0; k < 4; ++k) out[k] = -1;
    const int64_t mi = prim.integer("material", -1);
    if (mi < 0) return;
    const auto& mats = m.doc.array("materials");
    if (mi >= (int64_t)mats.size()) throw std::runtime_error("material index out of range");
    const Json& mat = mats[(size_t)mi];
    const int64_t ntex = (int64_t)m.doc.array("textures").size();
    auto ref = [&](const Json* holder, const char* key, int32_t* slot) {
        if (!holder) return;
        const Json* t = holder->get(key);
        if (!t) return;
        const int64_t i = t->integer("index", -1);
        if (i < 0 || i >= ntex) throw std::runtime_error(std::string(key) + " index out of range");
        *slot = (int32_t)i;
    };
    const Json* pbr = mat.get("pbrMetallicRoughness");
    ref(pbr, "baseColorTexture", out);
    ref(&mat, "emissiveTexture", out + 1);
    ref(pbr, "metallicRoughnessTexture", out + 2);
    ref(&mat, "normalTexture", out + 3);
}

// n floats per vertex of an optional FLOAT attribute, paired with the
// positions as parse_mesh pairs them: the k-th for vertex k, zeros past the
// accessor's count or where the attribute is absent or of another type (the
// reference reads FLOAT and skips what it does not handle, scene.cpp:188-265)
void per_vertex(const Model& m, const Json& attrs, const char* name, int ncomp, size_t nv, std::vector<float>& out) {
    size_t have = 0;
    Accessor a;
    if (const Json* j = attrs.get(name)) {
        a = m.accessor((int64_t)j->num);
        if (a.ctype == 5126 && a.ncomp == ncomp) have = std::min(a.count, nv);
    }
    for (size_t k = 0; k < nv; ++k) {
        float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (k < have) std::memcpy(v, a.data + k * a.stride, sizeof(float) * ncomp);
        out.insert(out.end(), v, v + ncomp);
    }
}

// Each texture's image ("source") and each image's "uri" or "bufferView"
// (scene.cpp:373-389 loads textures in this order).  Images are not decoded.
void add_textures(const Model& m, Scene& s) {
    const auto& images = m.doc.array("images");
    for (const Json& t : m.doc.array("textures")) {
        const int64_t src = t.integer("source", -1);
        s.tex_image.push_back(src >= 0 && src < (int64_t)images.size() ? (int32_t)src : -1);
    }
    const int64_t nviews = (int64_t)m.doc.array("bufferViews").size();
    for (const Json& im : images) {
        const Json* uri = im.get("uri");
        s.image_uri.push_back(uri && uri->kind == Json::String ? uri->str : std::string());
        const int64_t v = im.integer("bufferView", -1);
        s.image_view.push_back(v >= 0 && v < nviews ? (int32_t)v : -1);
    }
    for (const std::string& u : s.image_uri) s.image_uri_c.push_back(u.c_str());
}

void add_primitives(const Model& m, Scene& s) {
    const auto& meshes = m.doc.array("meshes");
    for (const Json& mesh : meshes) {
        s.mesh_first_prim.push_back((int32_t)(s.voff.size() - 1));
        int32_t count = 0;
        for (const Json& prim : mesh.array("primitives")) {
            const int64_t mode = prim.integer("mode", 4);
            if (mode != 4 && mode != 5 && mode != 6) continue;  // points and lines
            const Json& attrs = prim.at("attributes");
            const Json* pos_j = attrs.get("POSITION");
            if (!pos_j) throw std::runtime_error("primitive without POSITION");
            const Accessor pos = m.accessor((int64_t)pos_j->num);
            if (pos.ctype != 5126 || pos.ncomp != 3) throw std::runtime_error("POSITION must be FLOAT VEC3");
            const size_t nv = pos.count;
            std::vector<uint32_t> idx;
            const int64_t ii = prim.integer("indices", -1);
            if (ii >= 0) {
                const Accessor ia = m.accessor(ii);
                if (ia.ncomp != 1 || ia.ctype == 5126) throw std::runtime_error("indices must be integer SCALAR");
                idx.resize(ia.count);
                for (size_t k = 0; k < ia.count; ++k) idx[k] = index_at(ia, k);
            } else {
                idx.resize(nv);
                for (size_t k = 0; k < nv; ++k) idx[k] = (uint32_t)k;
            }
            std::vector<uint32_t> t;
            if (mode == 4) {
                t.assign(idx.begin(), idx.begin() + (idx.size() / 3) * 3);
            } else if (mode == 5) {  // strip: (k-2, k-1, k)
                for (size_t k = 2; k < idx.size(); ++k) t.insert(t.end(), {idx[k - 2], idx[k - 1], idx[k]});
            } else {  // fan: (0, k-1, k)
                for (size_t k = 2; k < idx.size(); ++k) t.insert(t.end(), {idx[0], idx[k - 1], idx[k]});
            }
            for (uint32_t v : t)
                if (v >= nv) throw std::runtime_error("index " + std::to_string(v) + " past " + std::to_string(nv) + " vertices");
            if (nv > (size_t)INT32_MAX) throw std::runtime_error("a primitive with more than 2^31 - 1 vertices");
            for (size_t k = 0; k < nv; ++k) {
                float p[3];
                std::memcpy(p, pos.data + k * pos.stride, 12);
                s.verts.insert(s.verts.end(), p, p + 3);
            }
            // normals as parse_mesh pairs them with positions: the k-th for
            // vertex k, zero past the accessor's count (scene.cpp:304-307)
            size_t nn = 0;
            Accessor na;
            if (const Json* n_j = attrs.get("NORMAL")) {
                na = m.accessor((int64_t)n_j->num);
                if (na.ctype != 5126 || na.ncomp != 3) throw std::runtime_error("NORMAL must be FLOAT VEC3");
                nn = std::min(na.count, nv);
            }
            for (size_t k = 0; k < nv; ++k) {
                float n[3] = {0.0f, 0.0f, 0.0f};
                if (k < nn) std::memcpy(n, na.data + k * na.stride, 12);
                s.normals.insert(s.normals.end(), n, n + 3);
            }
            per_vertex(m, attrs, "TEXCOORD_0", 2, nv, s.texcoords);
            per_vertex(m, attrs, "TANGENT", 4, nv, s.tangents);
            float mat[8];
            material_factors(m, prim, mat);
            s.materials.insert(s.materials.end(), mat, mat + 8);
            int32_t tex[4];
            material_textures(m, prim, tex);
            s.prim_tex.insert(s.prim_tex.end(), tex, tex + 4);
            for (uint32_t v : t) s.tris.push_back((int32_t)v);
            s.voff.push_back(s.voff.back() + (int64_t)nv);
            s.toff.push_back(s.toff.back() + (int64_t)(t.size() / 3));
            ++count;
        }
        s.mesh_num_prim.push_back(count);
    }
}

// 4 x 4 row-major products
void matmul(const float* a, const float* b, float* out) {
    float r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 4; ++k) acc += (double)a[4 * i + k] * b[4 * k + j];
            r[4 * i + j] = (float)acc;
        }
    std::memcpy(out, r, sizeof r);
}

void local_matrix(const Json& node, float* m) {
    const auto& mat = node.array("matrix");
    if (mat.size() == 16) {  // glTF stores column-major
        for (int c = 0; c < 4; ++c)
            for (int r = 0; r < 4; ++r) m[4 * r + c] = (float)mat[(size_t)(4 * c + r)].num;
        return;
    }
    double t[3] = {0, 0, 0}, q[4] = {0, 0, 0, 1}, s[3] = {1, 1, 1};
    const auto& tj = node.array("translation");
    const auto& qj = node.array("rotation");
    const auto& sj = node.array("scale");
    if (tj.size() == 3) for (int i = 0; i < 3; ++i) t[i] = tj[(size_t)i].num;
    if (qj.size() == 4) for (int i = 0; i < 4; ++i) q[i] = qj[(size_t)i].num;
    if (sj.size() == 3) for (int i = 0; i < 3; ++i) s[i] = sj[(size_t)i].num;
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
                         2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
                         2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)};
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) m[4 * r + c] = (float)(R[3 * r + c] * s[c]);
        m[4 * r + 3] = (float)t[r];
    }
    m[12] = m[13] = m[14] = 0.0f;
    m[15] = 1.0f;
}

void visit(const Model& m, Scene& s, int64_t n, const float* parent, int depth) {
    const auto& nodes = m.doc.array("nodes");
    if (n < 0 || n >= (int64_t)nodes.size()) throw std::runtime_error("node index out of range");
    if (depth > 1024) throw std::runtime_error("node hierarchy too deep (a cycle?)");
    const Json& node = nodes[(size_t)n];
    float local[16], world[16];
    local_matrix(node, local);
    matmul(parent, local, world);
    const int64_t mi = node.integer("mesh", -1);
    if (mi >= 0) {
        if (mi >= (int64_t)s.mesh_first_prim.size()) throw std::runtime_error("node mesh out of range");
        for (int32_t k = 0; k < s.mesh_num_prim[(size_t)mi]; ++k) {
            s.inst_prim.push_back(s.mesh_first_prim[(size_t)mi] + k);
            s.inst_world.insert(s.inst_world.end(), world, world + 16);
        }
    }
    for (const Json& c : node.array("children")) visit(m, s, (int64_t)c.num, world, depth + 1);
}

Model load_model(const std::string& path) {
    Model m;
    std::vector<uint8_t> file = read_file(path);
    std::vector<uint8_t> glb_bin;
    const char* json = reinterpret_cast<const char*>(file.data());
    size_t json_len = file.size();
    bool glb = false;
    if (file.size() >= 12 && std::memcmp(file.data(), "glTF", 4) == 0) {
        glb = true;
        if (rd32(file.data() + 4) != 2) throw std::runtime_error("only glTF 2.0 .glb is supported");
        const size_t total = std::min<size_t>(rd32(file.data() + 8), file.size());
        size_t off = 12;
        json = nullptr;
        while (off + 8 <= total) {
            const size_t len = rd32(file.data() + off), type = rd32(file.data() + off + 4);
            if (off + 8 + len > total) throw std::runtime_error(".glb chunk past the end of the file");
            if (type == 0x4E4F534Au && !json) {  // JSON
                json = reinterpret_cast<const char*>(file.data() + off + 8);
                json_len = len;
            } else if (type == 0x004E4942u && glb_bin.empty()) {  // BIN
                glb_bin.assign(file.data() + off + 8, file.data() + off + 8 + len);
            }
            off += 8 + ((len + 3) & ~size_t(3));
        }
        if (!json) throw std::runtime_error(".glb without a JSON chunk");
    }
    m.doc = JsonReader(json, json_len).parse();
    if (m.doc.kind != Json::Object) throw std::runtime_error("the document is not a JSON object");
    const std::string base = dir_of(path);
    const auto& bufs = m.doc.array("buffers");
    for (size_t i = 0; i < bufs.size(); ++i) {
        const Json* uri = bufs[i].get("uri");
        std::vector<uint8_t> data;
        if (!uri) {
            if (!glb || i != 0) throw std::runtime_error("buffer without uri");
            data = glb_bin;
        } else if (uri->str.rfind("data:", 0) == 0) {
            const size_t comma = uri->str.find(',');
            if (comma == std::string::npos || uri->str.find(";base64") == std::string::npos)
                throw std::runtime_error("only base64 data URIs are supported");
            data = base64(uri->str.substr(comma + 1));
        } else {
            data = read_file(base + uri_path(uri->str));
        }
        const size_t len = (size_t)bufs[i].integer("byteLength", (int64_t)data.size());
        if (len > data.size()) throw std::runtime_error("buffer shorter than its byteLength");
        data.resize(len);
        m.buffers.push_back(std::move(data));
    }
    return m;
}

}  // namespace

struct cp_gltf {
    Scene s;
};

extern "C" {

CP_API cp_status cp_gltf_load(const char* path, cp_gltf** out) {
    if (!path || !out) return cpq::set_error(CP_ERROR_INVALID_VALUE, "path or out is NULL");
    *out = nullptr;
    try {
        const Model m = load_model(path);
        auto g = std::make_unique<cp_gltf>();
        add_primitives(m, g->s);
        add_textures(m, g->s);
        const float I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        // every scene's root nodes, depth first, as Scene::load walks them
        for (const Json& scene : m.doc.array("scenes"))
            for (const Json& root : scene.array("nodes")) visit(m, g->s, (int64_t)root.num, I, 0);
        *out = g.release();
        return CP_SUCCESS;
    } catch (const std::exception& e) {
        return cpq::set_error(CP_ERROR_INVALID_VALUE, std::string("glTF ") + path + ": " + e.what());
    }
}

CP_API void cp_gltf_free(cp_gltf* g) { delete g; }

CP_API cp_status cp_gltf_primitives(const cp_gltf* g, int32_t* n, const float** verts, const int32_t** tris,
                                    const int64_t** vert_offsets, const int64_t** tri_offsets) {
    if (!g || !n) return cpq::set_error(CP_ERROR_INVALID_VALUE, "scene or count is NULL");
    *n = (int32_t)(g->s.voff.size() - 1);
    if (verts) *verts = g->s.verts.data();
    if (tris) *tris = g->s.tris.data();
    if (vert_offsets) *vert_offsets = g->s.voff.data();
    if (tri_offsets) *tri_offsets = g->s.toff.data();
    return CP_SUCCESS;
}

CP_API cp_status cp_gltf_shading(const cp_gltf* g, int32_t* n, const float** normals, const float** materials) {
    if (!g || !n) return cpq::set_error(CP_ERROR_INVALID_VALUE, "scene or count is NULL");
    *n = (int32_t)(g->s.voff.size() - 1);
    if (normals) *normals = g->s.normals.data();
    if (materials) *materials = g->s.materials.data();
    return CP_SUCCESS;
}

CP_API cp_status cp_gltf_textures(const cp_gltf* g, int32_t* n, const float** texcoords, const float** tangents,
                                  const int32_t** prim_tex, int32_t* num_textures, const int32_t** tex_image,
                                  int32_t* num_images, const char* const** image_uri, const int32_t** image_view) {
    if (!g || !n) return cpq::set_error(CP_ERROR_INVALID_VALUE, "scene or count is NULL");
    *n = (int32_t)(g->s.voff.size() - 1);
    if (texcoords) *texcoords = g->s.texcoords.data();
    if (tangents) *tangents = g->s.tangents.data();
    if (prim_tex) *prim_tex = g->s.prim_tex.data();
    if (num_textures) *num_textures = (int32_t)g->s.tex_image.size();
    if (tex_image) *tex_image = g->s.tex_image.data();
    if (num_images) *num_images = (int32_t)g->s.image_uri.size();
    if (image_uri) *image_uri = g->s.image_uri_c.data();
    if (image_view) *image_view = g->s.image_view.data();
    return CP_SUCCESS;
}

CP_API cp_status cp_gltf_instances(const cp_gltf* g, int32_t* n, const int32_t** primitive, const float** world) {
    if (!g || !n) return cpq::set_error(CP_ERROR_INVALID_VALUE, "scene or count is NULL");
    *n = (int32_t)g->s.inst_prim.size();
    if (primitive) *primitive = g->s.inst_prim.data();
    if (world) *world = g->s.inst_world.data();
    return CP_SUCCESS;
}

}  // extern "C"
