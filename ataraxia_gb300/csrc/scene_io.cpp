// Scene files and scene-graph flattening; see scene_io.h.
//
// The reference reads and writes scenes with nlohmann::json (Utils.cpp), which
// is not part of this build: the JSON reader and writer below are written for
// this library.  The reader is a plain recursive-descent parser of RFC 8259
// text; the writer reproduces json::dump(4)'s layout (sorted keys, four-space
// indent, one array element per line) and its number format (the shortest
// decimal that reads back to the same double, fixed notation for decimal
// exponents in (-4, 15], ".0" appended to integral values) so that a scene
// written by the reference reads and writes back byte for byte.
//
// The transform arithmetic is single precision in the order of the reference's
// vector library (glm): matrix products column by column as left-to-right sums,
// matrix-vector products as (c0*v0 + c1*v1) + (c2*v2 + c3*v3), vector length
// as sqrt((x*x + y*y) + z*z).  Contraction into FMA is disabled for this file.
#include "scene_io.h"

#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <utility>

#include "host_common.h"

namespace atx {

// ================================================================ JSON DOM

namespace {

struct JVal {
    enum Type { Null, Bool, Int, Float, Str, Arr, Obj } type = Null;
    bool b = false;
    int64_t i = 0;
    double d = 0.0;
    std::string s;
    std::vector<JVal> a;
    std::vector<std::pair<std::string, JVal>> o;

    const JVal* get(const char* key) const
    {
        if (type != Obj) return nullptr;
        for (const auto& kv : o)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    bool is_num() const { return type == Int || type == Float; }
    double num() const { return type == Int ? (double)i : d; }
};

class Parser {
public:
    Parser(const char* p, size_t n) : p_(p), end_(p + n), begin_(p) {}

    atx_status parse(JVal& out)
    {
        ws();
        ATX_TRY(value(out, 0));
        ws();
        if (p_ != end_) return err("trailing characters after the document");
        return ATX_OK;
    }

private:
    static constexpr int kMaxDepth = 256;

    atx_status err(const char* what)
    {
        int line = 1, col = 1;
        for (const char* q = begin_; q < p_ && q < end_; ++q) {
            if (*q == '\n') {
                ++line;
                col = 1;
            } else {
                ++col;
            }
        }
        return fail(ATX_ERR_PARSE, "scene json: line %d column %d: %s", line, col, what);
    }
    void ws()
    {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
    }
    bool lit(const char* word)
    {
        const size_t n = std::strlen(word);
        if ((size_t)(end_ - p_) < n || std::memcmp(p_, word, n) != 0) return false;
        p_ += n;
        return true;
    }

    atx_status value(JVal& v, int depth)
    {
        if (depth > kMaxDepth) return err("nesting too deep");
        if (p_ >= end_) return err("unexpected end of input");
        switch (*p_) {
        case '{': return object(v, depth);
        case '[': return array(v, depth);
        case '"': v.type = JVal::Str; return string(v.s);
        case 't':
            if (!lit("true")) return err("invalid literal");
            v.type = JVal::Bool;
            v.b = true;
            return ATX_OK;
        case 'f':
            if (!lit("false")) return err("invalid literal");
            v.type = JVal::Bool;
            v.b = false;
            return ATX_OK;
        case 'n':
            if (!lit("null")) return err("invalid literal");
            v.type = JVal::Null;
            return ATX_OK;
        default: return number(v);
        }
    }

    atx_status object(JVal& v, int depth)
    {
        v.type = JVal::Obj;
        ++p_;
        ws();
        if (p_ < end_ && *p_ == '}') {
            ++p_;
            return ATX_OK;
        }
        for (;;) {
            ws();
            if (p_ >= end_ || *p_ != '"') return err("expected a key string");
            std::string key;
            ATX_TRY(string(key));
            ws();
            if (p_ >= end_ || *p_ != ':') return err("expected ':'");
            ++p_;
            ws();
            JVal child;
            ATX_TRY(value(child, depth + 1));
            // duplicate keys: the last one wins, as with nlohmann's parser
            bool replaced = false;
            for (auto& kv : v.o)
                if (kv.first == key) {
                    kv.second = std::move(child);
                    replaced = true;
                    break;
                }
            if (!replaced) v.o.emplace_back(std::move(key), std::move(child));
            ws();
            if (p_ < end_ && *p_ == ',') {
                ++p_;
                continue;
            }
            if (p_ < end_ && *p_ == '}') {
                ++p_;
                return ATX_OK;
            }
            return err("expected ',' or '}'");
        }
    }

    atx_status array(JVal& v, int depth)
    {
        v.type = JVal::Arr;
        ++p_;
        ws();
        if (p_ < end_ && *p_ == ']') {
            ++p_;
            return ATX_OK;
        }
        for (;;) {
            ws();
            v.a.emplace_back();
            ATX_TRY(value(v.a.back(), depth + 1));
            ws();
            if (p_ < end_ && *p_ == ',') {
                ++p_;
                continue;
            }
            if (p_ < end_ && *p_ == ']') {
                ++p_;
                return ATX_OK;
            }
            return err("expected ',' or ']'");
        }
    }

    static void put_utf8(std::string& s, uint32_t cp)
    {
        if (cp < 0x80) {
            s += (char)cp;
        } else if (cp < 0x800) {
            s += (char)(0xC0 | (cp >> 6));
            s += (char)(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            s += (char)(0xE0 | (cp >> 12));
            s += (char)(0x80 | ((cp >> 6) & 0x3F));
            s += (char)(0x80 | (cp & 0x3F));
        } else {
            s += (char)(0xF0 | (cp >> 18));
            s += (char)(0x80 | ((cp >> 12) & 0x3F));
            s += (char)(0x80 | ((cp >> 6) & 0x3F));
            s += (char)(0x80 | (cp & 0x3F));
        }
    }

    bool hex4(uint32_t& out)
    {
        if (end_ - p_ < 4) return false;
        out = 0;
        for (int k = 0; k < 4; ++k) {
            const char c = p_[k];
            uint32_t d;
            if (c >= '0' && c <= '9') d = (uint32_t)(c - '0');
            else if (c >= 'a' && c <= 'f') d = (uint32_t)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') d = (uint32_t)(c - 'A' + 10);
            else return false;
            out = out * 16u + d;
        }
        p_ += 4;
        return true;
    }

    atx_status string(std::string& s)
    {
        ++p_;   // opening quote
        for (;;) {
            if (p_ >= end_) return err("unterminated string");
            const unsigned char c = (unsigned char)*p_;
            if (c == '"') {
                ++p_;
                return ATX_OK;
            }
            if (c < 0x20) return err("control character in string");
            if (c != '\\') {
                s += (char)c;
                ++p_;
                continue;
            }
            ++p_;
            if (p_ >= end_) return err("unterminated escape");
            const char e = *p_++;
            switch (e) {
            case '"': s += '"'; break;
            case '\\': s += '\\'; break;
            case '/': s += '/'; break;
            case 'b': s += '\b'; break;
            case 'f': s += '\f'; break;
            case 'n': s += '\n'; break;
            case 'r': s += '\r'; break;
            case 't': s += '\t'; break;
            case 'u': {
                uint32_t cp;
                if (!hex4(cp)) return err("invalid \\u escape");
                if (cp >= 0xD800 && cp <= 0xDBFF) {
                    uint32_t lo;
                    if (end_ - p_ < 2 || p_[0] != '\\' || p_[1] != 'u') return err("unpaired surrogate");
                    p_ += 2;
                    if (!hex4(lo) || lo < 0xDC00 || lo > 0xDFFF) return err("invalid low surrogate");
                    cp = 0x10000u + ((cp - 0xD800u) << 10) + (lo - 0xDC00u);
                } else if (cp >= 0xDC00 && cp <= 0xDFFF) {
                    return err("unpaired surrogate");
                }
                put_utf8(s, cp);
                break;
            }
            default: return err("invalid escape");
            }
        }
    }

    atx_status number(JVal& v)
    {
        const char* s = p_;
        const char* q = p_;
        bool is_float = false;
        if (q < end_ && *q == '-') ++q;
        if (q >= end_ || *q < '0' || *q > '9') return err("invalid value");
        if (*q == '0') {
            ++q;
        } else {
            while (q < end_ && *q >= '0' && *q <= '9') ++q;
        }
        if (q < end_ && *q == '.') {
            is_float = true;
            ++q;
            if (q >= end_ || *q < '0' || *q > '9') return err("invalid number");
            while (q < end_ && *q >= '0' && *q <= '9') ++q;
        }
        if (q < end_ && (*q == 'e' || *q == 'E')) {
            is_float = true;
            ++q;
            if (q < end_ && (*q == '+' || *q == '-')) ++q;
            if (q >= end_ || *q < '0' || *q > '9') return err("invalid number");
            while (q < end_ && *q >= '0' && *q <= '9') ++q;
        }
        if (!is_float) {
            int64_t iv = 0;
            const auto r = std::from_chars(s, q, iv);
            if (r.ec == std::errc() && r.ptr == q) {
                v.type = JVal::Int;
                v.i = iv;
                p_ = q;
                return ATX_OK;
            }
        }
        double dv = 0.0;
        const auto r = std::from_chars(s, q, dv);
        if (r.ptr != q || (r.ec != std::errc() && r.ec != std::errc::result_out_of_range))
            return err("invalid number");
        v.type = JVal::Float;
        v.d = dv;
        p_ = q;
        return ATX_OK;
    }

    const char* p_;
    const char* end_;
    const char* begin_;
};

// ------------------------------------------------------------ writer

void put_exponent(std::string& out, int e)
{
    out += (e < 0) ? '-' : '+';
    if (e < 0) e = -e;
    char b[8];
    if (e < 10) {
        std::snprintf(b, sizeof b, "0%d", e);
    } else {
        std::snprintf(b, sizeof b, "%d", e);
    }
    out += b;
}

// The shortest decimal that reads back to v, laid out as json::dump does.
void put_double(std::string& out, double v)
{
    if (!std::isfinite(v)) {
        out += "null";
        return;
    }
    if (v == 0.0) {
        out += std::signbit(v) ? "-0.0" : "0.0";
        return;
    }
    if (v < 0) {
        out += '-';
        v = -v;
    }
    char buf[64];
    const auto r = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::scientific);
    // buf = d[.ddd]e[+-]XX: digits D (k of them) and decimal point position n
    // with v = 0.D * 10^n
    std::string digits;
    const char* q = buf;
    for (; q < r.ptr && *q != 'e'; ++q)
        if (*q != '.') digits += *q;
    int e10 = 0;
    std::from_chars(*(q + 1) == '+' ? q + 2 : q + 1, r.ptr, e10);
    const int k = (int)digits.size();
    const int n = e10 + 1;
    constexpr int kMinExp = -4, kMaxExp = 15;
    if (k <= n && n <= kMaxExp) {
        out += digits;
        out.append((size_t)(n - k), '0');
        out += ".0";
    } else if (0 < n && n <= kMaxExp) {
        out += digits.substr(0, (size_t)n);
        out += '.';
        out += digits.substr((size_t)n);
    } else if (kMinExp < n && n <= 0) {
        out += "0.";
        out.append((size_t)(-n), '0');
        out += digits;
    } else {
        out += digits[0];
        if (k > 1) {
            out += '.';
            out += digits.substr(1);
        }
        out += 'e';
        put_exponent(out, n - 1);
    }
}

void put_string(std::string& out, const std::string& s)
{
    out += '"';
    for (const char ch : s) {
        const unsigned char c = (unsigned char)ch;
        switch (c) {
        case '"': out += "\\\""; break;
        case '\\': out += "\\\\"; break;
        case '\b': out += "\\b"; break;
        case '\f': out += "\\f"; break;
        case '\n': out += "\\n"; break;
        case '\r': out += "\\r"; break;
        case '\t': out += "\\t"; break;
        default:
            if (c < 0x20) {
                char b[8];
                std::snprintf(b, sizeof b, "\\u%04x", (unsigned)c);
                out += b;
            } else {
                out += (char)c;
            }
        }
    }
    out += '"';
}

// A small ordered tree for the writer: objects keep their keys sorted, as
// nlohmann's default std::map-backed object does.
struct WVal {
    enum Type { Num, Int, Bool, Str, Arr, Obj } type = Obj;
    double d = 0.0;
    int64_t i = 0;
    bool b = false;
    std::string s;
    std::vector<WVal> a;
    std::vector<std::pair<std::string, WVal>> o;

    static WVal num(double v) { WVal w; w.type = Num; w.d = v; return w; }
    static WVal integer(int64_t v) { WVal w; w.type = Int; w.i = v; return w; }
    static WVal boolean(bool v) { WVal w; w.type = Bool; w.b = v; return w; }
    static WVal str(const std::string& v) { WVal w; w.type = Str; w.s = v; return w; }
    static WVal arr() { WVal w; w.type = Arr; return w; }
    static WVal vec(const float* p, int n)
    {
        WVal w = arr();
        for (int k = 0; k < n; ++k) w.a.push_back(num((double)p[k]));
        return w;
    }
    WVal& set(const std::string& key, WVal v)
    {
        type = Obj;
        auto it = o.begin();
        while (it != o.end() && it->first < key) ++it;
        if (it != o.end() && it->first == key) {
            it->second = std::move(v);
            return it->second;
        }
        return o.insert(it, {key, std::move(v)})->second;
    }
};

void dump(std::string& out, const WVal& v, int level)
{
    const std::string pad((size_t)(4 * (level + 1)), ' ');
    const std::string pad0((size_t)(4 * level), ' ');
    switch (v.type) {
    case WVal::Num: put_double(out, v.d); break;
    case WVal::Int: out += std::to_string(v.i); break;
    case WVal::Bool: out += v.b ? "true" : "false"; break;
    case WVal::Str: put_string(out, v.s); break;
    case WVal::Arr:
        if (v.a.empty()) {
            out += "[]";
            break;
        }
        out += "[\n";
        for (size_t k = 0; k < v.a.size(); ++k) {
            out += pad;
            dump(out, v.a[k], level + 1);
            out += (k + 1 < v.a.size()) ? ",\n" : "\n";
        }
        out += pad0;
        out += ']';
        break;
    case WVal::Obj:
        if (v.o.empty()) {
            out += "{}";
            break;
        }
        out += "{\n";
        for (size_t k = 0; k < v.o.size(); ++k) {
            out += pad;
            put_string(out, v.o[k].first);
            out += ": ";
            dump(out, v.o[k].second, level + 1);
            out += (k + 1 < v.o.size()) ? ",\n" : "\n";
        }
        out += pad0;
        out += '}';
        break;
    }
}

// ------------------------------------------------------- schema reading

struct Reader {
    std::string path;   // for messages

    atx_status missing(const char* what) const
    {
        return fail(ATX_ERR_PARSE, "scene json: %s%s: missing or of the wrong type", path.c_str(), what);
    }
    const JVal* field(const JVal& obj, const char* key) const { return obj.get(key); }

    atx_status f32(const JVal& obj, const char* key, float& out) const
    {
        const JVal* v = obj.get(key);
        if (!v || !v->is_num()) return missing(key);
        out = (v->type == JVal::Int) ? (float)v->i : (float)v->d;
        return ATX_OK;
    }
    atx_status i32(const JVal& obj, const char* key, int32_t& out) const
    {
        const JVal* v = obj.get(key);
        if (!v || !v->is_num()) return missing(key);
        out = (v->type == JVal::Int) ? (int32_t)v->i : (int32_t)v->d;   // json::get<int> truncates
        return ATX_OK;
    }
    atx_status boolean(const JVal& obj, const char* key, bool& out) const
    {
        const JVal* v = obj.get(key);
        if (!v || v->type != JVal::Bool) return missing(key);
        out = v->b;
        return ATX_OK;
    }
    atx_status vec(const JVal& obj, const char* key, float* out, int n) const
    {
        const JVal* v = obj.get(key);
        if (!v || v->type != JVal::Arr || (int)v->a.size() < n) return missing(key);
        for (int k = 0; k < n; ++k) {
            const JVal& e = v->a[(size_t)k];
            if (!e.is_num()) return missing(key);
            out[k] = (e.type == JVal::Int) ? (float)e.i : (float)e.d;
        }
        return ATX_OK;
    }
};

atx_status read_node(const JVal& j, SceneGraph& g, uint32_t idx)
{
    Reader rd{"sceneGraph node: "};
    if (j.type != JVal::Obj) return rd.missing("node");
    GraphNode& n = g.nodes[idx];
    if (idx != 0) {   // the root keeps the name Scene() gave it (Utils.cpp:141-142)
        const JVal* name = j.get("name");
        if (!name || name->type != JVal::Str) return rd.missing("name");
        n.name = name->s;
    }
    const JVal* tr = j.get("transformation");
    if (!tr || tr->type != JVal::Obj) return rd.missing("transformation");
    ATX_TRY(rd.vec(*tr, "position", n.position, 3));
    ATX_TRY(rd.vec(*tr, "rotation", n.rotation, 4));   // stored x, y, z, w (Utils.cpp:143)
    ATX_TRY(rd.vec(*tr, "scale", n.scale, 3));
    if (const JVal* sp = j.get("spheres")) {
        if (sp->type != JVal::Arr && sp->type != JVal::Null) return rd.missing("spheres");
        for (const JVal& s : sp->a) {
            if (s.type != JVal::Obj) return rd.missing("spheres[]");
            atx_sphere out{};
            ATX_TRY(rd.vec(s, "center", out.center, 3));
            ATX_TRY(rd.f32(s, "radius", out.radius));
            ATX_TRY(rd.i32(s, "materialIndex", out.material));
            g.nodes[idx].spheres.push_back(out);
        }
    }
    if (const JVal* ch = j.get("children")) {
        if (ch->type != JVal::Arr && ch->type != JVal::Null) return rd.missing("children");
        for (const JVal& c : ch->a) {
            const uint32_t k = g.add_node(idx, "");
            if (k == kNoNode) return fail(ATX_ERR_PARSE, "scene json: scene graph nested too deeply");
            ATX_TRY(read_node(c, g, k));
        }
    }
    return ATX_OK;
}

// --------------------------------------------------------------- math

Mat4 identity()
{
    Mat4 r;
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) r.m[c][k] = (c == k) ? 1.0f : 0.0f;
    return r;
}

// m * v as (c0*v0 + c1*v1) + (c2*v2 + c3*v3)
void mat4_vec4(const Mat4& a, const float v[4], float out[4])
{
    for (int k = 0; k < 4; ++k) {
        const float p0 = a.m[0][k] * v[0];
        const float p1 = a.m[1][k] * v[1];
        const float p2 = a.m[2][k] * v[2];
        const float p3 = a.m[3][k] * v[3];
        out[k] = (p0 + p1) + (p2 + p3);
    }
}

float length3(const float* c)
{
    const float xx = c[0] * c[0];
    const float yy = c[1] * c[1];
    const float zz = c[2] * c[2];
    return std::sqrt((xx + yy) + zz);
}

void flatten_node(const SceneGraph& g, uint32_t idx, const Mat4& parent, std::vector<atx_sphere>& out)
{
    const GraphNode& n = g.nodes[idx];
    const Mat4 global = mat4_mul(parent, node_local_matrix(n));   // SceneNode.cpp:44-47
    const float scale = ((length3(global.m[0]) + length3(global.m[1])) + length3(global.m[2])) / 3.0f;
    for (const atx_sphere& s : n.spheres) {                        // Renderer.cu:75-89
        atx_sphere t = s;
        const float c[4] = {s.center[0], s.center[1], s.center[2], 1.0f};
        float w[4];
        mat4_vec4(global, c, w);
        t.center[0] = w[0] / w[3];
        t.center[1] = w[1] / w[3];
        t.center[2] = w[2] / w[3];
        t.radius = s.radius * scale;
        if ((uint32_t)t.material >= g.materials.size()) t.material = 0;   // Renderer.cu:30-37
        out.push_back(t);
    }
    for (const uint32_t c : n.children) flatten_node(g, c, global, out);   // Renderer.cu:91-94
}

}  // namespace

Mat4 mat4_mul(const Mat4& a, const Mat4& b)
{
    Mat4 r;
    for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) {
            float s = a.m[0][k] * b.m[c][0];
            s = s + a.m[1][k] * b.m[c][1];
            s = s + a.m[2][k] * b.m[c][2];
            s = s + a.m[3][k] * b.m[c][3];
            r.m[c][k] = s;
        }
    return r;
}

Mat4 node_local_matrix(const GraphNode& n)
{
    const Mat4 I = identity();
    // translate(I, p): column 3 = ((I0*px + I1*py) + I2*pz) + I3
    Mat4 T = I;
    for (int k = 0; k < 4; ++k) {
        float s = I.m[0][k] * n.position[0];
        s = s + I.m[1][k] * n.position[1];
        s = s + I.m[2][k] * n.position[2];
        T.m[3][k] = s + I.m[3][k];
    }
    // mat4_cast(q), the rotation matrix of q = (w; x, y, z), not normalised
    const float x = n.rotation[0], y = n.rotation[1], z = n.rotation[2], w = n.rotation[3];
    const float xx = x * x, yy = y * y, zz = z * z;
    const float xz = x * z, xy = x * y, yz = y * z;
    const float wx = w * x, wy = w * y, wz = w * z;
    Mat4 R = I;
    R.m[0][0] = 1.0f - 2.0f * (yy + zz);
    R.m[0][1] = 2.0f * (xy + wz);
    R.m[0][2] = 2.0f * (xz - wy);
    R.m[1][0] = 2.0f * (xy - wz);
    R.m[1][1] = 1.0f - 2.0f * (xx + zz);
    R.m[1][2] = 2.0f * (yz + wx);
    R.m[2][0] = 2.0f * (xz + wy);
    R.m[2][1] = 2.0f * (yz - wx);
    R.m[2][2] = 1.0f - 2.0f * (xx + yy);
    // scale(I, s): columns 0-2 scaled
    Mat4 S = I;
    for (int c = 0; c < 3; ++c)
        for (int k = 0; k < 4; ++k) S.m[c][k] = I.m[c][k] * n.scale[c];
    return mat4_mul(mat4_mul(T, R), S);
}

// ============================================================ SceneGraph

SceneGraph::SceneGraph()
{
    nodes.emplace_back();
    nodes[0].name = "Scene";
    camera = atx_camera{{0.0f, 0.0f, 3.0f}, {0.0f, 0.0f, -1.0f}, 45.0f, 0.1f, 100.0f};
    settings = atx_settings{1, 0, {0, 0}, 15};
}

uint32_t SceneGraph::add_node(uint32_t parent, const char* name)
{
    if (parent >= nodes.size() || nodes[parent].depth + 1 > kMaxNodeDepth) return kNoNode;
    const uint32_t k = (uint32_t)nodes.size();
    nodes.emplace_back();
    nodes.back().name = name ? name : "";
    nodes.back().depth = nodes[parent].depth + 1;
    nodes[parent].children.push_back(k);
    return k;
}

atx_status SceneGraph::parse(const char* text, size_t len)
{
    JVal j;
    Parser p(text, len);
    ATX_TRY(p.parse(j));
    Reader rd{""};
    if (j.type != JVal::Obj) return fail(ATX_ERR_PARSE, "scene json: the document is not an object");
    SceneGraph g;
    // camera (Utils.cpp:101-103); near and far keep the Camera defaults
    const JVal* cam = j.get("camera");
    if (!cam || cam->type != JVal::Obj) return rd.missing("camera");
    rd.path = "camera.";
    ATX_TRY(rd.vec(*cam, "position", g.camera.position, 3));
    ATX_TRY(rd.vec(*cam, "direction", g.camera.direction, 3));
    ATX_TRY(rd.f32(*cam, "fov", g.camera.fov_deg));
    // scene graph (Utils.cpp:105-109)
    if (const JVal* sg = j.get("sceneGraph")) ATX_TRY(read_node(*sg, g, 0));
    // materials (Utils.cpp:111-121): a missing list reads as empty
    rd.path = "materials[].";
    if (const JVal* ms = j.get("materials")) {
        if (ms->type != JVal::Arr && ms->type != JVal::Null) return rd.missing("");
        for (const JVal& m : ms->a) {
            if (m.type != JVal::Obj) return rd.missing("");
            atx_material out{};
            ATX_TRY(rd.vec(m, "albedo", out.albedo, 3));
            ATX_TRY(rd.f32(m, "roughness", out.roughness));
            ATX_TRY(rd.f32(m, "metallic", out.metallic));
            ATX_TRY(rd.vec(m, "F0", out.f0, 3));
            ATX_TRY(rd.f32(m, "emissionIntensity", out.emission_intensity));
            ATX_TRY(rd.vec(m, "emissionColor", out.emission_color, 3));
            out.id = 0;   // not stored in the file; Material::id defaults to 0
            g.materials.push_back(out);
        }
    }
    // lights (Utils.cpp:123-130)
    rd.path = "lights[].";
    if (const JVal* ls = j.get("lights")) {
        if (ls->type != JVal::Arr && ls->type != JVal::Null) return rd.missing("");
        for (const JVal& l : ls->a) {
            if (l.type != JVal::Obj) return rd.missing("");
            atx_light out{};
            ATX_TRY(rd.vec(l, "position", out.position, 3));
            ATX_TRY(rd.f32(l, "intensity", out.intensity));
            ATX_TRY(rd.vec(l, "color", out.color, 3));
            g.lights.push_back(out);
        }
    }
    // settings (Utils.cpp:132-134)
    const JVal* st = j.get("settings");
    rd.path = "settings.";
    if (!st || st->type != JVal::Obj) return rd.missing("");
    int32_t mb = 0;
    bool sky = false, acc = false;
    ATX_TRY(rd.i32(*st, "maxBounces", mb));
    ATX_TRY(rd.boolean(*st, "skyLight", sky));
    ATX_TRY(rd.boolean(*st, "accumulation", acc));
    g.settings.max_bounces = mb;
    g.settings.sky_light = sky ? 1 : 0;
    g.settings.accumulation = acc ? 1 : 0;
    *this = std::move(g);
    return ATX_OK;
}

namespace {

WVal node_json(const SceneGraph& g, uint32_t idx)   // Utils.cpp:64-95
{
    const GraphNode& n = g.nodes[idx];
    WVal j;
    j.set("name", WVal::str(n.name));
    WVal tr;
    tr.set("position", WVal::vec(n.position, 3));
    tr.set("rotation", WVal::vec(n.rotation, 4));
    tr.set("scale", WVal::vec(n.scale, 3));
    j.set("transformation", std::move(tr));
    if (!n.spheres.empty()) {
        WVal sp = WVal::arr();
        for (const atx_sphere& s : n.spheres) {
            WVal o;
            o.set("center", WVal::vec(s.center, 3));
            o.set("radius", WVal::num((double)s.radius));
            o.set("materialIndex", WVal::integer(s.material));
            sp.a.push_back(std::move(o));
        }
        j.set("spheres", std::move(sp));
    }
    if (!n.children.empty()) {
        WVal ch = WVal::arr();
        for (const uint32_t c : n.children) ch.a.push_back(node_json(g, c));
        j.set("children", std::move(ch));
    }
    return j;
}

}  // namespace

std::string SceneGraph::to_json() const
{
    WVal j;
    WVal cam;
    cam.set("position", WVal::vec(camera.position, 3));
    cam.set("direction", WVal::vec(camera.direction, 3));
    cam.set("fov", WVal::num((double)camera.fov_deg));
    j.set("camera", std::move(cam));
    j.set("sceneGraph", node_json(*this, 0));
    if (!materials.empty()) {
        WVal ms = WVal::arr();
        for (const atx_material& m : materials) {
            WVal o;
            o.set("albedo", WVal::vec(m.albedo, 3));
            o.set("roughness", WVal::num((double)m.roughness));
            o.set("metallic", WVal::num((double)m.metallic));
            o.set("F0", WVal::vec(m.f0, 3));
            o.set("emissionIntensity", WVal::num((double)m.emission_intensity));
            o.set("emissionColor", WVal::vec(m.emission_color, 3));
            ms.a.push_back(std::move(o));
        }
        j.set("materials", std::move(ms));
    }
    if (!lights.empty()) {
        WVal ls = WVal::arr();
        for (const atx_light& l : lights) {
            WVal o;
            o.set("position", WVal::vec(l.position, 3));
            o.set("intensity", WVal::num((double)l.intensity));
            o.set("color", WVal::vec(l.color, 3));
            ls.a.push_back(std::move(o));
        }
        j.set("lights", std::move(ls));
    }
    WVal st;
    st.set("maxBounces", WVal::integer(settings.max_bounces));
    st.set("skyLight", WVal::boolean(settings.sky_light != 0));
    st.set("accumulation", WVal::boolean(settings.accumulation != 0));
    j.set("settings", std::move(st));
    std::string out;
    dump(out, j, 0);
    return out;
}

void SceneGraph::flatten(std::vector<atx_sphere>& out) const
{
    out.clear();
    out.reserve(sphere_count());
    flatten_node(*this, 0, identity(), out);
}

size_t SceneGraph::sphere_count() const
{
    size_t n = 0;
    for (const GraphNode& g : nodes) n += g.spheres.size();
    return n;
}

}  // namespace atx
