// xml_scene.cpp — Scene::load (src/core/Scene.cpp:58-127) for the scene XML
// format, with the model and material conventions of the reference:
//   * <integrator><size width height/></integrator>, <sampler type="sobol"/>,
//     <camera><position/><angle/><fov/><lensRadius/><focalDistance/></camera>
//     (Scene.cpp:69-111), <modelInstances> (:112-122), <envMap path/> (:123-125);
//   * a model instance's matrix is translate * scale * rotX(+90 deg) *
//     rotZ(rx) * rotX(ry) * rotY(rz) (Model.cpp:6, :62-71); normals go through
//     transpose(inverse(mat3(model))) and are normalised (Scene.cpp:153-162);
//   * type="light" instances carry <radiance value/> = total power
//     (Scene.cpp:39-45, :235); other instances take the <material> of
//     MaterialLoader.cpp:5-68 for all their meshes ("default" keeps
//     Material's defaults).
// The reference imports meshes with assimp and images with stb_image, which
// are not part of this library: meshes are read from Wavefront OBJ files (v, vt,
// vn, f with fan triangulation, flipped texcoords, identical corners joined,
// smooth area-weighted normals when the file has none, mtllib / usemtl
// material slots with Kd and map_Kd), albedo textures from PPM or BMP files
// and the environment from a PFM float image.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "scene.h"
#include "zgl_internal.h"

namespace zgl {
namespace {

// ------------------------------------------------------------- tiny XML DOM
struct XmlNode {
    std::string name;
    std::map<std::string, std::string> attrs;
    std::vector<std::unique_ptr<XmlNode>> children;
    const XmlNode* child(const std::string& n) const {
        for (auto& c : children)
            if (c->name == n) return c.get();
        return nullptr;
    }
    std::string attr(const std::string& n) const {
        auto it = attrs.find(n);
        return it == attrs.end() ? std::string() : it->second;
    }
};

class XmlParser {
public:
    explicit XmlParser(const std::string& text) : s_(text) {}

    std::unique_ptr<XmlNode> parse() {
        auto root = std::make_unique<XmlNode>();
        root->name = "#document";
        while (true) {
            skip_misc();
            if (pos_ >= s_.size()) break;
            if (s_[pos_] != '<') fail(ZGL_ERR_PARSE, "XML: text outside the root element at byte %zu", pos_);
            root->children.push_back(element());
        }
        return root;
    }

private:
    void skip_ws() {
        while (pos_ < s_.size() && std::isspace((unsigned char)s_[pos_])) pos_++;
    }
    bool starts(const char* p) const { return s_.compare(pos_, std::strlen(p), p) == 0; }
    void skip_misc() {
        for (;;) {
            skip_ws();
            if (starts("<?")) {
                size_t e = s_.find("?>", pos_);
                if (e == std::string::npos) fail(ZGL_ERR_PARSE, "XML: unterminated declaration");
                pos_ = e + 2;
            } else if (starts("<!--")) {
                size_t e = s_.find("-->", pos_);
                if (e == std::string::npos) fail(ZGL_ERR_PARSE, "XML: unterminated comment");
                pos_ = e + 3;
            } else if (starts("<!")) {
                size_t e = s_.find('>', pos_);
                if (e == std::string::npos) fail(ZGL_ERR_PARSE, "XML: unterminated markup");
                pos_ = e + 1;
            } else {
                return;
            }
        }
    }
    std::string name() {
        size_t b = pos_;
        while (pos_ < s_.size() && (std::isalnum((unsigned char)s_[pos_]) || s_[pos_] == '_' || s_[pos_] == '-' ||
                                    s_[pos_] == ':' || s_[pos_] == '.'))
            pos_++;
        if (b == pos_) fail(ZGL_ERR_PARSE, "XML: expected a name at byte %zu", pos_);
        return s_.substr(b, pos_ - b);
    }
    static std::string unescape(const std::string& v) {
        std::string o;
        for (size_t i = 0; i < v.size(); i++) {
            if (v[i] == '&') {
                size_t e = v.find(';', i);
                if (e != std::string::npos) {
                    std::string ent = v.substr(i + 1, e - i - 1);
                    if (ent == "amp") o += '&';
                    else if (ent == "lt") o += '<';
                    else if (ent == "gt") o += '>';
                    else if (ent == "quot") o += '"';
                    else if (ent == "apos") o += '\'';
                    else o += v.substr(i, e - i + 1);
                    i = e;
                    continue;
                }
            }
            o += v[i];
        }
        return o;
    }
    std::unique_ptr<XmlNode> element() {
        pos_++;  // '<'
        auto n = std::make_unique<XmlNode>();
        n->name = name();
        for (;;) {
            skip_ws();
            if (pos_ >= s_.size()) fail(ZGL_ERR_PARSE, "XML: unterminated tag <%s>", n->name.c_str());
            if (starts("/>")) {
                pos_ += 2;
                return n;
            }
            if (s_[pos_] == '>') {
                pos_++;
                break;
            }
            std::string a = name();
            skip_ws();
            if (pos_ >= s_.size() || s_[pos_] != '=') fail(ZGL_ERR_PARSE, "XML: attribute %s without value", a.c_str());
            pos_++;
            skip_ws();
            if (pos_ >= s_.size() || (s_[pos_] != '"' && s_[pos_] != '\''))
                fail(ZGL_ERR_PARSE, "XML: unquoted attribute %s", a.c_str());
            char q = s_[pos_++];
            size_t e = s_.find(q, pos_);
            if (e == std::string::npos) fail(ZGL_ERR_PARSE, "XML: unterminated attribute %s", a.c_str());
            n->attrs[a] = unescape(s_.substr(pos_, e - pos_));
            pos_ = e + 1;
        }
        for (;;) {
            // text content is ignored (the format keeps values in attributes)
            while (pos_ < s_.size() && s_[pos_] != '<') pos_++;
            if (pos_ >= s_.size()) fail(ZGL_ERR_PARSE, "XML: <%s> is not closed", n->name.c_str());
            if (starts("<!--") || starts("<?") || starts("<!")) {
                skip_misc();
                continue;
            }
            if (starts("</")) {
                pos_ += 2;
                std::string cn = name();
                if (cn != n->name) fail(ZGL_ERR_PARSE, "XML: </%s> closes <%s>", cn.c_str(), n->name.c_str());
                skip_ws();
                if (pos_ >= s_.size() || s_[pos_] != '>') fail(ZGL_ERR_PARSE, "XML: malformed closing tag");
                pos_++;
                return n;
            }
            n->children.push_back(element());
        }
    }

    const std::string& s_;
    size_t pos_ = 0;
};

// ------------------------------------------------------------- small math
struct M4 {
    float m[4][4];  // m[col][row], like glm
};
M4 identity() {
    M4 r{};
    for (int i = 0; i < 4; i++) r.m[i][i] = 1.0f;
    return r;
}
M4 mul(const M4& a, const M4& b) {
    M4 r{};
    for (int c = 0; c < 4; c++)
        for (int rr = 0; rr < 4; rr++) {
            float s = 0.0f;
            for (int k = 0; k < 4; k++) s += a.m[k][rr] * b.m[c][k];
            r.m[c][rr] = s;
        }
    return r;
}
// rotation by `angle` radians about the unit axis (Rodrigues), as glm::rotate
M4 rotation(float angle, float ax, float ay, float az) {
    float len = std::sqrt(ax * ax + ay * ay + az * az);
    ax /= len;
    ay /= len;
    az /= len;
    float c = std::cos(angle), s = std::sin(angle), t = 1.0f - c;
    M4 r = identity();
    r.m[0][0] = c + t * ax * ax;
    r.m[0][1] = t * ax * ay + s * az;
    r.m[0][2] = t * ax * az - s * ay;
    r.m[1][0] = t * ay * ax - s * az;
    r.m[1][1] = c + t * ay * ay;
    r.m[1][2] = t * ay * az + s * ax;
    r.m[2][0] = t * az * ax + s * ay;
    r.m[2][1] = t * az * ay - s * ax;
    r.m[2][2] = c + t * az * az;
    return r;
}
const float kRad = 0.01745329251994329576923690768489f;

M4 model_matrix(const float pos[3], const float scale[3], const float rot[3]) {  // Model.cpp:62-71
    M4 t = identity();
    t.m[3][0] = pos[0];
    t.m[3][1] = pos[1];
    t.m[3][2] = pos[2];
    M4 s = identity();
    s.m[0][0] = scale[0];
    s.m[1][1] = scale[1];
    s.m[2][2] = scale[2];
    M4 m = mul(t, s);
    m = mul(m, rotation(90.0f * kRad, 1, 0, 0));  // ConstRot (Model.cpp:6)
    m = mul(m, rotation(rot[0] * kRad, 0, 0, 1));
    m = mul(m, rotation(rot[1] * kRad, 1, 0, 0));
    m = mul(m, rotation(rot[2] * kRad, 0, 1, 0));
    return m;
}

void parse_floats(const std::string& s, float* out, int n, const float* dflt) {
    std::istringstream is(s);
    for (int i = 0; i < n; i++) {
        float v;
        if (is >> v) out[i] = v;
        else out[i] = dflt[i];
    }
}

// ------------------------------------------------------------- OBJ meshes
// One material slot of a model: an .mtl material (Kd, map_Kd) or the OBJ
// importer's default material (diffuse 0.6, no texture) for faces without a
// known `usemtl`.  assimp makes one aiMaterial per slot and one mesh per slot
// (Resource.cpp:81-89, :148-165).
struct ObjSlot {
    std::string name;
    float kd[3] = {0.6f, 0.6f, 0.6f};
    std::string mapKd;  // path relative to the model file, "" = none
};

struct Mesh {
    std::vector<float> v, n, uv;  // 3, 3 and 2 per joined corner
    std::vector<uint32_t> idx;
    std::vector<int32_t> slot;    // per triangle
    std::vector<ObjSlot> slots;   // in order of first use
};

std::string dir_of(const std::string& path) {
    size_t slash = path.find_last_of('/');
    return slash == std::string::npos ? std::string() : path.substr(0, slash + 1);
}

// newmtl / Kd / map_Kd of a Wavefront material library (other keys ignored)
void load_mtl(const std::string& path, std::map<std::string, ObjSlot>& lib) {
    std::ifstream f(path);
    if (!f) return;  // a missing library leaves the default material, as the importer does
    std::string line;
    ObjSlot* cur = nullptr;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::string tag;
        if (!(is >> tag) || tag[0] == '#') continue;
        if (tag == "newmtl") {
            std::string name;
            std::getline(is >> std::ws, name);
            while (!name.empty() && std::isspace((unsigned char)name.back())) name.pop_back();
            cur = &lib[name];
            cur->name = name;
        } else if (cur && tag == "Kd") {
            float r, g, b;
            if (is >> r >> g >> b) cur->kd[0] = r, cur->kd[1] = g, cur->kd[2] = b;
        } else if (cur && tag == "map_Kd") {
            std::string tok, last;  // options (-s, -o, ...) come first; the file name is last
            while (is >> tok) last = tok;
            cur->mapKd = last;
        }
    }
}

// Wavefront OBJ with the post-processing the reference asks of assimp
// (Resource.cpp:44-54): polygons fan-triangulated, texcoords flipped
// (v -> 1 - v, aiProcess_FlipUVs), identical (position, texcoord, normal)
// corners joined, smooth area-weighted normals when the file has none; faces
// grouped into material slots by `usemtl` / `mtllib`.
namespace {

// Cursor over one line of an OBJ file.
struct LineScan {
    const char* p;
    const char* end;
    void skip_ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) p++;
    }
    bool at_end() {
        skip_ws();
        return p >= end;
    }
    // next whitespace-delimited token
    std::string token() {
        skip_ws();
        const char* b = p;
        while (p < end && *p != ' ' && *p != '\t' && *p != '\r') p++;
        return std::string(b, p);
    }
    // the rest of the line, trimmed
    std::string rest() {
        skip_ws();
        const char* e = end;
        while (e > p && (e[-1] == ' ' || e[-1] == '\t' || e[-1] == '\r')) e--;
        return std::string(p, e);
    }
    // a float as istream >> float reads it (strtof)
    bool number(float& out) {
        skip_ws();
        if (p >= end) return false;
        char buf[64];
        const char* b = p;
        while (p < end && *p != ' ' && *p != '\t' && *p != '\r') p++;
        size_t len = std::min<size_t>((size_t)(p - b), sizeof(buf) - 1);
        std::memcpy(buf, b, len);
        buf[len] = '\0';
        char* stop = nullptr;
        out = std::strtof(buf, &stop);
        return stop != buf && *stop == '\0';
    }
};

// one index of a face corner ("" = absent); false on a malformed number
bool corner_index(const char* b, const char* e, long& out) {
    out = 0;
    if (b == e) return true;
    bool neg = false;
    if (*b == '-' || *b == '+') {
        neg = *b == '-';
        b++;
    }
    if (b == e) return false;
    long v = 0;
    for (; b < e; b++) {
        if (*b < '0' || *b > '9' || v > 100000000000l) return false;
        v = 10 * v + (*b - '0');
    }
    out = neg ? -v : v;
    return true;
}

}  // namespace

Mesh load_obj(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) fail(ZGL_ERR_PARSE, "cannot open model '%s'", path.c_str());
    const std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    std::vector<float> P, N, T;
    std::map<std::string, ObjSlot> lib;
    std::map<std::string, int32_t> slotOf;
    Mesh m;
    // joined corners: per position a chain of its (texcoord, normal) variants
    std::vector<int32_t> head;  // per position: first corner id or -1
    std::vector<int32_t> next;  // per corner: next corner of the same position
    std::vector<std::tuple<long, long, long>> keys;
    int32_t cur = -1;
    auto slot_for = [&](const std::string& name) {
        auto it = slotOf.find(name);
        if (it != slotOf.end()) return it->second;
        ObjSlot sl;
        auto lt = lib.find(name);
        if (lt != lib.end()) sl = lt->second;
        sl.name = name;
        m.slots.push_back(sl);
        return slotOf[name] = (int32_t)m.slots.size() - 1;
    };
    std::vector<uint32_t> poly;
    size_t lineno = 0;
    const char* q = text.data();
    const char* const qend = q + text.size();
    while (q < qend) {
        const char* eol = static_cast<const char*>(std::memchr(q, '\n', (size_t)(qend - q)));
        if (!eol) eol = qend;
        LineScan ls{q, eol};
        q = eol + 1;
        lineno++;
        if (ls.at_end() || *ls.p == '#') continue;
        const std::string tag = ls.token();
        if (tag == "v") {
            float x, y, z;
            if (!ls.number(x) || !ls.number(y) || !ls.number(z))
                fail(ZGL_ERR_PARSE, "%s:%zu: bad vertex", path.c_str(), lineno);
            P.insert(P.end(), {x, y, z});
        } else if (tag == "vn") {
            float x, y, z;
            if (!ls.number(x) || !ls.number(y) || !ls.number(z))
                fail(ZGL_ERR_PARSE, "%s:%zu: bad normal", path.c_str(), lineno);
            N.insert(N.end(), {x, y, z});
        } else if (tag == "vt") {
            float u, v = 0.0f;
            if (!ls.number(u)) fail(ZGL_ERR_PARSE, "%s:%zu: bad texcoord", path.c_str(), lineno);
            ls.number(v);
            T.insert(T.end(), {u, 1.0f - v});
        } else if (tag == "mtllib") {
            while (!ls.at_end()) load_mtl(dir_of(path) + ls.token(), lib);
        } else if (tag == "usemtl") {
            cur = slot_for(ls.rest());
        } else if (tag == "f") {
            poly.clear();
            while (!ls.at_end()) {
                ls.skip_ws();
                const char* b = ls.p;
                while (ls.p < ls.end && *ls.p != ' ' && *ls.p != '\t' && *ls.p != '\r') ls.p++;
                const char* e = ls.p;
                const char* s1 = std::find(b, e, '/');
                const char* s2 = s1 == e ? e : std::find(s1 + 1, e, '/');
                long vi = 0, ti = 0, ni = 0;
                bool ok = s1 != b && corner_index(b, s1, vi);
                if (ok && s1 != e) ok = corner_index(s1 + 1, s2, ti);
                if (ok && s2 != e) ok = corner_index(s2 + 1, e, ni);
                if (!ok)
                    fail(ZGL_ERR_PARSE, "%s:%zu: bad face corner '%s'", path.c_str(), lineno,
                         std::string(b, e).c_str());
                const long nv = (long)P.size() / 3, nt = (long)T.size() / 2, nn = (long)N.size() / 3;
                if (vi < 0) vi += nv + 1;
                if (ti < 0) ti += nt + 1;
                if (ni < 0) ni += nn + 1;
                if (vi < 1 || vi > nv || ti < 0 || ti > nt || ni < 0 || ni > nn)
                    fail(ZGL_ERR_PARSE, "%s:%zu: face index out of range", path.c_str(), lineno);
                if (head.size() < (size_t)nv) head.resize((size_t)nv, -1);
                int32_t id = head[(size_t)vi - 1];
                while (id >= 0 && (std::get<1>(keys[(size_t)id]) != ti || std::get<2>(keys[(size_t)id]) != ni))
                    id = next[(size_t)id];
                if (id < 0) {
                    id = (int32_t)keys.size();
                    keys.emplace_back(vi, ti, ni);
                    next.push_back(head[(size_t)vi - 1]);
                    head[(size_t)vi - 1] = id;
                }
                poly.push_back((uint32_t)id);
            }
            if (poly.size() < 3) fail(ZGL_ERR_PARSE, "%s:%zu: face with fewer than 3 corners", path.c_str(), lineno);
            if (cur < 0) cur = slot_for("");
            for (size_t k = 1; k + 1 < poly.size(); k++) {
                m.idx.insert(m.idx.end(), {poly[0], poly[k], poly[k + 1]});
                m.slot.push_back(cur);
            }
        }
    }
    bool haveN = true;
    m.v.reserve(3 * keys.size());
    m.uv.reserve(2 * keys.size());
    for (auto& k : keys) {
        long vi = std::get<0>(k), ti = std::get<1>(k);
        m.v.insert(m.v.end(), {P[3 * (vi - 1)], P[3 * (vi - 1) + 1], P[3 * (vi - 1) + 2]});
        if (ti > 0) m.uv.insert(m.uv.end(), {T[2 * (ti - 1)], T[2 * (ti - 1) + 1]});
        else m.uv.insert(m.uv.end(), {0.0f, 0.0f});
        if (std::get<2>(k) == 0) haveN = false;
    }
    m.n.assign(m.v.size(), 0.0f);
    if (haveN) {
        for (size_t i = 0; i < keys.size(); i++)
            for (int c = 0; c < 3; c++) m.n[3 * i + c] = N[3 * (std::get<2>(keys[i]) - 1) + c];
    } else {
        // smooth normals: area-weighted face normals summed per position
        std::vector<float> acc(P.size(), 0.0f);
        for (size_t t = 0; t < m.idx.size() / 3; t++) {
            const float* a = &m.v[3 * m.idx[3 * t]];
            const float* b = &m.v[3 * m.idx[3 * t + 1]];
            const float* c = &m.v[3 * m.idx[3 * t + 2]];
            float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
            float fn[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            for (int j = 0; j < 3; j++) {
                float* sum = &acc[3 * (size_t)(std::get<0>(keys[m.idx[3 * t + j]]) - 1)];
                for (int c2 = 0; c2 < 3; c2++) sum[c2] += fn[c2];
            }
        }
        for (size_t i = 0; i < keys.size(); i++) {
            const float* sum = &acc[3 * (size_t)(std::get<0>(keys[i]) - 1)];
            float l = std::sqrt(sum[0] * sum[0] + sum[1] * sum[1] + sum[2] * sum[2]);
            for (int c = 0; c < 3; c++) m.n[3 * i + c] = l > 0.0f ? sum[c] / l : (c == 2 ? 1.0f : 0.0f);
        }
    }
    if (m.idx.empty()) fail(ZGL_ERR_PARSE, "model '%s' has no faces", path.c_str());
    return m;
}

// ------------------------------------------------------------- 8-bit images
// Albedo textures as 8-bit RGB, top row first (what stb_image returns for
// Image::createFromFile(path, Int8, 3), Image.cpp:10-32).  This library reads
// binary/ASCII PPM (P6/P3, maxval <= 255) and uncompressed 24/32-bit BMP;
// stb's PNG/JPEG/TGA decoders are not part of it.  Returns false when the
// file cannot be read, which leaves the mesh untextured as in
// Resource::addImage (Resource.cpp:24-35).
bool read_pnm_token(std::istream& f, long& out) {
    char c;
    while (f.get(c)) {
        if (c == '#') {
            std::string rest;
            std::getline(f, rest);
        } else if (!std::isspace((unsigned char)c)) {
            f.unget();
            return static_cast<bool>(f >> out);
        }
    }
    return false;
}

bool load_image_rgb8(const std::string& path, int& W, int& H, std::vector<uint8_t>& rgb) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    char m0 = 0, m1 = 0;
    f.get(m0);
    f.get(m1);
    if (m0 == 'P' && (m1 == '6' || m1 == '3')) {
        long w, h, maxv;
        if (!read_pnm_token(f, w) || !read_pnm_token(f, h) || !read_pnm_token(f, maxv)) return false;
        if (w <= 0 || h <= 0 || w > 16384 || h > 16384 || maxv <= 0 || maxv > 255) return false;
        W = (int)w;
        H = (int)h;
        rgb.assign((size_t)W * H * 3, 0);
        if (m1 == '6') {
            f.get();  // the single whitespace after maxval
            f.read(reinterpret_cast<char*>(rgb.data()), (std::streamsize)rgb.size());
            if (!f) return false;
        } else {
            for (auto& b : rgb) {
                long v;
                if (!read_pnm_token(f, v) || v < 0 || v > maxv) return false;
                b = (uint8_t)v;
            }
        }
        if (maxv != 255)
            for (auto& b : rgb) b = (uint8_t)((b * 255 + maxv / 2) / maxv);
        return true;
    }
    if (m0 == 'B' && m1 == 'M') {
        uint8_t hdr[52];
        f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
        if (!f) return false;
        auto u32 = [&](int o) { return (uint32_t)hdr[o] | ((uint32_t)hdr[o + 1] << 8) | ((uint32_t)hdr[o + 2] << 16) | ((uint32_t)hdr[o + 3] << 24); };
        auto u16 = [&](int o) { return (uint32_t)hdr[o] | ((uint32_t)hdr[o + 1] << 8); };
        uint32_t dataOff = u32(8);  // hdr[o] is file byte o + 2: bfOffBits, then BITMAPINFOHEADER
        int32_t w = (int32_t)u32(16), h = (int32_t)u32(20);
        uint32_t bpp = u16(26), comp = u32(28);
        if ((bpp != 24 && bpp != 32) || comp != 0 || w <= 0 || h == 0 || w > 16384 || h > 16384 || h < -16384)
            return false;
        bool topDown = h < 0;
        W = w;
        H = topDown ? -h : h;
        size_t stride = (((size_t)W * bpp / 8) + 3) & ~(size_t)3;
        std::vector<uint8_t> row(stride);
        rgb.assign((size_t)W * H * 3, 0);
        f.seekg(dataOff);
        for (int y = 0; y < H; y++) {
            f.read(reinterpret_cast<char*>(row.data()), (std::streamsize)stride);
            if (!f) return false;
            int dy = topDown ? y : H - 1 - y;
            for (int x = 0; x < W; x++) {
                const uint8_t* px = &row[(size_t)x * (bpp / 8)];
                uint8_t* o = &rgb[3 * ((size_t)dy * W + x)];
                o[0] = px[2];
                o[1] = px[1];
                o[2] = px[0];
            }
        }
        return true;
    }
    return false;
}

// PFM float image (bottom row first in the file); returned top row first.
std::vector<float> load_pfm(const std::string& path, int& W, int& H) {
    std::ifstream f(path, std::ios::binary);
    if (!f) fail(ZGL_ERR_PARSE, "cannot open environment map '%s'", path.c_str());
    std::string magic;
    double scale;
    f >> magic >> W >> H >> scale;
    f.get();
    if ((magic != "PF" && magic != "Pf") || W <= 0 || H <= 0 || (int64_t)W * H > (1ll << 28))
        fail(ZGL_ERR_PARSE, "'%s' is not a PFM image", path.c_str());
    int ch = magic == "PF" ? 3 : 1;
    std::vector<float> raw((size_t)W * H * ch);
    f.read(reinterpret_cast<char*>(raw.data()), (std::streamsize)(raw.size() * 4));
    if (!f) fail(ZGL_ERR_PARSE, "'%s' is truncated", path.c_str());
    if (scale > 0) {  // big-endian
        for (auto& v : raw) {
            uint32_t u;
            std::memcpy(&u, &v, 4);
            u = (u >> 24) | ((u >> 8) & 0xff00u) | ((u << 8) & 0xff0000u) | (u << 24);
            std::memcpy(&v, &u, 4);
        }
    }
    std::vector<float> rgb((size_t)W * H * 3);
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++)
            for (int c = 0; c < 3; c++)
                rgb[3 * ((size_t)(H - 1 - y) * W + x) + c] = raw[ch * ((size_t)y * W + x) + (ch == 3 ? c : 0)];
    return rgb;
}

std::string resolve_path(const std::string& base, const std::string& p) {
    if (p.empty() || p[0] == '/') return p;
    std::ifstream probe(p);
    if (probe) return p;  // relative to the working directory, like the reference
    size_t slash = base.find_last_of('/');
    return slash == std::string::npos ? p : base.substr(0, slash + 1) + p;
}

void material_from_xml(const XmlNode* node, float* out16, bool& useDefault) {
    // Material defaults (Material.h:32-53)
    float d[16] = {1, 1, 1, 1, 0, 0, 1, 1, 0, 1, 0, 0, 1.5f, 0, 0, 0};
    std::memcpy(out16, d, sizeof(d));
    int32_t type = 0;
    useDefault = false;
    std::string t = node ? node->attr("type") : std::string();
    auto val = [&](const char* n, float* dst, int cnt) {
        const XmlNode* c = node->child(n);
        if (!c) return;
        std::istringstream is(c->attr("value"));
        for (int i = 0; i < cnt; i++) {
            float v;
            if (is >> v) dst[i] = v;
        }
    };
    if (!node || t == "default") {
        useDefault = true;
    } else if (t == "principled") {
        val("baseColor", out16, 3);
        val("subsurface", out16 + 4, 1);
        val("metallic", out16 + 5, 1);
        val("roughness", out16 + 3, 1);
        val("specular", out16 + 6, 1);
        val("specularTint", out16 + 7, 1);
        val("sheen", out16 + 8, 1);
        val("sheenTint", out16 + 9, 1);
        val("clearcoat", out16 + 10, 1);
        val("clearcoatGloss", out16 + 11, 1);
        type = 1;
    } else if (t == "metalWorkflow") {
        val("baseColor", out16, 3);
        val("metallic", out16 + 5, 1);
        val("roughness", out16 + 3, 1);
        type = 2;
    } else if (t == "dielectric") {
        val("baseColor", out16, 3);
        val("ior", out16 + 12, 1);
        val("roughness", out16 + 3, 1);
        type = 3;
    } else if (t == "thinDielectric") {
        val("baseColor", out16, 3);
        val("ior", out16 + 12, 1);
        type = 4;
    } else if (t == "lambertian") {
        val("baseColor", out16, 3);
        type = 0;
    }
    std::memcpy(out16 + 13, &type, 4);
}

}  // namespace

// Parses the scene XML into world-space arrays and builds the scene.
zgl_scene* load_scene_xml(const std::string& path, int32_t flags) {
    std::ifstream f(path, std::ios::binary);
    if (!f) fail(ZGL_ERR_PARSE, "cannot open scene '%s'", path.c_str());
    std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    XmlParser parser(text);
    auto doc = parser.parse();
    const XmlNode* scene = doc->child("scene");
    if (!scene) fail(ZGL_ERR_PARSE, "'%s' has no <scene> element", path.c_str());

    zgl_scene_desc d{};
    const float zero3[3] = {0, 0, 0}, one3[3] = {1, 1, 1};
    if (const XmlNode* integ = scene->child("integrator"))
        if (const XmlNode* size = integ->child("size")) {
            d.film_width = std::atoi(size->attr("width").c_str());
            d.film_height = std::atoi(size->attr("height").c_str());
        }
    const XmlNode* sampler = scene->child("sampler");
    d.sampler = (sampler && sampler->attr("type") == "sobol") ? 1 : 0;
    if (const XmlNode* cam = scene->child("camera")) {
        auto get = [&](const char* n) { const XmlNode* c = cam->child(n); return c ? c->attr("value") : std::string(); };
        parse_floats(get("position"), d.cam_pos, 3, zero3);
        parse_floats(get("angle"), d.cam_angle, 3, zero3);
        d.cam_fov = (float)std::atof(get("fov").c_str());
        d.cam_lens_radius = (float)std::atof(get("lensRadius").c_str());
        d.cam_focal_dist = (float)std::atof(get("focalDistance").c_str());
    }
    std::vector<float> ov, on, ouv, lv, ln, lp, mats;
    std::vector<uint32_t> oi, li, lf{0};
    std::vector<int32_t> omt;
    // textures of the whole scene, one per distinct file (Resource::addImage)
    std::map<std::string, int32_t> texOf;
    std::vector<int32_t> texSize;
    std::vector<uint8_t> texRGB;
    auto add_image = [&](const std::string& file) -> int32_t {
        auto it = texOf.find(file);
        if (it != texOf.end()) return it->second;
        int W = 0, H = 0;
        std::vector<uint8_t> rgb;
        int32_t id = -1;
        if (load_image_rgb8(file, W, H, rgb)) {
            id = (int32_t)(texSize.size() / 2);
            texSize.insert(texSize.end(), {W, H});
            texRGB.insert(texRGB.end(), rgb.begin(), rgb.end());
        }
        return texOf[file] = id;
    };
    if (const XmlNode* insts = scene->child("modelInstances")) {
        for (auto& inst : insts->children) {
            const std::string objPath = resolve_path(path, inst->attr("path"));
            Mesh mesh = load_obj(objPath);
            float pos[3], scale[3], rot[3];
            const XmlNode* tr = inst->child("transform");
            parse_floats(tr ? tr->attr("translate") : "", pos, 3, zero3);
            parse_floats(tr ? tr->attr("scale") : "", scale, 3, one3);
            parse_floats(tr ? tr->attr("rotate") : "", rot, 3, zero3);
            M4 M = model_matrix(pos, scale, rot);
            // normal matrix = transpose(inverse(mat3(M)))
            float a[3][3];
            for (int c = 0; c < 3; c++)
                for (int r = 0; r < 3; r++) a[c][r] = M.m[c][r];
            float det = a[0][0] * (a[1][1] * a[2][2] - a[2][1] * a[1][2]) - a[1][0] * (a[0][1] * a[2][2] - a[2][1] * a[0][2]) +
                        a[2][0] * (a[0][1] * a[1][2] - a[1][1] * a[0][2]);
            if (det == 0.0f) fail(ZGL_ERR_INVALID_ARG, "model instance with a singular transform");
            float cof[3][3];  // cofactor matrix = transpose(inverse) * det
            cof[0][0] = a[1][1] * a[2][2] - a[2][1] * a[1][2];
            cof[0][1] = a[2][0] * a[1][2] - a[1][0] * a[2][2];
            cof[0][2] = a[1][0] * a[2][1] - a[2][0] * a[1][1];
            cof[1][0] = a[2][1] * a[0][2] - a[0][1] * a[2][2];
            cof[1][1] = a[0][0] * a[2][2] - a[2][0] * a[0][2];
            cof[1][2] = a[2][0] * a[0][1] - a[0][0] * a[2][1];
            cof[2][0] = a[0][1] * a[1][2] - a[1][1] * a[0][2];
            cof[2][1] = a[1][0] * a[0][2] - a[0][0] * a[1][2];
            cof[2][2] = a[0][0] * a[1][1] - a[1][0] * a[0][1];
            bool light = inst->attr("type") == "light";
            std::vector<float>& V = light ? lv : ov;
            std::vector<float>& Nn = light ? ln : on;
            uint32_t base = (uint32_t)(V.size() / 3);
            for (size_t i = 0; i < mesh.v.size() / 3; i++) {
                const float* p = &mesh.v[3 * i];
                for (int r = 0; r < 3; r++) V.push_back(M.m[0][r] * p[0] + M.m[1][r] * p[1] + M.m[2][r] * p[2] + M.m[3][r]);
                const float* q = &mesh.n[3 * i];
                float nn[3];
                for (int r = 0; r < 3; r++) nn[r] = (cof[0][r] * q[0] + cof[1][r] * q[1] + cof[2][r] * q[2]) / det;
                float l = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
                for (int r = 0; r < 3; r++) Nn.push_back(l > 0.0f ? nn[r] / l : 0.0f);
            }
            if (light) {
                for (uint32_t k : mesh.idx) li.push_back(base + k);
                lf.push_back((uint32_t)(li.size() / 3));
                float rad[3];
                const XmlNode* r = inst->child("radiance");
                parse_floats(r ? r->attr("value") : "", rad, 3, zero3);
                lp.insert(lp.end(), rad, rad + 3);
            } else {
                // one material per slot: the XML <material> for every slot
                // (Scene.cpp:47-53), else the slot's Kd on Material's
                // defaults; the slot's map_Kd texture either way
                float m16[16];
                bool dflt;
                material_from_xml(inst->child("material"), m16, dflt);
                const int32_t matBase = (int32_t)(mats.size() / 16);
                std::vector<int32_t> slotTex;
                for (const ObjSlot& sl : mesh.slots) {
                    float r[16];
                    std::memcpy(r, m16, sizeof(r));
                    if (dflt) std::memcpy(r, sl.kd, 3 * sizeof(float));
                    mats.insert(mats.end(), r, r + 16);
                    std::string tex = sl.mapKd;
                    if (!tex.empty() && tex[0] != '/') tex = dir_of(objPath) + tex;
                    slotTex.push_back(tex.empty() ? -1 : add_image(tex));
                }
                for (uint32_t k : mesh.idx) oi.push_back(base + k);
                ouv.insert(ouv.end(), mesh.uv.begin(), mesh.uv.end());
                for (size_t t = 0; t < mesh.idx.size() / 3; t++) {
                    const int32_t sl = mesh.slot[t];
                    omt.push_back((int32_t)(((uint32_t)slotTex[(size_t)sl] << 16) | (uint32_t)(matBase + sl)));
                }
            }
        }
    }
    std::vector<float> env;
    if (const XmlNode* e = scene->child("envMap")) {
        std::string p = e->attr("path");
        if (!p.empty()) {
            int W, H;
            env = load_pfm(resolve_path(path, p), W, H);
            d.env_width = W;
            d.env_height = H;
        }
    }
    d.obj_vertices = ov.data();
    d.obj_n_vertices = ov.size() / 3;
    d.obj_normals = on.data();
    d.obj_indices = oi.data();
    d.obj_n_triangles = oi.size() / 3;
    d.obj_mat_tex = omt.data();
    d.materials = mats.data();
    d.n_materials = mats.size() / 16;
    d.light_vertices = lv.data();
    d.light_n_vertices = lv.size() / 3;
    d.light_normals = ln.data();
    d.light_indices = li.data();
    d.light_n_triangles = li.size() / 3;
    d.light_first = lf.data();
    d.light_power = lp.data();
    d.n_light_instances = lp.size() / 3;
    d.env_rgb = env.empty() ? nullptr : env.data();
    d.obj_texcoords = ouv.empty() ? nullptr : ouv.data();
    d.n_textures = (int32_t)(texSize.size() / 2);
    d.tex_size = texSize.data();
    d.tex_rgb = texRGB.data();
    zgl_scene* out = nullptr;
    zgl_status st = zgl_scene_create(&d, flags, &out);
    if (st != ZGL_OK) throw Error{st};
    return out;
}

}  // namespace zgl

extern "C" zgl_status zgl_scene_load_xml(const char* path, int32_t flags, zgl_scene** out) {
    ZGL_API_BEGIN
    ZGL_RANGE("zgl_scene_load_xml");
    if (!path || !out) zgl::fail(ZGL_ERR_INVALID_ARG, "zgl_scene_load_xml: NULL argument");
    *out = nullptr;
    *out = zgl::load_scene_xml(path, flags);
    ZGL_API_END
}
