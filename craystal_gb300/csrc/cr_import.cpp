// cr_import.cpp -- Importer::import (Utils/Importer.cpp:203-236): an XML
// file with the camera and the emissive materials, next to an OBJ file of
// the same name holding the geometry and its MTL materials.
//
// The reference reads the XML with pugixml 1.15 and the OBJ/MTL with assimp
// 5.4.3 (post-processing Triangulate | GenNormals | CalcTangentSpace |
// JoinIdenticalVertices); neither library is used here.  What this file
// restates of them, because it decides the triangles, their order and the
// materials the path sees:
//   - the XML: the first top-level <camera> (attributes fovy, width,
//     height; children eye / lookat / up with x, y, z) and every top-level
//     <light mtlname=... radiance="r,g,b"> (Utils/Importer.cpp:17-78);
//   - assimp's OBJ parser: "DefaultMaterial" (diffuse 0.6) is material 0,
//     MTL materials follow in definition order and a usemtl of an unknown
//     name appends a default material of that name; o / g open an object
//     with a new mesh that takes the current material; usemtl opens a new
//     mesh only when the current one already has faces with another
//     material; meshes are emitted object by object and empty ones dropped;
//     numbers are parsed by assimp's fast_atof (integer digits, at most 15
//     fraction digits scaled by a power-of-ten table, then the exponent);
//     a single-number colour "Kd r" reads as (r, 0, 0);
//   - the post-processing: quads are split from their concave corner (or
//     corner 0) into (s, s+1, s+2), (s, s+2, s+3); a mesh without normals
//     gets flat face normals; corners equal in position, normal and
//     texture coordinates are joined in first-occurrence order.
// Differences, documented where they arise: polygons of more than four
// corners are fanned from corner 0 (assimp clips ears, which can choose
// other diagonals); only exactly equal corners are joined (assimp also
// joins corners closer than 1e-5); line and point elements are skipped.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "craystal_c.h"
#include "cr_io.h"

namespace cr {
namespace imp {

// ---------------------------------------------------------------------------
// assimp's fast_atof (include/assimp/fast_atof.h, 5.4.3) for ai_real = float
// ---------------------------------------------------------------------------
static const double kFracTable[16] = {0.0,  1e-1, 1e-2,  1e-3,  1e-4,  1e-5,  1e-6,  1e-7,
                                      1e-8, 1e-9, 1e-10, 1e-11, 1e-12, 1e-13, 1e-14, 1e-15};

// Decimal digits at c into an unsigned 64-bit value; with maxDigits set,
// stops counting after that many digits and skips the rest.
static uint64_t digits64(const char*& c, unsigned* maxDigits, bool& ok) {
    if (*c < '0' || *c > '9') {
        ok = false;
        return 0;
    }
    uint64_t v = 0;
    unsigned cur = 0;
    while (*c >= '0' && *c <= '9') {
        const uint64_t nv = v * 10u + (uint64_t)(*c - '0');
        if (nv < v) return 0;  // overflow: assimp returns 0
        v = nv;
        ++c;
        ++cur;
        if (maxDigits && *maxDigits == cur) {
            while (*c >= '0' && *c <= '9') ++c;
            return v;
        }
    }
    if (maxDigits) *maxDigits = cur;
    return v;
}

static bool iprefix(const char* c, const char* word) {
    for (; *word; ++c, ++word)
        if (std::tolower((unsigned char)*c) != *word) return false;
    return true;
}

// Returns false when the text does not start with a number.
bool fastAtof(const char* c, float& out) {
    float f = 0.0f;
    const bool inv = *c == '-';
    if (inv || *c == '+') ++c;
    if ((c[0] == 'n' || c[0] == 'N') && iprefix(c, "nan")) {
        out = NAN;
        return true;
    }
    if ((c[0] == 'i' || c[0] == 'I') && iprefix(c, "inf")) {
        out = inv ? -INFINITY : INFINITY;
        return true;
    }
    const bool digit0 = c[0] >= '0' && c[0] <= '9';
    if (!digit0 && !((c[0] == '.' || c[0] == ',') && c[1] >= '0' && c[1] <= '9')) return false;
    bool ok = true;
    if (*c != '.' && *c != ',') f = (float)digits64(c, nullptr, ok);
    if ((*c == '.' || *c == ',') && c[1] >= '0' && c[1] <= '9') {
        ++c;
        unsigned diff = 15;
        double pl = (double)digits64(c, &diff, ok);
        pl *= kFracTable[diff];
        f += (float)pl;
    } else if (*c == '.') {
        ++c;
    }
    if (*c == 'e' || *c == 'E') {
        ++c;
        const bool einv = *c == '-';
        if (einv || *c == '+') ++c;
        float e = (float)digits64(c, nullptr, ok);
        if (einv) e = -e;
        f *= std::pow(10.0f, e);
    }
    if (inv) f = -f;
    out = f;
    return ok;
}

// ---------------------------------------------------------------------------
// text helpers
// ---------------------------------------------------------------------------
static std::vector<std::string> splitWs(const std::string& s) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i < s.size()) {
        while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
        size_t j = i;
        while (j < s.size() && !std::isspace((unsigned char)s[j])) j++;
        if (j > i) out.push_back(s.substr(i, j - i));
        i = j;
    }
    return out;
}

static std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

// Lines of a text file; a backslash at the end of a line continues it.
static std::vector<std::string> textLines(const std::vector<uint8_t>& d) {
    std::vector<std::string> lines;
    std::string cur;
    for (size_t i = 0; i < d.size(); i++) {
        const char ch = (char)d[i];
        if (ch == '\n' || ch == '\r') {
            if (ch == '\r' && i + 1 < d.size() && d[i + 1] == '\n') i++;
            if (!cur.empty() && cur.back() == '\\') {
                cur.back() = ' ';
                continue;
            }
            lines.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(ch);
        }
    }
    if (!cur.empty()) lines.push_back(cur);
    return lines;
}

static std::string dirOf(const std::string& path) {
    const size_t s = path.find_last_of('/');
    return s == std::string::npos ? std::string() : path.substr(0, s + 1);
}

// ---------------------------------------------------------------------------
// XML (the subset a scene file uses: elements, attributes, comments,
// declarations; text content is ignored)
// ---------------------------------------------------------------------------
struct XmlNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XmlNode> children;
    const std::string* attr(const char* n) const {
        for (const auto& a : attrs)
            if (a.first == n) return &a.second;
        return nullptr;
    }
    const XmlNode* child(const char* n) const {
        for (const auto& c : children)
            if (c.name == n) return &c;
        return nullptr;
    }
};

class XmlParser {
   public:
    explicit XmlParser(const std::string& s) : s_(s) {}
    bool parseDocument(std::vector<XmlNode>& top, std::string& err) {
        while (true) {
            skipMisc();
            if (i_ >= s_.size()) return true;
            if (s_[i_] != '<') return failAt("text outside elements", err);
            XmlNode n;
            if (!parseElement(n, err)) return false;
            top.push_back(std::move(n));
        }
    }

   private:
    const std::string& s_;
    size_t i_ = 0;

    bool failAt(const char* why, std::string& err) {
        err = std::string("XML: ") + why + " at offset " + std::to_string(i_);
        return false;
    }
    void skipWs() {
        while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) i_++;
    }
    // whitespace, comments, <?...?> and <!...> declarations
    void skipMisc() {
        while (true) {
            skipWs();
            if (s_.compare(i_, 4, "<!--") == 0) {
                const size_t e = s_.find("-->", i_ + 4);
                i_ = e == std::string::npos ? s_.size() : e + 3;
            } else if (s_.compare(i_, 2, "<?") == 0) {
                const size_t e = s_.find("?>", i_ + 2);
                i_ = e == std::string::npos ? s_.size() : e + 2;
            } else if (s_.compare(i_, 2, "<!") == 0 && s_.compare(i_, 9, "<![CDATA[") != 0) {
                const size_t e = s_.find('>', i_ + 2);
                i_ = e == std::string::npos ? s_.size() : e + 1;
            } else {
                return;
            }
        }
    }
    static bool nameChar(char c) {
        return std::isalnum((unsigned char)c) || c == '_' || c == ':' || c == '-' || c == '.' || (unsigned char)c >= 0x80;
    }
    std::string name() {
        const size_t a = i_;
        while (i_ < s_.size() && nameChar(s_[i_])) i_++;
        return s_.substr(a, i_ - a);
    }
    static std::string unescape(const std::string& v) {
        std::string o;
        for (size_t k = 0; k < v.size(); k++) {
            if (v[k] != '&') {
                o.push_back(v[k]);
                continue;
            }
            const size_t e = v.find(';', k);
            if (e == std::string::npos) {
                o.push_back('&');
                continue;
            }
            const std::string ent = v.substr(k + 1, e - k - 1);
            if (ent == "lt") o.push_back('<');
            else if (ent == "gt") o.push_back('>');
            else if (ent == "amp") o.push_back('&');
            else if (ent == "quot") o.push_back('"');
            else if (ent == "apos") o.push_back('\'');
            else if (!ent.empty() && ent[0] == '#') {
                const long cp = ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X') ? std::strtol(ent.c_str() + 2, nullptr, 16)
                                                                                 : std::strtol(ent.c_str() + 1, nullptr, 10);
                if (cp < 0x80) {
                    o.push_back((char)cp);
                } else if (cp < 0x800) {
                    o.push_back((char)(0xC0 | (cp >> 6)));
                    o.push_back((char)(0x80 | (cp & 0x3F)));
                } else {
                    o.push_back((char)(0xE0 | ((cp >> 12) & 0x0F)));
                    o.push_back((char)(0x80 | ((cp >> 6) & 0x3F)));
                    o.push_back((char)(0x80 | (cp & 0x3F)));
                }
            } else {
                o += "&" + ent + ";";
            }
            k = e;
        }
        return o;
    }
    bool parseElement(XmlNode& n, std::string& err) {
        i_++;  // '<'
        n.name = name();
        if (n.name.empty()) return failAt("element name expected", err);
        while (true) {
            skipWs();
            if (i_ >= s_.size()) return failAt("unterminated tag", err);
            if (s_[i_] == '/') {
                if (s_.compare(i_, 2, "/>") != 0) return failAt("'/>' expected", err);
                i_ += 2;
                return true;
            }
            if (s_[i_] == '>') {
                i_++;
                break;
            }
            const std::string an = name();
            if (an.empty()) return failAt("attribute name expected", err);
            skipWs();
            if (i_ >= s_.size() || s_[i_] != '=') return failAt("'=' expected", err);
            i_++;
            skipWs();
            if (i_ >= s_.size() || (s_[i_] != '"' && s_[i_] != '\'')) return failAt("quoted value expected", err);
            const char q = s_[i_++];
            const size_t e = s_.find(q, i_);
            if (e == std::string::npos) return failAt("unterminated attribute value", err);
            n.attrs.emplace_back(an, unescape(s_.substr(i_, e - i_)));
            i_ = e + 1;
        }
        // content
        while (true) {
            if (i_ >= s_.size()) return failAt("unterminated element", err);
            if (s_.compare(i_, 9, "<![CDATA[") == 0) {
                const size_t e = s_.find("]]>", i_);
                if (e == std::string::npos) return failAt("unterminated CDATA", err);
                i_ = e + 3;
            } else if (s_.compare(i_, 4, "<!--") == 0 || s_.compare(i_, 2, "<?") == 0 ||
                       (s_.compare(i_, 2, "<!") == 0)) {
                skipMisc();
            } else if (s_.compare(i_, 2, "</") == 0) {
                i_ += 2;
                const std::string close = name();
                skipWs();
                if (close != n.name || i_ >= s_.size() || s_[i_] != '>') return failAt("mismatched end tag", err);
                i_++;
                return true;
            } else if (s_[i_] == '<') {
                XmlNode c;
                if (!parseElement(c, err)) return false;
                n.children.push_back(std::move(c));
            } else {
                i_++;  // text
            }
        }
    }
};

// pugixml's as_float / as_uint of a missing attribute is 0
static float xmlFloat(const XmlNode& n, const char* a) {
    const std::string* v = n.attr(a);
    return v ? (float)std::strtod(v->c_str(), nullptr) : 0.0f;
}
static uint32_t xmlUint(const XmlNode& n, const char* a) {
    const std::string* v = n.attr(a);
    if (!v) return 0;
    const char* c = v->c_str();
    while (std::isspace((unsigned char)*c)) c++;
    if (*c == '-') return 0;
    const unsigned long long x = std::strtoull(c, nullptr, 0);
    return x > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)x;
}

// ---------------------------------------------------------------------------
// OBJ / MTL model (assimp's ObjFile::Model)
// ---------------------------------------------------------------------------
constexpr uint32_t kNoMaterial = 0xFFFFFFFFu;

struct V3 {
    float x, y, z;
};

struct ObjMaterial {  // ObjFile::Material defaults
    std::string name;
    float kd[3] = {0.6f, 0.6f, 0.6f};
    float ks[3] = {0.0f, 0.0f, 0.0f};
    float alpha = 1.0f, shininess = 0.0f, ior = 1.0f;
    std::string mapKd;
};

struct ObjFace {
    std::vector<uint32_t> v, vt, vn;
};

struct ObjMesh {
    std::vector<ObjFace> faces;
    uint32_t material = kNoMaterial;
    bool hasNormals = false;
    size_t uvCount = 0;
};

struct ObjModel {
    std::vector<V3> v, vn, vt;
    std::vector<ObjMaterial> mats;  // mMaterialLib order
    std::map<std::string, uint32_t> matIndex;
    std::vector<ObjMesh> meshes;
    std::vector<std::vector<uint32_t>> objects;  // mesh ids per object
    std::vector<std::string> objectNames;
    int curObject = -1, curMesh = -1, curMaterial = -1;
    std::string activeGroup;

    ObjModel() { addMaterial("DefaultMaterial"); }
    uint32_t addMaterial(const std::string& name) {
        ObjMaterial m;
        m.name = name;
        mats.push_back(m);
        matIndex[name] = (uint32_t)mats.size() - 1;
        return (uint32_t)mats.size() - 1;
    }
    void createMesh() {
        meshes.emplace_back();
        curMesh = (int)meshes.size() - 1;
        if (curObject >= 0) objects[curObject].push_back((uint32_t)curMesh);
    }
    void createObject(const std::string& name) {
        objects.emplace_back();
        objectNames.push_back(name);
        curObject = (int)objects.size() - 1;
        createMesh();
        if (curMaterial >= 0) meshes[curMesh].material = (uint32_t)curMaterial;
    }
};

static int parseMtl(const std::vector<uint8_t>& d, ObjModel& m, std::string& err) {
    for (const std::string& raw : textLines(d)) {
        const std::string line = trim(raw);
        if (line.empty() || line[0] == '#') continue;
        const std::vector<std::string> t = splitWs(line);
        const std::string& k = t[0];
        auto rest = [&]() { return trim(line.substr(k.size())); };
        auto num = [&](size_t i, float& out) {
            if (i < t.size()) fastAtof(t[i].c_str(), out);
        };
        if (k == "newmtl") {
            const std::string name = rest();
            auto it = m.matIndex.find(name);
            m.curMaterial = it == m.matIndex.end() ? (int)m.addMaterial(name) : (int)it->second;
            if (it == m.matIndex.end() && m.curMesh >= 0) m.meshes[m.curMesh].material = (uint32_t)m.curMaterial;
            continue;
        }
        if (m.curMaterial < 0) continue;
        ObjMaterial& mt = m.mats[m.curMaterial];
        if (k == "Kd" || k == "Ks") {
            float* c = k == "Kd" ? mt.kd : mt.ks;
            float r = 0.0f, g = 0.0f, b = 0.0f;
            num(1, r);
            if (t.size() > 2) {  // "Kd r" alone reads as (r, 0, 0)
                num(2, g);
                num(3, b);
            }
            c[0] = r;
            c[1] = g;
            c[2] = b;
        } else if (k == "Ns") {
            num(1, mt.shininess);
        } else if (k == "Ni") {
            num(1, mt.ior);
        } else if (k == "d") {
            num(1, mt.alpha);
        } else if (k == "Tr") {
            float tr = 0.0f;
            num(1, tr);
            mt.alpha = 1.0f - tr;
        } else if (k == "map_Kd") {
            // texture options precede the file name
            static const std::map<std::string, int> optArgs = {
                {"-blendu", 1}, {"-blendv", 1}, {"-boost", 1}, {"-bm", 1},     {"-cc", 1},   {"-clamp", 1},
                {"-imfchan", 1}, {"-texres", 1}, {"-type", 1},  {"-mm", 2},    {"-o", 3},    {"-s", 3},
                {"-t", 3}};
            size_t i = 1;
            while (i < t.size() && !t[i].empty() && t[i][0] == '-') {
                auto it = optArgs.find(t[i]);
                i += 1 + (it == optArgs.end() ? 0 : (size_t)it->second);
            }
            std::string name;
            for (size_t j = i; j < t.size(); j++) name += (j > i ? " " : "") + t[j];
            mt.mapKd = name;
        }
    }
    (void)err;
    return CR_OK;
}

static bool faceIndex(const std::string& tok, size_t pos, size_t count, uint32_t& out) {
    const long v = std::strtol(tok.c_str() + pos, nullptr, 10);
    if (v > 0) {
        out = (uint32_t)(v - 1);
    } else if (v < 0) {
        if ((long)count + v < 0) return false;
        out = (uint32_t)((long)count + v);
    } else {
        return false;
    }
    return true;
}

static int parseObj(const std::string& objPath, ObjModel& m, std::string& err) {
    std::vector<uint8_t> d;
    if (!io::readFile(objPath, d)) {
        err = "cannot read " + objPath;
        return CR_ERR_IO;
    }
    const std::string dir = dirOf(objPath);
    size_t lineNo = 0;
    for (const std::string& raw : textLines(d)) {
        lineNo++;
        const std::string line = trim(raw);
        if (line.empty() || line[0] == '#') continue;
        std::vector<std::string> t = splitWs(line);
        // a comment ends the data of the line
        for (size_t i = 1; i < t.size(); i++)
            if (t[i][0] == '#') {
                t.resize(i);
                break;
            }
        const std::string& k = t[0];
        auto bad = [&](const char* why) {
            err = objPath + ":" + std::to_string(lineNo) + ": " + why;
            return CR_ERR_IO;
        };
        auto f = [&](size_t i) {
            float x = 0.0f;
            if (i < t.size()) fastAtof(t[i].c_str(), x);
            return x;
        };
        if (k == "v") {
            const size_t n = t.size() - 1;
            if (n == 3 || n == 6) {
                m.v.push_back({f(1), f(2), f(3)});
            } else if (n == 4) {
                const float w = f(4);
                if (w == 0.0f) return bad("homogeneous vertex with w = 0");
                m.v.push_back({f(1) / w, f(2) / w, f(3) / w});
            } else {
                return bad("vertex with an unexpected number of components");
            }
        } else if (k == "vn") {
            m.vn.push_back({f(1), f(2), f(3)});
        } else if (k == "vt") {
            const size_t n = t.size() - 1;
            if (n < 1 || n > 3) return bad("texture coordinate with an unexpected number of components");
            V3 c{f(1), n > 1 ? f(2) : 0.0f, n > 2 ? f(3) : 0.0f};
            if (!std::isfinite(c.x)) c.x = 0.0f;  // nan and inf read as the OBJ default 0
            if (!std::isfinite(c.y)) c.y = 0.0f;
            if (!std::isfinite(c.z)) c.z = 0.0f;
            m.vt.push_back(c);
        } else if (k == "f") {
            ObjFace face;
            bool hasNormal = false;
            for (size_t i = 1; i < t.size(); i++) {
                const std::string& tok = t[i];
                const size_t s1 = tok.find('/');
                const size_t s2 = s1 == std::string::npos ? std::string::npos : tok.find('/', s1 + 1);
                uint32_t idx;
                if (!faceIndex(tok, 0, m.v.size(), idx)) return bad("invalid face index");
                face.v.push_back(idx);
                if (s1 != std::string::npos && s1 + 1 < tok.size() && tok[s1 + 1] != '/') {
                    if (!faceIndex(tok, s1 + 1, m.vt.size(), idx)) return bad("invalid face index");
                    face.vt.push_back(idx);
                }
                if (s2 != std::string::npos && s2 + 1 < tok.size()) {
                    if (!faceIndex(tok, s2 + 1, m.vn.size(), idx)) return bad("invalid face index");
                    face.vn.push_back(idx);
                    hasNormal = true;
                }
            }
            if (face.v.size() < 3) continue;  // line-like faces are not triangles
            if (m.curObject < 0) m.createObject("defaultobject");
            if (m.curMesh < 0) m.createMesh();
            ObjMesh& mesh = m.meshes[m.curMesh];
            mesh.uvCount += face.vt.size();
            if (hasNormal) mesh.hasNormals = true;
            mesh.faces.push_back(std::move(face));
        } else if (k == "o") {
            const std::string name = trim(line.substr(1));
            int found = -1;
            for (size_t i = 0; i < m.objectNames.size(); i++)
                if (m.objectNames[i] == name) found = (int)i;
            if (found >= 0) {
                m.curObject = found;
            } else {
                m.createObject(name);
            }
        } else if (k == "g") {
            const std::string name = trim(line.substr(1));
            if (name != m.activeGroup) {
                m.createObject(name);
                m.activeGroup = name;
            }
        } else if (k == "usemtl") {
            const std::string name = trim(line.substr(6));
            if (m.curMaterial >= 0 && m.mats[m.curMaterial].name == name) continue;  // same material: ignored
            auto it = m.matIndex.find(name);
            const uint32_t idx = it == m.matIndex.end() ? m.addMaterial(name) : it->second;
            m.curMaterial = (int)idx;
            bool newMesh = m.curMesh < 0;
            if (!newMesh) {
                const ObjMesh& cur = m.meshes[m.curMesh];
                newMesh = cur.material != kNoMaterial && cur.material != idx && !cur.faces.empty();
            }
            if (newMesh) m.createMesh();
            m.meshes[m.curMesh].material = idx;
        } else if (k == "mtllib") {
            const std::string name = trim(line.substr(6));
            std::vector<uint8_t> md;
            if (io::readFile(dir + name, md)) {  // a missing library is not an error
                int rc = parseMtl(md, m, err);
                if (rc) return rc;
            }
        }
        // s, l, p, and anything else: ignored
    }
    return CR_OK;
}

// ---------------------------------------------------------------------------
// post-processing and the flat SceneData
// ---------------------------------------------------------------------------
static V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// aiVector3t::Normalize: divide by the length through its reciprocal, unless 0
static V3 normalizeAi(V3 a) {
    const float len = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    if (len == 0.0f) return a;
    const float inv = 1.0f / len;
    return {a.x * inv, a.y * inv, a.z * inv};
}

struct Corner {
    V3 p, n;
    float u, v;
};

struct Result {
    std::vector<float> pos, nrm, uv;
    std::vector<uint32_t> idx;
    std::vector<cr_mesh_desc> meshes;
    std::vector<cr_material> mats;
    std::vector<std::string> matNames;
    std::vector<uint32_t> matTex;
    std::vector<uint32_t> emissive;
    std::vector<io::Image> images;
    std::vector<std::vector<float>> texels;  // RGBA per texture
    std::vector<cr_texture> textures;
    cr_camera camera{};
};

static void emitMesh(const ObjModel& m, const ObjMesh& om, Result& r, std::string& err, int& rc) {
    // corners in face order (createVertexArray)
    std::vector<Corner> corners;
    std::vector<std::vector<uint32_t>> faces;
    const bool wantN = !m.vn.empty() && om.hasNormals;
    const bool wantUV = !m.vt.empty() && om.uvCount > 0;
    bool normalsOk = wantN, uvOk = wantUV;
    for (const ObjFace& f : om.faces) {
        std::vector<uint32_t> fi;
        for (size_t k = 0; k < f.v.size(); k++) {
            if (f.v[k] >= m.v.size()) {
                err = "OBJ: vertex index out of range";
                rc = CR_ERR_IO;
                return;
            }
            Corner c{m.v[f.v[k]], {0, 0, 0}, 0.0f, 0.0f};
            if (normalsOk && k < f.vn.size()) {
                if (f.vn[k] >= m.vn.size()) normalsOk = false;
                else c.n = m.vn[f.vn[k]];
            }
            if (uvOk && k < f.vt.size()) {
                if (f.vt[k] >= m.vt.size()) uvOk = false;
                else {
                    c.u = m.vt[f.vt[k]].x;
                    c.v = m.vt[f.vt[k]].y;
                }
            }
            fi.push_back((uint32_t)corners.size());
            corners.push_back(c);
        }
        faces.push_back(std::move(fi));
    }
    if (!normalsOk)
        for (Corner& c : corners) c.n = {0, 0, 0};
    if (!uvOk)
        for (Corner& c : corners) c.u = c.v = 0.0f;
    // Triangulate
    std::vector<uint32_t> tris;
    for (const auto& f : faces) {
        const size_t n = f.size();
        if (n == 3) {
            tris.insert(tris.end(), f.begin(), f.end());
        } else if (n == 4) {
            unsigned start = 0;
            for (unsigned i = 0; i < 4; ++i) {
                const V3 v = corners[f[i]].p;
                const V3 left = normalizeAi(sub(corners[f[(i + 3) % 4]].p, v));
                const V3 diag = normalizeAi(sub(corners[f[(i + 2) % 4]].p, v));
                const V3 right = normalizeAi(sub(corners[f[(i + 1) % 4]].p, v));
                const float angle = std::acos(dot(left, diag)) + std::acos(dot(right, diag));
                if (angle > 3.1415926538f) {  // the concave corner
                    start = i;
                    break;
                }
            }
            const uint32_t q[4] = {f[0], f[1], f[2], f[3]};
            tris.insert(tris.end(), {q[start], q[(start + 1) % 4], q[(start + 2) % 4]});
            tris.insert(tris.end(), {q[start], q[(start + 2) % 4], q[(start + 3) % 4]});
        } else {
            for (size_t k = 1; k + 1 < n; k++) tris.insert(tris.end(), {f[0], f[k], f[k + 1]});
        }
    }
    // GenNormals: flat face normals when the mesh has none
    if (!normalsOk) {
        for (size_t t = 0; t < tris.size(); t += 3) {
            const V3 p1 = corners[tris[t]].p, p2 = corners[tris[t + 1]].p, p3 = corners[tris[t + 2]].p;
            const V3 n = normalizeAi(cross(sub(p2, p1), sub(p3, p1)));
            for (int k = 0; k < 3; k++) corners[tris[t + k]].n = n;
        }
    }
    // JoinIdenticalVertices
    struct Key {
        uint32_t w[8];
        bool operator==(const Key& o) const { return std::memcmp(w, o.w, sizeof(w)) == 0; }
    };
    struct KeyHash {
        size_t operator()(const Key& k) const {
            uint64_t h = 1469598103934665603ull;
            for (uint32_t x : k.w) h = (h ^ x) * 1099511628211ull;
            return (size_t)h;
        }
    };
    std::unordered_map<Key, uint32_t, KeyHash> seen;
    std::vector<uint32_t> remap(corners.size());
    std::vector<Corner> unique;
    for (size_t i = 0; i < corners.size(); i++) {
        const Corner& c = corners[i];
        Key key;
        const float vals[8] = {c.p.x, c.p.y, c.p.z, c.n.x, c.n.y, c.n.z, c.u, c.v};
        for (int k = 0; k < 8; k++) {
            float v = vals[k] == 0.0f ? 0.0f : vals[k];  // -0 equals 0
            std::memcpy(&key.w[k], &v, 4);
        }
        auto it = seen.find(key);
        if (it == seen.end()) {
            it = seen.emplace(key, (uint32_t)unique.size()).first;
            unique.push_back(c);
        }
        remap[i] = it->second;
    }
    const uint32_t vOff = (uint32_t)(r.pos.size() / 3);
    const uint32_t iOff = (uint32_t)r.idx.size();
    for (const Corner& c : unique) {
        r.pos.insert(r.pos.end(), {c.p.x, c.p.y, c.p.z});
        r.nrm.insert(r.nrm.end(), {c.n.x, c.n.y, c.n.z});
        r.uv.insert(r.uv.end(), {c.u, c.v});
    }
    for (uint32_t t : tris) r.idx.push_back(vOff + remap[t]);
    cr_mesh_desc md;
    md.index_offset = iOff;
    md.index_count = (uint32_t)tris.size();
    md.vertex_offset = vOff;
    md.material_id = om.material == kNoMaterial ? 0u : om.material;
    r.meshes.push_back(md);
}

static int importXml(const std::string& path, Result& r, std::string& err) {
    if (path.size() < 4 || path.compare(path.size() - 4, 4, ".xml") != 0) {
        err = "Imported file must be xml file.";
        return CR_ERR_INVALID_ARGUMENT;
    }
    std::vector<uint8_t> d;
    if (!io::readFile(path, d)) {
        err = "Invalid XML file " + path + ".";
        return CR_ERR_IO;
    }
    std::vector<XmlNode> top;
    const std::string text(d.begin(), d.end());
    if (!XmlParser(text).parseDocument(top, err)) return CR_ERR_IO;
    const XmlNode* cam = nullptr;
    for (const XmlNode& n : top)
        if (n.name == "camera") {
            cam = &n;
            break;
        }
    if (!cam) {
        err = "No camera node found.";
        return CR_ERR_IO;
    }
    // createCamera, Utils/Importer.cpp:23-52, with the Camera defaults of
    // Core/CameraProxy.h:12-16
    cr_camera& c = r.camera;
    const float defPos[3] = {0, 0, 0}, defTarget[3] = {0, 0, -1}, defUp[3] = {0, 1, 0};
    std::memcpy(c.pos, defPos, sizeof(defPos));
    std::memcpy(c.target, defTarget, sizeof(defTarget));
    std::memcpy(c.up, defUp, sizeof(defUp));
    c.fov_y = xmlFloat(*cam, "fovy");
    auto f3 = [](const XmlNode* n, float* out) {
        if (!n) return;
        out[0] = xmlFloat(*n, "x");
        out[1] = xmlFloat(*n, "y");
        out[2] = xmlFloat(*n, "z");
    };
    f3(cam->child("eye"), c.pos);
    f3(cam->child("lookat"), c.target);
    f3(cam->child("up"), c.up);
    c.width = xmlUint(*cam, "width");
    c.height = xmlUint(*cam, "height");
    // createEmissiveDict, :54-78: "r,g,b" split at commas
    std::map<std::string, std::vector<float>> emissive;
    for (const XmlNode& n : top) {
        if (n.name != "light") continue;
        const std::string* mn = n.attr("mtlname");
        const std::string* rad = n.attr("radiance");
        std::vector<float> rgb(3, 0.0f);
        if (rad) {
            size_t start = 0;
            for (int i = 0; i < 3 && start <= rad->size(); i++) {
                size_t e = rad->find(',', start);
                if (e == std::string::npos) e = rad->size();
                const std::string tok = rad->substr(start, e - start);
                char* end = nullptr;
                const float v = std::strtof(tok.c_str(), &end);
                if (end != tok.c_str()) rgb[i] = v;
                start = e + 1;
                if (e == rad->size()) break;
            }
        }
        emissive[mn ? *mn : std::string()] = rgb;
    }
    // the geometry: the XML path with the extension .obj
    const std::string objPath = path.substr(0, path.size() - 4) + ".obj";
    ObjModel m;
    int rc = parseObj(objPath, m, err);
    if (rc) return rc;
    if (m.objects.empty()) {
        err = "OBJ: no geometry in " + objPath;
        return CR_ERR_IO;
    }
    // materials (createSceneData, :101-155)
    const std::string base = dirOf(path);
    for (const ObjMaterial& om : m.mats) {
        cr_material cm{};
        for (int k = 0; k < 3; k++) {
            cm.diffuse[k] = om.kd[k];
            cm.specular[k] = om.ks[k];
        }
        cm.shininess = om.shininess;
        cm.type = CR_MATERIAL_PHONG;
        cm.flags = 0;  // derived by finalize
        auto it = emissive.find(om.name);
        if (it != emissive.end())
            for (int k = 0; k < 3; k++) cm.emission[k] = it->second[k];
        uint32_t tex = CR_NO_TEXTURE;
        if (!om.mapKd.empty()) {
            io::Image img;
            rc = io::loadImage(base + om.mapKd, true, img, err);
            if (rc) return rc;
            tex = (uint32_t)r.images.size();
            r.images.push_back(std::move(img));
        }
        r.mats.push_back(cm);
        r.matNames.push_back(om.name);
        r.matTex.push_back(tex);
    }
    // meshes object by object, empty ones dropped (createNodes / createTopology)
    for (const auto& obj : m.objects)
        for (uint32_t id : obj) {
            const ObjMesh& om = m.meshes[id];
            if (om.faces.empty()) continue;
            rc = CR_OK;
            emitMesh(m, om, r, err, rc);
            if (rc) return rc;
        }
    // emitters: every triangle of a mesh with an emissive material
    uint32_t prim = 0;
    for (const cr_mesh_desc& md : r.meshes) {
        const cr_material& cm = r.mats[md.material_id];
        const bool em = std::max(std::max(cm.emission[0], cm.emission[1]), cm.emission[2]) != 0.0f;
        for (uint32_t t = 0; t < md.index_count / 3; t++, prim++)
            if (em) r.emissive.push_back(prim);
    }
    // textures as Texture(const Image&) fills them: RGBA, missing channels 0
    for (const io::Image& img : r.images) {
        std::vector<float> t((size_t)img.width * img.height * 4, 0.0f);
        for (size_t p = 0; p < (size_t)img.width * img.height; p++)
            for (uint32_t ch = 0; ch < std::min<uint32_t>(img.channels, 4); ch++)
                t[4 * p + ch] = img.pixels[p * img.channels + ch];
        r.texels.push_back(std::move(t));
    }
    for (size_t i = 0; i < r.images.size(); i++) {
        cr_texture ct;
        ct.width = r.images[i].width;
        ct.height = r.images[i].height;
        ct.texels = r.texels[i].data();
        r.textures.push_back(ct);
    }
    return CR_OK;
}

}  // namespace imp
}  // namespace cr

struct cr_import {
    cr::imp::Result r;
};

using namespace cr;

extern "C" {

int cr_import_xml(const char* path, cr_import** out) {
    clearError();
    if (!path || !out) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    std::unique_ptr<cr_import> imp(new cr_import);
    std::string err;
    const int rc = imp::importXml(path, imp->r, err);
    if (rc) return fail(rc, "%s", err.c_str());
    *out = imp.release();
    return CR_OK;
}

int cr_import_get(const cr_import* imp, cr_import_view* v) {
    clearError();
    if (!imp || !v) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    const imp::Result& r = imp->r;
    v->pos = r.pos.data();
    v->nrm = r.nrm.data();
    v->uv = r.uv.data();
    v->n_vertices = r.pos.size() / 3;
    v->idx = r.idx.data();
    v->n_tris = r.idx.size() / 3;
    v->meshes = r.meshes.data();
    v->n_meshes = (uint32_t)r.meshes.size();
    v->mats = r.mats.data();
    v->material_texture = r.matTex.data();
    v->n_mats = (uint32_t)r.mats.size();
    v->emissive = r.emissive.data();
    v->n_emissive = (uint32_t)r.emissive.size();
    v->textures = r.textures.data();
    v->n_textures = (uint32_t)r.textures.size();
    v->camera = r.camera;
    return CR_OK;
}

const char* cr_import_material_name(const cr_import* imp, uint32_t material) {
    if (!imp || material >= imp->r.matNames.size()) return "";
    return imp->r.matNames[material].c_str();
}

int cr_import_create_scene(const cr_import* imp, cr_scene** out) {
    clearError();
    if (!imp || !out) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    const imp::Result& r = imp->r;
    cr_scene* s = nullptr;
    int rc = cr_scene_create(r.pos.data(), r.nrm.data(), r.uv.data(), r.pos.size() / 3, r.idx.data(), r.idx.size() / 3,
                             r.meshes.data(), (uint32_t)r.meshes.size(), r.mats.data(), (uint32_t)r.mats.size(),
                             r.emissive.data(), (uint32_t)r.emissive.size(), &s);
    if (rc) return rc;
    if (!r.textures.empty())
        rc = cr_scene_set_diffuse_textures(s, r.textures.data(), (uint32_t)r.textures.size(), r.matTex.data(),
                                           (uint32_t)r.matTex.size());
    if (!rc && r.camera.width && r.camera.height) rc = cr_scene_set_camera(s, &r.camera);
    if (rc) {
        cr_scene_destroy(s);
        return rc;
    }
    *out = s;
    return CR_OK;
}

int cr_import_destroy(cr_import* imp) {
    delete imp;
    return CR_OK;
}

int cr_image_load(const char* path, int to_linear, cr_image* out) {
    clearError();
    if (!path || !out) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    io::Image img;
    std::string err;
    const int rc = io::loadImage(path, to_linear != 0, img, err);
    if (rc) return fail(rc, "%s", err.c_str());
    out->width = img.width;
    out->height = img.height;
    out->channels = img.channels;
    out->pixels = static_cast<float*>(std::malloc(std::max<size_t>(1, img.pixels.size()) * sizeof(float)));
    if (!out->pixels) return fail(CR_ERR_OUT_OF_MEMORY, "image of %zu floats", img.pixels.size());
    std::memcpy(out->pixels, img.pixels.data(), img.pixels.size() * sizeof(float));
    return CR_OK;
}

int cr_image_free(cr_image* img) {
    if (img) {
        std::free(img->pixels);
        img->pixels = nullptr;
    }
    return CR_OK;
}

int cr_image_write_exr(const char* path, uint32_t width, uint32_t height, uint32_t channels, const float* pixels) {
    clearError();
    if (!path || (width && height && !pixels)) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    const std::string p(path);
    if (p.size() < 4 || p.compare(p.size() - 4, 4, ".exr") != 0) return fail(CR_ERR_INVALID_ARGUMENT, "Output file must be .exr");
    if (!width || !height) return fail(CR_ERR_INVALID_ARGUMENT, "empty image");
    std::string err;
    const int rc = io::writeExr(p, width, height, channels, pixels, err);
    return rc ? fail(rc, "%s", err.c_str()) : CR_OK;
}

int cr_image_write_png(const char* path, uint32_t width, uint32_t height, uint32_t channels, const float* pixels,
                       int gamma_correct) {
    clearError();
    if (!path || (width && height && !pixels)) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    const std::string p(path);
    if (p.size() < 4 || p.compare(p.size() - 4, 4, ".png") != 0) return fail(CR_ERR_INVALID_ARGUMENT, "Output file must be .png");
    if (!width || !height) return fail(CR_ERR_INVALID_ARGUMENT, "empty image");
    std::string err;
    const int rc = io::writePng(p, width, height, channels, pixels, gamma_correct != 0, err);
    return rc ? fail(rc, "%s", err.c_str()) : CR_OK;
}

}  // extern "C"
