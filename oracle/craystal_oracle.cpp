// craystal_oracle.cpp -- CPU restatement of the CRaystal path-tracing hot path.
//
// TEST INFRASTRUCTURE ONLY: the checker for the CUDA product, never part of
// it.  Compiled with -O2 -ffp-contract=off -fno-fast-math so that every
// float operation is rounded on its own, in the order the reference source
// writes it (glm 1.0.1 evaluation order for dot, cross, normalize, reflect and
// mat3 * vec3).  Each function cites the reference file:line it restates.
//
// Parity pins: Tests/CameraTest.cpp:16-50 (camera rays), Tests/CoreTest.cpp
// :14-79 (spectrum arithmetic), :130-280 (sampler statistics).  The rest of
// the path has no known-answer vectors in the reference; the oracle is its
// source-level semantics.

#include "craystal_oracle.h"

#include <algorithm>
#include <atomic>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace orc {

constexpr float kEps = 1e-6f;                          // Math/MathDefs.h:12
constexpr float kPi = 3.14159265358979323846f;         // :13
constexpr float k2Pi = 2.f * kPi;                      // :14
constexpr float kInvPi = 1.f / kPi;                    // :15
constexpr float kInv2Pi = 0.5f / kPi;                  // :16
constexpr float kFltInf = std::numeric_limits<float>::infinity();
constexpr float kFltEps = std::numeric_limits<float>::epsilon();

// ---------------------------------------------------------------------------
// vector helpers with glm's evaluation order
// ---------------------------------------------------------------------------
struct V2 {
    float x, y;
};
struct V3 {
    float x, y, z;
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline V3 v3(float a) { return {a, a, a}; }
static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
static inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
static inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
// glm compute_dot<vec3>: tmp = a * b; return tmp.x + tmp.y + tmp.z
static inline float dot(V3 a, V3 b) {
    float x = a.x * b.x, y = a.y * b.y, z = a.z * b.z;
    return (x + y) + z;
}
static inline float absDot(V3 a, V3 b) { return std::fabs(dot(a, b)); }
// glm compute_cross
static inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
// glm normalize: v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x)
static inline V3 normalize(V3 a) {
    float inv = 1.0f / std::sqrt(dot(a, a));
    return a * inv;
}
static inline float length(V3 a) { return std::sqrt(dot(a, a)); }
// glm reflect: I - N * dot(N, I) * 2
static inline V3 reflect(V3 I, V3 N) { return I - (N * dot(N, I)) * 2.0f; }
// glm scalar min / max
static inline float gmin(float x, float y) { return (y < x) ? y : x; }
static inline float gmax(float x, float y) { return (x < y) ? y : x; }
static inline V3 vmin(V3 a, V3 b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
static inline V3 vmax(V3 a, V3 b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
static inline float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
// std::max / std::min
static inline float smax(float a, float b) { return (a < b) ? b : a; }
static inline float smin(float a, float b) { return (b < a) ? b : a; }

// float -> int conversion with x86 cvttss2si semantics (NaN and out-of-range
// give INT_MIN), so that the oracle agrees with itself on x86-64 and aarch64.
static inline int f2i_x86(float f) {
    if (!(f > -2147483904.0f && f < 2147483648.0f)) return INT32_MIN;
    return (int)f;
}

// ---------------------------------------------------------------------------
// RGB spectrum, Core/Spectrum.h:15-273
// ---------------------------------------------------------------------------
struct S3 {
    float c[3];
};
static inline S3 s3(float a) { return {{a, a, a}}; }
static inline S3 operator+(S3 a, S3 b) { return {{a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]}}; }
static inline S3 operator-(S3 a, S3 b) { return {{a.c[0] - b.c[0], a.c[1] - b.c[1], a.c[2] - b.c[2]}}; }
static inline S3 operator*(S3 a, S3 b) { return {{a.c[0] * b.c[0], a.c[1] * b.c[1], a.c[2] * b.c[2]}}; }
static inline S3 operator*(S3 a, float s) { return {{a.c[0] * s, a.c[1] * s, a.c[2] * s}}; }
static inline S3 operator*(float s, S3 a) { return {{s * a.c[0], s * a.c[1], s * a.c[2]}}; }
static inline S3 operator/(S3 a, float s) { return {{a.c[0] / s, a.c[1] / s, a.c[2] / s}}; }
static inline float maxValue(S3 a) {  // Spectrum.h:183-189
    float v = a.c[0];
    v = smax(v, a.c[1]);
    v = smax(v, a.c[2]);
    return v;
}
static inline float averageValue(S3 a) {  // Spectrum.h:199-205
    float v = 0.0f;
    v += a.c[0];
    v += a.c[1];
    v += a.c[2];
    return v / 3.0f;
}
static inline bool hasNaNOrInf(S3 a) {
    for (int i = 0; i < 3; i++)
        if (std::isnan(a.c[i]) || std::isinf(a.c[i])) return true;
    return false;
}

// ---------------------------------------------------------------------------
// Sampler, Core/Sampler.cu:4-31
// ---------------------------------------------------------------------------
struct Sampler {
    uint32_t state, inc;
    Sampler(uint32_t px, uint32_t py, uint32_t sampleIndex) {
        state = px * 2654435761u + py * 1597334677u + sampleIndex;
        inc = px * 1234567891u + py * 987654321u + 1u;
        for (int i = 0; i < 4; ++i) next();
    }
    uint32_t next() {
        uint32_t old = state;
        state = old * 747796405u + inc;
        old = ((old >> ((old >> 28u) + 4u)) ^ old) * 277803737u;
        return (old >> 22u) ^ old;
    }
    static float toFloat(uint32_t s) { return float(s) * (1.0f / 4294967296.0f); }
    float next1D() { return toFloat(next()); }
    // Float2(stateToFloat(nextState()), stateToFloat(nextState())): the
    // first draw goes to x.
    V2 next2D() {
        float a = toFloat(next());
        float b = toFloat(next());
        return {a, b};
    }
};

// ---------------------------------------------------------------------------
// Hero-wavelength spectral mode (an extension; the reference is RGB only):
// three wavelengths per path (hero ~ U[360, 830) nm from a hash of pixel and
// sample index, plus rotations by 470/3 nm), RGB upsampled with the
// partition of unity B_b = 1 - S((l-490)/15), B_r = S((l-590)/15),
// B_g = 1 - B_b - B_r, film conversion with the Wyman-Sloan-Shirley (2013)
// multi-lobe CIE 1931 fit and the IEC 61966-2-1 XYZ -> sRGB matrix,
// white-balanced to the flat spectrum.
// ---------------------------------------------------------------------------
static float sigmoidf(float x) { return 1.0f / (1.0f + std::exp(-x)); }
static float lobe(float l, float mu, float s1, float s2) {
    float t = (l - mu) / (l < mu ? s1 : s2);
    return std::exp(-0.5f * t * t);
}
static V3 cieXYZ(float l) {
    float x = 1.056f * lobe(l, 599.8f, 37.9f, 31.0f) + 0.362f * lobe(l, 442.0f, 16.0f, 26.7f) -
              0.065f * lobe(l, 501.1f, 20.4f, 26.2f);
    float y = 0.821f * lobe(l, 568.8f, 46.9f, 40.5f) + 0.286f * lobe(l, 530.9f, 16.3f, 31.1f);
    float z = 1.217f * lobe(l, 437.0f, 11.8f, 36.0f) + 0.681f * lobe(l, 459.0f, 26.0f, 13.8f);
    return {x, y, z};
}
static V3 xyzToSrgb(V3 c) {
    return {3.2404542f * c.x - 1.5371385f * c.y - 0.4985314f * c.z,
            -0.9692660f * c.x + 1.8760108f * c.y + 0.0415560f * c.z,
            0.0556434f * c.x - 0.2040259f * c.y + 1.0572252f * c.z};
}
struct Spectral {
    bool on = false;
    float lambda[3], br[3], bg[3], bb[3];
};
static uint32_t spectralHash(uint32_t x, uint32_t y, uint32_t s) {
    uint32_t h = x * 0x9E3779B1u ^ (y + 0x7F4A7C15u) * 0x85EBCA77u ^ (s + 0x165667B1u) * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h;
}
static Spectral makeSpectral(bool on, uint32_t x, uint32_t y, uint32_t s) {
    Spectral p;
    p.on = on;
    if (!on) return p;
    float u = (float)(spectralHash(x, y, s) >> 8) * (1.0f / 16777216.0f);
    for (int i = 0; i < 3; i++) {
        float t = u + (float)i / 3.0f;
        if (t >= 1.0f) t -= 1.0f;
        float l = 360.0f + 470.0f * t;
        p.lambda[i] = l;
        p.bb[i] = 1.0f - sigmoidf((l - 490.0f) / 15.0f);
        p.br[i] = sigmoidf((l - 590.0f) / 15.0f);
        p.bg[i] = 1.0f - p.bb[i] - p.br[i];
    }
    return p;
}
static S3 toPathSpec(const Spectral& p, const float c[3]) {
    if (!p.on) return {{c[0], c[1], c[2]}};
    S3 r;
    for (int i = 0; i < 3; i++) r.c[i] = (c[0] * p.br[i] + c[1] * p.bg[i]) + c[2] * p.bb[i];
    return r;
}
static V3 whiteBalanceOracle();
static S3 pathSpecToRgb(const Spectral& p, S3 L) {
    if (!p.on) return L;
    static const V3 wb = whiteBalanceOracle();
    V3 xyz{0, 0, 0};
    for (int i = 0; i < 3; i++) xyz = xyz + cieXYZ(p.lambda[i]) * L.c[i];
    xyz = xyz * (470.0f / 3.0f);
    V3 rgb = xyzToSrgb(xyz);
    return {{rgb.x * wb.x, rgb.y * wb.y, rgb.z * wb.z}};
}
static V3 whiteBalanceOracle() {
    double acc[3] = {0, 0, 0};
    const int n = 4700;
    const double dl = 470.0 / n;
    for (int i = 0; i < n; i++) {
        V3 c = cieXYZ((float)(360.0 + (i + 0.5) * dl));
        acc[0] += c.x * dl;
        acc[1] += c.y * dl;
        acc[2] += c.z * dl;
    }
    V3 rgb = xyzToSrgb({(float)acc[0], (float)acc[1], (float)acc[2]});
    return {1.0f / rgb.x, 1.0f / rgb.y, 1.0f / rgb.z};
}

// ---------------------------------------------------------------------------
// Ray, offset, AABB, Math/Ray.cu, Math/AABB.cu
// ---------------------------------------------------------------------------
struct Ray {
    V3 o;
    float tMin = 0.f;
    V3 d;
    float tMax = kFltInf;
};

static inline int floatAsInt(float f) {
    int i;
    std::memcpy(&i, &f, 4);
    return i;
}
static inline float intAsFloat(int i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}

// Math/Ray.cu:11-22 (Ray Tracing Gems ch. 6)
static V3 offsetRayOrigin(V3 p, V3 n) {
    const float kOrigin = 1.0f / 32.0f;
    const float kFltScale = 1.0f / 65535.0f;
    const float kIntScale = 256.0f;
    int ox = f2i_x86(kIntScale * n.x), oy = f2i_x86(kIntScale * n.y), oz = f2i_x86(kIntScale * n.z);
    auto nudge = [](float pc, int oc) {
        return intAsFloat((int)((uint32_t)floatAsInt(pc) + (uint32_t)((pc < 0) ? -oc : oc)));
    };
    float px = nudge(p.x, ox), py = nudge(p.y, oy), pz = nudge(p.z, oz);
    return {std::fabs(p.x) < kOrigin ? p.x + kFltScale * n.x : px,
            std::fabs(p.y) < kOrigin ? p.y + kFltScale * n.y : py,
            std::fabs(p.z) < kOrigin ? p.z + kFltScale * n.z : pz};
}

struct AABB {
    V3 mn = v3(kFltInf), mx = v3(-kFltInf);
    void include(V3 p) {  // AABB.h:63-68
        mn = vmin(mn, p);
        mx = vmax(mx, p);
    }
    void include(const AABB& b) {  // AABB.h:72-77
        mn = vmin(mn, b.mn);
        mx = vmax(mx, b.mx);
    }
    V3 diagonal() const { return mx - mn; }
};

// Math/AABB.cu:6-46
static bool aabbIntersect(const AABB& b, const Ray& ray, float& hitT) {
    float tMin = ray.tMin, tMax = ray.tMax;
    for (int i = 0; i < 3; ++i) {
        if (std::fabs(b.mx[i] - b.mn[i]) < kFltEps) {
            if (std::fabs(ray.d[i]) < kFltEps) {
                if (std::fabs(ray.o[i] - b.mn[i]) > kFltEps) return false;
                continue;
            }
            float t = (b.mn[i] - ray.o[i]) / ray.d[i];
            tMin = smax(tMin, t);
            tMax = smin(tMax, t);
        } else {
            float invD = 1.0f / ray.d[i];
            float t0 = (b.mn[i] - ray.o[i]) * invD;
            float t1 = (b.mx[i] - ray.o[i]) * invD;
            if (invD < 0.0f) std::swap(t0, t1);
            tMin = smax(tMin, t0);
            tMax = smin(tMax, t1);
        }
        if (tMin > tMax) return false;
    }
    if (tMin > ray.tMax || tMax < ray.tMin) return false;
    hitT = tMin;
    return true;
}

// Scene/Triangle.cu:40-75 (Moller-Trumbore)
static inline bool triIntersect(V3 v0, V3 v1, V3 v2, const Ray& ray, float& u,
                                float& v, float& t) {
    V3 e1 = v1 - v0;
    V3 e2 = v2 - v0;
    V3 p = cross(ray.d, e2);
    float det = dot(e1, p);
    if (std::fabs(det) < 1e-6f) return false;
    float invDet = 1.0f / det;
    V3 tvec = ray.o - v0;
    u = dot(tvec, p) * invDet;
    if (u < 0.0f || u > 1.0f) return false;
    V3 q = cross(tvec, e1);
    v = dot(ray.d, q) * invDet;
    if (v < 0.0f || u + v > 1.0f) return false;
    t = dot(e2, q) * invDet;
    if (t <= 0.0) return false;
    return true;
}

}  // namespace orc

using namespace orc;

// ---------------------------------------------------------------------------
// Scene + BVH
// ---------------------------------------------------------------------------
struct Node {  // Core/BVH.h:17-30
    AABB bounds;
    bool leaf;
    uint32_t a, b;  // leaf: offset, count; internal: left, right
};

struct orc_scene {
    std::vector<V3> pos, nrm;
    std::vector<V2> uv;
    std::vector<uint32_t> idx;
    std::vector<uint32_t> primToMesh;
    std::vector<orc_mesh_desc> meshes;
    std::vector<orc_material> mats;
    std::vector<uint32_t> emissive;
    // BVH
    std::vector<Node> nodes;
    std::vector<uint32_t> primMap;  // leaf slot -> primitive id
    AABB rootBounds;
    uint32_t rootIndex = 0;
    // lights beyond the reference (extensions)
    V3 env{0, 0, 0};
    std::vector<float> spheres;  // center xyz, radius, emission xyz per light (7 floats)
    // diffuse textures (Core/Texture.cu, Core/Material.h:29-36)
    std::vector<float> texels;         // RGBA per texel, all textures
    std::vector<uint32_t> texDescs;    // first texel, width, height per texture
    std::vector<uint32_t> matTex;      // texture per material or 0xFFFFFFFF
    // analytic spheres (Scene/Sphere.h:9-12) with a material each
    std::vector<float> sph;            // centre xyz, radius per sphere
    std::vector<uint32_t> sphMat;
    uint32_t maxDepth = 0, maxLeaf = 0, maxLeafDepth = 0;
};

namespace {

struct BuildTri {  // Core/BVH.h:73-78
    V3 centroid;
    AABB bounds;
    uint32_t tri;
};

struct Builder {
    std::vector<BuildTri> tris;
    std::vector<Node>& nodes;
    orc_scene& s;
    explicit Builder(orc_scene& sc) : nodes(sc.nodes), s(sc) {}

    static float surfaceArea(const AABB& b) {  // BVH.cu:284-287
        V3 d = b.diagonal();
        return (float)((double)((d.x * d.y + d.x * d.z) + d.y * d.z) * 2.0);
    }
    static float sah(const AABB& node, const AABB& l, const AABB& r, int nl, int nr) {
        // BVH.cu:289-301: 1 + 1 * (nL*SA_L + nR*SA_R) / SA_node
        float lsa = surfaceArea(l), rsa = surfaceArea(r), root = surfaceArea(node);
        return 1.0f + (1.0f * ((float)nl * lsa + (float)nr * rsa)) / root;
    }

    // BVH.cu:214-282
    void bestSplit(const std::vector<uint32_t>& ind, uint32_t start, uint32_t count,
                   const AABB& nb, uint32_t& axisOut, float& posOut) {
        const int NB = 32;
        float bestCost = kFltInf;
        uint32_t bestAxis = 0;
        float bestPos = 0.0f;
        for (uint32_t axis = 0; axis < 3; ++axis) {
            AABB bins[NB];
            int cnt[NB] = {0};
            V3 extent = nb.diagonal();
            float scale = (float)NB / extent[axis];
            for (uint32_t i = start; i < start + count; ++i) {
                const BuildTri& t = tris[ind[i]];
                int bi = std::min(NB - 1, f2i_x86((t.centroid[axis] - nb.mn[axis]) * scale));
                bi = std::clamp(bi, 0, NB - 1);
                bins[bi].include(t.bounds);
                cnt[bi]++;
            }
            AABB lb[NB - 1], rb[NB - 1];
            int lc[NB - 1], rc[NB - 1];
            AABB cur;
            int cc = 0;
            for (int i = 0; i < NB - 1; ++i) {
                cur.include(bins[i]);
                cc += cnt[i];
                lb[i] = cur;
                lc[i] = cc;
            }
            cur = AABB();
            cc = 0;
            for (int i = NB - 1; i > 0; --i) {
                cur.include(bins[i]);
                cc += cnt[i];
                rb[i - 1] = cur;
                rc[i - 1] = cc;
            }
            for (int i = 0; i < NB - 1; ++i) {
                float pos = nb.mn[axis] + ((float)(i + 1) * extent[axis]) / (float)NB;
                float cost = sah(nb, lb[i], rb[i], lc[i], rc[i]);
                if (cost < bestCost) {
                    bestCost = cost;
                    bestAxis = axis;
                    bestPos = pos;
                }
            }
        }
        axisOut = bestAxis;
        posOut = bestPos;
    }

    // std::partition as libstdc++ implements it for bidirectional iterators
    // (Hoare-style two-pointer swap), the order BVH.cu:177-181 produces.
    static uint32_t partition(std::vector<uint32_t>& ind, uint32_t first, uint32_t last,
                              const std::vector<BuildTri>& tris, uint32_t axis, float pos) {
        auto pred = [&](uint32_t id) { return tris[id].centroid[axis] < pos; };
        while (true) {
            while (true) {
                if (first == last) return first;
                if (pred(ind[first])) ++first;
                else break;
            }
            --last;
            while (true) {
                if (first == last) return first;
                if (!pred(ind[last])) --last;
                else break;
            }
            std::swap(ind[first], ind[last]);
            ++first;
        }
    }

    uint32_t makeLeaf(const AABB& b, uint32_t start, uint32_t count, uint32_t depth) {
        Node n;
        n.bounds = b;
        n.leaf = true;
        n.a = start;
        n.b = count;
        nodes.push_back(n);
        s.maxLeaf = std::max(s.maxLeaf, count);
        s.maxLeafDepth = std::max(s.maxLeafDepth, depth);
        return (uint32_t)nodes.size() - 1;
    }

    // BVH.cu:150-212
    uint32_t build(std::vector<uint32_t>& ind, uint32_t start, uint32_t count,
                   uint32_t depth, AABB& nb) {
        nb = AABB();
        for (uint32_t i = start; i < start + count; ++i) nb.include(tris[ind[i]].bounds);
        if (count <= 4 || depth >= 20) return makeLeaf(nb, start, count, depth);
        uint32_t axis;
        float pos;
        bestSplit(ind, start, count, nb, axis, pos);
        uint32_t mid = partition(ind, start, start + count, tris, axis, pos);
        uint32_t leftCount = mid - start;
        if (leftCount == 0 || leftCount == count) return makeLeaf(nb, start, count, depth);
        AABB lb, rb;
        uint32_t l = build(ind, start, leftCount, depth + 1, lb);
        uint32_t r = build(ind, start + leftCount, count - leftCount, depth + 1, rb);
        Node n;
        n.bounds = nb;
        n.leaf = false;
        n.a = l;
        n.b = r;
        nodes.push_back(n);
        s.maxDepth = std::max(s.maxDepth, depth);
        return (uint32_t)nodes.size() - 1;
    }

    void run() {
        const size_t nt = s.idx.size() / 3;
        tris.resize(nt);
        for (size_t i = 0; i < nt; ++i) {  // BVH.cu:120-148
            V3 v0 = s.pos[s.idx[3 * i]], v1 = s.pos[s.idx[3 * i + 1]], v2 = s.pos[s.idx[3 * i + 2]];
            BuildTri& t = tris[i];
            t.centroid = ((v0 + v1) + v2) / 3.0f;
            t.bounds.include(v0);
            t.bounds.include(v1);
            t.bounds.include(v2);
            t.tri = (uint32_t)i;
        }
        std::vector<uint32_t> ind(nt);
        for (size_t i = 0; i < nt; ++i) ind[i] = (uint32_t)i;
        nodes.clear();
        nodes.reserve(2 * nt + 1);
        s.rootIndex = build(ind, 0, (uint32_t)nt, 0, s.rootBounds);
        s.primMap.resize(nt);
        for (size_t i = 0; i < nt; ++i) s.primMap[i] = tris[ind[i]].tri;  // BVH.cu:322-338
    }
};

struct Hit {
    uint32_t prim = 0xFFFFFFFFu;
    float u = 0, v = 0;
    float t = kFltInf;
    bool tie = false;
};

struct Counters {
    uint64_t boxes = 0, tris = 0;
};

// Scene/Shape.h:16-37 + Scene/Triangle.cu:40-75
static inline bool intersectShape(const orc_scene& s, uint32_t prim, const Ray& ray, Hit& h) {
    V3 v0 = s.pos[s.idx[3 * prim]], v1 = s.pos[s.idx[3 * prim + 1]], v2 = s.pos[s.idx[3 * prim + 2]];
    float u, v, t = 0.0f;
    bool isHit = triIntersect(v0, v1, v2, ray, u, v, t);
    if (!isHit) return false;
    if (t < ray.tMin || t > ray.tMax) return false;
    if (t < h.t) {
        h.t = t;
        h.u = u;
        h.v = v;
        h.prim = prim;
        h.tie = false;
    } else if (t == h.t && prim != h.prim) {
        h.tie = true;
    }
    return true;
}

// SphereSOA::intersect, Scene/Sphere.cu:6-52
constexpr uint32_t kSphereBit = 0x80000000u;

static bool sphereIntersect(const float* g, const Ray& ray, float& hitT, float& u, float& v) {
    const V3 center{g[0], g[1], g[2]};
    const float radius = g[3];
    const V3 oc = ray.o - center;
    const float a = dot(ray.d, ray.d);
    const float b = 2.0f * dot(oc, ray.d);
    const float c = dot(oc, oc) - radius * radius;
    const float disc = b * b - 4.0f * a * c;
    if (disc < 0) return false;
    const float sq = std::sqrt(disc);
    float t0 = (-b - sq) / (2.0f * a);
    float t1 = (-b + sq) / (2.0f * a);
    if (t0 > t1) std::swap(t0, t1);
    if (t0 < ray.tMin || t0 > ray.tMax) {
        if (t1 < ray.tMin || t1 > ray.tMax) return false;
        t0 = t1;
    }
    hitT = t0;
    const V3 p = ray.o + ray.d * hitT;
    const V3 n = normalize(p - center);
    const float theta = std::acos(-n.y);
    const float phi = std::atan2(-n.z, n.x) + kPi;
    u = phi * (0.5f * kInvPi);
    v = theta * kInvPi;
    return true;
}

// The sphere loop of SceneView::intersect (Scene/Scene.cu:7-9) with the rule
// of intersectShape (Scene/Shape.h:16-37).
static bool spheresIntersect(const orc_scene& s, const Ray& ray, Hit& h) {
    bool any = false;
    for (size_t i = 0; i < s.sphMat.size(); i++) {
        float t, u, v;
        if (!sphereIntersect(&s.sph[4 * i], ray, t, u, v)) continue;
        if (t < ray.tMin || t > ray.tMax) continue;
        any = true;
        const uint32_t prim = kSphereBit | (uint32_t)i;
        if (t < h.t) {
            h.t = t;
            h.u = u;
            h.v = v;
            h.prim = prim;
            h.tie = false;
        } else if (t == h.t && prim != h.prim) {
            h.tie = true;
        }
    }
    return any;
}

// Core/BVH.cu:13-84
static bool bvhIntersect(const orc_scene& s, const Ray& ray, Hit& h, Counters* c) {
    float unused;
    if (c) c->boxes++;
    if (s.nodes.empty() || !aabbIntersect(s.rootBounds, ray, unused)) return false;
    struct Entry {
        uint32_t node;
        float tMin;
    };
    Entry stack[64];
    int sp = 0;
    stack[sp++] = {s.rootIndex, 0.0f};
    bool isHit = false;
    float closestT = h.t;
    while (sp > 0) {
        const Entry e = stack[--sp];
        const Node& node = s.nodes[e.node];
        if (e.tMin > closestT) continue;
        if (node.leaf) {
            for (uint32_t i = 0; i < node.b; ++i) {
                uint32_t prim = s.primMap[node.a + i];
                if (c) c->tris++;
                if (intersectShape(s, prim, ray, h)) {
                    isHit = true;
                    closestT = smin(closestT, h.t);
                }
            }
        } else {
            const Node& L = s.nodes[node.a];
            const Node& R = s.nodes[node.b];
            float lt = kFltInf, rt = kFltInf;
            bool hl = aabbIntersect(L.bounds, ray, lt);
            bool hr = aabbIntersect(R.bounds, ray, rt);
            if (c) c->boxes += 2;
            if (hl && hr) {
                if (lt > rt) {
                    if (lt < closestT) stack[sp++] = {node.a, lt};
                    if (rt < closestT) stack[sp++] = {node.b, rt};
                } else {
                    if (rt < closestT) stack[sp++] = {node.b, rt};
                    if (lt < closestT) stack[sp++] = {node.a, lt};
                }
            } else if (hl && lt < closestT) {
                stack[sp++] = {node.a, lt};
            } else if (hr && rt < closestT) {
                stack[sp++] = {node.b, rt};
            }
            if (sp > 62) {
                std::fprintf(stderr, "oracle: traversal stack overflow\n");
                std::abort();
            }
        }
    }
    return isHit;
}

template <class F>
static void parallelFor(uint64_t n, int threads, F&& f) {
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (threads == 1 || n < 1024) {
        f(0, n);
        return;
    }
    std::atomic<uint64_t> next{0};
    const uint64_t chunk = 4096;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([&]() {
            while (true) {
                uint64_t b = next.fetch_add(chunk);
                if (b >= n) break;
                f(b, std::min(n, b + chunk));
            }
        });
    }
    for (auto& th : pool) th.join();
}

static inline Ray toRay(const orc_ray& r) {
    Ray ray;
    ray.o = {r.o[0], r.o[1], r.o[2]};
    ray.tMin = r.tmin;
    ray.d = {r.d[0], r.d[1], r.d[2]};
    ray.tMax = r.tmax;
    return ray;
}

// ---------------------------------------------------------------------------
// Triangle attributes, Scene/Triangle.cu:9-38
// ---------------------------------------------------------------------------
struct VertexData {
    V3 p, n;
    V2 uv;
};
struct Triangle {
    VertexData v[3];
    V3 faceNormal() const { return normalize(cross(v[1].p - v[0].p, v[2].p - v[0].p)); }
    VertexData interpolate(V3 w) const {
        VertexData d;
        d.p = (v[0].p * w.x + v[1].p * w.y) + v[2].p * w.z;
        d.n = (v[0].n * w.x + v[1].n * w.y) + v[2].n * w.z;
        d.uv = {(v[0].uv.x * w.x + v[1].uv.x * w.y) + v[2].uv.x * w.z,
                (v[0].uv.y * w.x + v[1].uv.y * w.y) + v[2].uv.y * w.z};
        return d;
    }
    float area() const { return length(cross(v[0].p - v[1].p, v[2].p - v[1].p)) / 2.f; }
};
static Triangle getTriangle(const orc_scene& s, uint32_t prim) {
    Triangle t;
    for (int i = 0; i < 3; i++) {
        uint32_t vi = s.idx[3 * prim + i];
        t.v[i].p = s.pos[vi];
        t.v[i].n = s.nrm[vi];
        t.v[i].uv = s.uv[vi];
    }
    return t;
}
static const orc_material& materialOf(const orc_scene& s, uint32_t prim) {
    return s.mats[s.meshes[s.primToMesh[prim]].material_id];
}

// ---------------------------------------------------------------------------
// Frame + Intersection, Core/Frame.cu:6-30, Core/Intersection.cu:4-10
// ---------------------------------------------------------------------------
struct Frame {
    V3 T{1, 0, 0}, B{0, 1, 0}, N{0, 0, 1};
    explicit Frame(V3 n) {
        V3 t{0, 1, 0};
        if (1.0 - (double)absDot(n, t) < (double)kEps) t = {1, 0, 0};
        V3 bt = normalize(cross(n, t));
        T = normalize(cross(bt, n));
        N = n;
        B = cross(N, T);
    }
    // Float3x3(T.x, B.x, N.x, T.y, B.y, N.y, T.z, B.z, N.z) * w
    V3 toLocal(V3 w) const { return {dot(T, w), dot(B, w), dot(N, w)}; }
    // Float3x3(T, B, N) * l
    V3 toWorld(V3 l) const {
        return {(T.x * l.x + B.x * l.y) + N.x * l.z, (T.y * l.x + B.y * l.y) + N.y * l.z,
                (T.z * l.x + B.z * l.y) + N.z * l.z};
    }
};

struct Intersection {
    V3 posW, faceNormal, viewW;
    V2 uv;
    bool front;
    Frame frame;
    Intersection(V3 p, V3 fn, V3 sn, V3 vw, V2 t)
        : posW(p), faceNormal(fn), viewW(vw), uv(t), front(dot(vw, fn) > 0.0f), frame(front ? sn : -sn) {}
    V3 orientedFaceNormal() const { return front ? faceNormal : -faceNormal; }
};

// Scene/Scene.cu:31-59
static Intersection createIntersection(const orc_scene& s, const Ray& ray, const Hit& h) {
    V3 posW = ray.o + h.t * ray.d;
    V3 viewW = -normalize(ray.d);
    V3 w{(1.f - h.u) - h.v, h.u, h.v};
    Triangle tri = getTriangle(s, h.prim);
    V3 fn = tri.faceNormal();
    VertexData vd = tri.interpolate(w);
    V3 sn = normalize(vd.n);
    return Intersection(posW, fn, sn, viewW, vd.uv);
}

// createIntersection of a sphere hit (Scene/Scene.cu:43-47), with the
// sphere's own material (the reference reads a mesh table here)
static Intersection sphereIntersection(const orc_scene& s, const Ray& ray, const Hit& h) {
    const float* g = &s.sph[4 * (size_t)(h.prim & ~kSphereBit)];
    V3 posW = ray.o + h.t * ray.d;
    V3 viewW = -normalize(ray.d);
    V3 fn = normalize(posW - V3{g[0], g[1], g[2]});
    return Intersection(posW, fn, fn, viewW, V2{h.u, h.v});
}

// ---------------------------------------------------------------------------
// Sampling, Math/Sampling.cu
// ---------------------------------------------------------------------------
static V2 sampleBarycentric(V2 u) {  // :4-13
    float u1 = u.x, u2 = u.y;
    bool flip = (u1 + u2) > 1.0f;
    u1 = flip ? (1.0f - u1) : u1;
    u2 = flip ? (1.0f - u2) : u2;
    return {u1, u2};
}
static V3 cosineSampleHemisphere(V2 u) {  // :39-47
    float r = std::sqrt(u.x);
    float phi = 2.0f * kPi * u.y;
    float x = r * std::cos(phi);
    float y = r * std::sin(phi);
    float z = std::sqrt(smax(0.0f, (1.0f - x * x) - y * y));
    return {x, y, z};
}
static float cosinePdf(V3 d) { return smax(0.0f, d.z) * kInvPi; }
static float powerHeuristic(float f, float g) {  // :53-58, nf = ng = 1
    float a = 1.0f * f, b = 1.0f * g;
    return (a * a) / (a * a + b * b);
}
static float acosSafe(float v) {  // Math/CRayMath.cu:11-13
    return std::acos(gclamp(v, kEps, (float)(1.0 - (double)kEps)));
}

// ---------------------------------------------------------------------------
// TextureView::fetchTexel / sample, Core/Texture.cu:6-35
// ---------------------------------------------------------------------------
// static_cast<uint32_t>(float) as the device executes it: truncation toward
// zero, saturating (negative and NaN -> 0, >= 2^32 -> 2^32 - 1).
static uint32_t f2uDevice(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

struct RGBA {
    float v[4];
};

static RGBA texFetch(const orc_scene& s, const uint32_t* d, uint32_t x, uint32_t y) {
    x = std::clamp<uint32_t>(x, 0u, d[1] - 1u);
    y = std::clamp<uint32_t>(y, 0u, d[2] - 1u);
    const uint32_t index = y * d[1] + x;
    RGBA r;
    for (int k = 0; k < 4; k++) r.v[k] = s.texels[4 * ((size_t)d[0] + index) + k];
    return r;
}

static RGBA lerp4(const RGBA& a, const RGBA& b, float t) {  // Math/CRayMath.h:31-33
    RGBA r;
    for (int k = 0; k < 4; k++) r.v[k] = a.v[k] * (1.0f - t) + b.v[k] * t;
    return r;
}

static RGBA texSample(const orc_scene& s, uint32_t tex, V2 uv) {
    const uint32_t* d = &s.texDescs[3 * (size_t)tex];
    const float px = uv.x * (float)(d[1] - 1u);
    const float py = uv.y * (float)(d[2] - 1u);
    const uint32_t x0 = f2uDevice(std::floor(px));
    const uint32_t y0 = f2uDevice(std::floor(py));
    const uint32_t x1 = std::min<uint32_t>(x0 + 1u, d[1] - 1u);
    const uint32_t y1 = std::min<uint32_t>(y0 + 1u, d[2] - 1u);
    const float fx = px - (float)x0;
    const float fy = py - (float)y0;
    const RGBA c0 = lerp4(texFetch(s, d, x0, y0), texFetch(s, d, x1, y0), fx);
    const RGBA c1 = lerp4(texFetch(s, d, x0, y1), texFetch(s, d, x1, y1), fx);
    return lerp4(c0, c1, fy);
}

// ---------------------------------------------------------------------------
// BSDFs, Material/*.cu
// ---------------------------------------------------------------------------
struct Bsdf {
    uint32_t type;  // 0 Lambertian, 1 Principled, 2 Phong
    S3 kd, ks;
    float n;        // Phong exponent
    float dProb, sProb;
    float rough, metal;
    Frame frame;

    Bsdf(const orc_material& m, const Frame& f, const float* diffuse = nullptr) : frame(f) {
        type = m.type;
        if (!diffuse) diffuse = m.diffuse;
        kd = {{diffuse[0], diffuse[1], diffuse[2]}};
        ks = {{m.specular[0], m.specular[1], m.specular[2]}};
        n = m.shininess;
        if (type == 2) {  // PhongBRDF.cu:10-18
            dProb = smax(averageValue(kd), 0.0f);
            sProb = smax(averageValue(ks), 0.0f);
            float sum = gmax(dProb + sProb, kEps);
            dProb /= sum;
            sProb /= sum;
        } else if (type == 1) {  // PrincipledBRDF.cu:35-55
            float r = std::sqrt(2.0f / (m.shininess + 1.0f));
            float met = averageValue(ks);
            rough = std::clamp(r, 0.0f, 1.0f);
            metal = std::clamp(met, 0.0f, 1.0f);
            float sp = 0.1f * (1.0f - metal) + 1.0f * metal;
            dProb = 1.0f;
            sProb = sp;
            dProb /= (dProb + sProb);
            sProb /= (dProb + sProb);
        } else {
            dProb = 1.0f;
            sProb = 0.0f;
        }
    }

    // --- Phong, PhongBRDF.cu:20-68
    S3 phongEval(V3 wo, V3 wi) const {
        V3 r = reflect(-wo, V3{0, 0, 1});
        float c = smax(dot(r, wi), 0.0f);
        return kd * kInvPi + ((ks * (n + 2.0f)) * kInv2Pi) * std::pow(c, n);
    }
    float phongPdf(V3 wo, V3 wi) const {
        float dp = cosinePdf(wi);
        V3 r = reflect(-wo, V3{0, 0, 1});
        float ca = smax(dot(r, wi), 0.0f);
        float sp = (n + 1.0f) * kInv2Pi * std::pow(ca, n);
        return dp * dProb + sp * sProb;
    }
    V3 phongSample(V3 wo, V2 u, float& pdf) const {
        V2 u0 = u;
        V3 wi{0, 0, 0};
        pdf = 0.0f;
        bool hasD = dProb > 0.0f, hasS = sProb > 0.0f;
        if (hasD && u0.x < dProb) {
            u0.x /= dProb;
            wi = cosineSampleHemisphere(u0);
            pdf = cosinePdf(wi);
        } else if (hasS) {
            u0.x = (u0.x - dProb) / sProb;
            float alpha = acosSafe(std::pow(u0.x, 1.0f / (n + 1.0f)));
            float theta = gclamp(acosSafe(wo.z) + alpha, 0.0f, (float)((double)kPi / 2.0));
            float phi = k2Pi * u0.y;
            float st = std::sin(theta);
            wi = {st * std::cos(phi), st * std::sin(phi), (float)std::sqrt(1.0 - (double)(st * st))};
            pdf = (n + 1.0f) * kInv2Pi * std::pow(std::cos(alpha), n);
        }
        return wi;
    }

    // --- Principled, PrincipledBRDF.cu:9-150
    static float ndf(float r, float ch) {
        float a = r * r;
        float a2 = a * a;
        float c2 = ch * ch;
        float den = (float)(1.0 + ((double)a2 - 1.0) * (double)c2);
        return a2 * kInvPi / (den * den);
    }
    static float smithG1(float ag, float cv) {
        float a = ag * ag, b = cv * cv;
        return 1.0f / (cv + std::sqrt((a + b) - a * b));
    }
    static float geom(float r, float ci, float cv) {
        float alpha = (float)(0.5 + (double)r * 0.5);
        alpha *= alpha;
        return smithG1(alpha, ci) * smithG1(alpha, cv);
    }
    S3 princEval(V3 wo, V3 wi) const {
        if (wo.z <= 0.0f || wi.z <= 0.0f) return s3(0);
        V3 wh = normalize(wo + wi);
        float cv = wo.z, ci = wi.z, ch = wh.z;
        float cd = dot(wo, wh);
        // evaluateDiffuse (:132-138), double arithmetic as written
        float fd90 = (float)(0.5 + ((2.0 * (double)rough) * (double)cd) * (double)cd);
        float fl = (float)(1.0 + ((double)fd90 - 1.0) * std::pow(1.0 - (double)ci, 5.0));
        float fv = (float)(1.0 + ((double)fd90 - 1.0) * std::pow(1.0 - (double)cv, 5.0));
        S3 diffuse = (((kd * kInvPi) * fv) * fl) * (1.0f - metal);
        // evaluateSpecular (:140-147)
        float D = ndf(rough, ch);
        S3 f0 = kd * (1.0f - metal) + s3(0.04f) * metal;
        float v0 = 1.f - cd;
        float v1 = v0 * v0;
        S3 F = f0 + (((s3(1.0f) - f0) * v1) * v1) * v0;
        float G = geom(rough, ci, cv);
        float denom = (float)((4.0 * (double)ci) * (double)cv);
        S3 spec = ((D * F) * G) / denom;
        return diffuse + spec;
    }
    float princPdf(V3 wo, V3 wi) const {
        if (wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
        V3 wh = normalize(wo + wi);
        float ch = wh.z;
        float cd = dot(wo, wh);
        if (cd <= 0.0f) return 0.0f;
        float dp = cosinePdf(wi);
        float sp = 0.0f;
        if (ch > 0.0f) {
            float D = ndf(rough, ch);
            sp = D * ch / (4.0f * cd);
        }
        return dp * dProb + sp * sProb;
    }
    V3 princSample(V3 wo, V2 u, float& pdf) const {
        if (wo.z <= 0.0f) {
            pdf = 0.0f;
            return {0, 0, 0};
        }
        float u1 = u.x, u2 = u.y;
        V3 wi;
        if (u1 < sProb) {
            u1 /= sProb;
            float alpha = rough * rough;
            float a2 = alpha * alpha;
            float phi = u2 * k2Pi;
            float tan2 = a2 * u1 / (1.0f - u1);
            float ct = 1.0f / std::sqrt(1.0f + tan2);
            float r = std::sqrt(smax(1.0f - ct * ct, 0.0f));
            V3 wh{std::cos(phi) * r, std::sin(phi) * r, ct};
            wi = reflect(-wo, wh);
        } else {
            u1 = (u1 - sProb) / (1.0f - sProb);
            wi = cosineSampleHemisphere({u1, u2});
        }
        pdf = princPdf(wo, wi);
        return wi;
    }

    // --- Lambertian, LambertianBRDF.cu:6-25
    S3 lambEval() const { return kd * kInvPi; }

    // --- dispatch, Material/BSDF.h:30-57, BSDF.cu:36-103
    S3 evalLocal(V3 wo, V3 wi) const {
        S3 f = type == 2 ? phongEval(wo, wi) : (type == 1 ? princEval(wo, wi) : lambEval());
        return f * std::fabs(wi.z);
    }
    float pdfLocal(V3 wo, V3 wi) const {
        return type == 2 ? phongPdf(wo, wi) : (type == 1 ? princPdf(wo, wi) : cosinePdf(wi));
    }
    V3 sampleLocal(V3 wo, V2 u, float& pdf) const {
        if (type == 2) return phongSample(wo, u, pdf);
        if (type == 1) return princSample(wo, u, pdf);
        V3 wi = cosineSampleHemisphere(u);
        pdf = cosinePdf(wi);
        return wi;
    }
    S3 evaluate(V3 wo, V3 wi) const { return evalLocal(frame.toLocal(wo), frame.toLocal(wi)); }
    float evaluatePdf(V3 wo, V3 wi) const { return pdfLocal(frame.toLocal(wo), frame.toLocal(wi)); }
    S3 sampleEvaluate(V2 u, V3 wo, V3& wi, float& pdf) const {
        V3 woL = frame.toLocal(wo);
        pdf = 0.0f;
        V3 wiL = sampleLocal(woL, u, pdf);
        S3 f = evalLocal(woL, wiL);
        wi = frame.toWorld(wiL);
        return f;
    }
};


// ---------------------------------------------------------------------------
// Integrator, Core/Integrator.cu:13-227
// ---------------------------------------------------------------------------
// Ray / sphere (extension), nearest t in (tMin, tMax) or +inf.
static float raySphere(const Ray& r, const float* sph, float tMin, float tMax) {
    V3 oc = r.o - V3{sph[0], sph[1], sph[2]};
    float a = dot(r.d, r.d);
    float b = dot(oc, r.d) / a;
    float c = (dot(oc, oc) - sph[3] * sph[3]) / a;
    float disc = b * b - c;
    if (disc < 0.0f) return kFltInf;
    float q = std::sqrt(disc);
    float t0 = -b - q, t1 = -b + q;
    if (t0 > tMin && t0 < tMax) return t0;
    if (t1 > tMin && t1 < tMax) return t1;
    return kFltInf;
}

constexpr uint32_t kSpherePrim = 0xFFFFFF00u;

struct Tracer {
    const orc_scene& s;
    uint64_t rays = 0;
    Spectral spec;
    bool intersect(const Ray& r, Hit& h) {
        rays++;
        bool hit = spheresIntersect(s, r, h);
        hit |= bvhIntersect(s, r, h, nullptr);
        for (size_t i = 0; i < s.spheres.size() / 7; i++) {
            float t = raySphere(r, &s.spheres[7 * i], 0.0f, h.t);
            if (t < h.t) {
                h.t = t;
                h.prim = kSpherePrim + (uint32_t)i;
                hit = true;
            }
        }
        return hit;
    }
    bool occluded(const Ray& r) {
        rays++;
        for (size_t i = 0; i < s.spheres.size() / 7; i++)
            if (raySphere(r, &s.spheres[7 * i], 0.0f, r.tMax) < kFltInf) return true;
        Hit h;
        if (spheresIntersect(s, r, h)) return true;
        return bvhIntersect(s, r, h, nullptr);
    }
};

struct LightSample {
    S3 weight = s3(0);
    V3 dirW{0, 0, 0};
    float pdf = 0;
    uint32_t id = 0;
    float selectPdf = 0;
};

// Integrator.cu:21-72
static LightSample sampleLight(Tracer& tr, const Intersection& it, const Bsdf& bsdf, Sampler& sp) {
    const orc_scene& s = tr.s;
    int cnt = (int)s.emissive.size();
    if (cnt == 0) return {};
    int pick = std::min<int>(f2i_x86((float)cnt * sp.next1D()), cnt - 1);
    uint32_t id = s.emissive[pick];
    Triangle tri = getTriangle(s, id);
    V2 b = sampleBarycentric(sp.next2D());
    VertexData vd = tri.interpolate({(1.f - b.x) - b.y, b.x, b.y});
    V3 target = offsetRayOrigin(vd.p, tri.faceNormal());
    V3 toLight = target - it.posW;
    float distSqr = dot(toLight, toLight);
    float dist = std::sqrt(distSqr);
    V3 dir = toLight / dist;
    if (dot(it.orientedFaceNormal(), dir) < 0.0f || dot(vd.n, dir) > 0.0f || dist < kEps) return {};
    Ray sr;
    sr.o = offsetRayOrigin(it.posW, it.orientedFaceNormal());
    sr.d = dir;
    sr.tMax = length(sr.o - target) - kEps;
    if (tr.occluded(sr)) return {};
    LightSample ls;
    ls.weight = bsdf.evaluate(it.viewW, dir) * toPathSpec(tr.spec, materialOf(s, id).emission);
    ls.dirW = dir;
    ls.pdf = distSqr / (tri.area() * absDot(dir, vd.n));
    ls.id = id;
    ls.selectPdf = (float)(1.0 / (double)cnt);
    return ls;
}

// Integrator.cu:74-140
static S3 evalMIS(Tracer& tr, const Intersection& it, const Bsdf& bsdf, Sampler& sp) {
    const orc_scene& s = tr.s;
    S3 value = s3(0.0f);
    LightSample ls = sampleLight(tr, it, bsdf, sp);
    if (ls.pdf <= 0.0f) return value;
    {
        float lightPdf = ls.pdf;
        if (lightPdf > 0.0f) {
            float bsdfPdf = bsdf.evaluatePdf(it.viewW, ls.dirW);
            if (bsdfPdf > 0.0f) value = value + (powerHeuristic(lightPdf, bsdfPdf) * ls.weight) / lightPdf;
        }
    }
    {
        V3 dir;
        float bsdfPdf = 0.0f;
        S3 w = bsdf.sampleEvaluate(sp.next2D(), it.viewW, dir, bsdfPdf);
        if (maxValue(w) > 0.0f && bsdfPdf > 0.0f) {
            Ray r;
            r.o = offsetRayOrigin(it.posW, it.orientedFaceNormal());
            r.d = dir;
            Hit h;
            if (tr.intersect(r, h) && h.prim == ls.id) {
                Intersection li = createIntersection(s, r, h);
                const orc_material& m = materialOf(s, h.prim);
                if (m.flags & 1u) {
                    S3 em = toPathSpec(tr.spec, m.emission);
                    V3 toLight = li.posW - it.posW;
                    float distSqr = dot(toLight, toLight);
                    V3 lv = toLight / std::sqrt(distSqr);
                    float cosL = absDot(lv, li.faceNormal);
                    if (cosL != 0.0f) {
                        float area = getTriangle(s, h.prim).area();
                        float lightPdf = distSqr / (area * cosL);
                        value = value + ((powerHeuristic(bsdfPdf, lightPdf) * em) * w) / bsdfPdf;
                    }
                }
            }
        }
    }
    return value / ls.selectPdf;
}

struct CameraData {
    V3 pos, U, V, W;
    float fovY;
    uint32_t width, height;
    float halfH;
};

// Core/Camera.cu:35-39
static CameraData makeCamera(const orc_camera& c) {
    CameraData d;
    d.pos = {c.pos[0], c.pos[1], c.pos[2]};
    V3 target{c.target[0], c.target[1], c.target[2]};
    V3 up{c.up[0], c.up[1], c.up[2]};
    d.W = normalize(target - d.pos);
    d.U = normalize(cross(d.W, up));
    d.V = normalize(cross(d.U, d.W));
    d.fovY = c.fov_y;
    d.width = c.width;
    d.height = c.height;
    // std::tan(radians(fovY * 0.5)) evaluated in double, stored as Float
    d.halfH = (float)std::tan(((double)c.fov_y * 0.5) * 0.01745329251994329576923690768489);
    return d;
}

// Core/CameraProxy.h:25-40
static Ray generateRay(const CameraData& c, V2 sp) {
    float u = 2.0f * (sp.x / (float)c.width) - 1.0f;
    float v = 1.0f - 2.0f * (sp.y / (float)c.height);
    float aspect = (float)c.width / (float)c.height;
    float halfW = aspect * c.halfH;
    V3 dir = normalize((c.U * (u * halfW) + c.V * (v * c.halfH)) + c.W);
    Ray r;
    r.o = c.pos;
    r.d = dir;
    return r;
}

// Core/Integrator.cu:142-227 for one (pixel, sample index); returns the
// radiance and the jittered film position.
static S3 tracePath(Tracer& tr, const CameraData& cam, const orc_integrator_config& cfg,
                    uint32_t x, uint32_t y, uint32_t sampleIndex, V2& pixel) {
    const orc_scene& s = tr.s;
    tr.spec = makeSpectral((cfg.flags & 1u) != 0, x, y, sampleIndex);
    Sampler sp(x, y, sampleIndex);
    V2 j = sp.next2D();
    pixel = {(float)x + j.x, (float)y + j.y};
    Ray ray = generateRay(cam, pixel);
    S3 radiance = s3(0.0f), beta = s3(1.0f);
    for (uint32_t depth = 0; depth < cfg.max_depth; depth++) {
        bool terminate = false;
        Hit h;
        if (tr.intersect(ray, h)) {
            if (h.prim >= kSpherePrim) {  // sphere light (extension)
                const float* sl = &s.spheres[7 * (h.prim - kSpherePrim)];
                radiance = radiance + toPathSpec(tr.spec, sl + 4) * beta;
                break;
            }
            const bool sphere = h.prim >= kSphereBit && h.prim < kSpherePrim;
            Intersection it = sphere ? sphereIntersection(s, ray, h) : createIntersection(s, ray, h);
            const orc_material& m = sphere ? s.mats[s.sphMat[h.prim & ~kSphereBit]] : materialOf(s, h.prim);
            if (m.flags & 1u) {
                radiance = radiance + toPathSpec(tr.spec, m.emission) * beta;
                break;
            }
            // getBSDF, Material/BSDF.cu:11-15: a textured material's diffuse
            // reflectance is the texture sampled at the hit
            const float* diffuse = m.diffuse;
            float texRgb[3];
            const uint32_t mid =
                sphere ? s.sphMat[h.prim & ~kSphereBit] : s.meshes[s.primToMesh[h.prim]].material_id;
            if (mid < s.matTex.size() && s.matTex[mid] != 0xFFFFFFFFu) {
                const RGBA t = texSample(s, s.matTex[mid], it.uv);
                texRgb[0] = t.v[0];
                texRgb[1] = t.v[1];
                texRgb[2] = t.v[2];
                diffuse = texRgb;
            }
            Bsdf bsdf(m, it.frame, diffuse);
            if (tr.spec.on) {
                bsdf.kd = toPathSpec(tr.spec, diffuse);
                bsdf.ks = toPathSpec(tr.spec, m.specular);
            }
            if (cfg.use_mis) {
                radiance = radiance + evalMIS(tr, it, bsdf, sp) * beta;
            } else {
                LightSample ls = sampleLight(tr, it, bsdf, sp);
                if (ls.pdf > 0.0f) radiance = radiance + ((ls.weight * beta) / ls.pdf) / ls.selectPdf;
            }
            V3 wi;
            float pdf = 0.0f;
            S3 f = bsdf.sampleEvaluate(sp.next2D(), it.viewW, wi, pdf);
            if (pdf <= 0.0f) break;
            beta = beta * (f / pdf);
            ray.o = offsetRayOrigin(it.posW, it.orientedFaceNormal());
            ray.d = wi;
        } else {
            if (s.env.x > 0.0f || s.env.y > 0.0f || s.env.z > 0.0f) {  // environment (extension)
                const float e[3] = {s.env.x, s.env.y, s.env.z};
                radiance = radiance + toPathSpec(tr.spec, e) * beta;
            }
            terminate = true;
        }
        if (sp.next1D() < cfg.rr_threshold) terminate = true;
        if (terminate) break;
        if (depth > 5) {
            float q = std::clamp(smax(cfg.rr_threshold, 1.0f - maxValue(beta)), 0.0f, 1.0f);
            if (sp.next1D() < q) break;
            beta = beta / (1.0f - q);
        }
    }
    return radiance;
}

// Core/Sensor.cu:19-43 with an FP64 film
static void addSample(double* rgb, double* w, uint32_t W, uint32_t H, int rowOff,
                      int rows, S3 sample, V2 xy) {
    if (hasNaNOrInf(sample)) return;
    int x0 = (int)std::floor(xy.x - 1.0f), y0 = (int)std::floor(xy.y - 1.0f);
    int x1 = (int)std::ceil(xy.x + 1.0f), y1 = (int)std::ceil(xy.y + 1.0f);
    x0 = std::max(x0, 0);
    y0 = std::max(y0, 0);
    x1 = std::min(x1, (int)W - 1);
    y1 = std::min(y1, (int)H - 1);
    for (int y = y0; y <= y1; y++) {
        for (int x = x0; x <= x1; x++) {
            float dx = xy.x - ((float)x + 0.5f), dy = xy.y - ((float)y + 0.5f);
            float fw = smax(0.0f, 1.0f - std::fabs(dx)) * smax(0.0f, 1.0f - std::fabs(dy));
            int ry = y - rowOff;
            if (ry < 0 || ry >= rows) continue;
            size_t idx = (size_t)ry * W + x;
            for (int c = 0; c < 3; c++) rgb[3 * idx + c] += (double)sample.c[c] * (double)fw;
            w[idx] += (double)fw;
        }
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void orc_sampler_draws(uint32_t px, uint32_t py, uint32_t si, uint32_t n, float* out) {
    Sampler s(px, py, si);
    for (uint32_t i = 0; i < n; i++) out[i] = s.next1D();
}

void orc_sampler_raw(uint32_t px, uint32_t py, uint32_t si, uint32_t n, uint32_t* out) {
    Sampler s(px, py, si);
    for (uint32_t i = 0; i < n; i++) out[i] = s.next();
}

void orc_camera_basis(const orc_camera* cam, float out[9]) {
    CameraData c = makeCamera(*cam);
    V3 b[3] = {c.U, c.V, c.W};
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) out[3 * i + k] = b[i][k];
}

void orc_camera_rays(const orc_camera* cam, const float* sp, uint64_t n, orc_ray* out) {
    CameraData c = makeCamera(*cam);
    for (uint64_t i = 0; i < n; i++) {
        Ray r = generateRay(c, {sp[2 * i], sp[2 * i + 1]});
        out[i] = {{r.o.x, r.o.y, r.o.z}, r.tMin, {r.d.x, r.d.y, r.d.z}, r.tMax};
    }
}

void orc_offset_ray_origin(const float* p, const float* n, uint64_t count, float* out) {
    for (uint64_t i = 0; i < count; i++) {
        V3 r = offsetRayOrigin({p[3 * i], p[3 * i + 1], p[3 * i + 2]}, {n[3 * i], n[3 * i + 1], n[3 * i + 2]});
        out[3 * i] = r.x;
        out[3 * i + 1] = r.y;
        out[3 * i + 2] = r.z;
    }
}

void orc_aabb_intersect(const float* bmin, const float* bmax, const orc_ray* rays, uint64_t n,
                        uint8_t* hit, float* t) {
    for (uint64_t i = 0; i < n; i++) {
        AABB b;
        b.mn = {bmin[3 * i], bmin[3 * i + 1], bmin[3 * i + 2]};
        b.mx = {bmax[3 * i], bmax[3 * i + 1], bmax[3 * i + 2]};
        float tt = kFltInf;
        hit[i] = aabbIntersect(b, toRay(rays[i]), tt) ? 1 : 0;
        t[i] = tt;
    }
}

void orc_triangle_intersect(const float* v0, const float* v1, const float* v2, const orc_ray* rays,
                            uint64_t n, uint8_t* hit, float* t, float* u, float* v) {
    for (uint64_t i = 0; i < n; i++) {
        float uu = 0, vv = 0, tt = 0;
        bool h = triIntersect({v0[3 * i], v0[3 * i + 1], v0[3 * i + 2]}, {v1[3 * i], v1[3 * i + 1], v1[3 * i + 2]},
                              {v2[3 * i], v2[3 * i + 1], v2[3 * i + 2]}, toRay(rays[i]), uu, vv, tt);
        hit[i] = h ? 1 : 0;
        t[i] = h ? tt : 0.0f;
        u[i] = h ? uu : 0.0f;
        v[i] = h ? vv : 0.0f;
    }
}

orc_scene* orc_scene_create(const float* pos, const float* nrm, const float* uv, uint64_t nv,
                            const uint32_t* idx, uint64_t nt, const orc_mesh_desc* meshes,
                            uint32_t n_meshes, const orc_material* mats, uint32_t n_mats,
                            const uint32_t* emissive, uint32_t n_emissive) {
    orc_scene* s = new orc_scene();
    s->pos.resize(nv);
    s->nrm.resize(nv);
    s->uv.resize(nv);
    for (uint64_t i = 0; i < nv; i++) {
        s->pos[i] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        s->nrm[i] = nrm ? V3{nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]} : V3{0, 0, 0};
        s->uv[i] = uv ? V2{uv[2 * i], uv[2 * i + 1]} : V2{0, 0};
    }
    s->idx.assign(idx, idx + 3 * nt);
    s->meshes.assign(meshes, meshes + n_meshes);
    s->mats.assign(mats, mats + n_mats);
    s->emissive.assign(emissive, emissive + n_emissive);
    // Scene/Triangle.cu:121-131: primitive -> mesh
    s->primToMesh.assign(nt, 0);
    for (uint32_t m = 0; m < n_meshes; m++) {
        uint32_t start = meshes[m].index_offset / 3u, count = meshes[m].index_count / 3u;
        for (uint32_t k = 0; k < count && start + k < nt; k++) s->primToMesh[start + k] = m;
    }
    Builder b(*s);
    if (nt > 0) b.run();
    return s;
}

void orc_scene_destroy(orc_scene* s) { delete s; }

void orc_scene_set_lights(orc_scene* s, const float* env3, const float* spheres7, uint32_t n_spheres) {
    s->env = env3 ? V3{env3[0], env3[1], env3[2]} : V3{0, 0, 0};
    s->spheres.assign(spheres7, spheres7 + 7 * (size_t)n_spheres);
}

void orc_scene_set_spheres(orc_scene* s, const float* geom4, const uint32_t* mats, uint32_t n) {
    s->sph.assign(geom4, geom4 + 4 * (size_t)n);
    s->sphMat.assign(mats, mats + n);
}

void orc_scene_set_textures(orc_scene* s, const float* texels, const uint32_t* descs, uint32_t n_tex,
                            const uint32_t* mat_tex, uint32_t n_mats) {
    size_t total = 0;
    for (uint32_t t = 0; t < n_tex; t++) total = std::max<size_t>(total, (size_t)descs[3 * t] + (size_t)descs[3 * t + 1] * descs[3 * t + 2]);
    s->texels.assign(texels, texels + 4 * total);
    s->texDescs.assign(descs, descs + 3 * (size_t)n_tex);
    s->matTex.assign(mat_tex, mat_tex + n_mats);
}

void orc_texture_sample(const orc_scene* s, uint32_t tex, const float* uv, uint64_t n, float* rgba) {
    for (uint64_t i = 0; i < n; i++) {
        const RGBA r = texSample(*s, tex, V2{uv[2 * i], uv[2 * i + 1]});
        for (int k = 0; k < 4; k++) rgba[4 * i + k] = r.v[k];
    }
}

void orc_scene_bvh_stats(const orc_scene* s, orc_bvh_stats* o) {
    std::memset(o, 0, sizeof(*o));
    o->node_count = (uint32_t)s->nodes.size();
    uint32_t leaves = 0;
    for (const Node& n : s->nodes) leaves += n.leaf ? 1 : 0;
    o->leaf_count = leaves;
    o->root_index = s->rootIndex;
    o->max_depth = s->maxDepth;
    o->max_leaf_size = s->maxLeaf;
    o->max_leaf_depth = s->maxLeafDepth;
    for (int k = 0; k < 3; k++) {
        o->root_min[k] = s->rootBounds.mn[k];
        o->root_max[k] = s->rootBounds.mx[k];
    }
}

void orc_scene_bvh_export(const orc_scene* s, orc_bvh_node* nodes, uint32_t* prim_map) {
    for (size_t i = 0; i < s->nodes.size(); i++) {
        const Node& n = s->nodes[i];
        for (int k = 0; k < 3; k++) {
            nodes[i].bmin[k] = n.bounds.mn[k];
            nodes[i].bmax[k] = n.bounds.mx[k];
        }
        nodes[i].is_leaf = n.leaf ? 1 : 0;
        nodes[i].a = n.a;
        nodes[i].b = n.b;
    }
    if (prim_map) std::memcpy(prim_map, s->primMap.data(), s->primMap.size() * 4);
}

void orc_trace_closest(const orc_scene* s, const orc_ray* rays, uint64_t n, orc_hit* hits,
                       uint8_t* ties, int threads, orc_trace_counters* counters) {
    std::atomic<uint64_t> boxes{0}, tris{0}, tieCount{0};
    parallelFor(n, threads, [&](uint64_t b, uint64_t e) {
        Counters c;
        uint64_t tc = 0;
        for (uint64_t i = b; i < e; i++) {
            Hit h;
            const Ray r = toRay(rays[i]);
            bool hit = spheresIntersect(*s, r, h);  // SceneView::intersect: spheres, then the BVH
            hit |= bvhIntersect(*s, r, h, counters ? &c : nullptr);
            if (hit) hits[i] = {h.prim, h.t, h.u, h.v};
            else hits[i] = {0xFFFFFFFFu, kFltInf, 0.0f, 0.0f};
            if (ties) ties[i] = (hit && h.tie) ? 1 : 0;
            tc += (hit && h.tie) ? 1 : 0;
        }
        boxes += c.boxes;
        tris += c.tris;
        tieCount += tc;
    });
    if (counters) {
        counters->rays = n;
        counters->boxes = boxes;
        counters->tris = tris;
        counters->map_reads = tris;
        counters->ties = tieCount;
    }
}

void orc_trace_occluded(const orc_scene* s, const orc_ray* rays, uint64_t n, uint8_t* occ, int threads) {
    parallelFor(n, threads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; i++) {
            Hit h;
            const Ray r = toRay(rays[i]);
            occ[i] = (spheresIntersect(*s, r, h) || bvhIntersect(*s, r, h, nullptr)) ? 1 : 0;
        }
    });
}

void orc_trace_brute(const orc_scene* s, const orc_ray* rays, uint64_t n, orc_hit* hits, int threads) {
    const uint32_t nt = (uint32_t)(s->idx.size() / 3);
    parallelFor(n, threads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; i++) {
            Ray r = toRay(rays[i]);
            Hit h;
            bool any = false;
            any |= spheresIntersect(*s, r, h);
            for (uint32_t p = 0; p < nt; p++) any |= intersectShape(*s, p, r, h);
            if (any) hits[i] = {h.prim, h.t, h.u, h.v};
            else hits[i] = {0xFFFFFFFFu, kFltInf, 0.0f, 0.0f};
        }
    });
}

void orc_bsdf_eval(const orc_material* m, const float* n, const float* wo, const float* wi,
                   uint64_t count, float* f, float* pdf) {
    for (uint64_t i = 0; i < count; i++) {
        Frame fr({n[3 * i], n[3 * i + 1], n[3 * i + 2]});
        Bsdf b(*m, fr);
        V3 o{wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]}, w{wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]};
        S3 v = b.evaluate(o, w);
        for (int c = 0; c < 3; c++) f[3 * i + c] = v.c[c];
        pdf[i] = b.evaluatePdf(o, w);
    }
}

void orc_bsdf_sample(const orc_material* m, const float* n, const float* wo, const float* u,
                     uint64_t count, float* wi, float* f, float* pdf) {
    for (uint64_t i = 0; i < count; i++) {
        Frame fr({n[3 * i], n[3 * i + 1], n[3 * i + 2]});
        Bsdf b(*m, fr);
        V3 o{wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]};
        V3 w;
        float p = 0.0f;
        S3 v = b.sampleEvaluate({u[2 * i], u[2 * i + 1]}, o, w, p);
        for (int c = 0; c < 3; c++) {
            f[3 * i + c] = v.c[c];
            wi[3 * i + c] = w[c];
        }
        pdf[i] = p;
    }
}

void orc_render(const orc_scene* s, const orc_camera* cam, const orc_integrator_config* cfg,
                uint32_t spp, uint32_t first, uint32_t row_begin, uint32_t row_end,
                double* film_rgb, double* film_w, int threads, uint64_t* rays_traced) {
    CameraData c = makeCamera(*cam);
    const uint32_t W = c.width, H = c.height;
    uint32_t y0 = 0, y1 = H;
    if (row_end > row_begin) {
        y0 = row_begin;
        y1 = std::min(row_end, H);
    }
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    const uint32_t rows = y1 - y0;
    threads = (int)std::max<uint32_t>(1, std::min<uint32_t>((uint32_t)threads, rows));
    std::vector<std::vector<double>> bandRgb(threads), bandW(threads);
    std::vector<uint64_t> rayCount(threads, 0);
    std::vector<std::thread> pool;
    std::atomic<uint32_t> nextRow{y0};
    // Rows are handed out dynamically; each thread keeps a full-height film so
    // that the merge is a plain sum.  Sample order per pixel: index first..
    for (int t = 0; t < threads; t++) {
        pool.emplace_back([&, t]() {
            std::vector<double>& rgb = bandRgb[t];
            std::vector<double>& w = bandW[t];
            rgb.assign((size_t)W * H * 3, 0.0);
            w.assign((size_t)W * H, 0.0);
            Tracer tr{*s};
            while (true) {
                uint32_t y = nextRow.fetch_add(1);
                if (y >= y1) break;
                for (uint32_t x = 0; x < W; x++) {
                    for (uint32_t k = 0; k < spp; k++) {
                        V2 pix;
                        S3 L = pathSpecToRgb(tr.spec, tracePath(tr, c, *cfg, x, y, first + k, pix));
                        addSample(rgb.data(), w.data(), W, H, 0, (int)H, L, pix);
                    }
                }
            }
            rayCount[t] = tr.rays;
        });
    }
    for (auto& th : pool) th.join();
    uint64_t total = 0;
    for (int t = 0; t < threads; t++) {
        total += rayCount[t];
        for (size_t i = 0; i < (size_t)W * H * 3; i++) film_rgb[i] += bandRgb[t][i];
        for (size_t i = 0; i < (size_t)W * H; i++) film_w[i] += bandW[t][i];
    }
    if (rays_traced) *rays_traced = total;
}

void orc_spectral_cmf(const float* lambda, uint64_t n, float* xyz) {
    for (uint64_t i = 0; i < n; i++) {
        V3 c = cieXYZ(lambda[i]);
        xyz[3 * i] = c.x;
        xyz[3 * i + 1] = c.y;
        xyz[3 * i + 2] = c.z;
    }
}

void orc_spectral_white_balance(float* out3) {
    V3 w = whiteBalanceOracle();
    out3[0] = w.x;
    out3[1] = w.y;
    out3[2] = w.z;
}

void orc_spectral_upsample(const float* rgb, const float* lambda, uint64_t n, float* out) {
    for (uint64_t i = 0; i < n; i++) {
        float l = lambda[i];
        float bb = 1.0f - sigmoidf((l - 490.0f) / 15.0f), br = sigmoidf((l - 590.0f) / 15.0f);
        float bg = 1.0f - bb - br;
        out[i] = (rgb[3 * i] * br + rgb[3 * i + 1] * bg) + rgb[3 * i + 2] * bb;
    }
}

int orc_hardware_threads(void) { return (int)std::max(1u, std::thread::hardware_concurrency()); }

}  // extern "C"
