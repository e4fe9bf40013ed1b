// cr_shading.cuh -- sampler, shading frame, BSDFs and hit reconstruction of
// the CRaystal path tracer, as device functions.
//
// Each function restates the reference: Core/Sampler.cu:4-31,
// Math/Ray.cu:11-22, Core/Frame.cu:6-30, Core/Intersection.cu:4-10,
// Scene/Scene.cu:31-59, Scene/Triangle.cu:9-38, Math/Sampling.cu:4-58,
// Math/CRayMath.cu:11-13, Material/BSDF.cu:6-103, Material/PhongBRDF.cu,
// Material/PrincipledBRDF.cu, Material/LambertianBRDF.cu, Material/Fresnel.cu.
// Where the reference computes in double (a double literal promotes the
// expression) the device code does too.
#pragma once

#include "cr_internal.cuh"
#include "cr_math.cuh"

namespace cr {

// ---------------------------------------------------------------------------
// Sampler (PCG variant), Core/Sampler.cu:4-31
// ---------------------------------------------------------------------------
struct Sampler {
    uint32_t state, inc;
    Sampler() = default;
    // a sampler resumed from a saved (state, inc)
    __device__ __forceinline__ static Sampler resume(uint32_t state, uint32_t inc) {
        Sampler s;
        s.state = state;
        s.inc = inc;
        return s;
    }
    __device__ __forceinline__ Sampler(uint32_t px, uint32_t py, uint32_t sampleIndex) {
        state = px * 2654435761u + py * 1597334677u + sampleIndex;
        inc = px * 1234567891u + py * 987654321u + 1u;
        for (int i = 0; i < 4; ++i) next();
    }
    __device__ __forceinline__ uint32_t next() {
        uint32_t old = state;
        state = old * 747796405u + inc;
        old = ((old >> ((old >> 28u) + 4u)) ^ old) * 277803737u;
        return (old >> 22u) ^ old;
    }
    __device__ __forceinline__ static float toFloat(uint32_t s) { return (float)s * (1.0f / 4294967296.0f); }
    __device__ __forceinline__ float next1D() { return toFloat(next()); }
    // Float2(stateToFloat(nextState()), stateToFloat(nextState())): the first
    // draw is x.
    __device__ __forceinline__ float2 next2D() {
        float a = toFloat(next());
        float b = toFloat(next());
        return make_float2(a, b);
    }
};

// Math/Ray.cu:11-22 (Ray Tracing Gems, chapter 6)
__device__ __forceinline__ float3 offsetRayOrigin(float3 p, float3 n) {
    const float kOrigin = 1.0f / 32.0f;
    const float kFltScale = 1.0f / 65535.0f;
    const float kIntScale = 256.0f;
    const int ox = f2iX86(kIntScale * n.x), oy = f2iX86(kIntScale * n.y), oz = f2iX86(kIntScale * n.z);
    const float px = __int_as_float(__float_as_int(p.x) + ((p.x < 0) ? -ox : ox));
    const float py = __int_as_float(__float_as_int(p.y) + ((p.y < 0) ? -oy : oy));
    const float pz = __int_as_float(__float_as_int(p.z) + ((p.z < 0) ? -oz : oz));
    return mk3(fabsf(p.x) < kOrigin ? p.x + kFltScale * n.x : px, fabsf(p.y) < kOrigin ? p.y + kFltScale * n.y : py,
               fabsf(p.z) < kOrigin ? p.z + kFltScale * n.z : pz);
}

// ---------------------------------------------------------------------------
// Frame, Core/Frame.cu:6-30
// ---------------------------------------------------------------------------
struct Frame {
    float3 T, B, N;
    __device__ __forceinline__ void build(float3 n) {
        float3 t = mk3(0.0f, 1.0f, 0.0f);
        if (1.0 - (double)absDot(n, t) < (double)kEps) t = mk3(1.0f, 0.0f, 0.0f);
        const float3 bt = normalize(cross(n, t));
        T = normalize(cross(bt, n));
        N = n;
        B = cross(N, T);
    }
    __device__ __forceinline__ float3 toLocal(float3 w) const { return mk3(dot(T, w), dot(B, w), dot(N, w)); }
    __device__ __forceinline__ float3 toWorld(float3 l) const {
        return mk3((T.x * l.x + B.x * l.y) + N.x * l.z, (T.y * l.x + B.y * l.y) + N.y * l.z,
                   (T.z * l.x + B.z * l.y) + N.z * l.z);
    }
};

// Intersection, Core/Intersection.h:11-26
struct Isect {
    float3 posW, faceN, viewW;
    bool front;
    Frame frame;
    __device__ __forceinline__ float3 orientedFaceNormal() const { return front ? faceN : neg(faceN); }
};

struct TriVerts {
    float3 p[3], n[3];
};

__device__ __forceinline__ TriVerts loadTriangle(const SceneView& sc, uint32_t prim) {
    TriVerts t;
    for (int k = 0; k < 3; k++) {
        const uint32_t vi = __ldg(sc.idx + 3 * prim + k);
        t.p[k] = sc.pos[vi];
        t.n[k] = sc.nrm[vi];
    }
    return t;
}
// TriangleData::getFaceNormal / interpolate / getArea, Scene/Triangle.cu:9-38
__device__ __forceinline__ float3 faceNormal(const TriVerts& t) {
    return normalize(cross(sub(t.p[1], t.p[0]), sub(t.p[2], t.p[0])));
}
__device__ __forceinline__ float3 interp(const float3 v[3], float3 w) {
    return add(add(mul(v[0], w.x), mul(v[1], w.y)), mul(v[2], w.z));
}
__device__ __forceinline__ float triArea(const TriVerts& t) {
    return length(cross(sub(t.p[0], t.p[1]), sub(t.p[2], t.p[1]))) / 2.f;
}

// SceneView::createIntersection, Scene/Scene.cu:31-59
__device__ __forceinline__ Isect makeIsect(const SceneView& sc, float3 o, float3 d, float t, float u, float v,
                                           uint32_t prim) {
    Isect it;
    it.posW = add(o, mul(t, d));
    it.viewW = neg(normalize(d));
    const float3 w = mk3((1.f - u) - v, u, v);
    const TriVerts tri = loadTriangle(sc, prim);
    it.faceN = faceNormal(tri);
    const float3 sn = normalize(interp(tri.n, w));
    it.front = dot(it.viewW, it.faceN) > 0.0f;
    it.frame.build(it.front ? sn : neg(sn));
    return it;
}

// createIntersection of a sphere hit (Scene/Scene.cu:43-47): the face and
// shading normal point from the centre to the hit point.
__device__ __forceinline__ Isect makeIsectSphere(const SceneView& sc, float3 o, float3 d, float t, uint32_t id) {
    Isect it;
    it.posW = add(o, mul(t, d));
    it.viewW = neg(normalize(d));
    const float4 g = __ldg(sc.sphGeom + id);
    it.faceN = normalize(sub(it.posW, mk3(g.x, g.y, g.z)));
    it.front = dot(it.viewW, it.faceN) > 0.0f;
    it.frame.build(it.front ? it.faceN : neg(it.faceN));
    return it;
}

__device__ __forceinline__ const MaterialGpu& materialOf(const SceneView& sc, uint32_t prim) {
    return sc.mats[sc.meshes[sc.primToMesh[prim]].material_id];
}

// Interpolated texture coordinates of a hit (TriangleData::interpolate,
// Scene/Triangle.cu:18-30, with the weights of HitInfo::getBarycentricWeights,
// Core/Hit.h:20-23).
__device__ __forceinline__ float2 texCoordAt(const SceneView& sc, uint32_t prim, float u, float v) {
    const float w0 = (1.f - u) - v;
    float2 t[3];
    for (int k = 0; k < 3; k++) t[k] = sc.uv[__ldg(sc.idx + 3 * prim + k)];
    return make_float2((t[0].x * w0 + t[1].x * u) + t[2].x * v, (t[0].y * w0 + t[1].y * u) + t[2].y * v);
}

// TextureView::fetchTexel (Core/Texture.cu:6-13): clamp to the last texel.
__device__ __forceinline__ float4 texFetch(const SceneView& sc, uint4 d, uint32_t x, uint32_t y) {
    x = (d.y - 1u) < x ? d.y - 1u : x;
    y = (d.z - 1u) < y ? d.z - 1u : y;
    return __ldg(sc.texels + d.x + (y * d.y + x));
}

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t) {
    const float s = 1.0f - t;
    return make_float4(a.x * s + b.x * t, a.y * s + b.y * t, a.z * s + b.z * t, a.w * s + b.w * t);
}

// TextureView::sample (Core/Texture.cu:15-35): bilinear over texel centres
// at uv * (size - 1).  The float -> uint32 conversions are the device's
// (truncating and saturating: a negative coordinate gives texel 0 and a
// negative fraction, which extrapolates as the reference does).
__device__ __forceinline__ float4 texSample(const SceneView& sc, uint32_t tex, float2 uv) {
    const uint4 d = __ldg(sc.texDescs + tex);
    const float px = uv.x * (float)(d.y - 1u);
    const float py = uv.y * (float)(d.z - 1u);
    const uint32_t x0 = __float2uint_rz(floorf(px));
    const uint32_t y0 = __float2uint_rz(floorf(py));
    const uint32_t x1 = min(x0 + 1u, d.y - 1u);
    const uint32_t y1 = min(y0 + 1u, d.z - 1u);
    const float fx = px - (float)x0;
    const float fy = py - (float)y0;
    const float4 c0 = lerp4(texFetch(sc, d, x0, y0), texFetch(sc, d, x1, y0), fx);
    const float4 c1 = lerp4(texFetch(sc, d, x0, y1), texFetch(sc, d, x1, y1), fx);
    return lerp4(c0, c1, fy);
}

// ---------------------------------------------------------------------------
// Math/Sampling.cu, Math/CRayMath.cu
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 sampleBarycentric(float2 u) {
    float u1 = u.x, u2 = u.y;
    const bool flip = (u1 + u2) > 1.0f;
    u1 = flip ? (1.0f - u1) : u1;
    u2 = flip ? (1.0f - u2) : u2;
    return make_float2(u1, u2);
}
__device__ __forceinline__ float3 cosineSampleHemisphere(float2 u) {
    const float r = sqrtf(u.x);
    const float phi = 2.0f * kPi * u.y;
    const float x = r * cosf(phi);
    const float y = r * sinf(phi);
    const float z = sqrtf(smax(0.0f, (1.0f - x * x) - y * y));
    return mk3(x, y, z);
}
__device__ __forceinline__ float cosinePdf(float3 d) { return smax(0.0f, d.z) * kInvPi; }
__device__ __forceinline__ float powerHeuristic(float f, float g) {
    const float a = 1.0f * f, b = 1.0f * g;
    return (a * a) / (a * a + b * b);
}
__device__ __forceinline__ float acosSafe(float v) { return acosf(gclamp(v, kEps, (float)(1.0 - (double)kEps))); }
// x^5 in double, the value std::pow(x, 5.0) rounds to before the float
// conversion that follows it in PrincipledBRDF.cu:134-135
__device__ __forceinline__ double pow5d(double x) {
    const double x2 = x * x;
    return (x2 * x2) * x;
}

// ---------------------------------------------------------------------------
// BSDF, Material/BSDF.{h,cu} + the three lobes
// ---------------------------------------------------------------------------
struct Bsdf {
    uint32_t type;
    Spec kd, ks;
    float n, dProb, sProb, rough, metal;
    Frame frame;

    __device__ __forceinline__ void init(const MaterialGpu& m, const Frame& f) {
        type = m.type;
        kd = sp(m.kd[0], m.kd[1], m.kd[2]);
        ks = sp(m.ks[0], m.ks[1], m.ks[2]);
        n = m.shininess;
        dProb = m.dProb;
        sProb = m.sProb;
        rough = m.rough;
        metal = m.metal;
        frame = f;
    }

    // PhongBRDF.cu:20-68
    __device__ __forceinline__ Spec phongEval(float3 wo, float3 wi) const {
        const float3 r = reflect(neg(wo), mk3(0.0f, 0.0f, 1.0f));
        const float c = smax(dot(r, wi), 0.0f);
        return add(mul(kd, kInvPi), mul(mul(mul(ks, n + 2.0f), kInv2Pi), powf(c, n)));
    }
    __device__ __forceinline__ float phongPdf(float3 wo, float3 wi) const {
        const float dp = cosinePdf(wi);
        const float3 r = reflect(neg(wo), mk3(0.0f, 0.0f, 1.0f));
        const float ca = smax(dot(r, wi), 0.0f);
        const float spdf = (n + 1.0f) * kInv2Pi * powf(ca, n);
        return dp * dProb + spdf * sProb;
    }
    __device__ __forceinline__ float3 phongSample(float3 wo, float2 u, float& pdf) const {
        float2 u0 = u;
        float3 wi = mk3(0.0f, 0.0f, 0.0f);
        pdf = 0.0f;
        const bool hasD = dProb > 0.0f, hasS = sProb > 0.0f;
        if (hasD && u0.x < dProb) {
            u0.x /= dProb;
            wi = cosineSampleHemisphere(u0);
            pdf = cosinePdf(wi);
        } else if (hasS) {
            u0.x = (u0.x - dProb) / sProb;
            const float alpha = acosSafe(powf(u0.x, 1.0f / (n + 1.0f)));
            const float theta = gclamp(acosSafe(wo.z) + alpha, 0.0f, (float)((double)kPi / 2.0));
            const float phi = k2Pi * u0.y;
            const float st = sinf(theta);
            wi = mk3(st * cosf(phi), st * sinf(phi), (float)sqrt(1.0 - (double)(st * st)));
            pdf = (n + 1.0f) * kInv2Pi * powf(cosf(alpha), n);
        }
        return wi;
    }

    // PrincipledBRDF.cu:9-150
    __device__ __forceinline__ static float ndf(float r, float ch) {
        const float a = r * r;
        const float a2 = a * a;
        const float c2 = ch * ch;
        const float den = (float)(1.0 + ((double)a2 - 1.0) * (double)c2);
        return a2 * kInvPi / (den * den);
    }
    __device__ __forceinline__ static float smithG1(float ag, float cv) {
        const float a = ag * ag, b = cv * cv;
        return 1.0f / (cv + sqrtf((a + b) - a * b));
    }
    __device__ __forceinline__ static float geom(float r, float ci, float cv) {
        float alpha = (float)(0.5 + (double)r * 0.5);
        alpha *= alpha;
        return smithG1(alpha, ci) * smithG1(alpha, cv);
    }
    __device__ __forceinline__ Spec princEval(float3 wo, float3 wi) const {
        if (wo.z <= 0.0f || wi.z <= 0.0f) return sp(0.0f);
        const float3 wh = normalize(add(wo, wi));
        const float cv = wo.z, ci = wi.z, ch = wh.z;
        const float cd = dot(wo, wh);
        const float fd90 = (float)(0.5 + ((2.0 * (double)rough) * (double)cd) * (double)cd);
        const float fl = (float)(1.0 + ((double)fd90 - 1.0) * pow5d(1.0 - (double)ci));
        const float fv = (float)(1.0 + ((double)fd90 - 1.0) * pow5d(1.0 - (double)cv));
        const Spec diffuse = mul(mul(mul(mul(kd, kInvPi), fv), fl), 1.0f - metal);
        const float D = ndf(rough, ch);
        const Spec f0 = add(mul(kd, 1.0f - metal), mul(sp(0.04f), metal));
        const float v0 = 1.f - cd;
        const float v1 = v0 * v0;
        const Spec F = add(f0, mul(mul(mul(sub(sp(1.0f), f0), v1), v1), v0));
        const float G = geom(rough, ci, cv);
        const float denom = (float)((4.0 * (double)ci) * (double)cv);
        const Spec spec = divs(mul(mul(D, F), G), denom);
        return add(diffuse, spec);
    }
    __device__ __forceinline__ float princPdf(float3 wo, float3 wi) const {
        if (wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
        const float3 wh = normalize(add(wo, wi));
        const float ch = wh.z;
        const float cd = dot(wo, wh);
        if (cd <= 0.0f) return 0.0f;
        const float dp = cosinePdf(wi);
        float spdf = 0.0f;
        if (ch > 0.0f) {
            const float D = ndf(rough, ch);
            spdf = D * ch / (4.0f * cd);
        }
        return dp * dProb + spdf * sProb;
    }
    __device__ __forceinline__ float3 princSample(float3 wo, float2 u, float& pdf) const {
        if (wo.z <= 0.0f) {
            pdf = 0.0f;
            return mk3(0.0f, 0.0f, 0.0f);
        }
        float u1 = u.x;
        const float u2 = u.y;
        float3 wi;
        if (u1 < sProb) {
            u1 /= sProb;
            const float alpha = rough * rough;
            const float a2 = alpha * alpha;
            const float phi = u2 * k2Pi;
            const float tan2 = a2 * u1 / (1.0f - u1);
            const float ct = 1.0f / sqrtf(1.0f + tan2);
            const float r = sqrtf(smax(1.0f - ct * ct, 0.0f));
            const float3 wh = mk3(cosf(phi) * r, sinf(phi) * r, ct);
            wi = reflect(neg(wo), wh);
        } else {
            u1 = (u1 - sProb) / (1.0f - sProb);
            wi = cosineSampleHemisphere(make_float2(u1, u2));
        }
        pdf = princPdf(wo, wi);
        return wi;
    }

    // dispatch, Material/BSDF.h:30-57 and Material/BSDF.cu:36-103.
    // kPrincipled = false: code for a scene without Principled materials,
    // whose shading kernels then carry only the Lambertian and Phong lobes.
    template <bool kPrincipled = true>
    __device__ __forceinline__ Spec evalLocal(float3 wo, float3 wi) const {
        Spec f;
        if (type == CR_MATERIAL_PHONG) f = phongEval(wo, wi);
        else if (kPrincipled && type == CR_MATERIAL_PRINCIPLED) f = princEval(wo, wi);
        else f = mul(kd, kInvPi);
        return mul(f, fabsf(wi.z));
    }
    template <bool kPrincipled = true>
    __device__ __forceinline__ float pdfLocal(float3 wo, float3 wi) const {
        if (type == CR_MATERIAL_PHONG) return phongPdf(wo, wi);
        if (kPrincipled && type == CR_MATERIAL_PRINCIPLED) return princPdf(wo, wi);
        return cosinePdf(wi);
    }
    template <bool kPrincipled = true>
    __device__ __forceinline__ float3 sampleLocal(float3 wo, float2 u, float& pdf) const {
        if (type == CR_MATERIAL_PHONG) return phongSample(wo, u, pdf);
        if (kPrincipled && type == CR_MATERIAL_PRINCIPLED) return princSample(wo, u, pdf);
        const float3 wi = cosineSampleHemisphere(u);
        pdf = cosinePdf(wi);
        return wi;
    }
    template <bool kPrincipled = true>
    __device__ __forceinline__ Spec evaluate(float3 wo, float3 wi) const {
        return evalLocal<kPrincipled>(frame.toLocal(wo), frame.toLocal(wi));
    }
    template <bool kPrincipled = true>
    __device__ __forceinline__ float evaluatePdf(float3 wo, float3 wi) const {
        return pdfLocal<kPrincipled>(frame.toLocal(wo), frame.toLocal(wi));
    }
    template <bool kPrincipled = true>
    __device__ __forceinline__ Spec sampleEvaluate(float2 u, float3 wo, float3& wi, float& pdf) const {
        const float3 woL = frame.toLocal(wo);
        pdf = 0.0f;
        const float3 wiL = sampleLocal<kPrincipled>(woL, u, pdf);
        const Spec f = evalLocal<kPrincipled>(woL, wiL);
        wi = frame.toWorld(wiL);
        return f;
    }
};

}  // namespace cr
