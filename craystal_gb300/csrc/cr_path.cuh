// cr_path.cuh -- the path-tracing loop of pathTraceKernel<useMIS>
// (Core/Integrator.cu:142-227) with sampleLight (:21-72) and evalMIS
// (:74-140), shared by the plain megakernel (cr_render.cu) and the
// radiance-cache integrator (cr_cache.cu) through a hook called at every
// surface vertex.
#pragma once

#include "cr_internal.cuh"
#include "cr_math.cuh"
#include "cr_shading.cuh"
#include "cr_spectral.cuh"
#include "cr_traverse.cuh"

namespace cr {

struct Params {
    uint32_t maxDepth;
    float rrThreshold;
    uint32_t useMIS;
    uint32_t spp;
    uint32_t first;
    uint32_t sppPerBlock;
    uint32_t spectral;  // CR_RENDER_SPECTRAL: channels carry three wavelengths
    float3 wb;          // white balance of the spectral film conversion
};

struct PathCtx {
    const SceneView& sc;
    uint32_t rays;
    SpectralPath spec;  // set by tracePath
};

__device__ __forceinline__ Spec emissionOf(const PathCtx& c, const MaterialGpu& m) {
    return toPathSpec(c.spec, m.em[0], m.em[1], m.em[2]);
}

// What a scene's shading code must handle.  kFullScene = false: no
// Principled material, no diffuse texture and no analytic spheres (sphere
// lights are still handled); the wavefront's shade stage is instantiated
// both ways and a scene takes the lean form when its materials and
// geometry allow (5 % faster renders of the Cornell box on GB300: smaller
// code, fewer spilled registers).  Everything else defaults to the full form.

// getBSDF (Material/BSDF.cu:7-31): the material's lobes, with the diffuse
// reflectance of a textured material sampled at the hit.
template <bool kFullScene = true>
__device__ __forceinline__ void initBsdf(const PathCtx& c, Bsdf& b, const MaterialGpu& m, const Frame& f,
                                         uint32_t prim, float u, float v) {
    b.init(m, f);
    if (kFullScene && m.tex != CR_NO_TEXTURE) {
        // a sphere's texture coordinates are its hit's (u, v), Scene/Scene.cu:41
        const float2 tc = isSphereHit(prim) ? make_float2(u, v) : texCoordAt(c.sc, prim, u, v);
        const float4 t = texSample(c.sc, m.tex, tc);
        b.kd = sp(t.x, t.y, t.z);
        if (m.type == CR_MATERIAL_PHONG) phongLobeProbs(b.kd, b.ks, kEps, b.dProb, b.sProb);
    }
    if (c.spec.on) {
        b.kd = toPathSpec(c.spec, b.kd.r, b.kd.g, b.kd.b);
        b.ks = toPathSpec(c.spec, m.ks[0], m.ks[1], m.ks[2]);
    }
}

// Nearest intersection t of a ray with a sphere (centre c, radius r) in
// (tMin, tMax), or INFINITY (geometric form: oc = o - c, b = oc.d / d.d).
__device__ __forceinline__ float raySphere(float3 o, float3 d, float4 s, float tMin, float tMax) {
    const float3 oc = sub(o, mk3(s.x, s.y, s.z));
    const float a = dot(d, d);
    const float b = dot(oc, d) / a;
    const float c = (dot(oc, oc) - s.w * s.w) / a;
    const float disc = b * b - c;
    if (disc < 0.0f) return INFINITY;
    const float q = sqrtf(disc);
    const float t0 = -b - q, t1 = -b + q;
    if (t0 > tMin && t0 < tMax) return t0;
    if (t1 > tMin && t1 < tMax) return t1;
    return INFINITY;
}


// SceneView::intersect (Scene/Scene.cu:5-14): the BVH, then the sphere
// lights (an extension) under the closest-hit rule.
template <int kShared = 0, bool kFullScene = true>
__device__ __forceinline__ bool closest(PathCtx& c, float3 o, float3 d, THit& h,
                                        uint2 (*shStack)[kStackBlock] = nullptr) {
    c.rays++;
    h.t = INFINITY;
    h.prim = CR_MISS;
    h.u = h.v = 0.0f;
    const TRay r = makeTRay(o, 0.0f, d, INFINITY);
    bool hit = false;
    if (kFullScene && c.sc.sph.hasRoot) hit = traverseSpheres<false, kShared>(c.sc, r, h, shStack);
    hit |= traverse<false, kShared>(c.sc, r, h, shStack);
    for (uint32_t i = 0; i < c.sc.nSpheres; i++) {
        const float t = raySphere(o, d, __ldg(c.sc.spheres + i), 0.0f, h.t);
        if (t < h.t) {
            h.t = t;
            h.prim = kSpherePrim + i;
            hit = true;
        }
    }
    return hit;
}

// SceneView::intersectOcclusion (Scene/Scene.cu:16-29), spheres included.
template <bool kFullScene = true>
__device__ __forceinline__ bool occluded(PathCtx& c, float3 o, float3 d, float tMax) {
    c.rays++;
    for (uint32_t i = 0; i < c.sc.nSpheres; i++)
        if (raySphere(o, d, __ldg(c.sc.spheres + i), 0.0f, tMax) < INFINITY) return true;
    THit h;
    h.t = INFINITY;
    const TRay r = makeTRay(o, 0.0f, d, tMax);
    if (kFullScene && c.sc.sph.hasRoot && traverseSpheres<true>(c.sc, r, h)) return true;
    return traverse<true>(c.sc, r, h);
}

// The shadow and MIS rays' queries, inline (kOutOfLine = false) or as calls
// to one out-of-line copy.  The megakernel and the wavefront's shade stage
// inline them.  With the earlier whole-leaf traversal step, calls made
// wavefront shading 1.6x faster on a small scene (fewer instruction-fetch
// stalls); with the one-slot step, inline is 1-4 % faster on every scene
// measured.  kWfFinish, which runs few paths, keeps the calls.
static __device__ __noinline__ bool closestOutOfLine(PathCtx* c, float3 o, float3 d, THit* h) {
    return closest(*c, o, d, *h);
}
static __device__ __noinline__ bool occludedOutOfLine(PathCtx* c, float3 o, float3 d, float tMax) {
    return occluded(*c, o, d, tMax);
}
template <bool kOutOfLine, bool kFullScene = true>
__device__ __forceinline__ bool closestSecondary(PathCtx& c, float3 o, float3 d, THit& h) {
    if (kOutOfLine) return closestOutOfLine(&c, o, d, &h);
    return closest<0, kFullScene>(c, o, d, h);
}
template <bool kOutOfLine, bool kFullScene = true>
__device__ __forceinline__ bool occludedSecondary(PathCtx& c, float3 o, float3 d, float tMax) {
    if (kOutOfLine) return occludedOutOfLine(&c, o, d, tMax);
    return occluded<kFullScene>(c, o, d, tMax);
}

struct LightSample {
    Spec weight;
    float3 dirW;
    float pdf;
    uint32_t id;
    float selectPdf;
};

// sampleLight, Core/Integrator.cu:21-72
template <bool kOutOfLine = false, bool kFullScene = true>
__device__ __forceinline__ LightSample sampleLight(PathCtx& c, const Isect& it, const Bsdf& bsdf, Sampler& smp) {
    const SceneView& sc = c.sc;
    LightSample ls;
    ls.weight = sp(0.0f);
    ls.dirW = mk3(0.0f, 0.0f, 0.0f);
    ls.pdf = 0.0f;
    ls.id = 0;
    ls.selectPdf = 0.0f;
    const int cnt = (int)sc.nEmissive;
    if (cnt == 0) return ls;
    const int pick = min(f2iX86((float)cnt * smp.next1D()), cnt - 1);
    const uint32_t id = sc.emissive[pick];
    const TriVerts tri = loadTriangle(sc, id);
    const float2 b = sampleBarycentric(smp.next2D());
    const float3 w = mk3((1.f - b.x) - b.y, b.x, b.y);
    const float3 vp = interp(tri.p, w);
    const float3 vn = interp(tri.n, w);
    const float3 target = offsetRayOrigin(vp, faceNormal(tri));
    const float3 toLight = sub(target, it.posW);
    const float distSqr = dot(toLight, toLight);
    const float dist = sqrtf(distSqr);
    const float3 dir = divs(toLight, dist);
    const float3 ofn = it.orientedFaceNormal();
    if (dot(ofn, dir) < 0.0f || dot(vn, dir) > 0.0f || dist < kEps) return ls;
    const float3 so = offsetRayOrigin(it.posW, ofn);
    const float tMax = length(sub(so, target)) - kEps;
    if (occludedSecondary<kOutOfLine, kFullScene>(c, so, dir, tMax)) return ls;
    const MaterialGpu& m = materialOf(sc, id);
    ls.weight = mul(bsdf.evaluate<kFullScene>(it.viewW, dir), emissionOf(c, m));
    ls.dirW = dir;
    ls.pdf = distSqr / (triArea(tri) * absDot(dir, vn));
    ls.id = id;
    ls.selectPdf = (float)(1.0 / (double)cnt);
    return ls;
}

// evalMIS, Core/Integrator.cu:74-140
template <bool kOutOfLine = false, bool kFullScene = true>
__device__ __forceinline__ Spec evalMIS(PathCtx& c, const Isect& it, const Bsdf& bsdf, Sampler& smp) {
    const SceneView& sc = c.sc;
    Spec value = sp(0.0f);
    const LightSample ls = sampleLight<kOutOfLine, kFullScene>(c, it, bsdf, smp);
    if (ls.pdf <= 0.0f) return value;
    {
        const float lightPdf = ls.pdf;
        if (lightPdf > 0.0f) {
            const float bsdfPdf = bsdf.evaluatePdf<kFullScene>(it.viewW, ls.dirW);
            if (bsdfPdf > 0.0f) value = add(value, divs(mul(powerHeuristic(lightPdf, bsdfPdf), ls.weight), lightPdf));
        }
    }
    {
        float3 dir;
        float bsdfPdf = 0.0f;
        const Spec w = bsdf.sampleEvaluate<kFullScene>(smp.next2D(), it.viewW, dir, bsdfPdf);
        if (maxValue(w) > 0.0f && bsdfPdf > 0.0f) {
            const float3 o = offsetRayOrigin(it.posW, it.orientedFaceNormal());
            THit h;
            if (closestSecondary<kOutOfLine, kFullScene>(c, o, dir, h) && h.prim == ls.id) {
                // createIntersection of the light hit: only its position and
                // face normal are read
                const TriVerts tri = loadTriangle(sc, h.prim);
                const float3 lpos = add(o, mul(h.t, dir));
                const float3 lfn = faceNormal(tri);
                const MaterialGpu& m = materialOf(sc, h.prim);
                if (m.flags & CR_MATERIAL_EMISSIVE) {
                    const Spec em = emissionOf(c, m);
                    const float3 toLight = sub(lpos, it.posW);
                    const float distSqr = dot(toLight, toLight);
                    const float3 lv = divs(toLight, sqrtf(distSqr));
                    const float cosL = absDot(lv, lfn);
                    if (cosL != 0.0f) {
                        const float area = triArea(tri);
                        const float lightPdf = distSqr / (area * cosL);
                        value = add(value, divs(mul(mul(powerHeuristic(bsdfPdf, lightPdf), em), w), bsdfPdf));
                    }
                }
            }
        }
    }
    return divs(value, ls.selectPdf);
}

// CameraProxy::generateRay, Core/CameraProxy.h:25-40
__device__ __forceinline__ float3 cameraDir(const CameraGpu& cam, float2 s) {
    const float u = 2.0f * (s.x / (float)cam.width) - 1.0f;
    const float v = 1.0f - 2.0f * (s.y / (float)cam.height);
    return normalize(add(add(mul(cam.U, u * cam.halfW), mul(cam.V, v * cam.halfH)), cam.W));
}

// Hooks of tracePath: called at every surface vertex before it is shaded
// (depth = vertex index, 0 = the camera ray's hit); returning true ends the
// path there.  The plain integrator uses NoHooks.
struct NoHooks {
    __device__ __forceinline__ bool atVertex(uint32_t, const Isect&, const MaterialGpu&, const Spec&, const Spec&) {
        return false;
    }
};

// One bounce of pathTraceKernel<useMIS> after its closest-hit query
// (Core/Integrator.cu:170-225): h is the query's hit (h.prim == CR_MISS for
// a miss).  Updates the ray, throughput and radiance; returns false when the
// path ends.  Shared by the megakernel (tracePath) and the wavefront shade
// stage (cr_wavefront.cu), so both consume the sampler identically.
template <class Hooks, bool kOutOfLine = false, bool kFullScene = true>
__device__ __forceinline__ bool shadeBounce(PathCtx& c, const Params& p, Sampler& smp, uint32_t depth, const THit& h,
                                            float3& ro, float3& rd, Spec& beta, Spec& radiance, Hooks& hk) {
    const SceneView& sc = c.sc;
    bool terminate = false;
    if (h.prim != CR_MISS) {
        if (h.prim >= kSpherePrim) {  // a sphere light (extension)
            const float4 e = __ldg(sc.sphereEm + (h.prim - kSpherePrim));
            radiance = add(radiance, mul(toPathSpec(c.spec, e.x, e.y, e.z), beta));
            return false;
        }
        const bool sphere = kFullScene && isSphereHit(h.prim);
        const Isect it = sphere ? makeIsectSphere(sc, ro, rd, h.t, h.prim & ~kSphereBit)
                                : makeIsect(sc, ro, rd, h.t, h.u, h.v, h.prim);
        const MaterialGpu& m = sphere ? sc.mats[__ldg(sc.sphMat + (h.prim & ~kSphereBit))] : materialOf(sc, h.prim);
        if (hk.atVertex(depth, it, m, beta, radiance)) return false;
        if (m.flags & CR_MATERIAL_EMISSIVE) {
            radiance = add(radiance, mul(emissionOf(c, m), beta));
            return false;
        }
        Bsdf bsdf;
        initBsdf<kFullScene>(c, bsdf, m, it.frame, h.prim, h.u, h.v);
        if (p.useMIS) {
            radiance = add(radiance, mul(evalMIS<kOutOfLine, kFullScene>(c, it, bsdf, smp), beta));
        } else {
            const LightSample ls = sampleLight<kOutOfLine, kFullScene>(c, it, bsdf, smp);
            if (ls.pdf > 0.0f) radiance = add(radiance, divs(divs(mul(ls.weight, beta), ls.pdf), ls.selectPdf));
        }
        float3 wi;
        float pdf = 0.0f;
        const Spec f = bsdf.sampleEvaluate<kFullScene>(smp.next2D(), it.viewW, wi, pdf);
        if (pdf <= 0.0f) return false;
        beta = mul(beta, divs(f, pdf));
        ro = offsetRayOrigin(it.posW, it.orientedFaceNormal());
        rd = wi;
    } else {
        // a miss ends the path (Core/Integrator.cu:205-207), after
        // collecting the constant environment when there is one (extension)
        if (sc.env.x > 0.0f || sc.env.y > 0.0f || sc.env.z > 0.0f)
            radiance = add(radiance, mul(toPathSpec(c.spec, sc.env.x, sc.env.y, sc.env.z), beta));
        terminate = true;
    }
    if (smp.next1D() < p.rrThreshold) terminate = true;
    if (terminate) return false;
    if (depth > 5) {
        float q = smax(p.rrThreshold, 1.0f - maxValue(beta));
        q = q < 0.0f ? 0.0f : (1.0f < q ? 1.0f : q);
        if (smp.next1D() < q) return false;
        beta = divs(beta, 1.0f - q);
    }
    return true;
}

// The camera ray of a (pixel, sample index): the sampler's first 2D draw
// jitters the film position (Core/Integrator.cu:150-156).
__device__ __forceinline__ void cameraRay(const CameraGpu& cam, Sampler& smp, uint32_t x, uint32_t y, float2& pixel,
                                          float3& ro, float3& rd) {
    const float2 j = smp.next2D();
    pixel = make_float2((float)x + j.x, (float)y + j.y);
    ro = cam.pos;
    rd = cameraDir(cam, pixel);
}

// pathTraceKernel body for one (pixel, sample index).
template <class Hooks>
__device__ __forceinline__ Spec tracePath(PathCtx& c, const CameraGpu& cam, const Params& p, uint32_t x, uint32_t y,
                                          uint32_t si, float2& pixel, Hooks& hk) {
    c.spec = makeSpectralPath(p.spectral != 0, x, y, si);
    Sampler smp(x, y, si);
    float3 ro, rd;
    cameraRay(cam, smp, x, y, pixel, ro, rd);
    Spec radiance = sp(0.0f), beta = sp(1.0f);
    for (uint32_t depth = 0; depth < p.maxDepth; depth++) {
        THit h;
        closest(c, ro, rd, h);
        if (!shadeBounce(c, p, smp, depth, h, ro, rd, beta, radiance, hk)) break;
    }
    return radiance;
}

}  // namespace cr
