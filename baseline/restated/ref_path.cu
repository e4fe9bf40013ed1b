// ref_path.cu -- the reference's path tracer restated as a measurement
// comparator (not part of the product): pathTraceKernel<useMIS>
// (Core/Integrator.cu:142-227) with sampleLight (:21-72) and evalMIS
// (:74-140), launched as PathTraceIntegrator::dispatch does (:233-262): a
// W x H grid of 16 x 16 blocks (each pixel's thread in its own 256-thread
// block, the rest of the block exiting), one launch and one
// cudaDeviceSynchronize per sample.  Its traversal is the restated
// BVHData::intersect over 36-byte nodes (ref_bvh.cu, separately compiled),
// also for shadow rays, which the reference traces as full closest-hit
// queries (SceneView::intersectOcclusion, Scene/Scene.cu:16-29); the film
// is SensorData::addSample with global atomics (Core/Sensor.cu:19-43).
// The BSDF, sampler, frame and camera arithmetic is the product's
// restatement of the reference's (cr_shading.cuh), called through
// out-of-line functions as the reference's separately compiled BSDF code
// is.  Built with nvcc's default flags (FMA contraction on).
#include "cr_shading.cuh"
#include "ref_common.cuh"

namespace refk {

struct PathScene {
    Bvh bvh;
    Mesh mesh;
    const float3* nrm;
    const uint32_t* primToMesh;
    const uint32_t* meshMaterial;
    const cr::MaterialGpu* mats;
    const uint32_t* emissive;
    uint32_t nEmissive;
};

struct PathParams {
    uint32_t maxDepth;
    float rrThreshold;
};

struct Isect {
    float3 posW, faceN, viewW;
    bool front;
    cr::Frame frame;
    __device__ float3 oriented() const { return front ? faceN : cr::neg(faceN); }
};

__device__ static float3 f3(const Vec3& v) { return make_float3(v.x, v.y, v.z); }

__device__ static Ray makeRay(float3 o, float3 d, float tMax) {
    Ray r;
    r.origin = {o.x, o.y, o.z};
    r.tMin = 0.0f;
    r.direction = {d.x, d.y, d.z};
    r.tMax = tMax;
    return r;
}

// SceneView::intersect (no spheres in the compared scenes)
__device__ static bool sceneIntersect(const PathScene& s, RayHit& rh) { return bvhIntersect(s.bvh, s.mesh, rh); }

// SceneView::intersectOcclusion: a full closest-hit traversal
__device__ static bool sceneOccluded(const PathScene& s, const Ray& r) {
    RayHit rh;
    rh.ray = r;
    rh.t = INFINITY;
    rh.hit = HitInfo{0, 0, 0, 0xffffffffu};
    return bvhIntersect(s.bvh, s.mesh, rh);
}

__device__ static void triangle(const PathScene& s, uint32_t prim, float3 p[3], float3 n[3]) {
    for (int k = 0; k < 3; k++) {
        const uint32_t vi = s.mesh.idx[3 * prim + k];
        p[k] = f3(s.mesh.pos[vi]);
        n[k] = s.nrm[vi];
    }
}

__device__ static float3 faceNormal(const float3 p[3]) {
    return cr::normalize(cr::cross(cr::sub(p[1], p[0]), cr::sub(p[2], p[0])));
}

__device__ static float3 interp(const float3 v[3], float3 w) {
    return cr::add(cr::add(cr::mul(v[0], w.x), cr::mul(v[1], w.y)), cr::mul(v[2], w.z));
}

// SceneView::createIntersection (Scene/Scene.cu:31-59) + Intersection
__device__ static Isect createIntersection(const PathScene& s, const RayHit& rh) {
    Isect it;
    const float3 o = f3(rh.ray.origin), d = f3(rh.ray.direction);
    it.posW = cr::add(o, cr::mul(rh.t, d));
    it.viewW = cr::neg(cr::normalize(d));
    float3 p[3], n[3];
    triangle(s, rh.hit.prim, p, n);
    it.faceN = faceNormal(p);
    const float3 w = make_float3((1.f - rh.hit.u) - rh.hit.v, rh.hit.u, rh.hit.v);
    const float3 sn = cr::normalize(interp(n, w));
    it.front = cr::dot(it.viewW, it.faceN) > 0.0f;
    it.frame.build(it.front ? sn : cr::neg(sn));
    return it;
}

__device__ static const cr::MaterialGpu& materialOf(const PathScene& s, uint32_t prim) {
    return s.mats[s.meshMaterial[s.primToMesh[prim]]];
}

// the BSDF entry points, out of line as the reference's separately compiled ones
__device__ __noinline__ cr::Spec bsdfEvaluate(const cr::Bsdf& b, float3 wo, float3 wi) { return b.evaluate(wo, wi); }
__device__ __noinline__ float bsdfPdf(const cr::Bsdf& b, float3 wo, float3 wi) { return b.evaluatePdf(wo, wi); }
__device__ __noinline__ cr::Spec bsdfSample(const cr::Bsdf& b, float2 u, float3 wo, float3& wi, float& pdf) {
    return b.sampleEvaluate(u, wo, wi, pdf);
}

struct LightSample {
    cr::Spec weight;
    float3 dir;
    float pdf;
    uint32_t id;
    float selectPdf;
};

__device__ static LightSample sampleLight(const PathScene& s, const Isect& it, const cr::Bsdf& bsdf, cr::Sampler& smp,
                                          uint32_t& rays) {
    LightSample ls{cr::sp(0.0f), make_float3(0, 0, 0), 0.0f, 0, 0.0f};
    const int cnt = (int)s.nEmissive;
    if (cnt == 0) return ls;
    const int pick = min(cr::f2iX86((float)cnt * smp.next1D()), cnt - 1);
    const uint32_t id = s.emissive[pick];
    float3 p[3], n[3];
    triangle(s, id, p, n);
    const float2 b = cr::sampleBarycentric(smp.next2D());
    const float3 w = make_float3((1.f - b.x) - b.y, b.x, b.y);
    const float3 vp = interp(p, w), vn = interp(n, w);
    const float3 target = cr::offsetRayOrigin(vp, faceNormal(p));
    const float3 toLight = cr::sub(target, it.posW);
    const float distSqr = cr::dot(toLight, toLight);
    const float dist = sqrtf(distSqr);
    const float3 dir = cr::divs(toLight, dist);
    if (cr::dot(it.oriented(), dir) < 0.0f || cr::dot(vn, dir) > 0.0f || dist < cr::kEps) return ls;
    const float3 so = cr::offsetRayOrigin(it.posW, it.oriented());
    rays++;
    if (sceneOccluded(s, makeRay(so, dir, cr::length(cr::sub(so, target)) - cr::kEps))) return ls;
    const cr::MaterialGpu& m = materialOf(s, id);
    const float area = cr::length(cr::cross(cr::sub(p[0], p[1]), cr::sub(p[2], p[1]))) / 2.f;
    ls.weight = cr::mul(bsdfEvaluate(bsdf, it.viewW, dir), cr::sp(m.em[0], m.em[1], m.em[2]));
    ls.dir = dir;
    ls.pdf = distSqr / (area * cr::absDot(dir, vn));
    ls.id = id;
    ls.selectPdf = (float)(1.0 / (double)cnt);
    return ls;
}

__device__ static cr::Spec evalMIS(const PathScene& s, const Isect& it, const cr::Bsdf& bsdf, cr::Sampler& smp,
                                   uint32_t& rays) {
    cr::Spec value = cr::sp(0.0f);
    const LightSample ls = sampleLight(s, it, bsdf, smp, rays);
    if (ls.pdf <= 0.0f) return value;
    const float bp = bsdfPdf(bsdf, it.viewW, ls.dir);
    if (bp > 0.0f) value = cr::add(value, cr::divs(cr::mul(cr::powerHeuristic(ls.pdf, bp), ls.weight), ls.pdf));
    float3 dir;
    float bsdfPdfV = 0.0f;
    const cr::Spec w = bsdfSample(bsdf, smp.next2D(), it.viewW, dir, bsdfPdfV);
    if (cr::maxValue(w) > 0.0f && bsdfPdfV > 0.0f) {
        const float3 o = cr::offsetRayOrigin(it.posW, it.oriented());
        RayHit rh;
        rh.ray = makeRay(o, dir, INFINITY);
        rh.t = INFINITY;
        rh.hit = HitInfo{0, 0, 0, 0xffffffffu};
        rays++;
        if (sceneIntersect(s, rh) && rh.hit.prim == ls.id) {
            float3 p[3], n[3];
            triangle(s, rh.hit.prim, p, n);
            const float3 lpos = cr::add(o, cr::mul(rh.t, dir));
            const cr::MaterialGpu& m = materialOf(s, rh.hit.prim);
            if (m.flags & CR_MATERIAL_EMISSIVE) {
                const float3 toLight = cr::sub(lpos, it.posW);
                const float distSqr = cr::dot(toLight, toLight);
                const float cosL = cr::absDot(cr::divs(toLight, sqrtf(distSqr)), faceNormal(p));
                if (cosL != 0.0f) {
                    const float area = cr::length(cr::cross(cr::sub(p[0], p[1]), cr::sub(p[2], p[1]))) / 2.f;
                    const float lightPdf = distSqr / (area * cosL);
                    value = cr::add(value, cr::divs(cr::mul(cr::mul(cr::powerHeuristic(bsdfPdfV, lightPdf),
                                                                    cr::sp(m.em[0], m.em[1], m.em[2])),
                                                            w),
                                                    bsdfPdfV));
                }
            }
        }
    }
    return cr::divs(value, ls.selectPdf);
}

// SensorData::addSample (Core/Sensor.cu:19-43)
__device__ static void addSample(const cr::CameraGpu& cam, float* filmRgb, float* filmW, cr::Spec L, float2 pix) {
    if (isnan(L.r) || isnan(L.g) || isnan(L.b) || isinf(L.r) || isinf(L.g) || isinf(L.b)) return;
    const int xa = max((int)floorf(pix.x - 1.0f), 0), ya = max((int)floorf(pix.y - 1.0f), 0);
    const int xb = min((int)ceilf(pix.x + 1.0f), (int)cam.width - 1), yb = min((int)ceilf(pix.y + 1.0f), (int)cam.height - 1);
    for (int yy = ya; yy <= yb; yy++)
        for (int xx = xa; xx <= xb; xx++) {
            const float w = cr::smax(0.0f, 1.0f - fabsf(pix.x - ((float)xx + 0.5f))) *
                            cr::smax(0.0f, 1.0f - fabsf(pix.y - ((float)yy + 0.5f)));
            const size_t pi = (size_t)yy * cam.width + xx;
            atomicAdd(filmRgb + 3 * pi + 0, L.r * w);
            atomicAdd(filmRgb + 3 * pi + 1, L.g * w);
            atomicAdd(filmRgb + 3 * pi + 2, L.b * w);
            atomicAdd(filmW + pi, w);
        }
}

template <bool kMIS>
__global__ void pathTraceKernel(uint32_t frameIdx, const PathParams* pIntegrator, const PathScene* pScene,
                                const cr::CameraGpu* pCamera, float* filmRgb, float* filmW,
                                unsigned long long* rayCounter) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const cr::CameraGpu& cam = *pCamera;
    if (x >= cam.width || y >= cam.height) return;
    const PathScene& s = *pScene;
    cr::Sampler smp(x, y, frameIdx);
    const float2 j = smp.next2D();
    const float2 pixel = make_float2((float)x + j.x, (float)y + j.y);
    const float u = 2.0f * (pixel.x / (float)cam.width) - 1.0f;
    const float v = 1.0f - 2.0f * (pixel.y / (float)cam.height);
    float3 ro = cam.pos;
    float3 rd = cr::normalize(cr::add(cr::add(cr::mul(cam.U, u * cam.halfW), cr::mul(cam.V, v * cam.halfH)), cam.W));
    cr::Spec radiance = cr::sp(0.0f), beta = cr::sp(1.0f);
    uint32_t rays = 0;
    for (uint32_t depth = 0; depth < pIntegrator->maxDepth; depth++) {
        RayHit rh;
        rh.ray = makeRay(ro, rd, INFINITY);
        rh.t = INFINITY;
        rh.hit = HitInfo{0, 0, 0, 0xffffffffu};
        bool terminate = false;
        rays++;
        if (sceneIntersect(s, rh)) {
            const Isect it = createIntersection(s, rh);
            const cr::MaterialGpu m = materialOf(s, rh.hit.prim);  // by value, as the reference copies it
            if (m.flags & CR_MATERIAL_EMISSIVE) {
                radiance = cr::add(radiance, cr::mul(cr::sp(m.em[0], m.em[1], m.em[2]), beta));
                break;
            }
            cr::Bsdf bsdf;
            bsdf.init(m, it.frame);
            if (kMIS) {
                radiance = cr::add(radiance, cr::mul(evalMIS(s, it, bsdf, smp, rays), beta));
            } else {
                const LightSample ls = sampleLight(s, it, bsdf, smp, rays);
                if (ls.pdf > 0.0f) radiance = cr::add(radiance, cr::divs(cr::divs(cr::mul(ls.weight, beta), ls.pdf), ls.selectPdf));
            }
            float3 wi;
            float pdf = 0.0f;
            const cr::Spec f = bsdfSample(bsdf, smp.next2D(), it.viewW, wi, pdf);
            if (pdf <= 0.0f) break;
            beta = cr::mul(beta, cr::divs(f, pdf));
            ro = cr::offsetRayOrigin(it.posW, it.oriented());
            rd = wi;
        } else {
            terminate = true;
        }
        if (smp.next1D() < pIntegrator->rrThreshold) terminate = true;
        if (terminate) break;
        if (depth > 5) {
            float q = cr::smax(pIntegrator->rrThreshold, 1.0f - cr::maxValue(beta));
            q = q < 0.0f ? 0.0f : (1.0f < q ? 1.0f : q);
            if (smp.next1D() < q) break;
            beta = cr::divs(beta, 1.0f - q);
        }
    }
    addSample(cam, filmRgb, filmW, radiance, pixel);
    atomicAdd(rayCounter, (unsigned long long)rays);
}

}  // namespace refk

// Inputs are device pointers: the reference-layout BVH (nodes, prim map),
// the global vertex arrays, primitive -> mesh, mesh -> material,
// per-material records as the product derives them (cr::MaterialGpu), the
// emitter list; camera as cr_camera.  Renders spp samples (indices 0..spp-1)
// into film_rgb / film_w and counts rays.
extern "C" int refk_render(const void* nodes, uint32_t root_index, const float* root_min, const float* root_max,
                           const uint32_t* prim_map, const float* pos, const float* nrm, const uint32_t* idx,
                           const uint32_t* prim_to_mesh, const uint32_t* mesh_material, const void* materials,
                           const uint32_t* emissive, uint32_t n_emissive, const cr_camera* cam, uint32_t max_depth,
                           float rr_threshold, int use_mis, uint32_t spp, float* film_rgb, float* film_w,
                           unsigned long long* rays) {
    using namespace refk;
    PathScene s;
    s.bvh.rootBounds = {{root_min[0], root_min[1], root_min[2]}, {root_max[0], root_max[1], root_max[2]}};
    s.bvh.rootIndex = root_index;
    s.bvh.nodes = static_cast<const Node*>(nodes);
    s.bvh.primMap = prim_map;
    s.mesh = Mesh{reinterpret_cast<const Vec3*>(pos), idx};
    s.nrm = reinterpret_cast<const float3*>(nrm);
    s.primToMesh = prim_to_mesh;
    s.meshMaterial = mesh_material;
    s.mats = static_cast<const cr::MaterialGpu*>(materials);
    s.emissive = emissive;
    s.nEmissive = n_emissive;
    // Camera::calculateCameraData (Core/Camera.cu:35-39, Core/CameraProxy.h:32-35)
    cr::CameraGpu c;
    const float3 p = make_float3(cam->pos[0], cam->pos[1], cam->pos[2]);
    c.pos = p;
    c.W = cr::normalize(cr::sub(make_float3(cam->target[0], cam->target[1], cam->target[2]), p));
    c.U = cr::normalize(cr::cross(c.W, make_float3(cam->up[0], cam->up[1], cam->up[2])));
    c.V = cr::normalize(cr::cross(c.U, c.W));
    c.halfH = (float)std::tan(((double)cam->fov_y * 0.5) * 0.01745329251994329576923690768489);
    c.halfW = ((float)cam->width / (float)cam->height) * c.halfH;
    c.width = cam->width;
    c.height = cam->height;
    PathParams pp{max_depth, rr_threshold};
    // device views, as the reference's DeviceBuffer copies of its views
    PathScene* dS = nullptr;
    cr::CameraGpu* dC = nullptr;
    PathParams* dP = nullptr;
    if (cudaMalloc(&dS, sizeof(s)) || cudaMalloc(&dC, sizeof(c)) || cudaMalloc(&dP, sizeof(pp))) return 1;
    cudaMemcpy(dS, &s, sizeof(s), cudaMemcpyHostToDevice);
    cudaMemcpy(dC, &c, sizeof(c), cudaMemcpyHostToDevice);
    cudaMemcpy(dP, &pp, sizeof(pp), cudaMemcpyHostToDevice);
    int rc = 0;
    for (uint32_t i = 0; i < spp && !rc; i++) {
        if (use_mis)
            pathTraceKernel<true><<<dim3(c.width, c.height, 1), dim3(16, 16, 1)>>>(i, dP, dS, dC, film_rgb, film_w, rays);
        else
            pathTraceKernel<false><<<dim3(c.width, c.height, 1), dim3(16, 16, 1)>>>(i, dP, dS, dC, film_rgb, film_w, rays);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = 2;
    }
    cudaFree(dS);
    cudaFree(dC);
    cudaFree(dP);
    return rc;
}
