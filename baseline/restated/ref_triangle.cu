// TriangleMeshSOA::intersect (Scene/Triangle.cu:40-75) with its indexed
// vertex fetches, and the closest-hit rule intersectShape (Scene/Shape.h:16-37).
#include "ref_common.cuh"

namespace refk {

__device__ static Vec3 sub(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ static Vec3 cross(Vec3 a, Vec3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
__device__ static float dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ bool triangleIntersect(const Mesh& mesh, uint32_t prim, const Ray& ray, HitInfo& hit, float& t) {
    const uint32_t i = prim * 3;
    const uint32_t vi[3] = {mesh.idx[i], mesh.idx[i + 1], mesh.idx[i + 2]};
    const Vec3 v0 = mesh.pos[vi[0]], v1 = mesh.pos[vi[1]], v2 = mesh.pos[vi[2]];
    const Vec3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    const Vec3 p = cross(ray.direction, e2);
    const float det = dot(e1, p);
    if (fabsf(det) < 1e-6f) return false;
    const float invDet = 1.0f / det;
    const Vec3 tv = sub(ray.origin, v0);
    const float u = dot(tv, p) * invDet;
    if (u < 0.0f || u > 1.0f) return false;
    const Vec3 q = cross(tv, e1);
    const float v = dot(ray.direction, q) * invDet;
    if (v < 0.0f || u + v > 1.0f) return false;
    const float tt = dot(e2, q) * invDet;
    if (tt <= 0.0f) return false;
    hit.u = u;
    hit.v = v;
    t = tt;
    return true;
}

__device__ bool intersectShape(uint32_t prim, const Mesh& mesh, RayHit& rh) {
    HitInfo hit;
    float t = 0.0f;
    hit.type = 1;
    const bool isHit = triangleIntersect(mesh, prim, rh.ray, hit, t);
    hit.prim = prim;
    if (t < rh.ray.tMin || t > rh.ray.tMax) return false;
    if (isHit && t < rh.t) {
        rh.hit = hit;
        rh.t = t;
    }
    return isHit;
}

}  // namespace refk
