// AABB::intersect as the reference writes it (Math/AABB.cu:6-46): a
// division 1/d per axis per test, std::max / std::min, a swap for negative d.
#include <cfloat>

#include "ref_common.cuh"

namespace refk {

__device__ static float comp(const Vec3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

__device__ bool aabbIntersect(const Aabb& box, const Ray& ray, float& hitT) {
    float tMin = ray.tMin, tMax = ray.tMax;
    for (int i = 0; i < 3; ++i) {
        const float mn = comp(box.pMin, i), mx = comp(box.pMax, i);
        const float o = comp(ray.origin, i), d = comp(ray.direction, i);
        if (fabsf(mx - mn) < FLT_EPSILON) {
            if (fabsf(d) < FLT_EPSILON) {
                if (fabsf(o - mn) > FLT_EPSILON) return false;
                continue;
            }
            const float t = (mn - o) / d;
            tMin = tMin < t ? t : tMin;
            tMax = t < tMax ? t : tMax;
        } else {
            const float invD = 1.0f / d;
            float t0 = (mn - o) * invD, t1 = (mx - o) * invD;
            if (invD < 0.0f) {
                const float tmp = t0;
                t0 = t1;
                t1 = tmp;
            }
            tMin = tMin < t0 ? t0 : tMin;
            tMax = t1 < tMax ? t1 : tMax;
        }
        if (tMin > tMax) return false;
    }
    if (tMin > ray.tMax || tMax < ray.tMin) return false;
    hitT = tMin;
    return true;
}

}  // namespace refk
