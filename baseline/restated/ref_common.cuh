// ref_common.cuh -- types of the restated reference traversal (a measurement
// comparator, not part of the product).  Layouts follow the reference:
// glm-style vec3 of three floats (12 B, 4-byte aligned), Ray
// (Math/Ray.h:8-13), AABB (Math/AABB.h:12-14), BVHNode holding a
// std::variant<LeafProp, InternalProp> followed by its AABB
// (Core/BVH.h:17-30; 8 bytes of alternative, a one-byte index padded to 4,
// then 24 bytes of bounds: 36 B), RayHit (Core/Hit.h:26-30).
#pragma once
#include <cstdint>

namespace refk {

struct Vec3 {
    float x, y, z;
};

struct Ray {
    Vec3 origin;
    float tMin;
    Vec3 direction;
    float tMax;
};

struct Aabb {
    Vec3 pMin, pMax;
};

struct Node {
    uint32_t a, b;      // leaf: (leafOffset, leafCount); internal: (left, right)
    uint8_t index;      // variant index: 0 = LeafProp, 1 = InternalProp
    uint8_t pad[3];
    Aabb bounds;
};
static_assert(sizeof(Node) == 36, "reference node size");

struct HitInfo {
    float u, v;
    uint32_t type;
    uint32_t prim;
};

struct RayHit {
    Ray ray;
    HitInfo hit;
    float t;
};

struct Mesh {
    const Vec3* pos;
    const uint32_t* idx;
};

struct Bvh {
    Aabb rootBounds;
    uint32_t rootIndex;
    const Node* nodes;
    const uint32_t* primMap;
};

// separately compiled device functions (relocatable device code, as the
// reference builds with CUDA_SEPARABLE_COMPILATION, Source/CRaystal/CMakeLists.txt:93)
__device__ bool aabbIntersect(const Aabb& box, const Ray& ray, float& hitT);
__device__ bool triangleIntersect(const Mesh& mesh, uint32_t prim, const Ray& ray, HitInfo& hit, float& t);
__device__ bool intersectShape(uint32_t prim, const Mesh& mesh, RayHit& rh);
__device__ bool bvhIntersect(const Bvh& bvh, const Mesh& mesh, RayHit& rh);

}  // namespace refk
