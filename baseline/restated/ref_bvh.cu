// BVHData::intersect (Core/BVH.cu:13-84): root box test, a 64-entry stack of
// {node, tEntry} in local memory, both children loaded as 36-byte nodes and
// tested, far child pushed before near, per-entry culling; and a batch
// kernel with one thread per ray (the reference has no batch entry point;
// this is its traversal as a ray-cast comparator).
#include <cmath>

#include "ref_common.cuh"

namespace refk {

struct StackEntry {
    uint32_t node;
    float tMin;
};

__device__ bool bvhIntersect(const Bvh& bvh, const Mesh& mesh, RayHit& rh) {
    float unused;
    if (!aabbIntersect(bvh.rootBounds, rh.ray, unused)) return false;
    StackEntry stack[64];
    int sp = 0;
    stack[sp++] = {bvh.rootIndex, 0.0f};
    bool isHit = false;
    float closest = rh.t;
    while (sp > 0) {
        const StackEntry e = stack[--sp];
        const Node& node = bvh.nodes[e.node];
        if (e.tMin > closest) continue;
        if (node.index == 0) {
            for (uint32_t i = 0; i < node.b; ++i) {
                const uint32_t prim = bvh.primMap[node.a + i];
                if (intersectShape(prim, mesh, rh)) {
                    isHit = true;
                    closest = fminf(closest, rh.t);
                }
            }
        } else {
            const Node& l = bvh.nodes[node.a];
            const Node& r = bvh.nodes[node.b];
            float lt = INFINITY, rt = INFINITY;
            const bool hl = aabbIntersect(l.bounds, rh.ray, lt);
            const bool hr = aabbIntersect(r.bounds, rh.ray, rt);
            if (hl && hr) {
                if (lt > rt) {
                    if (lt < closest) stack[sp++] = {node.a, lt};
                    if (rt < closest) stack[sp++] = {node.b, rt};
                } else {
                    if (rt < closest) stack[sp++] = {node.b, rt};
                    if (lt < closest) stack[sp++] = {node.a, lt};
                }
            } else if (hl && lt < closest) {
                stack[sp++] = {node.a, lt};
            } else if (hr && rt < closest) {
                stack[sp++] = {node.b, rt};
            }
        }
    }
    return isHit;
}

__global__ void kRefTrace(Bvh bvh, Mesh mesh, const Ray* rays, uint64_t n, float4* hits) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    RayHit rh;
    rh.ray = rays[i];
    rh.t = INFINITY;
    rh.hit = HitInfo{0, 0, 0, 0xffffffffu};
    const bool hit = bvhIntersect(bvh, mesh, rh);
    hits[i] = hit ? make_float4(__uint_as_float(rh.hit.prim), rh.t, rh.hit.u, rh.hit.v)
                  : make_float4(__uint_as_float(0xffffffffu), INFINITY, 0.0f, 0.0f);
}

}  // namespace refk

// nodes: node_count 36-byte reference nodes (post-order, root last);
// prim_map: leaf slot -> primitive; pos / idx: the mesh; rays (32 B each) and
// hits (prim, t, u, v) are device pointers.
extern "C" int refk_trace_closest(const void* nodes, uint32_t root_index, const float* root_min,
                                  const float* root_max, const uint32_t* prim_map, const float* pos,
                                  const uint32_t* idx, const void* rays, uint64_t n, void* hits, void* stream) {
    refk::Bvh bvh;
    bvh.rootBounds = {{root_min[0], root_min[1], root_min[2]}, {root_max[0], root_max[1], root_max[2]}};
    bvh.rootIndex = root_index;
    bvh.nodes = static_cast<const refk::Node*>(nodes);
    bvh.primMap = prim_map;
    refk::Mesh mesh{reinterpret_cast<const refk::Vec3*>(pos), idx};
    const unsigned blocks = (unsigned)((n + 127) / 128);
    refk::kRefTrace<<<blocks, 128, 0, static_cast<cudaStream_t>(stream)>>>(
        bvh, mesh, static_cast<const refk::Ray*>(rays), n, static_cast<float4*>(hits));
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
