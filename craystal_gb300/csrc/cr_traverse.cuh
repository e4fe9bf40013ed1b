// cr_traverse.cuh -- ray / box, ray / triangle and BVH traversal device code.
//
// The arithmetic is the reference's: Math/AABB.cu:6-46 (slab test),
// Scene/Triangle.cu:40-75 (Moller-Trumbore with the absolute 1e-6
// determinant cull), Scene/Shape.h:16-37 (closest-hit update rule) and
// Core/BVH.cu:13-84 (near-first binary traversal with per-entry culling).
// Only the memory layout differs: both children's boxes sit in one 64-byte
// NodePair, the inverse direction is computed once per ray (the value
// 1/d the reference recomputes per box is the same float), and each leaf
// slot holds a pre-gathered 48-byte triangle block (v0, e1, e2) whose
// edges are the differences the reference forms per test.
#pragma once

#include "cr_internal.cuh"
#include "cr_math.cuh"

namespace cr {

struct TRay {
    float3 o;
    float tMin;
    float3 d;
    float tMax;
    float3 inv;
};

__device__ __forceinline__ TRay makeTRay(float3 o, float tMin, float3 d, float tMax) {
    TRay r;
    r.o = o;
    r.tMin = tMin;
    r.d = d;
    r.tMax = tMax;
    r.inv = mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    return r;
}

struct THit {
    float t;
    float u, v;
    uint32_t prim;
};

// One slab of Math/AABB.cu:10-29.  Returns false for the degenerate-slab
// early out; the per-axis "tMin > tMax" test of the reference is folded into
// the final test, which is equivalent because tMin only grows and tMax only
// shrinks afterwards.
__device__ __forceinline__ bool slab(float mn, float mx, float o, float d, float inv, bool degenerate,
                                     float& tMin, float& tMax) {
    if (degenerate) {
        if (fabsf(d) < kFltEps) return fabsf(o - mn) <= kFltEps;
        float t = (mn - o) / d;
        tMin = smax(tMin, t);
        tMax = smin(tMax, t);
        return true;
    }
    float t0 = (mn - o) * inv;
    float t1 = (mx - o) * inv;
    float tn = (inv < 0.0f) ? t1 : t0;
    float tf = (inv < 0.0f) ? t0 : t1;
    tMin = smax(tMin, tn);
    tMax = smin(tMax, tf);
    return true;
}

// AABB::intersect (Math/AABB.cu:6-46); flags bits 0-2 = degenerate axes.
__device__ __forceinline__ bool boxTest(float3 mn, float3 mx, uint32_t flags, const TRay& r, float& tEntry) {
    float tMin = r.tMin, tMax = r.tMax;
    bool ok = slab(mn.x, mx.x, r.o.x, r.d.x, r.inv.x, flags & 1u, tMin, tMax);
    ok &= slab(mn.y, mx.y, r.o.y, r.d.y, r.inv.y, flags & 2u, tMin, tMax);
    ok &= slab(mn.z, mx.z, r.o.z, r.d.z, r.inv.z, flags & 4u, tMin, tMax);
    if (!ok || tMin > tMax) return false;
    if (tMin > r.tMax || tMax < r.tMin) return false;
    tEntry = tMin;
    return true;
}

__host__ __device__ __forceinline__ uint32_t degenerateFlags(float3 mn, float3 mx) {
    return (fabsf(mx.x - mn.x) < kFltEps ? 1u : 0u) | (fabsf(mx.y - mn.y) < kFltEps ? 2u : 0u) |
           (fabsf(mx.z - mn.z) < kFltEps ? 4u : 0u);
}

// TriangleMeshSOA::intersect (Scene/Triangle.cu:40-75) on a pre-gathered block.
__device__ __forceinline__ bool triTest(const float3& v0, const float3& e1, const float3& e2, const TRay& r,
                                        float& t, float& u, float& v) {
    float3 p = cross(r.d, e2);
    float det = dot(e1, p);
    if (fabsf(det) < 1e-6f) return false;
    float invDet = 1.0f / det;
    float3 tv = sub(r.o, v0);
    u = dot(tv, p) * invDet;
    if (u < 0.0f || u > 1.0f) return false;
    float3 q = cross(tv, e1);
    v = dot(r.d, q) * invDet;
    if (v < 0.0f || u + v > 1.0f) return false;
    t = dot(e2, q) * invDet;
    if (t <= 0.0f) return false;
    return true;
}

__device__ __forceinline__ void loadTri(const TriBlock* tris, uint32_t slot, float3& v0, float3& e1, float3& e2,
                                        uint32_t& prim) {
    const float4* p = reinterpret_cast<const float4*>(tris + slot);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    v0 = mk3(a.x, a.y, a.z);
    prim = __float_as_uint(a.w);
    e1 = mk3(b.x, b.y, b.z);
    e2 = mk3(c.x, c.y, c.z);
}

constexpr int kStackSize = 32;  // depth <= 20 bounds a near-first stack by 21

// BVHData::intersect (Core/BVH.cu:13-84).  h.t must hold the initial
// closest t (infinity for a fresh RayHit).  Returns whether any triangle
// was hit inside [tMin, tMax] (not only closer ones), as the reference does.
template <bool kAnyHit>
__device__ __forceinline__ bool traverse(const SceneView& sc, const TRay& r, THit& h) {
    if (!sc.hasRoot) return false;
    float tr;
    if (!boxTest(sc.rootMin, sc.rootMax, sc.rootFlags, r, tr)) return false;
    uint2 stack[kStackSize];
    int sp = 0;
    stack[sp++] = make_uint2(sc.rootRef, __float_as_uint(0.0f));
    bool isHit = false;
    while (sp > 0) {
        const uint2 e = stack[--sp];
        if (__uint_as_float(e.y) > h.t) continue;
        if (e.x & kLeafBit) {
            const uint2 leaf = __ldg(sc.leaves + (e.x & ~kLeafBit));
            for (uint32_t i = 0; i < leaf.y; ++i) {
                float3 v0, e1, e2;
                uint32_t prim;
                loadTri(sc.tris, leaf.x + i, v0, e1, e2, prim);
                float t, u, v;
                if (triTest(v0, e1, e2, r, t, u, v)) {
                    if (t < r.tMin || t > r.tMax) continue;
                    isHit = true;
                    if (kAnyHit) return true;
                    if (t < h.t) {
                        h.t = t;
                        h.u = u;
                        h.v = v;
                        h.prim = prim;
                    }
                }
            }
        } else {
            const float4* np = reinterpret_cast<const float4*>(sc.pairs + e.x);
            const float4 p0 = __ldg(np), p1 = __ldg(np + 1), p2 = __ldg(np + 2);
            const uint4 ref = __ldg(reinterpret_cast<const uint4*>(np + 3));
            float lt = INFINITY, rt = INFINITY;
            bool hl = boxTest(mk3(p0.x, p0.y, p0.z), mk3(p0.w, p1.x, p1.y), ref.z & 7u, r, lt);
            bool hr = boxTest(mk3(p1.z, p1.w, p2.x), mk3(p2.y, p2.z, p2.w), (ref.z >> 3) & 7u, r, rt);
            const float ct = h.t;
            if (hl && hr) {
                if (lt > rt) {
                    if (lt < ct) stack[sp++] = make_uint2(ref.x, __float_as_uint(lt));
                    if (rt < ct) stack[sp++] = make_uint2(ref.y, __float_as_uint(rt));
                } else {
                    if (rt < ct) stack[sp++] = make_uint2(ref.y, __float_as_uint(rt));
                    if (lt < ct) stack[sp++] = make_uint2(ref.x, __float_as_uint(lt));
                }
            } else if (hl && lt < ct) {
                stack[sp++] = make_uint2(ref.x, __float_as_uint(lt));
            } else if (hr && rt < ct) {
                stack[sp++] = make_uint2(ref.y, __float_as_uint(rt));
            }
            if (sp > kStackSize - 2) {  // unreachable for depth <= 20; never overrun
                atomicOr(sc.errFlags, kErrStackOverflow);
                break;
            }
        }
    }
    return isHit;
}

}  // namespace cr
