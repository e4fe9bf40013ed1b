// cr_traverse.cuh -- ray / box, ray / triangle and BVH traversal device code.
//
// The arithmetic is the reference's: Math/AABB.cu:6-46 (slab test),
// Scene/Triangle.cu:40-75 (Moller-Trumbore with the absolute 1e-6
// determinant cull), Scene/Shape.h:16-37 (closest-hit update rule) and
// Core/BVH.cu:13-84 (near-first binary traversal with per-entry culling).
// What differs is the memory layout and the unit of work: both children's
// boxes sit in one 64-byte NodePair (read as two 32-byte loads), small
// leaves carry their slot range in the child ref, the inverse direction is
// computed once per ray (the value 1/d the reference recomputes per box is
// the same float), each leaf slot holds a pre-gathered 48-byte triangle
// block (v0, e1, e2) whose edges are the differences the reference forms
// per test, and a traversal step is one node or one leaf slot (travStep).
//
// Visiting order.  The reference pushes the far child, then the near child,
// and pops the near child at once; here the near child becomes the current
// node directly and only the far child is pushed.  That is the same order
// with the same culling decisions: nothing changes closestT between the push
// and the pop of the near child, so its pop-time test "tEntry > closestT" is
// the push-time test "tEntry < closestT" negated.
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

// One slab of Math/AABB.cu:10-29.
//
// fmaxf / fminf stand for the reference's std::max / std::min: they differ
// only for a NaN second operand, where both keep the first (a NaN slab
// distance arises as 0 * inf when the origin lies on the slab plane and the
// direction component is zero; tMin / tMax themselves never become NaN), and
// in the sign of a zero result, which no comparison downstream can see.
// The per-axis "tMin > tMax" early out of the reference is folded into one
// final test: tMin only grows and tMax only shrinks, and tMin starts at
// ray.tMin, tMax at ray.tMax, so the final "tMin > ray.tMax || tMax <
// ray.tMin" test is implied by "tMin > tMax" as well.
__device__ __forceinline__ void slabFast(float mn, float mx, float o, float inv, float& tMin, float& tMax) {
    const float t0 = (mn - o) * inv;
    const float t1 = (mx - o) * inv;
    const bool neg = inv < 0.0f;
    tMin = fmaxf(tMin, neg ? t1 : t0);
    tMax = fminf(tMax, neg ? t0 : t1);
}

// Degenerate slab (|max - min| < FLT_EPSILON), Math/AABB.cu:11-19.  Returns
// false for the early out of a ray parallel to the slab and outside it.
__device__ __forceinline__ bool slabDegenerate(float mn, float o, float d, float& tMin, float& tMax) {
    if (fabsf(d) < kFltEps) return !(fabsf(o - mn) > kFltEps);
    const float t = (mn - o) / d;
    tMin = fmaxf(tMin, t);
    tMax = fminf(tMax, t);
    return true;
}

// AABB::intersect (Math/AABB.cu:6-46); flags bits 0-2 = degenerate axes.
__device__ __forceinline__ bool boxTest(float3 mn, float3 mx, uint32_t flags, const TRay& r, float& tEntry) {
    float tMin = r.tMin, tMax = r.tMax;
    bool ok = true;
    if (flags == 0u) {
        slabFast(mn.x, mx.x, r.o.x, r.inv.x, tMin, tMax);
        slabFast(mn.y, mx.y, r.o.y, r.inv.y, tMin, tMax);
        slabFast(mn.z, mx.z, r.o.z, r.inv.z, tMin, tMax);
    } else {
        if (flags & 1u) ok &= slabDegenerate(mn.x, r.o.x, r.d.x, tMin, tMax);
        else slabFast(mn.x, mx.x, r.o.x, r.inv.x, tMin, tMax);
        if (flags & 2u) ok &= slabDegenerate(mn.y, r.o.y, r.d.y, tMin, tMax);
        else slabFast(mn.y, mx.y, r.o.y, r.inv.y, tMin, tMax);
        if (flags & 4u) ok &= slabDegenerate(mn.z, r.o.z, r.d.z, tMin, tMax);
        else slabFast(mn.z, mx.z, r.o.z, r.inv.z, tMin, tMax);
    }
    tEntry = tMin;
    return ok && !(tMin > tMax);
}

__host__ __device__ __forceinline__ uint32_t degenerateFlags(float3 mn, float3 mx) {
    return (fabsf(mx.x - mn.x) < kFltEps ? 1u : 0u) | (fabsf(mx.y - mn.y) < kFltEps ? 2u : 0u) |
           (fabsf(mx.z - mn.z) < kFltEps ? 4u : 0u);
}

// TriangleMeshSOA::intersect (Scene/Triangle.cu:40-75) on a pre-gathered block.
//
// The reference leaves at the first failed test (determinant, u, v, t); here
// every quantity is formed and the tests are combined at the end.  The
// values are the same floats, and t, u, v are only used when every test
// passes, so the result is the reference's.  One branch instead of four
// keeps the lanes of a warp together: 4 % faster closest-hit ray casts.
__device__ __forceinline__ bool triTest(const float3& v0, const float3& e1, const float3& e2, const TRay& r,
                                        float& t, float& u, float& v) {
    const float3 p = cross(r.d, e2);
    const float det = dot(e1, p);
    const float invDet = 1.0f / det;
    const float3 tv = sub(r.o, v0);
    u = dot(tv, p) * invDet;
    const float3 q = cross(tv, e1);
    v = dot(r.d, q) * invDet;
    t = dot(e2, q) * invDet;
    return !(fabsf(det) < 1e-6f) & !(u < 0.0f) & !(u > 1.0f) & !(v < 0.0f) & !(u + v > 1.0f) & !(t <= 0.0f);
}

__device__ __forceinline__ void loadTri(const TriBlock* tris, uint32_t slot, float3& v0, float3& e1, float3& e2,
                                        uint32_t& prim) {
    const float4* p = reinterpret_cast<const float4*>(tris + slot);
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    v0 = mk3(a.x, a.y, a.z);
    prim = __float_as_uint(a.w);
    e1 = mk3(b.x, b.y, b.z);
    e2 = mk3(c.x, c.y, c.z);
}

constexpr int kStackSize = 32;  // depth <= 20 bounds a near-first stack by 21

// Where the traversal stack lives.  kShared = 0: all kStackSize entries in
// the thread's local memory.  kShared > 0: the first kShared entries in a
// shared-memory area of kShared rows x kStackBlock columns (one column per
// thread; entry-major, so the lanes of a warp touch consecutive 8-byte words
// at any depth and never conflict), the deeper ones in local memory.  Keeping
// the top of the stack out of L1 leaves L1 to the node and triangle data:
// 3 % faster closest-hit ray casts on GB300.  A kernel using it runs blocks
// of exactly kStackBlock threads and declares the area as SharedStackArea.
constexpr int kStackBlock = 128;
constexpr int kSharedStack = 16;
typedef uint2 SharedStackArea[kSharedStack][kStackBlock];

template <int kShared>
struct TravStack {
    static_assert(kShared >= 0 && kShared < kStackSize, "stack split");
    uint2 (*sh)[kStackBlock];
    uint2 loc[kStackSize - kShared];
    __device__ __forceinline__ void put(int sp, uint2 v) {
        if (kShared > 0 && sp < kShared) sh[sp][threadIdx.x] = v;
        else loc[sp - kShared] = v;
    }
    __device__ __forceinline__ uint2 get(int sp) const {
        if (kShared > 0 && sp < kShared) return sh[sp][threadIdx.x];
        return loc[sp - kShared];
    }
};

// 32 bytes in one load (ld.global.nc.v4.b64, sm_100 and later) from a
// 32-byte aligned address.  A NodePair is two such loads instead of four
// 16-byte ones: the lanes of a warp visit scattered nodes, and the L1 data
// stage serves each lane's line once per load instruction, so half the
// instructions is half the L1 wavefronts per visit (7 % faster ray casts,
// where that stage was 88 % busy).  Pair arrays come from cudaMalloc and
// the records are 64-byte aligned.
struct Float8 {
    float4 a, b;
};

__device__ __forceinline__ Float8 ldg32(const void* p) {
    unsigned long long x, y, z, w;
    asm("ld.global.nc.v4.b64 {%0, %1, %2, %3}, [%4];" : "=l"(x), "=l"(y), "=l"(z), "=l"(w) : "l"(p));
    Float8 r;
    r.a = make_float4(__uint_as_float((uint32_t)x), __uint_as_float((uint32_t)(x >> 32)),
                      __uint_as_float((uint32_t)y), __uint_as_float((uint32_t)(y >> 32)));
    r.b = make_float4(__uint_as_float((uint32_t)z), __uint_as_float((uint32_t)(z >> 32)),
                      __uint_as_float((uint32_t)w), __uint_as_float((uint32_t)(w >> 32)));
    return r;
}

// The slot range [first, first + count) of a leaf ref: from the ref itself
// (kInlineLeafBit) or from the leaf table.
__device__ __forceinline__ void openLeaf(const uint2* leaves, uint32_t ref, uint32_t& ts, uint32_t& te) {
    if (ref & kInlineLeafBit) {
        ts = ref & kInlineSlotMask;
        te = ts + ((ref >> 27) & kInlineMaxCount);
    } else {
        const uint2 leaf = __ldg(leaves + (ref & ~(kLeafBit | kInlineLeafBit)));
        ts = leaf.x;
        te = leaf.x + leaf.y;
    }
}

// Leaf slot tests, one slot per call.  Each returns true when an any-hit
// query can stop.
//
// Triangles: the closest-hit rule of Scene/Shape.h:26-31; the traversal
// calls it on a leaf's slots in order.
template <bool kAnyHit>
struct TriLeaf {
    const TriBlock* tris;
    __device__ __forceinline__ bool operator()(const TRay& r, THit& h, bool& isHit, uint32_t slot) const {
        float3 v0, e1, e2;
        uint32_t prim;
        loadTri(tris, slot, v0, e1, e2, prim);
        float t, u, v;
        if (!triTest(v0, e1, e2, r, t, u, v) || t < r.tMin || t > r.tMax) return false;
        isHit = true;
        if (kAnyHit) return true;
        if (t < h.t) {
            h.t = t;
            h.u = u;
            h.v = v;
            h.prim = prim;
        }
        return false;
    }
};

// SphereSOA::intersect (Scene/Sphere.cu:6-38): the nearer root of
// |o + t d - c|^2 = r^2 inside [tMin, tMax], else the farther one.
__device__ __forceinline__ bool sphereTest(float4 s, const TRay& r, float& t) {
    const float3 oc = sub(r.o, mk3(s.x, s.y, s.z));
    const float a = dot(r.d, r.d);
    const float b = 2.0f * dot(oc, r.d);
    const float c = dot(oc, oc) - s.w * s.w;
    const float disc = b * b - 4.0f * a * c;
    if (disc < 0.0f) return false;
    const float sq = sqrtf(disc);
    float t0 = (-b - sq) / (2.0f * a);
    float t1 = (-b + sq) / (2.0f * a);
    if (t0 > t1) {
        const float x = t0;
        t0 = t1;
        t1 = x;
    }
    if (t0 < r.tMin || t0 > r.tMax) {
        if (t1 < r.tMin || t1 > r.tMax) return false;
        t0 = t1;
    }
    t = t0;
    return true;
}

// The spherical coordinates a sphere hit reports as its (u, v)
// (Scene/Sphere.cu:39-49).
__device__ __forceinline__ float2 sphereUV(float4 s, const TRay& r, float t) {
    const float3 p = add(r.o, mul(r.d, t));
    const float3 n = normalize(sub(p, mk3(s.x, s.y, s.z)));
    const float theta = acosf(-n.y);
    const float phi = atan2f(-n.z, n.x) + kPi;
    return make_float2(phi * (0.5f * kInvPi), theta * kInvPi);
}

// Spheres, tested before the triangles as SceneView::intersect does
// (Scene/Scene.cu:5-14).  The reference loops over the spheres in index
// order with the strict closest-hit rule, so of spheres hit at the same t
// the lowest index wins; the BVH visits them in another order and breaks
// such ties by index explicitly.
template <bool kAnyHit>
struct SphereLeaf {
    const SphereBlock* blocks;
    __device__ __forceinline__ bool operator()(const TRay& r, THit& h, bool& isHit, uint32_t slot) const {
        const float4* p = reinterpret_cast<const float4*>(blocks + slot);
        const float4 g = __ldg(p);
        float t;
        if (!sphereTest(g, r, t)) return false;
        isHit = true;
        if (kAnyHit) return true;
        const uint32_t id = kSphereBit | __ldg(reinterpret_cast<const uint32_t*>(p + 1));
        if (t < h.t || (t == h.t && id < h.prim)) {
            const float2 uv = sphereUV(g, r, t);
            h.t = t;
            h.u = uv.x;
            h.v = uv.y;
            h.prim = id;
        }
        return false;
    }
};

// BVHData::intersect (Core/BVH.cu:13-84) for one ray over one BVH, as a
// resumable traversal: travBegin() tests the root box, each travStep() is
// one unit of work: one interior node (both child boxes), one leaf slot, or
// a culled entry.  The scalar state (TravState) is kept apart from the stack
// array so that it stays in registers.
//
// The entry e being visited lives in registers.  When both children pass,
// the far one is pushed and the near one becomes e (the reference pushes
// both and pops the near one at once); an entry taken from the stack is
// culled when its distance is beyond the closest hit, as at
// Core/BVH.cu:34-36.  A leaf that is not culled opens its slot range
// [ts, te), and the following steps test one slot each, in order, before
// the next entry is taken: the reference's visiting order, split into
// steps of similar length so that the lanes of a warp (each at its own
// place in its own ray's traversal) run the same code at the same time.
// Every path through a step ends at one pop site.  h.t must hold the
// initial closest t (infinity for a fresh RayHit).  isHit: whether any
// primitive was hit inside [tMin, tMax] (not only closer ones), as the
// reference returns.
struct TravState {
    uint2 e;
    int sp;
    bool isHit;
    uint32_t ts, te;  // the open leaf's slots still to test
};

// false: the ray misses the root box and there is nothing to visit
__device__ __forceinline__ bool travBegin(TravState& s, const BvhView& bv, const TRay& r) {
    s.sp = 0;
    s.isHit = false;
    s.ts = s.te = 0;
    s.e = make_uint2(bv.rootRef, __float_as_uint(0.0f));
    float tr;
    return bv.hasRoot && boxTest(bv.rootMin, bv.rootMax, bv.rootFlags, r, tr);
}

// One binary level: both child boxes of the pair (w0, w1), the reference's
// near-first choice, the far child pushed when both pass.  Returns 1 when
// s.e is now the near child, 0 when neither child passes (pop), -1 on a
// stack overflow (reported through errFlags).
template <class Stack>
__device__ __forceinline__ int nodeLevel(const Float8& w0, const Float8& w1, TravState& s, Stack& stack,
                                         uint32_t* errFlags, const TRay& r, float ct) {
    const float4 p0 = w0.a, p1 = w0.b, p2 = w1.a;
    const uint4 ref = make_uint4(__float_as_uint(w1.b.x), __float_as_uint(w1.b.y), __float_as_uint(w1.b.z), 0u);
    float lt = INFINITY, rt = INFINITY;
    const bool hl = boxTest(mk3(p0.x, p0.y, p0.z), mk3(p0.w, p1.x, p1.y), ref.z & 7u, r, lt);
    const bool hr = boxTest(mk3(p1.z, p1.w, p2.x), mk3(p2.y, p2.z, p2.w), (ref.z >> 3) & 7u, r, rt);
    const bool gl = hl && lt < ct, gr = hr && rt < ct;
    // near = the child the reference pushes last: right when lt > rt
    const bool rightNear = gl && gr ? lt > rt : gr;
    if (gl && gr) {
        if (s.sp >= kStackSize) {  // unreachable for depth <= 20; never overrun
            atomicOr(errFlags, kErrStackOverflow);
            return -1;
        }
        stack.put(s.sp++, rightNear ? make_uint2(ref.x, __float_as_uint(lt)) : make_uint2(ref.y, __float_as_uint(rt)));
    }
    s.e = rightNear ? make_uint2(ref.y, __float_as_uint(rt)) : make_uint2(ref.x, __float_as_uint(lt));
    return (gl || gr) ? 1 : 0;
}

// One step; false once the traversal is over (an any-hit query that found
// a hit stops at once).
//
// kTwoLevel: the view's pairs are the grouped copy (kGroupTopBit).  At a
// group top whose near child is interior, the near child's level runs in
// the same step, on the next pair of the group: two binary levels per step,
// fetched from adjacent records.  Nothing
// changes closestT between the two levels, so the reference's pop-time cull
// of the near child (Core/BVH.cu:34-36) never fires there and the visiting
// order, the culling and the hits are those of the one-level step.  Measured
// on GB300 it is slower than one level per step at every tree size tried
// (the one-level step is the default; cr_scene_set_traversal).
template <bool kAnyHit, class Leaf, class Stack, bool kTwoLevel = false>
__device__ __forceinline__ bool travStep(TravState& s, Stack& stack, const BvhView& bv, uint32_t* errFlags,
                                         const Leaf& leaf, const TRay& r, THit& h) {
    bool pop = true;
    const bool culled = __uint_as_float(s.e.y) > h.t;
    if (s.ts < s.te || (s.e.x & kLeafBit) || culled) {
        if (s.ts >= s.te && (s.e.x & kLeafBit) && !culled) openLeaf(bv.leaves, s.e.x, s.ts, s.te);
        if (s.ts < s.te) {
            if (leaf(r, h, s.isHit, s.ts)) return false;
            pop = ++s.ts >= s.te;
        }
    } else {
        const uint32_t ref = s.e.x;
        const NodePair* np = bv.pairs + (kTwoLevel ? ref & kPairIndexMask : ref);
        const float ct = h.t;
        int st = nodeLevel(ldg32(&np->p0), ldg32(&np->p2), s, stack, errFlags, r, ct);
        if (st < 0) return false;
        if (kTwoLevel && st > 0 && (ref & kGroupTopBit) && !(s.e.x & kLeafBit)) {
            // s.e is now the near child, a second-level pair of this group
            const NodePair* cp = bv.pairs + s.e.x;
            st = nodeLevel(ldg32(&cp->p0), ldg32(&cp->p2), s, stack, errFlags, r, ct);
            if (st < 0) return false;
        }
        pop = st == 0;
    }
    if (pop) {
        if (s.sp == 0) return false;
        s.e = stack.get(--s.sp);
    }
    return true;
}

// The whole traversal of one ray; returns isHit.
template <bool kAnyHit, class Leaf, int kShared = 0>
__device__ __forceinline__ bool traverseBvh(const BvhView& bv, uint32_t* errFlags, const Leaf& leaf, const TRay& r,
                                            THit& h, uint2 (*shStack)[kStackBlock] = nullptr) {
    TravStack<kShared> stack;
    stack.sh = shStack;
    TravState s;
    if (!travBegin(s, bv, r)) return false;
    while (travStep<kAnyHit>(s, stack, bv, errFlags, leaf, r, h)) {
    }
    return s.isHit;
}

// The triangle BVH of the scene.
template <bool kAnyHit, int kShared = 0>
__device__ __forceinline__ bool traverse(const SceneView& sc, const TRay& r, THit& h,
                                         uint2 (*shStack)[kStackBlock] = nullptr) {
    const BvhView bv{sc.pairs, sc.leaves, sc.rootRef, sc.rootFlags, sc.rootMin, sc.rootMax, sc.hasRoot};
    const TriLeaf<kAnyHit> leaf{sc.tris};
    return traverseBvh<kAnyHit, TriLeaf<kAnyHit>, kShared>(bv, sc.errFlags, leaf, r, h, shStack);
}

// The sphere BVH of the scene (no spheres: no work).
template <bool kAnyHit, int kShared = 0>
__device__ __forceinline__ bool traverseSpheres(const SceneView& sc, const TRay& r, THit& h,
                                                uint2 (*shStack)[kStackBlock] = nullptr) {
    const SphereLeaf<kAnyHit> leaf{sc.sphBlocks};
    return traverseBvh<kAnyHit, SphereLeaf<kAnyHit>, kShared>(sc.sph, sc.errFlags, leaf, r, h, shStack);
}

}  // namespace cr
