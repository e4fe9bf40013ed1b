// cr_internal.cuh -- types and device helpers shared by the craystal_gb300
// translation units.
//
// Every translation unit is compiled with -fmad=false (device) and
// -ffp-contract=off (host): each float multiply and add is rounded on its
// own, in the order written, which is the order of the reference source
// (glm 1.0.1 for dot / cross / normalize / reflect / mat3 * vec3).  Division
// and square root are IEEE round-to-nearest (-prec-div / -prec-sqrt on).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "craystal_c.h"

namespace cr {

// ---------------------------------------------------------------------------
// error plumbing
// ---------------------------------------------------------------------------
void setError(const char* fmt, ...);
void clearError();
int fail(int code, const char* fmt, ...);
void countLaunch(uint64_t n = 1);

#define CR_CUDA(call)                                                              \
    do {                                                                           \
        cudaError_t _e = (call);                                                   \
        if (_e != cudaSuccess) {                                                   \
            return ::cr::fail(_e == cudaErrorMemoryAllocation ? CR_ERR_OUT_OF_MEMORY \
                                                             : CR_ERR_CUDA,        \
                              "%s failed: %s (%s:%d)", #call,                      \
                              cudaGetErrorString(_e), __FILE__, __LINE__);         \
        }                                                                          \
    } while (0)

#define CR_LAUNCH_CHECK()                                                          \
    do {                                                                           \
        ::cr::countLaunch();                                                       \
        cudaError_t _e = cudaGetLastError();                                       \
        if (_e != cudaSuccess)                                                     \
            return ::cr::fail(CR_ERR_CUDA, "kernel launch failed: %s (%s:%d)",      \
                              cudaGetErrorString(_e), __FILE__, __LINE__);         \
    } while (0)

// ---------------------------------------------------------------------------
// constants, Math/MathDefs.h:12-20
// ---------------------------------------------------------------------------
constexpr float kEps = 1e-6f;
constexpr float kPi = 3.14159265358979323846f;
constexpr float k2Pi = 2.f * kPi;
constexpr float kInvPi = 1.f / kPi;
constexpr float kInv2Pi = 0.5f / kPi;
constexpr float kFltEps = 1.19209290e-07f;  // std::numeric_limits<float>::epsilon()

// Device error flags (bits of Scene::errFlags).
constexpr uint32_t kErrStackOverflow = 1u;

// ---------------------------------------------------------------------------
// GPU-resident scene layout
// ---------------------------------------------------------------------------

// One interior node of the binary BVH with both children's boxes in one
// 64-byte record, so a visit is four coalesced 16-byte loads.
//   p0 = (L.min.x, L.min.y, L.min.z, L.max.x)
//   p1 = (L.max.y, L.max.z, R.min.x, R.min.y)
//   p2 = (R.min.z, R.max.x, R.max.y, R.max.z)
//   ref = (L.ref, R.ref, flags, 0).  A child ref with bit 31 clear points
//         at the pair of an interior child (its index and the group flags,
//         kGroupTopBit below); with bit 31 set it is a leaf, whose slot
//         range is in the ref itself or in the leaf table
//         (kInlineLeafBit, below).  flags bits 0-2
//         (left) and 3-5 (right) mark box axes thinner than FLT_EPSILON,
//         which take the degenerate-slab branch of Math/AABB.cu:10-19.
struct __align__(64) NodePair {
    float4 p0, p1, p2;
    uint4 ref;
};

// Triangle block per leaf slot (48 B): v0 with the primitive id in .w,
// e1 = v1 - v0 and e2 = v2 - v0 exactly as Moller-Trumbore forms them.
struct __align__(16) TriBlock {
    float4 v0;
    float4 e1;
    float4 e2;
};

// Sphere block per leaf slot of the sphere BVH (32 B): centre and radius,
// then (sphere id, 0, 0, 0).
struct __align__(16) SphereBlock {
    float4 geom;
    uint4 meta;
};

// One binary BVH in the traversal layout: interior NodePairs, the leaf
// table (first slot, count) and the root (its ref, degenerate-axis flags
// and box).
struct BvhView {
    const NodePair* pairs;
    const uint2* leaves;
    uint32_t rootRef;
    uint32_t rootFlags;
    float3 rootMin, rootMax;
    uint32_t hasRoot;
};

// Node produced by the GPU builder (breadth-first numbering).
struct __align__(16) BuildNode {
    float4 lo;   // min.xyz
    float4 hi;   // max.xyz
    uint4 info;  // (a, b, isLeaf, depth): leaf (start, count), interior (left, right)
};

struct MaterialGpu {
    float kd[3];
    float ks[3];
    float em[3];
    float shininess;
    uint32_t type;
    uint32_t flags;
    // derived once per material, as the BSDF constructors compute them
    float dProb, sProb;       // lobe selection (Phong, Principled)
    float rough, metal;       // Principled
    uint32_t tex;             // diffuse texture or CR_NO_TEXTURE
};

struct CameraGpu {
    float3 pos, U, V, W;
    float halfH, halfW;
    uint32_t width, height;
};

// Child refs.  Bit 31 clear: the pair index of an interior child.  Bit 31
// set: a leaf.  A leaf of 1 to 7 slots that start below 2^27 carries its
// range in the ref itself (bit 30 set, count in bits 27-29, first slot in
// bits 0-26), so that opening it needs no load; any other leaf has bit 30
// clear and bits 0-29 index the leaf table (first slot, count).
//
// The grouped copy of the pairs (built for the two-level traversal step,
// cr_scene_set_traversal) stores them in two-level groups instead: the pair
// of every interior node at even depth (the root's depth is 0) is followed
// directly by the pairs of its interior children, left before right.  There
// an interior ref holds the pair index in bits 0-27; a ref to the top of a
// group has bit 30 set, bit 29 when the node's left child is interior (its
// pair is the next one) and bit 28 when its right child is (the pair after
// that, or the next one when the left child is a leaf); a ref to the second
// pair of a group carries no flags.  Leaf refs are the same in both layouts.
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kInlineLeafBit = 0x40000000u;
constexpr uint32_t kInlineSlotMask = (1u << 27) - 1u;
constexpr uint32_t kInlineMaxCount = 7u;
constexpr uint32_t kGroupTopBit = 0x40000000u;
constexpr uint32_t kGroupLeftBit = 0x20000000u;
constexpr uint32_t kGroupRightBit = 0x10000000u;
constexpr uint32_t kPairIndexMask = 0x0FFFFFFFu;
constexpr uint32_t kMaxPairs = kPairIndexMask + 1u;

__host__ __device__ __forceinline__ uint32_t leafRef(uint32_t tableIndex, uint32_t first, uint32_t count) {
    if (count >= 1u && count <= kInlineMaxCount && first <= kInlineSlotMask)
        return kLeafBit | kInlineLeafBit | (count << 27) | first;
    return kLeafBit | tableIndex;
}

// Everything a traversal or render kernel reads, passed by value.

struct SceneView {
    const NodePair* pairs;
    const uint2* leaves;
    const TriBlock* tris;
    const float3* pos;
    const float3* nrm;
    const float2* uv;
    const uint32_t* idx;
    const uint32_t* primToMesh;
    const cr_mesh_desc* meshes;
    const MaterialGpu* mats;
    const uint32_t* emissive;
    uint32_t nEmissive;
    uint32_t rootRef;              // same encoding as a child ref
    uint32_t rootFlags;            // degenerate axes of the root box
    float3 rootMin, rootMax;
    uint32_t hasRoot;
    uint32_t* errFlags;
    float3 env;                    // constant environment radiance (0 = none)
    uint32_t nSpheres;             // sphere lights
    const float4* spheres;         // (center, radius)
    const float4* sphereEm;        // (emission, 0)
    const float4* texels;          // all diffuse textures, row-major RGBA
    const uint4* texDescs;         // (first texel, width, height, 0) per texture
    // analytic spheres with materials (Scene/Sphere.cu), in their own BVH
    BvhView sph;
    const SphereBlock* sphBlocks;  // per leaf slot
    const float4* sphGeom;         // per sphere id: centre, radius
    const uint32_t* sphMat;        // per sphere id: material
};

constexpr uint32_t kSpherePrim = 0xFFFFFF00u;  // hit ids kSpherePrim + i for sphere light i
constexpr uint32_t kMaxSphereLights = 64;
constexpr uint32_t kSphereBit = 0x80000000u;   // hit ids kSphereBit | i for sphere i
constexpr uint32_t kMaxSpheres = 0x7FFFFF00u;

__host__ __device__ __forceinline__ bool isSphereHit(uint32_t prim) { return prim >= kSphereBit && prim < kSpherePrim; }

}  // namespace cr

struct cr_scene {
    int device = 0;
    uint64_t nv = 0, nt = 0;
    uint32_t nMeshes = 0, nMats = 0, nEmissive = 0;
    float3* pos = nullptr;
    float3* nrm = nullptr;
    float2* uv = nullptr;
    uint32_t* idx = nullptr;
    uint32_t* primToMesh = nullptr;
    cr_mesh_desc* meshes = nullptr;
    cr::MaterialGpu* mats = nullptr;
    uint32_t* emissive = nullptr;
    // BVH
    cr::NodePair* pairs = nullptr;
    uint32_t nPairs = 0;
    uint2* leaves = nullptr;
    uint32_t nLeaves = 0;
    cr::TriBlock* tris = nullptr;
    uint32_t* slotToPrim = nullptr;
    cr::BuildNode* buildNodes = nullptr;
    uint32_t nBuildNodes = 0;
    uint32_t rootRef = 0, rootFlags = 0, hasRoot = 0;
    float3 rootMin{0, 0, 0}, rootMax{0, 0, 0};
    cr_bvh_stats stats{};
    uint32_t traversal = CR_TRAVERSAL_ONE_LEVEL;  // of the ray-cast queries
    bool hasPrincipled = false;                   // a material of type CR_MATERIAL_PRINCIPLED
    bool hasTextures = false;                     // a material with a diffuse texture
    cr::NodePair* groupPairs = nullptr;           // the grouped copy (two-level step only)
    uint32_t groupRootRef = 0;
    uint32_t* errFlags = nullptr;
    // camera + film
    bool hasCamera = false;
    cr::CameraGpu cam{};
    float* filmRgb = nullptr;
    float* filmW = nullptr;
    unsigned long long* rayCounter = nullptr;
    // host trace staging
    cudaStream_t streams[2] = {nullptr, nullptr};
    cr_ray* stageRays[2] = {nullptr, nullptr};
    cr_hit* stageHits[2] = {nullptr, nullptr};
    uint8_t* stageOcc[2] = {nullptr, nullptr};
    uint64_t stageCap = 0;
    // buffers of the radiance-cache integrator (cr_cache.cu), created on first use
    void* cacheBuffers = nullptr;
    // path state of the wavefront integrator (cr_wavefront.cu), created on first use
    void* wfBuffers = nullptr;
    // lights beyond the reference
    float3 env{0, 0, 0};
    uint32_t nSpheres = 0;
    float4* spheres = nullptr;
    float4* sphereEm = nullptr;
    // diffuse textures
    float4* texels = nullptr;
    uint4* texDescs = nullptr;
    uint32_t nTex = 0;
    // spheres and their BVH
    uint32_t nSph = 0;
    float4* sphGeom = nullptr;
    uint32_t* sphMat = nullptr;
    cr::NodePair* sphPairs = nullptr;
    uint2* sphLeaves = nullptr;
    cr::SphereBlock* sphBlocks = nullptr;
    uint32_t sphRootRef = 0, sphRootFlags = 0, sphHasRoot = 0;
    float3 sphRootMin{0, 0, 0}, sphRootMax{0, 0, 0};

    cr::SceneView view() const {
        cr::SceneView v;
        v.pairs = pairs;
        v.leaves = leaves;
        v.tris = tris;
        v.pos = pos;
        v.nrm = nrm;
        v.uv = uv;
        v.idx = idx;
        v.primToMesh = primToMesh;
        v.meshes = meshes;
        v.mats = mats;
        v.emissive = emissive;
        v.nEmissive = nEmissive;
        v.rootRef = rootRef;
        v.rootFlags = rootFlags;
        v.rootMin = rootMin;
        v.rootMax = rootMax;
        v.hasRoot = hasRoot;
        v.errFlags = errFlags;
        v.env = env;
        v.nSpheres = nSpheres;
        v.spheres = spheres;
        v.sphereEm = sphereEm;
        v.texels = texels;
        v.texDescs = texDescs;
        v.sph.pairs = sphPairs;
        v.sph.leaves = sphLeaves;
        v.sph.rootRef = sphRootRef;
        v.sph.rootFlags = sphRootFlags;
        v.sph.rootMin = sphRootMin;
        v.sph.rootMax = sphRootMax;
        v.sph.hasRoot = sphHasRoot;
        v.sphBlocks = sphBlocks;
        v.sphGeom = sphGeom;
        v.sphMat = sphMat;
        return v;
    }
};

namespace cr {

// implemented in cr_core.cu: reports and clears the scene's device error word
int takeDeviceErrors(cr_scene* s, const char* what);
// implemented in cr_bvh.cu
int buildBvh(cr_scene* s);
int buildSphereBvh(cr_scene* s);
int exportBvh(const cr_scene* s, cr_bvh_node* nodes, uint32_t* primMap);
int importBvh(cr_scene* s, const cr_bvh_node* nodes, uint32_t nodeCount, const uint32_t* primMap);
int buildGroupedPairs(cr_scene* s);
// implemented in cr_trace.cu
// mayAllocate = false: no device allocation (the no-allocation entry point)
int traceClosestDevice(cr_scene* s, const cr_ray* rays, uint64_t n, cr_hit* hits, cudaStream_t st,
                       bool mayAllocate = true);
int traceOccludedDevice(cr_scene* s, const cr_ray* rays, uint64_t n, uint8_t* occ, cudaStream_t st);
// implemented in cr_render.cu
int renderWavefront(cr_scene* s, const cr_integrator_config* cfg, uint32_t spp, uint32_t first,
                    cudaStream_t stream);
void freeWavefrontBuffers(void* p);
int renderDevice(cr_scene* s, const cr_integrator_config* cfg, uint32_t spp, uint32_t first,
                 cudaStream_t st);
int resolveFilm(cr_scene* s, float* rgbHost);
// implemented in cr_cache.cu
void freeCacheBuffers(void* buffers);
struct MlpState;
int checkCachedConfig(const cr_integrator_config* cfg, const cr_cache_config* cc);
int renderCachedMany(cr_scene* const* scenes, const cr_integrator_config* cfgs, const uint32_t* frames,
                     const uint32_t* firsts, MlpState* const* mlps, const cr_cache_config* cc,
                     const cudaStream_t* streams, uint32_t n, cr_cache_stats* stats, uint32_t* cnt);

}  // namespace cr
