// cr_bvh.cu -- GPU binned-SAH BVH builder with a Morton presort.
//
// The tree is the one BVH::build (Core/BVH.cu:88-338) makes: top-down,
// 32 centroid bins on each of the three axes, SAH cost
// 1 + (nL * SA_L + nR * SA_R) / SA_node (:289-301), the first (axis, bin)
// reaching the minimum cost wins (:244-279), partition by
// centroid[axis] < pMin + (i + 1) * extent / 32, a leaf when count <= 4 or
// depth >= 20 (:161) or when the split leaves one side empty (:186-195).
// Every quantity the split decision reads (node bounds, bin bounds and
// counts) is a min / max / count over a set, so the decisions, and with them
// the tree's topology and boxes, do not depend on the order in which the GPU
// visits primitives.  Two things do differ from the host build: nodes are
// numbered breadth-first (cr_scene_bvh_export renumbers them post-order),
// and primitives inside a leaf keep their Morton order (a stable partition)
// where the reference's std::partition leaves its own swap order; the two
// can only disagree on which of two triangles hit at exactly the same t is
// reported.
//
// Schedule: nodes with more than kTile primitives are processed one level
// at a time by multi-CTA kernels (bounds, binning, split, count, scan,
// scatter, children); every smaller subtree is then built to completion by
// one warp, with its bins in shared memory.

#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <vector>

#include "cr_internal.cuh"
#include "cr_math.cuh"
#include "cr_traverse.cuh"

namespace cr {
namespace {

constexpr int kBins = 32;
constexpr int kBinWords = 7;                         // lo.xyz, hi.xyz (encoded), count
constexpr int kBinBlock = 3 * kBins * kBinWords;     // 672 words per node
constexpr uint32_t kTile = 2048;                     // primitives per CTA tile
constexpr int kTileThreads = 256;
constexpr int kItems = kTile / kTileThreads;         // 8
constexpr uint32_t kMaxDepth = 20;                   // BVH.h:106
constexpr uint32_t kLeafMax = 4;                     // BVH.h:105
constexpr int kSubtreeWarps = 8;
constexpr int kSubtreeStack = 48;

struct __align__(16) PrimRec {
    float4 c;   // centroid, w = primitive id bits
    float4 lo;  // bounds min
    float4 hi;  // bounds max
};

struct BigTask {
    uint32_t start, count, node, firstTile;
    uint32_t nTiles, leftCount, axis, isLeaf;
    float pos;
    uint32_t pad[3];
};

struct Tile {
    uint32_t task, begin, end, pad;
};

struct SmallTask {
    uint32_t start, count, node, depth;
    uint32_t buf, pad[3];
};

struct Counters {
    uint32_t nodes;
    uint32_t nextBig;
    uint32_t nextTiles;
    uint32_t small;
    uint32_t leafCount;
    uint32_t maxLeafSize;
    uint32_t maxLeafDepth;
    uint32_t maxDepth;
    uint32_t cminEnc[3];
    uint32_t cmaxEnc[3];
    uint32_t overflow;   // set when a capacity check refused a write
};

__device__ __forceinline__ float comp(const float4& v, uint32_t a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
__device__ __forceinline__ float comp3(const float3& v, uint32_t a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// calcAABBSurfaceArea, Core/BVH.cu:284-287
__device__ __forceinline__ float surfaceArea(float3 lo, float3 hi) {
    float3 d = sub(hi, lo);
    return ((d.x * d.y + d.x * d.z) + d.y * d.z) * 2.0f;
}

// BVH::evaluateSAH, Core/BVH.cu:289-301
__device__ __forceinline__ float sahCost(float rootSA, float3 llo, float3 lhi, float3 rlo, float3 rhi, int nl,
                                         int nr) {
    float lsa = surfaceArea(llo, lhi), rsa = surfaceArea(rlo, rhi);
    return 1.0f + (1.0f * ((float)nl * lsa + (float)nr * rsa)) / rootSA;
}

// Bin index of Core/BVH.cu:228-235 (min(31, int(...)) then clamp to [0, 31]).
__device__ __forceinline__ int binIndex(float c, float mn, float scale) {
    int b = min(kBins - 1, f2iX86((c - mn) * scale));
    return b < 0 ? 0 : (b > kBins - 1 ? kBins - 1 : b);
}

__device__ __forceinline__ uint32_t laneId() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t warpUmin(uint32_t v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ uint32_t warpUmax(uint32_t v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Best split of one node from its 3 x 32 bins (words laid out as
// bins[(axis * 32 + bin) * 7 + k]), Core/BVH.cu:214-282.  Called by a full
// warp; lane i evaluates the split after bin i on each axis.  Returns false
// when no cost is below +inf, in which case the reference keeps
// (axis 0, position 0).
__device__ void warpBestSplit(const uint32_t* bins, float3 mn, float3 mx, uint32_t& axisOut, float& posOut) {
    const uint32_t lane = laneId();
    const float3 ext = sub(mx, mn);
    const float rootSA = surfaceArea(mn, mx);
    float bestCost = INFINITY;
    uint32_t bestAxis = 0;
    float bestPos = 0.0f;
    for (uint32_t a = 0; a < 3; ++a) {
        const uint32_t* b = bins + (a * kBins + lane) * kBinWords;
        uint32_t lo[3] = {b[0], b[1], b[2]}, hi[3] = {b[3], b[4], b[5]};
        int cnt = (int)b[6];
        // inclusive prefix (bins 0..lane) and suffix (bins lane..31)
        uint32_t plo[3], phi[3], slo[3], shi[3];
        int pc = cnt, sc = cnt;
        for (int k = 0; k < 3; k++) {
            plo[k] = slo[k] = lo[k];
            phi[k] = shi[k] = hi[k];
        }
        for (int o = 1; o < 32; o <<= 1) {
            int upc = __shfl_up_sync(0xffffffffu, pc, o);
            int dnc = __shfl_down_sync(0xffffffffu, sc, o);
            uint32_t ul[3], uh[3], dl[3], dh[3];
            for (int k = 0; k < 3; k++) {
                ul[k] = __shfl_up_sync(0xffffffffu, plo[k], o);
                uh[k] = __shfl_up_sync(0xffffffffu, phi[k], o);
                dl[k] = __shfl_down_sync(0xffffffffu, slo[k], o);
                dh[k] = __shfl_down_sync(0xffffffffu, shi[k], o);
            }
            if (lane >= (uint32_t)o) {
                pc += upc;
                for (int k = 0; k < 3; k++) {
                    plo[k] = min(plo[k], ul[k]);
                    phi[k] = max(phi[k], uh[k]);
                }
            }
            if (lane + o < 32u) {
                sc += dnc;
                for (int k = 0; k < 3; k++) {
                    slo[k] = min(slo[k], dl[k]);
                    shi[k] = max(shi[k], dh[k]);
                }
            }
        }
        // right side of split i = suffix starting at bin i + 1
        int rc = __shfl_down_sync(0xffffffffu, sc, 1);
        uint32_t rlo[3], rhi[3];
        for (int k = 0; k < 3; k++) {
            rlo[k] = __shfl_down_sync(0xffffffffu, slo[k], 1);
            rhi[k] = __shfl_down_sync(0xffffffffu, shi[k], 1);
        }
        float cost = INFINITY;
        if (lane < (uint32_t)(kBins - 1)) {
            cost = sahCost(rootSA, mk3(fdec(plo[0]), fdec(plo[1]), fdec(plo[2])),
                           mk3(fdec(phi[0]), fdec(phi[1]), fdec(phi[2])),
                           mk3(fdec(rlo[0]), fdec(rlo[1]), fdec(rlo[2])),
                           mk3(fdec(rhi[0]), fdec(rhi[1]), fdec(rhi[2])), pc, rc);
        }
        // first lane with the smallest cost strictly below +inf
        bool valid = cost < INFINITY;
        float c = valid ? cost : INFINITY;
        uint32_t idx = valid ? lane : 0xffffffffu;
        for (int o = 16; o > 0; o >>= 1) {
            float oc = __shfl_xor_sync(0xffffffffu, c, o);
            uint32_t oi = __shfl_xor_sync(0xffffffffu, idx, o);
            bool take = (oi != 0xffffffffu) && (idx == 0xffffffffu || oc < c || (oc == c && oi < idx));
            if (take) {
                c = oc;
                idx = oi;
            }
        }
        if (idx != 0xffffffffu && c < bestCost) {
            bestCost = c;
            bestAxis = a;
            bestPos = comp3(mn, a) + ((float)(idx + 1) * comp3(ext, a)) / (float)kBins;
        }
    }
    axisOut = bestAxis;
    posOut = bestPos;
}

// ---------------------------------------------------------------------------
// preparation: centroids, bounds, Morton codes
// ---------------------------------------------------------------------------
__global__ void kPrep(const float3* __restrict__ pos, const uint32_t* __restrict__ idx, uint32_t n,
                      PrimRec* __restrict__ out, Counters* __restrict__ ctr) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cl[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, ch[3] = {0u, 0u, 0u};
    if (i < n) {
        float3 v0 = pos[idx[3 * i]], v1 = pos[idx[3 * i + 1]], v2 = pos[idx[3 * i + 2]];
        // gatherTriangles, Core/BVH.cu:120-148
        float3 c = divs(add(add(v0, v1), v2), 3.0f);
        float3 lo = mk3(INFINITY, INFINITY, INFINITY), hi = mk3(-INFINITY, -INFINITY, -INFINITY);
        const float3 vs[3] = {v0, v1, v2};
        for (int k = 0; k < 3; k++) {
            lo = mk3(gmin(lo.x, vs[k].x), gmin(lo.y, vs[k].y), gmin(lo.z, vs[k].z));
            hi = mk3(gmax(hi.x, vs[k].x), gmax(hi.y, vs[k].y), gmax(hi.z, vs[k].z));
        }
        PrimRec r;
        r.c = make_float4(c.x, c.y, c.z, __uint_as_float(i));
        r.lo = make_float4(lo.x, lo.y, lo.z, 0.0f);
        r.hi = make_float4(hi.x, hi.y, hi.z, 0.0f);
        out[i] = r;
        cl[0] = ch[0] = fenc(c.x);
        cl[1] = ch[1] = fenc(c.y);
        cl[2] = ch[2] = fenc(c.z);
    }
    for (int k = 0; k < 3; k++) {
        uint32_t a = warpUmin(cl[k]), b = warpUmax(ch[k]);
        if (laneId() == 0) {
            atomicMin(&ctr->cminEnc[k], a);
            atomicMax(&ctr->cmaxEnc[k], b);
        }
    }
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void kMorton(const PrimRec* __restrict__ rec, uint32_t n, const Counters* __restrict__ ctr,
                        uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 c = rec[i].c;
    uint32_t q[3];
    for (int k = 0; k < 3; k++) {
        float mn = fdec(ctr->cminEnc[k]), mx = fdec(ctr->cmaxEnc[k]);
        float e = mx - mn;
        float t = (e > 0.0f) ? (comp(c, k) - mn) / e : 0.0f;
        t = fminf(fmaxf(t, 0.0f), 1.0f);  // NaN -> 0
        q[k] = (uint32_t)(t * 1023.0f);
    }
    keys[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
    vals[i] = i;
}

__global__ void kGather(const PrimRec* __restrict__ src, const uint32_t* __restrict__ order, uint32_t n,
                        PrimRec* __restrict__ dst) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[order[i]];
}

// ---------------------------------------------------------------------------
// breadth-first levels for nodes larger than one tile
// ---------------------------------------------------------------------------
__global__ void kBigInit(uint32_t nTasks, uint32_t* __restrict__ bounds, uint32_t* __restrict__ bins) {
    uint32_t t = blockIdx.x;
    if (t >= nTasks) return;
    for (uint32_t j = threadIdx.x; j < 6; j += blockDim.x) bounds[t * 6 + j] = j < 3 ? fenc(INFINITY) : fenc(-INFINITY);
    for (uint32_t j = threadIdx.x; j < (uint32_t)kBinBlock; j += blockDim.x) {
        uint32_t k = j % kBinWords;
        bins[(size_t)t * kBinBlock + j] = k < 3 ? fenc(INFINITY) : (k < 6 ? fenc(-INFINITY) : 0u);
    }
}

// Block-wide min/max of six encoded words; result valid in thread 0.
__device__ void blockMinMax6(uint32_t v[6], uint32_t* sh /* 6 * 32 */) {
    for (int k = 0; k < 6; k++) v[k] = k < 3 ? warpUmin(v[k]) : warpUmax(v[k]);
    const uint32_t w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (laneId() == 0)
        for (int k = 0; k < 6; k++) sh[k * 32 + w] = v[k];
    __syncthreads();
    if (w == 0) {
        for (int k = 0; k < 6; k++) {
            uint32_t x = laneId() < nw ? sh[k * 32 + laneId()] : (k < 3 ? 0xffffffffu : 0u);
            v[k] = k < 3 ? warpUmin(x) : warpUmax(x);
        }
    }
}

__global__ void kBigBounds(const Tile* __restrict__ tiles, const PrimRec* __restrict__ src,
                           uint32_t* __restrict__ bounds) {
    __shared__ uint32_t sh[6 * 32];
    const Tile tl = tiles[blockIdx.x];
    uint32_t v[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    for (uint32_t i = tl.begin + threadIdx.x; i < tl.end; i += blockDim.x) {
        const float4 lo = src[i].lo, hi = src[i].hi;
        v[0] = min(v[0], fenc(lo.x));
        v[1] = min(v[1], fenc(lo.y));
        v[2] = min(v[2], fenc(lo.z));
        v[3] = max(v[3], fenc(hi.x));
        v[4] = max(v[4], fenc(hi.y));
        v[5] = max(v[5], fenc(hi.z));
    }
    blockMinMax6(v, sh);
    if (threadIdx.x == 0) {
        uint32_t* b = bounds + tl.task * 6;
        for (int k = 0; k < 3; k++) atomicMin(b + k, v[k]);
        for (int k = 3; k < 6; k++) atomicMax(b + k, v[k]);
    }
}

__device__ __forceinline__ void statLeaf(Counters* ctr, uint32_t count, uint32_t depth) {
    atomicAdd(&ctr->leafCount, 1u);
    atomicMax(&ctr->maxLeafSize, count);
    atomicMax(&ctr->maxLeafDepth, depth);
}

__global__ void kBigNode(BigTask* __restrict__ tasks, uint32_t nTasks, uint32_t level,
                         const uint32_t* __restrict__ bounds, BuildNode* __restrict__ nodes,
                         Counters* __restrict__ ctr) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nTasks) return;
    BigTask& tk = tasks[t];
    const uint32_t* b = bounds + t * 6;
    BuildNode& nd = nodes[tk.node];
    nd.lo = make_float4(fdec(b[0]), fdec(b[1]), fdec(b[2]), 0.0f);
    nd.hi = make_float4(fdec(b[3]), fdec(b[4]), fdec(b[5]), 0.0f);
    tk.isLeaf = 0;
    if (tk.count <= kLeafMax || level >= kMaxDepth) {
        tk.isLeaf = 1;
        nd.info = make_uint4(tk.start, tk.count, 1u, level);
        statLeaf(ctr, tk.count, level);
    }
}

__global__ void kBigBin(const Tile* __restrict__ tiles, const BigTask* __restrict__ tasks,
                        const PrimRec* __restrict__ src, const uint32_t* __restrict__ bounds,
                        uint32_t* __restrict__ bins) {
    __shared__ uint32_t sb[kBinBlock];
    const Tile tl = tiles[blockIdx.x];
    if (tasks[tl.task].isLeaf) return;
    for (uint32_t j = threadIdx.x; j < (uint32_t)kBinBlock; j += blockDim.x) {
        uint32_t k = j % kBinWords;
        sb[j] = k < 3 ? fenc(INFINITY) : (k < 6 ? fenc(-INFINITY) : 0u);
    }
    const uint32_t* bb = bounds + tl.task * 6;
    const float3 mn = mk3(fdec(bb[0]), fdec(bb[1]), fdec(bb[2]));
    const float3 mx = mk3(fdec(bb[3]), fdec(bb[4]), fdec(bb[5]));
    const float3 ext = sub(mx, mn);
    const float sc[3] = {(float)kBins / ext.x, (float)kBins / ext.y, (float)kBins / ext.z};
    const float mnv[3] = {mn.x, mn.y, mn.z};
    __syncthreads();
    for (uint32_t i = tl.begin + threadIdx.x; i < tl.end; i += blockDim.x) {
        const PrimRec r = src[i];
        const uint32_t e[6] = {fenc(r.lo.x), fenc(r.lo.y), fenc(r.lo.z), fenc(r.hi.x), fenc(r.hi.y), fenc(r.hi.z)};
        for (uint32_t a = 0; a < 3; a++) {
            int bi = binIndex(comp(r.c, a), mnv[a], sc[a]);
            uint32_t* w = sb + (a * kBins + bi) * kBinWords;
            atomicMin(w + 0, e[0]);
            atomicMin(w + 1, e[1]);
            atomicMin(w + 2, e[2]);
            atomicMax(w + 3, e[3]);
            atomicMax(w + 4, e[4]);
            atomicMax(w + 5, e[5]);
            atomicAdd(w + 6, 1u);
        }
    }
    __syncthreads();
    uint32_t* g = bins + (size_t)tl.task * kBinBlock;
    for (uint32_t j = threadIdx.x; j < 3u * kBins; j += blockDim.x) {
        const uint32_t* w = sb + j * kBinWords;
        if (w[6] == 0) continue;
        uint32_t* gw = g + j * kBinWords;
        atomicMin(gw + 0, w[0]);
        atomicMin(gw + 1, w[1]);
        atomicMin(gw + 2, w[2]);
        atomicMax(gw + 3, w[3]);
        atomicMax(gw + 4, w[4]);
        atomicMax(gw + 5, w[5]);
        atomicAdd(gw + 6, w[6]);
    }
}

__global__ void kBigSplit(BigTask* __restrict__ tasks, uint32_t nTasks, const uint32_t* __restrict__ bounds,
                          const uint32_t* __restrict__ bins) {
    const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (t >= nTasks) return;
    BigTask& tk = tasks[t];
    if (tk.isLeaf) return;
    const uint32_t* bb = bounds + t * 6;
    uint32_t axis;
    float pos;
    warpBestSplit(bins + (size_t)t * kBinBlock, mk3(fdec(bb[0]), fdec(bb[1]), fdec(bb[2])),
                  mk3(fdec(bb[3]), fdec(bb[4]), fdec(bb[5])), axis, pos);
    if (laneId() == 0) {
        tk.axis = axis;
        tk.pos = pos;
    }
}

__device__ __forceinline__ int blockSumInt(int v, int* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const uint32_t w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (laneId() == 0) sh[w] = v;
    __syncthreads();
    int s = 0;
    for (uint32_t k = 0; k < nw; k++) s += sh[k];
    return s;
}

__global__ void kBigCount(const Tile* __restrict__ tiles, const BigTask* __restrict__ tasks,
                          const PrimRec* __restrict__ src, uint32_t* __restrict__ tileLeft) {
    __shared__ int sh[32];
    const Tile tl = tiles[blockIdx.x];
    const BigTask tk = tasks[tl.task];
    if (tk.isLeaf) return;
    int c = 0;
    for (uint32_t i = tl.begin + threadIdx.x; i < tl.end; i += blockDim.x) c += comp(src[i].c, tk.axis) < tk.pos ? 1 : 0;
    int s = blockSumInt(c, sh);
    if (threadIdx.x == 0) tileLeft[blockIdx.x] = (uint32_t)s;
}

// Per task (one warp): exclusive prefix of its tiles' left counts.
__global__ void kBigScan(BigTask* __restrict__ tasks, uint32_t nTasks, const uint32_t* __restrict__ tileLeft,
                         uint32_t* __restrict__ tilePrefix) {
    const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (t >= nTasks) return;
    BigTask& tk = tasks[t];
    if (tk.isLeaf) return;
    const uint32_t lane = laneId();
    uint32_t run = 0;
    for (uint32_t base = 0; base < tk.nTiles; base += 32) {
        uint32_t j = base + lane;
        uint32_t v = j < tk.nTiles ? tileLeft[tk.firstTile + j] : 0u;
        uint32_t incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += u;
        }
        if (j < tk.nTiles) tilePrefix[tk.firstTile + j] = run + incl - v;
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) tk.leftCount = run;
}

// Stable partition of one tile into dst.
__global__ void __launch_bounds__(kTileThreads) kBigScatter(const Tile* __restrict__ tiles,
                                                            const BigTask* __restrict__ tasks,
                                                            const uint32_t* __restrict__ tilePrefix,
                                                            const PrimRec* __restrict__ src,
                                                            PrimRec* __restrict__ dst) {
    __shared__ uint32_t warpTot[kTileThreads / 32];
    const Tile tl = tiles[blockIdx.x];
    const BigTask tk = tasks[tl.task];
    if (tk.isLeaf) return;
    const uint32_t first = tl.begin + threadIdx.x * kItems;
    uint32_t flags = 0, nLeft = 0, nValid = 0;
    for (int k = 0; k < kItems; k++) {
        uint32_t i = first + k;
        if (i < tl.end) {
            nValid++;
            if (comp(src[i].c, tk.axis) < tk.pos) {
                flags |= 1u << k;
                nLeft++;
            }
        }
    }
    // block exclusive scan of nLeft
    const uint32_t lane = laneId(), w = threadIdx.x >> 5;
    uint32_t incl = nLeft;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += u;
    }
    if (lane == 31) warpTot[w] = incl;
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t k = 0; k < w; k++) before += warpTot[k];
    const uint32_t leftBefore = before + incl - nLeft;                   // within tile
    const uint32_t tileLeftBefore = tilePrefix[blockIdx.x];              // within task
    const uint32_t tileOffset = tl.begin - tk.start;                     // prims of task before tile
    const uint32_t itemOffset = threadIdx.x * kItems;                    // prims of tile before thread
    uint32_t l = tk.start + tileLeftBefore + leftBefore;
    uint32_t r = tk.start + tk.leftCount + (tileOffset - tileLeftBefore) + (itemOffset - leftBefore);
    for (int k = 0; k < kItems; k++) {
        if ((uint32_t)k >= nValid) break;
        const PrimRec rec = src[first + k];
        if (flags & (1u << k)) dst[l++] = rec;
        else dst[r++] = rec;
    }
}

__global__ void kBigChildren(BigTask* __restrict__ tasks, uint32_t nTasks, uint32_t level, uint32_t dstBuf,
                             BuildNode* __restrict__ nodes, BigTask* __restrict__ nextTasks,
                             Tile* __restrict__ nextTiles, SmallTask* __restrict__ small,
                             Counters* __restrict__ ctr, uint32_t capBig, uint32_t capTiles, uint32_t capSmall,
                             uint32_t capNodes) {
    const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (t >= nTasks) return;
    BigTask& tk = tasks[t];
    if (tk.isLeaf) return;
    const uint32_t lane = laneId();
    const uint32_t L = tk.leftCount;
    if (L == 0 || L == tk.count) {  // Core/BVH.cu:186-195
        if (lane == 0) {
            tk.isLeaf = 1;
            nodes[tk.node].info = make_uint4(tk.start, tk.count, 1u, level);
            statLeaf(ctr, tk.count, level);
        }
        return;
    }
    uint32_t ln = 0;
    if (lane == 0) {
        ln = atomicAdd(&ctr->nodes, 2u);
        if (ln + 2 > capNodes) {
            ctr->overflow = 1;
        } else {
            nodes[tk.node].info = make_uint4(ln, ln + 1, 0u, level);
            atomicMax(&ctr->maxDepth, level);
        }
    }
    ln = __shfl_sync(0xffffffffu, ln, 0);
    if (ln + 2 > capNodes) return;
    for (int side = 0; side < 2; side++) {
        const uint32_t cs = side == 0 ? tk.start : tk.start + L;
        const uint32_t cc = side == 0 ? L : tk.count - L;
        const uint32_t node = ln + side;
        if (cc > kTile) {
            const uint32_t nt = (cc + kTile - 1) / kTile;
            uint32_t bt = 0, ft = 0;
            if (lane == 0) {
                bt = atomicAdd(&ctr->nextBig, 1u);
                ft = atomicAdd(&ctr->nextTiles, nt);
                if (bt >= capBig || ft + nt > capTiles) ctr->overflow = 1;
            }
            bt = __shfl_sync(0xffffffffu, bt, 0);
            ft = __shfl_sync(0xffffffffu, ft, 0);
            if (bt >= capBig || ft + nt > capTiles) continue;
            if (lane == 0) {
                BigTask c;
                memset(&c, 0, sizeof(c));
                c.start = cs;
                c.count = cc;
                c.node = node;
                c.firstTile = ft;
                c.nTiles = nt;
                nextTasks[bt] = c;
            }
            for (uint32_t j = lane; j < nt; j += 32) {
                Tile tl;
                tl.task = bt;
                tl.begin = cs + j * kTile;
                tl.end = min(cs + (j + 1) * kTile, cs + cc);
                tl.pad = 0;
                nextTiles[ft + j] = tl;
            }
        } else if (lane == 0) {
            uint32_t st = atomicAdd(&ctr->small, 1u);
            if (st >= capSmall) {
                ctr->overflow = 1;
                continue;
            }
            SmallTask s;
            s.start = cs;
            s.count = cc;
            s.node = node;
            s.depth = level + 1;
            s.buf = dstBuf;
            s.pad[0] = s.pad[1] = s.pad[2] = 0;
            small[st] = s;
        }
    }
}

__global__ void kBigFinalize(const Tile* __restrict__ tiles, const BigTask* __restrict__ tasks,
                             const PrimRec* __restrict__ src, uint32_t* __restrict__ order) {
    const Tile tl = tiles[blockIdx.x];
    if (!tasks[tl.task].isLeaf) return;
    for (uint32_t i = tl.begin + threadIdx.x; i < tl.end; i += blockDim.x) order[i] = __float_as_uint(src[i].c.w);
}

// ---------------------------------------------------------------------------
// one warp builds a whole subtree of <= kTile primitives
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kSubtreeWarps * 32) kSubtree(const SmallTask* __restrict__ tasks, uint32_t nTasks,
                                                               PrimRec* buf0, PrimRec* buf1,
                                                               BuildNode* __restrict__ nodes,
                                                               uint32_t* __restrict__ order,
                                                               Counters* __restrict__ ctr, uint32_t capNodes) {
    __shared__ uint32_t sbins[kSubtreeWarps][kBinBlock];
    __shared__ SmallTask sstack[kSubtreeWarps][kSubtreeStack];
    const uint32_t w = threadIdx.x >> 5, lane = laneId();
    const uint32_t t = blockIdx.x * kSubtreeWarps + w;
    if (t >= nTasks) return;
    uint32_t* bins = sbins[w];
    SmallTask* stack = sstack[w];
    int sp = 0;
    if (lane == 0) stack[0] = tasks[t];
    sp = 1;
    __syncwarp();
    while (sp > 0) {
        const SmallTask tk = stack[--sp];
        __syncwarp();
        PrimRec* src = tk.buf ? buf1 : buf0;
        PrimRec* dst = tk.buf ? buf0 : buf1;
        // node bounds (Core/BVH.cu:153-157)
        uint32_t v[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
        for (uint32_t i = lane; i < tk.count; i += 32) {
            const float4 lo = src[tk.start + i].lo, hi = src[tk.start + i].hi;
            v[0] = min(v[0], fenc(lo.x));
            v[1] = min(v[1], fenc(lo.y));
            v[2] = min(v[2], fenc(lo.z));
            v[3] = max(v[3], fenc(hi.x));
            v[4] = max(v[4], fenc(hi.y));
            v[5] = max(v[5], fenc(hi.z));
        }
        for (int k = 0; k < 6; k++) v[k] = k < 3 ? warpUmin(v[k]) : warpUmax(v[k]);
        const float3 mn = mk3(fdec(v[0]), fdec(v[1]), fdec(v[2]));
        const float3 mx = mk3(fdec(v[3]), fdec(v[4]), fdec(v[5]));
        if (lane == 0) {
            nodes[tk.node].lo = make_float4(mn.x, mn.y, mn.z, 0.0f);
            nodes[tk.node].hi = make_float4(mx.x, mx.y, mx.z, 0.0f);
        }
        // a full stack cannot happen for depth <= 20 (at most 22 entries); the
        // check keeps every write in bounds regardless
        bool leaf = tk.count <= kLeafMax || tk.depth >= kMaxDepth || sp + 2 > kSubtreeStack;
        if (sp + 2 > kSubtreeStack && lane == 0) ctr->overflow = 1;
        uint32_t axis = 0, leftTotal = 0;
        float pos = 0.0f;
        if (!leaf) {
            for (uint32_t j = lane; j < (uint32_t)kBinBlock; j += 32) {
                uint32_t k = j % kBinWords;
                bins[j] = k < 3 ? fenc(INFINITY) : (k < 6 ? fenc(-INFINITY) : 0u);
            }
            __syncwarp();
            const float3 ext = sub(mx, mn);
            const float sc[3] = {(float)kBins / ext.x, (float)kBins / ext.y, (float)kBins / ext.z};
            const float mnv[3] = {mn.x, mn.y, mn.z};
            for (uint32_t i = lane; i < tk.count; i += 32) {
                const PrimRec r = src[tk.start + i];
                const uint32_t e[6] = {fenc(r.lo.x), fenc(r.lo.y), fenc(r.lo.z),
                                       fenc(r.hi.x), fenc(r.hi.y), fenc(r.hi.z)};
                for (uint32_t a = 0; a < 3; a++) {
                    int bi = binIndex(comp(r.c, a), mnv[a], sc[a]);
                    uint32_t* wd = bins + (a * kBins + bi) * kBinWords;
                    atomicMin(wd + 0, e[0]);
                    atomicMin(wd + 1, e[1]);
                    atomicMin(wd + 2, e[2]);
                    atomicMax(wd + 3, e[3]);
                    atomicMax(wd + 4, e[4]);
                    atomicMax(wd + 5, e[5]);
                    atomicAdd(wd + 6, 1u);
                }
            }
            __syncwarp();
            warpBestSplit(bins, mn, mx, axis, pos);
            for (uint32_t base = 0; base < tk.count; base += 32) {
                uint32_t i = base + lane;
                bool p = i < tk.count && comp(src[tk.start + i].c, axis) < pos;
                leftTotal += __popc(__ballot_sync(0xffffffffu, p));
            }
            leaf = leftTotal == 0 || leftTotal == tk.count;
        }
        if (leaf) {
            for (uint32_t i = lane; i < tk.count; i += 32) order[tk.start + i] = __float_as_uint(src[tk.start + i].c.w);
            if (lane == 0) {
                nodes[tk.node].info = make_uint4(tk.start, tk.count, 1u, tk.depth);
                statLeaf(ctr, tk.count, tk.depth);
            }
            __syncwarp();
            continue;
        }
        // stable partition src -> dst
        const uint32_t ltMask = (1u << lane) - 1u;
        uint32_t nl = 0, nr = 0;
        for (uint32_t base = 0; base < tk.count; base += 32) {
            uint32_t i = base + lane;
            bool valid = i < tk.count;
            PrimRec r;
            bool p = false;
            if (valid) {
                r = src[tk.start + i];
                p = comp(r.c, axis) < pos;
            }
            uint32_t bl = __ballot_sync(0xffffffffu, valid && p);
            uint32_t br = __ballot_sync(0xffffffffu, valid && !p);
            if (valid) {
                if (p) dst[tk.start + nl + __popc(bl & ltMask)] = r;
                else dst[tk.start + leftTotal + nr + __popc(br & ltMask)] = r;
            }
            nl += __popc(bl);
            nr += __popc(br);
        }
        __syncwarp();
        uint32_t ln = 0;
        if (lane == 0) ln = atomicAdd(&ctr->nodes, 2u);
        ln = __shfl_sync(0xffffffffu, ln, 0);
        if (ln + 2 > capNodes) {  // cannot happen: a split always leaves both sides non-empty
            if (lane == 0) ctr->overflow = 1;
            break;
        }
        if (lane == 0) {
            nodes[tk.node].info = make_uint4(ln, ln + 1, 0u, tk.depth);
            atomicMax(&ctr->maxDepth, tk.depth);
            SmallTask a, b;
            a.start = tk.start + leftTotal;
            a.count = tk.count - leftTotal;
            a.node = ln + 1;
            a.depth = tk.depth + 1;
            a.buf = tk.buf ^ 1u;
            b.start = tk.start;
            b.count = leftTotal;
            b.node = ln;
            b.depth = tk.depth + 1;
            b.buf = tk.buf ^ 1u;
            a.pad[0] = a.pad[1] = a.pad[2] = b.pad[0] = b.pad[1] = b.pad[2] = 0;
            stack[sp] = a;
            stack[sp + 1] = b;
        }
        sp += 2;
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// traversal layout
// ---------------------------------------------------------------------------
__global__ void kLeafFlags(const BuildNode* __restrict__ nodes, uint32_t n, uint32_t* __restrict__ isLeaf) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) isLeaf[i] = nodes[i].info.z;
}

__host__ __device__ __forceinline__ uint32_t childRef(const BuildNode* nodes, const uint32_t* leafPrefix, uint32_t c) {
    const BuildNode& n = nodes[c];
    return n.info.z ? leafRef(leafPrefix[c], n.info.x, n.info.y) : (c - leafPrefix[c]);
}

// The NodePair of interior node i: both children's boxes, refs and
// degenerate-axis flags.  Interior node i becomes pair i - leafPrefix[i].
__host__ __device__ __forceinline__ NodePair pairOf(const BuildNode* nodes, const uint32_t* leafPrefix, uint32_t i) {
    const BuildNode& nd = nodes[i];
    const BuildNode& L = nodes[nd.info.x];
    const BuildNode& R = nodes[nd.info.y];
    NodePair p;
    p.p0 = make_float4(L.lo.x, L.lo.y, L.lo.z, L.hi.x);
    p.p1 = make_float4(L.hi.y, L.hi.z, R.lo.x, R.lo.y);
    p.p2 = make_float4(R.lo.z, R.hi.x, R.hi.y, R.hi.z);
    uint32_t fl = degenerateFlags(mk3(L.lo.x, L.lo.y, L.lo.z), mk3(L.hi.x, L.hi.y, L.hi.z)) |
                  (degenerateFlags(mk3(R.lo.x, R.lo.y, R.lo.z), mk3(R.hi.x, R.hi.y, R.hi.z)) << 3);
    p.ref = make_uint4(childRef(nodes, leafPrefix, nd.info.x), childRef(nodes, leafPrefix, nd.info.y), fl, 0u);
    return p;
}

__global__ void kLayout(const BuildNode* __restrict__ nodes, uint32_t n, const uint32_t* __restrict__ leafPrefix,
                        NodePair* __restrict__ pairs, uint2* __restrict__ leaves) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const BuildNode nd = nodes[i];
    if (nd.info.z) {
        leaves[leafPrefix[i]] = make_uint2(nd.info.x, nd.info.y);
        return;
    }
    pairs[i - leafPrefix[i]] = pairOf(nodes, leafPrefix, i);
}

// ---------------------------------------------------------------------------
// the grouped copy of the pairs, for the two-level traversal step
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ bool isInterior(const BuildNode* nodes, uint32_t c) { return nodes[c].info.z == 0u; }

// Pairs in node i's group: 1 + its interior children for an interior node at
// even depth (a group top), 0 for any other node (a leaf, or an interior
// node at odd depth, whose pair sits in its parent's group).
__host__ __device__ __forceinline__ uint32_t groupSize(const BuildNode* nodes, uint32_t i) {
    const BuildNode& nd = nodes[i];
    if (nd.info.z || (nd.info.w & 1u)) return 0u;
    return 1u + (isInterior(nodes, nd.info.x) ? 1u : 0u) + (isInterior(nodes, nd.info.y) ? 1u : 0u);
}

// The ref of group top g: its pair index and the flags that say which of
// its children's pairs follow it.
__host__ __device__ __forceinline__ uint32_t topRef(const BuildNode* nodes, const uint32_t* groupStart, uint32_t g) {
    const BuildNode& nd = nodes[g];
    return groupStart[g] | kGroupTopBit | (isInterior(nodes, nd.info.x) ? kGroupLeftBit : 0u) |
           (isInterior(nodes, nd.info.y) ? kGroupRightBit : 0u);
}

// The NodePair of interior node i at grouped index p.  The children of a
// group top (top = true) are the group's second-level pairs at p + 1 and
// after; the interior children of a second-level node are group tops.
__host__ __device__ __forceinline__ NodePair groupPair(const BuildNode* nodes, const uint32_t* leafPrefix,
                                                       const uint32_t* groupStart, uint32_t i, bool top, uint32_t p) {
    NodePair q = pairOf(nodes, leafPrefix, i);
    const BuildNode& nd = nodes[i];
    uint32_t next = p + 1u;
    uint32_t* ref[2] = {&q.ref.x, &q.ref.y};
    for (int k = 0; k < 2; k++) {
        const uint32_t c = k == 0 ? nd.info.x : nd.info.y;
        if (!isInterior(nodes, c)) continue;  // leaf refs are the same in both layouts
        *ref[k] = top ? next++ : topRef(nodes, groupStart, c);
    }
    return q;
}

// Group top i: its own pair and its second-level pairs.  Every interior
// node's pair is written exactly once, by the top of its group.
__global__ void kGroupLayout(const BuildNode* __restrict__ nodes, uint32_t n, const uint32_t* __restrict__ leafPrefix,
                             const uint32_t* __restrict__ groupStart, NodePair* __restrict__ pairs,
                             uint32_t* __restrict__ rootRef) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || groupSize(nodes, i) == 0u) return;
    const BuildNode nd = nodes[i];
    const uint32_t p = groupStart[i];
    pairs[p] = groupPair(nodes, leafPrefix, groupStart, i, true, p);
    uint32_t q = p + 1u;
    for (uint32_t c : {nd.info.x, nd.info.y})
        if (isInterior(nodes, c)) {
            pairs[q] = groupPair(nodes, leafPrefix, groupStart, c, false, q);
            q++;
        }
    if (i == 0) *rootRef = topRef(nodes, groupStart, 0);  // node 0 is the root
}

__global__ void kGroupFlags(const BuildNode* __restrict__ nodes, uint32_t n, uint32_t* __restrict__ isLeaf,
                            uint32_t* __restrict__ group) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        isLeaf[i] = nodes[i].info.z;
        group[i] = groupSize(nodes, i);
    }
}

__global__ void kTriBlocks(const float3* __restrict__ pos, const uint32_t* __restrict__ idx,
                           const uint32_t* __restrict__ order, uint32_t n, TriBlock* __restrict__ out) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    uint32_t prim = order[s];
    float3 v0 = pos[idx[3 * prim]], v1 = pos[idx[3 * prim + 1]], v2 = pos[idx[3 * prim + 2]];
    float3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    TriBlock b;
    b.v0 = make_float4(v0.x, v0.y, v0.z, __uint_as_float(prim));
    b.e1 = make_float4(e1.x, e1.y, e1.z, 0.0f);
    b.e2 = make_float4(e2.x, e2.y, e2.z, 0.0f);
    out[s] = b;
}

// Sphere records: the centre as centroid, the box centre +- radius widened
// by a small margin, so that a box's entry distance never exceeds the
// computed distance of a sphere hit inside it (the quadratic's rounding)
// and the traversal's culling drops no sphere the linear loop of
// SceneView::intersect would find.
__global__ void kPrepSpheres(const float4* __restrict__ geom, uint32_t n, PrimRec* __restrict__ out,
                             Counters* __restrict__ ctr) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cl[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, ch[3] = {0u, 0u, 0u};
    if (i < n) {
        const float4 g = geom[i];
        const float ext = g.w * 1.0009765625f + 1e-6f * fmaxf(fmaxf(fabsf(g.x), fabsf(g.y)), fabsf(g.z));
        PrimRec r;
        r.c = make_float4(g.x, g.y, g.z, __uint_as_float(i));
        r.lo = make_float4(g.x - ext, g.y - ext, g.z - ext, 0.0f);
        r.hi = make_float4(g.x + ext, g.y + ext, g.z + ext, 0.0f);
        out[i] = r;
        cl[0] = ch[0] = fenc(g.x);
        cl[1] = ch[1] = fenc(g.y);
        cl[2] = ch[2] = fenc(g.z);
    }
    for (int k = 0; k < 3; k++) {
        uint32_t a = warpUmin(cl[k]), b = warpUmax(ch[k]);
        if (laneId() == 0) {
            atomicMin(&ctr->cminEnc[k], a);
            atomicMax(&ctr->cmaxEnc[k], b);
        }
    }
}

__global__ void kSphereBlocks(const float4* __restrict__ geom, const uint32_t* __restrict__ order, uint32_t n,
                              SphereBlock* __restrict__ out) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t id = order[s];
    SphereBlock b;
    b.geom = geom[id];
    b.meta = make_uint4(id, 0u, 0u, 0u);
    out[s] = b;
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)); }
    T* release() {
        T* r = p;
        p = nullptr;
        return r;
    }
};

inline unsigned blocksFor(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

namespace {

// A built BVH in the traversal layout, plus the build records.
struct BuiltBvh {
    NodePair* pairs = nullptr;
    uint32_t nPairs = 0;
    uint2* leaves = nullptr;
    uint32_t nLeaves = 0;
    uint32_t* order = nullptr;  // leaf slot -> primitive
    BuildNode* nodes = nullptr;
    uint32_t nNodes = 0;
    uint32_t levels = 0;
    Counters counters{};
    BuildNode root{};
};

// The GPU binned-SAH build over N primitive records that prep(rec, ctr)
// writes (centroid with the primitive id in .w, bounds; centroid bounds
// into the counters): Morton presort, breadth-first levels for tasks above
// kTile primitives, a warp per smaller subtree, then the NodePair layout.
template <class Prep>
int buildGeneric(uint32_t N, Prep prep, BuiltBvh& out) {
    DevBuf<PrimRec> recA, recB;
    DevBuf<Counters> ctr;
    DevBuf<uint32_t> order, keysIn, keysOut, valsIn, valsOut;
    CR_CUDA(recA.alloc(N));
    CR_CUDA(recB.alloc(N));
    CR_CUDA(ctr.alloc(1));
    CR_CUDA(order.alloc(N));
    CR_CUDA(cudaMemset(order.p, 0, (size_t)N * sizeof(uint32_t)));
    Counters h0;
    std::memset(&h0, 0, sizeof(h0));
    h0.nodes = 1;
    for (int k = 0; k < 3; k++) {
        h0.cminEnc[k] = 0xffffffffu;
        h0.cmaxEnc[k] = 0u;
    }
    CR_CUDA(cudaMemcpy(ctr.p, &h0, sizeof(h0), cudaMemcpyHostToDevice));

    // 1. centroids, bounds, Morton presort
    prep(recA.p, ctr.p);
    CR_LAUNCH_CHECK();
    CR_CUDA(keysIn.alloc(N));
    CR_CUDA(keysOut.alloc(N));
    CR_CUDA(valsIn.alloc(N));
    CR_CUDA(valsOut.alloc(N));
    kMorton<<<blocksFor(N, 256), 256>>>(recA.p, N, ctr.p, keysIn.p, valsIn.p);
    CR_LAUNCH_CHECK();
    size_t tempBytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tempBytes, keysIn.p, keysOut.p, valsIn.p, valsOut.p, (int)N, 0, 30);
    DevBuf<uint8_t> temp;
    CR_CUDA(temp.alloc(tempBytes));
    CR_CUDA(cub::DeviceRadixSort::SortPairs(temp.p, tempBytes, keysIn.p, keysOut.p, valsIn.p, valsOut.p, (int)N, 0,
                                            30));
    countLaunch(4);
    kGather<<<blocksFor(N, 256), 256>>>(recA.p, valsOut.p, N, recB.p);
    CR_LAUNCH_CHECK();
    PrimRec* bufs[2] = {recB.p, recA.p};  // level 0 reads bufs[0]

    // 2. nodes, tasks
    const uint32_t maxNodes = 2 * N;
    DevBuf<BuildNode> nodes;
    CR_CUDA(nodes.alloc(maxNodes));
    const uint32_t capBig = N / kTile + 2;                   // tasks with > kTile prims per level
    const uint32_t capTiles = 2 * (N / kTile) + 4;           // ceil per task
    DevBuf<BigTask> bigA, bigB;
    DevBuf<Tile> tilesA, tilesB;
    DevBuf<uint32_t> bounds, bins, tileLeft, tilePrefix;
    DevBuf<SmallTask> small;
    CR_CUDA(bigA.alloc(capBig));
    CR_CUDA(bigB.alloc(capBig));
    CR_CUDA(tilesA.alloc(capTiles));
    CR_CUDA(tilesB.alloc(capTiles));
    CR_CUDA(bounds.alloc((size_t)capBig * 6));
    CR_CUDA(bins.alloc((size_t)capBig * kBinBlock));
    CR_CUDA(tileLeft.alloc(capTiles));
    CR_CUDA(tilePrefix.alloc(capTiles));
    CR_CUDA(small.alloc(N + 1));

    uint32_t nBig = 0, nTiles = 0, level = 0;
    if (N > kTile) {
        BigTask root;
        std::memset(&root, 0, sizeof(root));
        root.count = N;
        root.node = 0;
        root.nTiles = (N + kTile - 1) / kTile;
        CR_CUDA(cudaMemcpy(bigA.p, &root, sizeof(root), cudaMemcpyHostToDevice));
        std::vector<Tile> tl(root.nTiles);
        for (uint32_t j = 0; j < root.nTiles; j++) tl[j] = Tile{0, j * kTile, std::min((j + 1) * kTile, N), 0};
        CR_CUDA(cudaMemcpy(tilesA.p, tl.data(), tl.size() * sizeof(Tile), cudaMemcpyHostToDevice));
        nBig = 1;
        nTiles = root.nTiles;
    } else {
        SmallTask root{0, N, 0, 0, 0, {0, 0, 0}};
        CR_CUDA(cudaMemcpy(small.p, &root, sizeof(root), cudaMemcpyHostToDevice));
        uint32_t one = 1;
        CR_CUDA(cudaMemcpy(&ctr.p->small, &one, 4, cudaMemcpyHostToDevice));
    }
    BigTask* cur = bigA.p;
    BigTask* nxt = bigB.p;
    Tile* curT = tilesA.p;
    Tile* nxtT = tilesB.p;
    uint32_t curBuf = 0;
    while (nBig > 0) {
        const uint32_t dstBuf = curBuf ^ 1u;
        uint32_t zero3[3] = {0, 0, 0};
        CR_CUDA(cudaMemcpy(&ctr.p->nextBig, zero3, 8, cudaMemcpyHostToDevice));
        kBigInit<<<nBig, 256>>>(nBig, bounds.p, bins.p);
        CR_LAUNCH_CHECK();
        kBigBounds<<<nTiles, kTileThreads>>>(curT, bufs[curBuf], bounds.p);
        CR_LAUNCH_CHECK();
        kBigNode<<<blocksFor(nBig, 128), 128>>>(cur, nBig, level, bounds.p, nodes.p, ctr.p);
        CR_LAUNCH_CHECK();
        kBigBin<<<nTiles, kTileThreads>>>(curT, cur, bufs[curBuf], bounds.p, bins.p);
        CR_LAUNCH_CHECK();
        kBigSplit<<<blocksFor((uint64_t)nBig * 32, 128), 128>>>(cur, nBig, bounds.p, bins.p);
        CR_LAUNCH_CHECK();
        kBigCount<<<nTiles, kTileThreads>>>(curT, cur, bufs[curBuf], tileLeft.p);
        CR_LAUNCH_CHECK();
        kBigScan<<<blocksFor((uint64_t)nBig * 32, 128), 128>>>(cur, nBig, tileLeft.p, tilePrefix.p);
        CR_LAUNCH_CHECK();
        kBigScatter<<<nTiles, kTileThreads>>>(curT, cur, tilePrefix.p, bufs[curBuf], bufs[dstBuf]);
        CR_LAUNCH_CHECK();
        kBigChildren<<<blocksFor((uint64_t)nBig * 32, 128), 128>>>(cur, nBig, level, dstBuf, nodes.p, nxt, nxtT,
                                                                   small.p, ctr.p, capBig, capTiles, N + 1,
                                                                   maxNodes);
        CR_LAUNCH_CHECK();
        kBigFinalize<<<nTiles, kTileThreads>>>(curT, cur, bufs[curBuf], order.p);
        CR_LAUNCH_CHECK();
        Counters hc;
        CR_CUDA(cudaMemcpy(&hc, ctr.p, sizeof(hc), cudaMemcpyDeviceToHost));
        if (hc.overflow || hc.nextBig > capBig || hc.nextTiles > capTiles)
            return fail(CR_ERR_DEVICE, "BVH build: task capacity exceeded (%u / %u)", hc.nextBig, hc.nextTiles);
        nBig = hc.nextBig;
        nTiles = hc.nextTiles;
        std::swap(cur, nxt);
        std::swap(curT, nxtT);
        curBuf = dstBuf;
        level++;
    }
    Counters hc;
    CR_CUDA(cudaMemcpy(&hc, ctr.p, sizeof(hc), cudaMemcpyDeviceToHost));
    if (hc.small > 0) {
        kSubtree<<<blocksFor(hc.small, kSubtreeWarps), kSubtreeWarps * 32>>>(small.p, hc.small, bufs[0], bufs[1],
                                                                            nodes.p, order.p, ctr.p, maxNodes);
        CR_LAUNCH_CHECK();
    }
    CR_CUDA(cudaMemcpy(&hc, ctr.p, sizeof(hc), cudaMemcpyDeviceToHost));
    const uint32_t nNodes = hc.nodes;
    if (hc.overflow || nNodes > maxNodes) return fail(CR_ERR_DEVICE, "BVH build: node count %u exceeds %u", nNodes, maxNodes);

    // 3. traversal layout
    DevBuf<uint32_t> isLeaf, leafPrefix;
    CR_CUDA(isLeaf.alloc(nNodes));
    CR_CUDA(leafPrefix.alloc(nNodes));
    kLeafFlags<<<blocksFor(nNodes, 256), 256>>>(nodes.p, nNodes, isLeaf.p);
    CR_LAUNCH_CHECK();
    size_t scanBytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, isLeaf.p, leafPrefix.p, (int)nNodes);
    DevBuf<uint8_t> scanTemp;
    CR_CUDA(scanTemp.alloc(scanBytes));
    CR_CUDA(cub::DeviceScan::ExclusiveSum(scanTemp.p, scanBytes, isLeaf.p, leafPrefix.p, (int)nNodes));
    countLaunch(1);
    const uint32_t nLeaves = hc.leafCount;
    if (nLeaves > ~(kLeafBit | kInlineLeafBit))  // leaf-table refs have 30 index bits
        return fail(CR_ERR_UNSUPPORTED, "BVH has %u leaves; the limit is 2^30-1", nLeaves);
    const uint32_t nPairs = nNodes - nLeaves;
    DevBuf<NodePair> pairs;
    DevBuf<uint2> leaves;
    CR_CUDA(pairs.alloc(nPairs));
    CR_CUDA(leaves.alloc(nLeaves));
    kLayout<<<blocksFor(nNodes, 256), 256>>>(nodes.p, nNodes, leafPrefix.p, pairs.p, leaves.p);
    CR_LAUNCH_CHECK();
    CR_CUDA(cudaMemcpy(&out.root, nodes.p, sizeof(BuildNode), cudaMemcpyDeviceToHost));
    out.pairs = pairs.release();
    out.nPairs = nPairs;
    out.leaves = leaves.release();
    out.nLeaves = nLeaves;
    out.order = order.release();
    out.nodes = nodes.release();
    out.nNodes = nNodes;
    out.levels = level;
    out.counters = hc;
    return CR_OK;
}

void freeBuilt(BuiltBvh& b) {
    void* ptrs[] = {b.pairs, b.leaves, b.order, b.nodes};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    b = BuiltBvh{};
}

}  // namespace

int buildBvh(cr_scene* s) {
    const uint32_t N = (uint32_t)s->nt;
    s->hasRoot = 0;
    s->stats = cr_bvh_stats{};
    if (N == 0) return CR_OK;
    if (s->nt >= 0x7fffffffull) return fail(CR_ERR_UNSUPPORTED, "scene has %llu triangles; the limit is 2^31-1",
                                            (unsigned long long)s->nt);
    cudaEvent_t e0, e1;
    CR_CUDA(cudaEventCreate(&e0));
    CR_CUDA(cudaEventCreate(&e1));
    CR_CUDA(cudaEventRecord(e0, 0));
    BuiltBvh b;
    const float3* pos = s->pos;
    const uint32_t* idx = s->idx;
    int rc = buildGeneric(N, [&](PrimRec* rec, Counters* ctr) {
        kPrep<<<blocksFor(N, 256), 256>>>(pos, idx, N, rec, ctr);
    }, b);
    if (rc) {
        freeBuilt(b);
        return rc;
    }
    DevBuf<TriBlock> tris;
    CR_CUDA(tris.alloc(N));
    kTriBlocks<<<blocksFor(N, 256), 256>>>(s->pos, s->idx, b.order, N, tris.p);
    CR_LAUNCH_CHECK();
    CR_CUDA(cudaEventRecord(e1, 0));
    CR_CUDA(cudaEventSynchronize(e1));
    float ms = 0.0f;
    CR_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);

    const BuildNode& root = b.root;
    s->pairs = b.pairs;
    s->nPairs = b.nPairs;
    s->leaves = b.leaves;
    s->nLeaves = b.nLeaves;
    s->tris = tris.release();
    s->slotToPrim = b.order;
    s->buildNodes = b.nodes;
    s->nBuildNodes = b.nNodes;
    s->hasRoot = 1;
    s->rootMin = mk3(root.lo.x, root.lo.y, root.lo.z);
    s->rootMax = mk3(root.hi.x, root.hi.y, root.hi.z);
    s->rootFlags = degenerateFlags(s->rootMin, s->rootMax);
    s->rootRef = root.info.z ? kLeafBit : 0u;

    const Counters& hc = b.counters;
    cr_bvh_stats& st = s->stats;
    st.node_count = b.nNodes;
    st.leaf_count = b.nLeaves;
    st.max_depth = hc.maxDepth;
    st.max_leaf_size = hc.maxLeafSize;
    st.max_leaf_depth = hc.maxLeafDepth;
    st.levels = b.levels;
    st.root_min[0] = root.lo.x;
    st.root_min[1] = root.lo.y;
    st.root_min[2] = root.lo.z;
    st.root_max[0] = root.hi.x;
    st.root_max[1] = root.hi.y;
    st.root_max[2] = root.hi.z;
    st.build_ms = ms;
    st.device_bytes = (uint64_t)b.nPairs * sizeof(NodePair) + (uint64_t)b.nLeaves * sizeof(uint2) +
                      (uint64_t)N * sizeof(TriBlock);
    return CR_OK;
}

// The sphere BVH over s->sphGeom (s->nSph spheres), replacing any earlier one.
int buildSphereBvh(cr_scene* s) {
    void* old[] = {s->sphPairs, s->sphLeaves, s->sphBlocks};
    for (void* p : old)
        if (p) cudaFree(p);
    s->sphPairs = nullptr;
    s->sphLeaves = nullptr;
    s->sphBlocks = nullptr;
    s->sphHasRoot = 0;
    const uint32_t N = s->nSph;
    if (N == 0) return CR_OK;
    BuiltBvh b;
    const float4* geom = s->sphGeom;
    int rc = buildGeneric(N, [&](PrimRec* rec, Counters* ctr) {
        kPrepSpheres<<<blocksFor(N, 256), 256>>>(geom, N, rec, ctr);
    }, b);
    if (rc) {
        freeBuilt(b);
        return rc;
    }
    DevBuf<SphereBlock> blocks;
    CR_CUDA(blocks.alloc(N));
    kSphereBlocks<<<blocksFor(N, 256), 256>>>(geom, b.order, N, blocks.p);
    CR_LAUNCH_CHECK();
    CR_CUDA(cudaDeviceSynchronize());
    s->sphPairs = b.pairs;
    s->sphLeaves = b.leaves;
    s->sphBlocks = blocks.release();
    cudaFree(b.order);
    cudaFree(b.nodes);
    const BuildNode& root = b.root;
    s->sphRootMin = mk3(root.lo.x, root.lo.y, root.lo.z);
    s->sphRootMax = mk3(root.hi.x, root.hi.y, root.hi.z);
    s->sphRootFlags = degenerateFlags(s->sphRootMin, s->sphRootMax);
    s->sphRootRef = root.info.z ? kLeafBit : 0u;
    s->sphHasRoot = 1;
    return CR_OK;
}

int exportBvh(const cr_scene* s, cr_bvh_node* out, uint32_t* primMap) {
    if (!s->hasRoot) return CR_OK;
    std::vector<BuildNode> nodes(s->nBuildNodes);
    CR_CUDA(cudaMemcpy(nodes.data(), s->buildNodes, nodes.size() * sizeof(BuildNode), cudaMemcpyDeviceToHost));
    if (primMap) CR_CUDA(cudaMemcpy(primMap, s->slotToPrim, s->nt * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (!out) return CR_OK;
    // post-order numbering, left subtree first (Core/BVH.cu:199-211)
    std::vector<uint32_t> post(nodes.size(), 0xffffffffu);
    struct Frame {
        uint32_t node;
        uint32_t state;
    };
    std::vector<Frame> st;
    st.push_back({0, 0});
    uint32_t next = 0;
    while (!st.empty()) {
        Frame& f = st.back();
        const BuildNode& n = nodes[f.node];
        if (n.info.z || f.state == 2) {
            post[f.node] = next++;
            st.pop_back();
            continue;
        }
        uint32_t child = f.state == 0 ? n.info.x : n.info.y;
        f.state++;
        st.push_back({child, 0});
    }
    for (uint32_t i = 0; i < nodes.size(); i++) {
        const BuildNode& n = nodes[i];
        if (post[i] == 0xffffffffu) continue;
        cr_bvh_node& o = out[post[i]];
        o.bmin[0] = n.lo.x;
        o.bmin[1] = n.lo.y;
        o.bmin[2] = n.lo.z;
        o.bmax[0] = n.hi.x;
        o.bmax[1] = n.hi.y;
        o.bmax[2] = n.hi.z;
        o.is_leaf = n.info.z;
        o.a = n.info.z ? n.info.x : post[n.info.x];
        o.b = n.info.z ? n.info.y : post[n.info.y];
    }
    return CR_OK;
}

}  // namespace cr

namespace cr {

// Replaces the scene's triangle BVH with a tree given in the reference's
// layout (BVHData, Core/BVH.h:17-30, as BVH::createFinalBVH fills it,
// Core/BVH.cu:303-338): nodes in any order with the root last, interior
// children by index, leaves as (first slot, count) ranges of primMap, which
// maps each of the n_tris leaf slots to a triangle.  The tree is checked
// (every index in range, every node reached once from the root, depth within
// the traversal stack), renumbered breadth-first and laid out as NodePairs
// and triangle blocks like a built tree; traversal then visits it in the
// reference's order with the reference's culling.
int importBvh(cr_scene* s, const cr_bvh_node* in, uint32_t nodeCount, const uint32_t* primMap) {
    if (s->nt == 0) {
        if (nodeCount) return fail(CR_ERR_INVALID_ARGUMENT, "the scene has no triangles; pass node_count 0");
        return CR_OK;
    }
    if (!in || nodeCount == 0 || !primMap) return fail(CR_ERR_INVALID_ARGUMENT, "nodes / prim_map is NULL or empty");
    const uint64_t nSlots = s->nt;
    for (uint64_t i = 0; i < nSlots; i++)
        if (primMap[i] >= s->nt)
            return fail(CR_ERR_INVALID_ARGUMENT, "prim_map[%llu] = %u is not a triangle", (unsigned long long)i,
                        primMap[i]);
    // breadth-first renumbering from the root (the last node), with checks
    std::vector<uint32_t> order;  // new index -> input index
    std::vector<uint32_t> depth;
    std::vector<uint8_t> seen(nodeCount, 0);
    order.reserve(nodeCount);
    order.push_back(nodeCount - 1);
    depth.push_back(0);
    seen[nodeCount - 1] = 1;
    uint32_t maxDepth = 0, maxLeafDepth = 0, maxLeafSize = 0, nLeaves = 0;
    for (size_t k = 0; k < order.size(); k++) {
        const cr_bvh_node& n = in[order[k]];
        if (n.is_leaf > 1) return fail(CR_ERR_INVALID_ARGUMENT, "node %u: is_leaf = %u", order[k], n.is_leaf);
        if (n.is_leaf) {
            if ((uint64_t)n.a + n.b > nSlots)
                return fail(CR_ERR_INVALID_ARGUMENT, "leaf %u: slots %u + %u run past the %llu slots", order[k], n.a,
                            n.b, (unsigned long long)nSlots);
            nLeaves++;
            maxLeafSize = std::max(maxLeafSize, n.b);
            maxLeafDepth = std::max(maxLeafDepth, depth[k]);
            continue;
        }
        maxDepth = std::max(maxDepth, depth[k]);
        // a near-first traversal holds at most one pushed entry per level
        // above the current node, so pushing at an interior node of depth d
        // needs d + 1 stack entries
        if (depth[k] + 1 > (uint32_t)kStackSize)
            return fail(CR_ERR_UNSUPPORTED,
                        "node %u is an interior node at depth %u; the %d-entry traversal stack holds depths up to %d",
                        order[k], depth[k], kStackSize, kStackSize - 1);
        for (uint32_t c : {n.a, n.b}) {
            if (c >= nodeCount) return fail(CR_ERR_INVALID_ARGUMENT, "node %u: child %u of %u", order[k], c, nodeCount);
            if (seen[c]) return fail(CR_ERR_INVALID_ARGUMENT, "node %u is reached twice (not a tree)", c);
            seen[c] = 1;
            order.push_back(c);
            depth.push_back(depth[k] + 1);
        }
    }
    if (order.size() != nodeCount)
        return fail(CR_ERR_INVALID_ARGUMENT, "%u of %u nodes are not reached from the root (node %u)",
                    (uint32_t)(nodeCount - order.size()), nodeCount, nodeCount - 1);
    if (nLeaves > ~(kLeafBit | kInlineLeafBit)) return fail(CR_ERR_UNSUPPORTED, "%u leaves", nLeaves);
    std::vector<uint32_t> newIndex(nodeCount);
    for (uint32_t k = 0; k < nodeCount; k++) newIndex[order[k]] = k;
    std::vector<BuildNode> nodes(nodeCount);
    std::vector<uint32_t> leafPrefix(nodeCount);
    uint32_t leavesBefore = 0;
    for (uint32_t k = 0; k < nodeCount; k++) {
        const cr_bvh_node& n = in[order[k]];
        BuildNode& b = nodes[k];
        b.lo = make_float4(n.bmin[0], n.bmin[1], n.bmin[2], 0.0f);
        b.hi = make_float4(n.bmax[0], n.bmax[1], n.bmax[2], 0.0f);
        b.info = n.is_leaf ? make_uint4(n.a, n.b, 1u, depth[k]) : make_uint4(newIndex[n.a], newIndex[n.b], 0u, depth[k]);
        leafPrefix[k] = leavesBefore;
        leavesBefore += n.is_leaf;
    }
    const uint32_t nPairs = nodeCount - nLeaves;
    std::vector<NodePair> pairs(std::max<uint32_t>(nPairs, 1));
    std::vector<uint2> leaves(std::max<uint32_t>(nLeaves, 1));
    for (uint32_t k = 0; k < nodeCount; k++) {
        if (nodes[k].info.z) leaves[leafPrefix[k]] = make_uint2(nodes[k].info.x, nodes[k].info.y);
        else pairs[k - leafPrefix[k]] = pairOf(nodes.data(), leafPrefix.data(), k);
    }
    DevBuf<NodePair> dPairs;
    DevBuf<uint2> dLeaves;
    DevBuf<BuildNode> dNodes;
    DevBuf<uint32_t> dOrder;
    DevBuf<TriBlock> dTris;
    CR_CUDA(dPairs.alloc(nPairs));
    CR_CUDA(dLeaves.alloc(nLeaves));
    CR_CUDA(dNodes.alloc(nodeCount));
    CR_CUDA(dOrder.alloc(nSlots));
    CR_CUDA(dTris.alloc(nSlots));
    CR_CUDA(cudaMemcpy(dPairs.p, pairs.data(), (size_t)nPairs * sizeof(NodePair), cudaMemcpyHostToDevice));
    CR_CUDA(cudaMemcpy(dLeaves.p, leaves.data(), (size_t)nLeaves * sizeof(uint2), cudaMemcpyHostToDevice));
    CR_CUDA(cudaMemcpy(dNodes.p, nodes.data(), (size_t)nodeCount * sizeof(BuildNode), cudaMemcpyHostToDevice));
    CR_CUDA(cudaMemcpy(dOrder.p, primMap, nSlots * sizeof(uint32_t), cudaMemcpyHostToDevice));
    kTriBlocks<<<blocksFor(nSlots, 256), 256>>>(s->pos, s->idx, dOrder.p, (uint32_t)nSlots, dTris.p);
    CR_LAUNCH_CHECK();
    CR_CUDA(cudaDeviceSynchronize());
    // the new tree is complete: drop the old one (cudaFree waits for queries still using it)
    void* old[] = {s->pairs, s->leaves, s->tris, s->slotToPrim, s->buildNodes, s->groupPairs};
    for (void* p : old)
        if (p) cudaFree(p);
    s->groupPairs = nullptr;
    const BuildNode& root = nodes[0];
    s->pairs = dPairs.release();
    s->nPairs = nPairs;
    s->leaves = dLeaves.release();
    s->nLeaves = nLeaves;
    s->tris = dTris.release();
    s->slotToPrim = dOrder.release();
    s->buildNodes = dNodes.release();
    s->nBuildNodes = nodeCount;
    s->rootMin = mk3(root.lo.x, root.lo.y, root.lo.z);
    s->rootMax = mk3(root.hi.x, root.hi.y, root.hi.z);
    s->rootFlags = degenerateFlags(s->rootMin, s->rootMax);
    s->rootRef = root.info.z ? kLeafBit : 0u;
    s->hasRoot = 1;
    cr_bvh_stats& st = s->stats;
    st = cr_bvh_stats{};
    st.node_count = nodeCount;
    st.leaf_count = nLeaves;
    st.max_depth = maxDepth;
    st.max_leaf_size = maxLeafSize;
    st.max_leaf_depth = maxLeafDepth;
    st.levels = 0;
    for (int k = 0; k < 3; k++) {
        st.root_min[k] = k == 0 ? root.lo.x : (k == 1 ? root.lo.y : root.lo.z);
        st.root_max[k] = k == 0 ? root.hi.x : (k == 1 ? root.hi.y : root.hi.z);
    }
    st.build_ms = 0.0;
    st.device_bytes = (uint64_t)nPairs * sizeof(NodePair) + (uint64_t)nLeaves * sizeof(uint2) + nSlots * sizeof(TriBlock);
    return s->traversal == CR_TRAVERSAL_TWO_LEVEL ? buildGroupedPairs(s) : CR_OK;
}

// The scene's pairs again, laid out in two-level groups for the two-level
// step: from the kept build records (breadth-first, depths included), with
// the same leaf table.  Replaces an earlier grouped copy.
int buildGroupedPairs(cr_scene* s) {
    if (s->groupPairs) cudaFree(s->groupPairs);
    s->groupPairs = nullptr;
    s->groupRootRef = s->rootRef;
    if (!s->hasRoot || s->nPairs == 0) return CR_OK;  // a leaf root: nothing to group
    if (s->nPairs > kMaxPairs)
        return fail(CR_ERR_UNSUPPORTED, "the two-level step takes at most 2^28 interior nodes (the tree has %u)",
                    s->nPairs);
    const uint32_t n = s->nBuildNodes;
    DevBuf<uint32_t> isLeaf, leafPrefix, group, groupStart, rootRef;
    CR_CUDA(isLeaf.alloc(n));
    CR_CUDA(leafPrefix.alloc(n));
    CR_CUDA(group.alloc(n));
    CR_CUDA(groupStart.alloc(n));
    CR_CUDA(rootRef.alloc(1));
    kGroupFlags<<<blocksFor(n, 256), 256>>>(s->buildNodes, n, isLeaf.p, group.p);
    CR_LAUNCH_CHECK();
    size_t scanBytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, isLeaf.p, leafPrefix.p, (int)n);
    DevBuf<uint8_t> scanTemp;
    CR_CUDA(scanTemp.alloc(scanBytes));
    CR_CUDA(cub::DeviceScan::ExclusiveSum(scanTemp.p, scanBytes, isLeaf.p, leafPrefix.p, (int)n));
    CR_CUDA(cub::DeviceScan::ExclusiveSum(scanTemp.p, scanBytes, group.p, groupStart.p, (int)n));
    countLaunch(2);
    DevBuf<NodePair> pairs;
    CR_CUDA(pairs.alloc(s->nPairs));
    kGroupLayout<<<blocksFor(n, 256), 256>>>(s->buildNodes, n, leafPrefix.p, groupStart.p, pairs.p, rootRef.p);
    CR_LAUNCH_CHECK();
    uint32_t rr = 0;
    CR_CUDA(cudaMemcpy(&rr, rootRef.p, sizeof(rr), cudaMemcpyDeviceToHost));
    s->groupPairs = pairs.release();
    s->groupRootRef = rr;
    return CR_OK;
}

}  // namespace cr
