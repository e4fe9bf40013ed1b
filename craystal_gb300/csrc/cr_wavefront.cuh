// cr_wavefront.cuh -- the wavefront variant of pathTraceKernel<useMIS>
// (Core/Integrator.cu:142-227): paths live in HBM between bounces and each
// bounce is three launches over the live paths,
//   extend   the closest-hit query of every live path (a pure traversal
//            kernel), with the hit's material as a sort key;
//   sort     the live paths by material (a counting sort: block-aggregated
//            histogram, scan, block-aggregated scatter), so that the warps of
//            the shade stage run one BSDF and touch one material's data;
//   shade    the bounce after the query (shadeBounce, the megakernel's own
//            code: next-event estimation and MIS with their shadow and BSDF
//            rays, continuation sampling, Russian roulette); surviving paths
//            are appended to the next bounce's queue, ending paths go to the
//            integrator's Mode (the plain tracer splats them into the film,
//            cr_wavefront.cu; the cached one records them, cr_cache.cu).
// Per path the arithmetic and the sampler's sequence are the megakernel's,
// so the plain film equals cr_render's up to the order of its float adds.
//
// Path state (structure of arrays, 16-byte records):
//   ro    (origin, film x)        rd    (direction, film y)
//   beta  (throughput, depth)     rad   (radiance, 0)
//   meta  (x, y, sample index, sampler state)   inc (sampler increment)
//   hit   (prim, t, u, v) of the extend stage
//   aux   per-path state of the Mode's hooks
// Paths run in waves of at most kWaveCap (the whole image x spp when it
// fits), 132 bytes each.  Every stage reads the live-path count from device
// memory, so a render is a fixed sequence of launches on one stream: no
// host synchronisation, and it can be captured into a CUDA graph.

#pragma once

#include "cr_internal.cuh"
#include "cr_math.cuh"
#include "cr_path.cuh"
#include "cr_shading.cuh"
#include "cr_tile.cuh"
#include "cr_traverse.cuh"

namespace cr {

// Path state and queues, kept with the scene and grown on demand.
struct WfBuffers {
    uint32_t cap = 0, keyCap = 0;
    float4 *ro = nullptr, *rd = nullptr, *beta = nullptr, *rad = nullptr, *hit = nullptr;
    uint4 *meta = nullptr, *aux = nullptr;
    uint32_t *inc = nullptr, *item = nullptr, *qa = nullptr, *qb = nullptr, *keys = nullptr, *sorted = nullptr,
             *counts = nullptr, *hist = nullptr;
    void release() {
        void* ptrs[] = {ro, rd, beta, rad, hit, meta, aux, inc, item, qa, qb, keys, sorted, counts, hist};
        for (void* q : ptrs)
            if (q) cudaFree(q);
        *this = WfBuffers{};
    }
};

template <class T>
inline cudaError_t wfAlloc(T*& p, size_t n) {
    return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
}

inline int ensureWavefrontBuffers(void*& slot, uint32_t cap, uint32_t nKeys, WfBuffers*& out) {
    WfBuffers* b = static_cast<WfBuffers*>(slot);
    if (!b) {
        b = new WfBuffers;
        slot = b;
    }
    if (b->cap < cap || b->keyCap < nKeys) {
        CR_CUDA(cudaDeviceSynchronize());  // earlier renders may still use the old buffers
        b->release();
        CR_CUDA(wfAlloc(b->ro, cap));
        CR_CUDA(wfAlloc(b->rd, cap));
        CR_CUDA(wfAlloc(b->beta, cap));
        CR_CUDA(wfAlloc(b->rad, cap));
        CR_CUDA(wfAlloc(b->hit, cap));
        CR_CUDA(wfAlloc(b->meta, cap));
        CR_CUDA(wfAlloc(b->aux, cap));
        CR_CUDA(wfAlloc(b->inc, cap));
        CR_CUDA(wfAlloc(b->item, cap));
        CR_CUDA(wfAlloc(b->qa, cap));
        CR_CUDA(wfAlloc(b->qb, cap));
        CR_CUDA(wfAlloc(b->keys, cap));
        CR_CUDA(wfAlloc(b->sorted, cap));
        CR_CUDA(wfAlloc(b->counts, 4));  // live paths, next queue, extension and shade fetch counters
        CR_CUDA(wfAlloc(b->hist, nKeys));
        b->cap = cap;
        b->keyCap = nKeys;
    }
    out = b;
    return CR_OK;
}

namespace {


// Waves of up to 2^26 paths (8.8 GB of path state).  Every wave ends with a
// tail of bounces in which few paths are left and most SMs idle, so fewer,
// larger waves render faster: on GB300, 2^21 / 2^23 / 2^25 / 2^26-path waves
// take 0.42 / 0.24 / 0.195 / 0.187 s for 1920x1080 at 64 spp (depth 16) and
// 2.19 / 1.19 / 0.83 / 0.77 s for 3840x2160 at 32 spp.  A render whose path
// state cannot be allocated halves its wave, down to kWaveCapMin.
constexpr uint32_t kWaveCap = 1u << 26;
constexpr uint32_t kWaveCapMin = 1u << 20;
constexpr int kWfThreads = 128;

// Path state for waves of up to `want` paths, halving the wave while the
// allocation fails; cap receives the wave size in use.
inline int ensureWavefrontWave(void*& slot, uint64_t want, uint32_t nKeys, WfBuffers*& out, uint32_t& cap) {
    cap = (uint32_t)std::min<uint64_t>(want, kWaveCap);
    while (true) {
        const int rc = ensureWavefrontBuffers(slot, cap, nKeys, out);
        if (rc != CR_ERR_OUT_OF_MEMORY || cap <= kWaveCapMin) return rc;
        (void)cudaGetLastError();  // a failed allocation leaves no sticky error
        static_cast<WfBuffers*>(slot)->release();
        cap /= 2;
    }
}

struct WfState {
    float4* ro;
    float4* rd;
    float4* beta;
    float4* rad;
    uint4* meta;
    uint32_t* inc;
    float4* hit;
    uint4* aux;       // per-path state of the integrator's hooks
    uint32_t* item;   // the path's scene (many-scene sources)
};

// Rays traced by each lane, added to its scene's counter: one atomic per
// group of lanes with the same counter.
__device__ __forceinline__ void addRays(unsigned long long* counter, uint32_t rays) {
    const unsigned act = __activemask();
    const unsigned grp = __match_any_sync(act, (unsigned long long)counter);
    const uint32_t sum = __reduce_add_sync(grp, rays);
    if ((int)(threadIdx.x & 31) == __ffs(grp) - 1 && sum) atomicAdd(counter, (unsigned long long)sum);
}

// What a wave renders.  A source maps path g of its sequence to a scene
// (item), a pixel and a sample index, and gives each item's scene, camera,
// integrator parameters, film and key range of the material sort.
//
// One scene: path g is pixel g mod (w h) at sample p.first + g / (w h).
struct OneScene {
    // 96 registers: spills a little, 2 % faster than 4 blocks of 128; 6, 7 and
    // 8 blocks (80, 72, 64 registers) measured within 1 % of 5
    static constexpr int kShadeMinBlocks = 5;
    static constexpr bool kAllowLean = true;   // its shade stage has a lean form (kFullScene = false)
    SceneView view;
    CameraGpu cam;
    Params p;
    float* filmRgb;
    float* filmW;
    unsigned long long* rayCounter;
    uint32_t nMats;
    __device__ __forceinline__ const SceneView& sceneOf(uint32_t) const { return view; }
    __device__ __forceinline__ const CameraGpu& camOf(uint32_t) const { return cam; }
    __device__ __forceinline__ const Params& paramsOf(uint32_t) const { return p; }
    __device__ __forceinline__ float* filmRgbOf(uint32_t) const { return filmRgb; }
    __device__ __forceinline__ float* filmWOf(uint32_t) const { return filmW; }
    __device__ __forceinline__ unsigned long long* raysOf(uint32_t) const { return rayCounter; }
    __device__ __forceinline__ uint32_t keyBase(uint32_t) const { return 0u; }
    __device__ __forceinline__ uint32_t nMatsOf(uint32_t) const { return nMats; }
    __device__ __forceinline__ void locate(uint64_t g, uint32_t& item, uint32_t& x, uint32_t& y,
                                           uint32_t& si) const {
        const uint64_t area = (uint64_t)cam.width * cam.height;
        const uint32_t px = (uint32_t)(g % area);
        item = 0;
        x = px % cam.width;
        y = px / cam.width;
        si = p.first + (uint32_t)(g / area);
    }
};

// One scene of a many-scene source; its paths are [pathBase, pathBase +
// width * height * p.spp) of the source's sequence, its sort keys
// [keyBase, keyBase + nMats + 2).
struct __align__(16) WfScene {
    SceneView view;
    CameraGpu cam;
    Params p;
    float* filmRgb;
    float* filmW;
    unsigned long long* rayCounter;
    uint64_t pathBase;
    uint32_t keyBase, nMats;
};

struct ManyScenes {
    // 128 registers: it spills there, but 3 blocks of 168 measured 10 % slower
    static constexpr int kShadeMinBlocks = 4;
    static constexpr bool kAllowLean = false;
    const WfScene* scenes;
    uint32_t n;
    __device__ __forceinline__ const SceneView& sceneOf(uint32_t i) const { return scenes[i].view; }
    __device__ __forceinline__ const CameraGpu& camOf(uint32_t i) const { return scenes[i].cam; }
    __device__ __forceinline__ const Params& paramsOf(uint32_t i) const { return scenes[i].p; }
    __device__ __forceinline__ float* filmRgbOf(uint32_t i) const { return scenes[i].filmRgb; }
    __device__ __forceinline__ float* filmWOf(uint32_t i) const { return scenes[i].filmW; }
    __device__ __forceinline__ unsigned long long* raysOf(uint32_t i) const { return scenes[i].rayCounter; }
    __device__ __forceinline__ uint32_t keyBase(uint32_t i) const { return scenes[i].keyBase; }
    __device__ __forceinline__ uint32_t nMatsOf(uint32_t i) const { return scenes[i].nMats; }
    __device__ __forceinline__ void locate(uint64_t g, uint32_t& item, uint32_t& x, uint32_t& y,
                                           uint32_t& si) const {
        uint32_t lo = 0, hi = n - 1;  // the last scene whose pathBase <= g
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) / 2;
            if (scenes[mid].pathBase <= g) lo = mid;
            else hi = mid - 1;
        }
        item = lo;
        const WfScene& s = scenes[lo];
        const uint64_t k = g - s.pathBase;
        const uint64_t area = (uint64_t)s.cam.width * s.cam.height;
        const uint32_t px = (uint32_t)(k % area);
        x = px % s.cam.width;
        y = px / s.cam.width;
        si = s.p.first + (uint32_t)(k / area);
    }
};

// Camera rays of paths [base, base + n) of the source's sequence.
//
// With waveBase set, the wave starts at *waveBase and holds min(n, total -
// *waveBase) paths (a wave graph replayed over a long sequence).
__device__ __forceinline__ uint32_t waveSize(uint64_t& base, uint32_t n, const uint64_t* waveBase, uint64_t total) {
    if (!waveBase) return n;
    base = *waveBase;
    if (base >= total) return 0u;
    const uint64_t left = total - base;
    return left < (uint64_t)n ? (uint32_t)left : n;
}

template <class Src>
__global__ void __launch_bounds__(kWfThreads) kWfInit(const __grid_constant__ Src src, WfState st, uint64_t base,
                                                      uint32_t n, const uint64_t* __restrict__ waveBase,
                                                      uint64_t total) {
    n = waveSize(base, n, waveBase, total);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t item, x, y, si;
    src.locate(base + i, item, x, y, si);
    Sampler smp(x, y, si);
    float2 pix;
    float3 ro, rd;
    cameraRay(src.camOf(item), smp, x, y, pix, ro, rd);
    st.ro[i] = make_float4(ro.x, ro.y, ro.z, pix.x);
    st.rd[i] = make_float4(rd.x, rd.y, rd.z, pix.y);
    st.beta[i] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(0u));
    st.rad[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    st.meta[i] = make_uint4(x, y, si, smp.state);
    st.inc[i] = smp.inc;
    st.aux[i] = make_uint4(CR_MISS, CR_MISS, 0u, 0u);
    st.item[i] = item;
}

// The closest-hit query of every live path; key = the scene's key base plus
// the material to shade (nMats for a miss, nMats + 1 for a sphere light).
//
// Persistent blocks with dynamic fetch: the lanes of a warp take queue
// entries from counts[2] (zeroed by the kernel before) as they finish, at
// least kWfRefill at a time (checked every kWfSteps traversal steps), so
// that a warp keeps most lanes busy until the queue runs out instead of
// waiting for its slowest ray: 10 % faster on a 500k-triangle box clutter.  Each query is the
// closest() of the megakernel: the analytic-sphere BVH first (run whole when
// the scene has one), then the triangle BVH one cursor step per round, then
// the sphere lights; only the lane that carries a path changes.
// Refill at 8 idle lanes, 4 steps per round: the best of refill 4 / 8 / 16
// and 1 / 2 / 4 / 8 steps on the 2.6M-triangle 1080p scene (0.134 s against
// 0.136-0.141 s), and within 1 % of the best on the Cornell box.
constexpr int kWfRefill = 8;
constexpr int kWfSteps = 4;

template <class Src>
__global__ void __launch_bounds__(kWfThreads) kWfExtend(const __grid_constant__ Src src, WfState st,
                                                        const uint32_t* __restrict__ queue,
                                                        uint32_t* __restrict__ counts,
                                                        uint32_t* __restrict__ keys) {
    static_assert(kWfThreads == kStackBlock, "the extension query keeps the top of its stack in shared memory");
    __shared__ SharedStackArea stk;
    const uint32_t n = counts[0];
    if (blockIdx.x * blockDim.x >= n) return;  // more blocks than the queue needs (uniform per block)
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    TravStack<kSharedStack> stack;
    stack.sh = stk;
    TravState cur;
    TRay r;
    THit h;
    bool active = false, exhausted = false;
    uint32_t i = 0, k = 0, item = 0;
    // rays traced and not yet added to the counter of scene rayItem
    uint32_t pending = 0, rayItem = 0;
    auto finish = [&]() {
        const SceneView& sc = src.sceneOf(item);
        for (uint32_t q = 0; q < sc.nSpheres; q++) {
            const float t = raySphere(r.o, r.d, __ldg(sc.spheres + q), 0.0f, h.t);
            if (t < h.t) {
                h.t = t;
                h.prim = kSpherePrim + q;
            }
        }
        st.hit[k] = make_float4(__uint_as_float(h.prim), h.t, h.u, h.v);
        const uint32_t nMats = src.nMatsOf(item);
        uint32_t key;
        if (h.prim == CR_MISS) key = nMats;
        else if (h.prim >= kSpherePrim) key = nMats + 1;
        else if (isSphereHit(h.prim)) key = __ldg(sc.sphMat + (h.prim & ~kSphereBit));
        else key = sc.meshes[sc.primToMesh[h.prim]].material_id;
        keys[i] = src.keyBase(item) + key;
    };
    while (true) {
        const unsigned idle = __ballot_sync(full, !active);
        if (!exhausted && __popc(idle) >= kWfRefill) {
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(counts + 2, (uint32_t)__popc(idle));
            base = __shfl_sync(full, base, leader);
            if (base + (uint32_t)__popc(idle) >= n) exhausted = true;
            if (!active) {
                i = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (i < n) {
                    k = queue[i];
                    item = st.item[k];
                    if (item != rayItem) {
                        if (pending) atomicAdd(src.raysOf(rayItem), (unsigned long long)pending);
                        pending = 0;
                        rayItem = item;
                    }
                    pending++;
                    const SceneView& sc = src.sceneOf(item);
                    const float4 o = st.ro[k], d = st.rd[k];
                    r = makeTRay(mk3(o.x, o.y, o.z), 0.0f, mk3(d.x, d.y, d.z), INFINITY);
                    h.t = INFINITY;
                    h.prim = CR_MISS;
                    h.u = h.v = 0.0f;
                    if (sc.sph.hasRoot) traverseSpheres<false, kSharedStack>(sc, r, h, stk);
                    const BvhView bv{sc.pairs, sc.leaves, sc.rootRef, sc.rootFlags, sc.rootMin, sc.rootMax, sc.hasRoot};
                    if (travBegin(cur, bv, r)) active = true;
                    else finish();
                }
            }
        }
        if (!__any_sync(full, active)) {
            if (exhausted) break;
            continue;  // every lane idle: the next round refills all 32
        }
        // kWfSteps steps per refill round: the vote costs less than a step
        // here, where paths traverse shorter than the ray cast's rays
#pragma unroll 1
        for (int j = 0; j < kWfSteps; j++) {
            if (active) {
                const SceneView& sc = src.sceneOf(item);
                const BvhView bv{sc.pairs, sc.leaves, sc.rootRef, sc.rootFlags, sc.rootMin, sc.rootMax, sc.hasRoot};
                const TriLeaf<false> leaf{sc.tris};
                if (!travStep<false>(cur, stack, bv, sc.errFlags, leaf, r, h)) {
                    finish();
                    active = false;
                }
            }
        }
    }
    addRays(src.raysOf(rayItem), pending);
}

// Resident blocks of kernel K across the current device's SMs (cached per
// kernel and device ordinal; host threads that both ask store the same
// value).
constexpr int kWfOccDevices = 64;
template <auto K>
unsigned residentBlocks() {
    static std::atomic<int> occ[kWfOccDevices];
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int o = dev >= 0 && dev < kWfOccDevices ? occ[dev].load(std::memory_order_relaxed) : 0;
    if (!o) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, K, kWfThreads, 0);
        o = b > 0 ? b : 1;
        if (dev >= 0 && dev < kWfOccDevices) occ[dev].store(o, std::memory_order_relaxed);
    }
    return (unsigned)(sms * o);
}

// Blocks of the persistent extension kernel: as many as stay resident.
template <class Src>
unsigned wfExtendBlocks() {
    return residentBlocks<kWfExtend<Src>>();
}

// The capped grid of the histogram and scatter: four rounds of resident
// blocks striding over the live paths (their per-path work is uniform, so a
// fixed assignment balances; waves of up to about 1.2M paths keep one block
// per 128 paths).  With 64 rounds, the late bounces of a 2^26-path wave still
// spent 80 us per launch on empty blocks.
template <auto K>
unsigned bounceBlocks() {
    return 4u * residentBlocks<K>();
}

// Counting sort of the live paths by key.  Keys beyond kSmemKeys bins fall
// back to global atomics per path.
constexpr uint32_t kSmemKeys = 2048;

//
// The per-path kernels of a bounce run capped grids on large waves (the
// histogram and the scatter stride over the live paths, bounceBlocks; the
// shade stage's resident blocks take chunks from a counter): the live count
// is known only on the device, and a grid sized for the whole wave would
// launch, in the late bounces of a 2^26-path wave, half a million blocks that
// read the count and exit.
__global__ void __launch_bounds__(kWfThreads) kWfHistogram(const uint32_t* __restrict__ keys,
                                                           const uint32_t* __restrict__ count, uint32_t nKeys,
                                                           uint32_t* __restrict__ hist) {
    __shared__ uint32_t local[kSmemKeys];
    const uint32_t n = *count;
    if (blockIdx.x * blockDim.x >= n) return;
    const uint32_t stride = gridDim.x * blockDim.x;
    const bool smem = nKeys <= kSmemKeys;
    if (smem) {
        for (uint32_t k = threadIdx.x; k < nKeys; k += blockDim.x) local[k] = 0;
        __syncthreads();
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) atomicAdd(&local[keys[i]], 1u);
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < nKeys; k += blockDim.x)
            if (local[k]) atomicAdd(&hist[k], local[k]);
    } else {
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) atomicAdd(&hist[keys[i]], 1u);
    }
}

// Exclusive scan of the histogram into bin offsets (one block).
__global__ void __launch_bounds__(1024) kWfScan(uint32_t* __restrict__ hist, uint32_t nKeys) {
    __shared__ uint32_t partial[1024];
    const uint32_t per = (nKeys + blockDim.x - 1) / blockDim.x;
    const uint32_t b = threadIdx.x * per, e = min(nKeys, b + per);
    uint32_t sum = 0;
    for (uint32_t k = b; k < e; k++) sum += hist[k];
    partial[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t t = 0; t < blockDim.x; t++) {
            const uint32_t v = partial[t];
            partial[t] = run;
            run += v;
        }
    }
    __syncthreads();
    uint32_t run = partial[threadIdx.x];
    for (uint32_t k = b; k < e; k++) {
        const uint32_t v = hist[k];
        hist[k] = run;
        run += v;
    }
}

// Scatter: each block reserves its range in every bin once, then places its
// paths with shared-memory counters.
__global__ void __launch_bounds__(kWfThreads) kWfScatter(const uint32_t* __restrict__ keys,
                                                         const uint32_t* __restrict__ queue,
                                                         const uint32_t* __restrict__ count, uint32_t nKeys,
                                                         uint32_t* __restrict__ offsets,
                                                         uint32_t* __restrict__ sorted) {
    __shared__ uint32_t local[kSmemKeys];
    const uint32_t n = *count;
    const uint32_t stride = gridDim.x * blockDim.x;
    // block-uniform loop over chunks of blockDim.x paths
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        const uint32_t i = i0 + threadIdx.x;
        if (nKeys <= kSmemKeys) {
            for (uint32_t k = threadIdx.x; k < nKeys; k += blockDim.x) local[k] = 0;
            __syncthreads();
            uint32_t key = 0, rank = 0;
            if (i < n) {
                key = keys[i];
                rank = atomicAdd(&local[key], 1u);
            }
            __syncthreads();
            for (uint32_t k = threadIdx.x; k < nKeys; k += blockDim.x)
                if (local[k]) local[k] = atomicAdd(&offsets[k], local[k]);
            __syncthreads();
            if (i < n) sorted[local[key] + rank] = queue[i];
            __syncthreads();  // local[] is cleared for the next chunk
        } else if (i < n) {
            sorted[atomicAdd(&offsets[keys[i]], 1u)] = queue[i];
        }
    }
}

// Between bounces: the next queue's count becomes the live count, and the
// counters the next bounce accumulates into are cleared.
__global__ void kWfAdvance(uint32_t* __restrict__ counts, uint32_t* __restrict__ hist, uint32_t nKeys) {
    for (uint32_t k = threadIdx.x; k < nKeys; k += blockDim.x) hist[k] = 0;
    if (threadIdx.x == 0) {
        counts[0] = counts[1];
        counts[1] = 0;
        counts[2] = 0;
        counts[3] = 0;
    }
}

// The bounce after the query, for the live paths in material order.  Mode
// supplies the hooks of shadeBounce (with their per-path state in st.aux)
// and what happens to a path that ends.
template <class Src, class Mode, bool kDynamicFetch = false, bool kFullScene = true>
__global__ void __launch_bounds__(kWfThreads, Src::kShadeMinBlocks) kWfShade(const __grid_constant__ Src src, WfState st,
                                                       const __grid_constant__ Mode mode,
                                                       const uint32_t* __restrict__ order,
                                                       uint32_t* __restrict__ counts, uint32_t depth,
                                                       uint32_t* __restrict__ next,
                                                       uint32_t* __restrict__ nextCount) {
    // kDynamicFetch = false: block b shades live paths [128 b, 128 b + 128) (a
    // grid of one block per 128 paths of the wave).  true (waves too large
    // for that grid to be cheap in their late bounces): the resident blocks
    // take chunks of 128 live paths from counts[3] (zeroed before the launch)
    // as they free up, until none are left.
    __shared__ uint32_t chunk;
    const uint32_t n = counts[0];
    for (uint32_t round = 0;; round++) {
        uint32_t i0 = blockIdx.x * blockDim.x;
        if (kDynamicFetch) {
            if (threadIdx.x == 0) chunk = atomicAdd(counts + 3, 1u);
            __syncthreads();
            i0 = chunk * blockDim.x;
            __syncthreads();  // every thread has read chunk before thread 0 overwrites it
        } else if (round) {
            break;
        }
        if (i0 >= n) break;
        const uint32_t i = i0 + threadIdx.x;
        bool push = false;
        uint32_t k = 0, item = 0, rays = 0;
        if (i < n) {
            k = order[i];
            item = st.item[k];
            const Params& p = src.paramsOf(item);
            PathCtx c{src.sceneOf(item), 0u, SpectralPath{}};
            const uint4 meta = st.meta[k];
            c.spec = makeSpectralPath(p.spectral != 0, meta.x, meta.y, meta.z);
            Sampler smp = Sampler::resume(meta.w, st.inc[k]);
            const float4 o = st.ro[k], d = st.rd[k], b = st.beta[k], r = st.rad[k], hv = st.hit[k];
            float3 ro = mk3(o.x, o.y, o.z), rd = mk3(d.x, d.y, d.z);
            Spec beta = sp(b.x, b.y, b.z), radiance = sp(r.x, r.y, r.z);
            THit h;
            h.prim = __float_as_uint(hv.x);
            h.t = hv.y;
            h.u = hv.z;
            h.v = hv.w;
            typename Mode::Hooks hk = mode.hooks(st, k, meta);
            const bool alive =
                shadeBounce<typename Mode::Hooks, false, kFullScene>(c, p, smp, depth, h, ro, rd, beta, radiance, hk);
            if (alive && depth + 1 < p.maxDepth) {
                push = true;
                st.ro[k] = make_float4(ro.x, ro.y, ro.z, o.w);
                st.rd[k] = make_float4(rd.x, rd.y, rd.z, d.w);
                st.beta[k] = make_float4(beta.r, beta.g, beta.b, __uint_as_float(depth + 1));
                st.rad[k] = make_float4(radiance.r, radiance.g, radiance.b, 0.0f);
                st.meta[k] = make_uint4(meta.x, meta.y, meta.z, smp.state);
                mode.keep(st, k, hk);
            } else {
                mode.end(src, item, st, k, meta, c, radiance, make_float2(o.w, d.w), hk);
            }
            rays = c.rays;
        }
        // warp-aggregated append to the next queue
        const unsigned act = __activemask();
        const unsigned m = __ballot_sync(act, push);
        if (m) {
            const int lane = threadIdx.x & 31;
            const int leader = __ffs(m) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(nextCount, (uint32_t)__popc(m));
            base = __shfl_sync(act, base, leader);
            if (push) next[base + __popc(m & ((1u << lane) - 1u))] = k;
        }
        addRays(src.raysOf(item), rays);
    }
}

// Paths whose scene allows no bounce (max depth 0) end with zero radiance;
// the others form the first queue.
//
// allTraced: every path's scene allows a bounce (a single scene with max
// depth > 0): the first queue is every path of the wave in order, written
// without the append's atomics (which cost 1.5 ms on a 2^26-path wave).
template <class Src, class Mode>
__global__ void __launch_bounds__(kWfThreads) kWfEndUntraced(const __grid_constant__ Src src, WfState st,
                                                             const __grid_constant__ Mode mode, uint32_t n,
                                                             const uint64_t* __restrict__ waveBase, uint64_t total,
                                                             uint32_t* __restrict__ queue,
                                                             uint32_t* __restrict__ liveCount, int allTraced) {
    uint64_t base = 0;
    n = waveSize(base, n, waveBase, total);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (allTraced) {
        if (i < n) queue[i] = i;
        if (i == 0) *liveCount = n;
        return;
    }
    bool push = false;
    if (i < n) {
        const uint32_t item = st.item[i];
        const Params& p = src.paramsOf(item);
        if (p.maxDepth > 0) {
            push = true;
        } else {
            const uint4 meta = st.meta[i];
            PathCtx c{src.sceneOf(item), 0u, SpectralPath{}};
            c.spec = makeSpectralPath(p.spectral != 0, meta.x, meta.y, meta.z);
            typename Mode::Hooks hk = mode.hooks(st, i, meta);
            mode.end(src, item, st, i, meta, c, sp(0.0f), make_float2(st.ro[i].w, st.rd[i].w), hk);
        }
    }
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, push);
    if (m) {
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(m) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(liveCount, (uint32_t)__popc(m));
        base = __shfl_sync(act, base, leader);
        if (push) queue[base + __popc(m & ((1u << lane) - 1u))] = i;
    }
}

// The remaining bounces of every live path in one launch, from bounce
// depth0 on: closest() and shadeBounce() in a loop per path, the
// megakernel's form resumed from the wave's path state.  The cached
// integrator uses it once only its training paths (one pixel in hundreds)
// are left: a wavefront bounce per remaining depth would cost six launches
// for a few thousand paths each.  The same operations in the same order as
// the bounce-by-bounce form, so the results are those of kWfShade.
//
// fewMax > 0: only when at most fewMax paths are live (the tail of a wave,
// where each further bounce would cost its launches and the latency of its
// slowest query for a handful of paths); kWfDrainIfFew then empties the
// queue, so that the remaining launches of the wave find no live path.
template <class Src, class Mode>
__global__ void __launch_bounds__(kWfThreads) kWfFinish(const __grid_constant__ Src src, WfState st,
                                                        const __grid_constant__ Mode mode,
                                                        const uint32_t* __restrict__ queue,
                                                        const uint32_t* __restrict__ count, uint32_t depth0,
                                                        uint32_t fewMax = 0) {
    const uint32_t n = *count;
    if (fewMax && n > fewMax) return;
    if (blockIdx.x * blockDim.x >= n) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t item = 0, rays = 0;
    if (i < n) {
        const uint32_t k = queue[i];
        item = st.item[k];
        const Params& p = src.paramsOf(item);
        PathCtx c{src.sceneOf(item), 0u, SpectralPath{}};
        const uint4 meta = st.meta[k];
        c.spec = makeSpectralPath(p.spectral != 0, meta.x, meta.y, meta.z);
        Sampler smp = Sampler::resume(meta.w, st.inc[k]);
        const float4 o = st.ro[k], d = st.rd[k], b = st.beta[k], r = st.rad[k];
        float3 ro = mk3(o.x, o.y, o.z), rd = mk3(d.x, d.y, d.z);
        Spec beta = sp(b.x, b.y, b.z), radiance = sp(r.x, r.y, r.z);
        typename Mode::Hooks hk = mode.hooks(st, k, meta);
        for (uint32_t depth = depth0; depth < p.maxDepth; depth++) {
            THit h;
            closest(c, ro, rd, h);
            if (!shadeBounce<typename Mode::Hooks, true>(c, p, smp, depth, h, ro, rd, beta, radiance, hk)) break;
        }
        mode.end(src, item, st, k, meta, c, radiance, make_float2(o.w, d.w), hk);
        rays = c.rays;
    }
    addRays(src.raysOf(item), rays);
}

__global__ void kWfNextWave(uint64_t* __restrict__ waveBase, uint32_t cap) { *waveBase += cap; }

__global__ void kWfDrainIfFew(uint32_t* __restrict__ counts, uint32_t fewMax) {
    if (counts[0] <= fewMax) counts[0] = 0;
}

__global__ void kWfStart(uint32_t* __restrict__ counts, uint32_t* __restrict__ hist, uint32_t nKeys) {
    for (uint32_t k = threadIdx.x; k < nKeys; k += blockDim.x) hist[k] = 0;
    if (threadIdx.x == 0) {
        counts[0] = 0;
        counts[1] = 0;
        counts[2] = 0;
        counts[3] = 0;
    }
}

inline unsigned blocks(uint64_t n) { return (unsigned)((n + kWfThreads - 1) / kWfThreads); }

// Whether every path of a source takes at least one bounce, as the host
// knows it: a single scene with max depth > 0.  (A many-scene source keeps
// its scenes' parameters in device memory.)
inline bool allTraced(const OneScene& s) { return s.p.maxDepth > 0; }
inline bool allTraced(const ManyScenes&) { return false; }

// One wave of n paths (path k of the wave is path base + k of the source):
// camera rays, then per bounce extend, histogram, scan, scatter, shade and
// advance, on `stream` without waiting on the host.  maxDepth bounds every
// scene's max depth, nKeys the sort keys of all scenes.
//
// With waveBase set (device memory), the wave starts at *waveBase, holds
// min(n, total - *waveBase) paths and advances *waveBase by n at its end, so
// that the same launch sequence (a captured graph) replays wave after wave.
//
// finishFrom < maxDepth: the bounces from finishFrom on run as one kWfFinish
// launch over the paths still live then.  fewMax > 0: before each bounce
// after the first, the live paths finish in one kWfFinish launch once at most
// fewMax of them are left.
template <class Src, class Mode>
int runWave(const Src& src, const Mode& mode, WfBuffers* b, uint64_t base, uint32_t n, uint32_t maxDepth,
            uint32_t nKeys, cudaStream_t stream, uint64_t* waveBase = nullptr, uint64_t total = 0,
            uint32_t finishFrom = 0xffffffffu, uint32_t fewMax = 0, bool lean = false) {
    const WfState st{b->ro, b->rd, b->beta, b->rad, b->meta, b->inc, b->hit, b->aux, b->item};
    kWfInit<Src><<<blocks(n), kWfThreads, 0, stream>>>(src, st, base, n, waveBase, total);
    CR_LAUNCH_CHECK();
    kWfStart<<<1, 256, 0, stream>>>(b->counts, b->hist, nKeys);
    CR_LAUNCH_CHECK();
    // the paths of scenes with max depth 0 end here; the others form the first queue
    kWfEndUntraced<Src, Mode><<<blocks(n), kWfThreads, 0, stream>>>(src, st, mode, n, waveBase, total, b->qa,
                                                                     b->counts, allTraced(src) ? 1 : 0);
    CR_LAUNCH_CHECK();
    uint32_t* live = b->qa;
    uint32_t* nextQ = b->qb;
    // measured on GB300: one block per 128 paths is faster up to waves of a
    // few million paths (1M: 2.94 against 2.89 ms per Cornell render; 4M box
    // clutter: 32.1 against 30.9 ms); beyond, half a million mostly empty
    // blocks per late bounce cost more (1080p x 64 spp in 2^26-path waves:
    // 0.140 against 0.161 s)
    const unsigned shadeResident = residentBlocks<kWfShade<Src, Mode, true>>();
    const bool shadeDynamic = blocks(n) > 64u * shadeResident;
    const uint32_t bounces = std::min(maxDepth, finishFrom);
    for (uint32_t depth = 0; depth < bounces; depth++) {
        if (fewMax && depth > 0) {
            kWfFinish<Src, Mode><<<blocks(std::min(n, fewMax)), kWfThreads, 0, stream>>>(src, st, mode, live, b->counts,
                                                                                         depth, fewMax);
            CR_LAUNCH_CHECK();
            kWfDrainIfFew<<<1, 1, 0, stream>>>(b->counts, fewMax);
            CR_LAUNCH_CHECK();
        }
        kWfExtend<Src><<<std::min(blocks(n), wfExtendBlocks<Src>()), kWfThreads, 0, stream>>>(src, st, live,
                                                                                              b->counts, b->keys);
        CR_LAUNCH_CHECK();
        kWfHistogram<<<std::min(blocks(n), bounceBlocks<kWfHistogram>()), kWfThreads, 0, stream>>>(b->keys, b->counts,
                                                                                                 nKeys, b->hist);
        CR_LAUNCH_CHECK();
        kWfScan<<<1, 1024, 0, stream>>>(b->hist, nKeys);
        CR_LAUNCH_CHECK();
        kWfScatter<<<std::min(blocks(n), bounceBlocks<kWfScatter>()), kWfThreads, 0, stream>>>(b->keys, live, b->counts,
                                                                                             nKeys, b->hist, b->sorted);
        CR_LAUNCH_CHECK();
        bool launched = false;
        if constexpr (Src::kAllowLean && Mode::kAllowLean) {
            if (lean) {
                if (shadeDynamic)
                    kWfShade<Src, Mode, true, false><<<residentBlocks<kWfShade<Src, Mode, true, false>>(), kWfThreads, 0,
                                                       stream>>>(src, st, mode, b->sorted, b->counts, depth, nextQ,
                                                                 b->counts + 1);
                else
                    kWfShade<Src, Mode, false, false><<<blocks(n), kWfThreads, 0, stream>>>(
                        src, st, mode, b->sorted, b->counts, depth, nextQ, b->counts + 1);
                launched = true;
            }
        }
        if (!launched) {
            if (shadeDynamic)
                kWfShade<Src, Mode, true><<<shadeResident, kWfThreads, 0, stream>>>(src, st, mode, b->sorted, b->counts,
                                                                                     depth, nextQ, b->counts + 1);
            else
                kWfShade<Src, Mode, false><<<blocks(n), kWfThreads, 0, stream>>>(src, st, mode, b->sorted, b->counts,
                                                                                  depth, nextQ, b->counts + 1);
        }
        CR_LAUNCH_CHECK();
        kWfAdvance<<<1, 256, 0, stream>>>(b->counts, b->hist, nKeys);
        CR_LAUNCH_CHECK();
        std::swap(live, nextQ);
    }
    if (bounces < maxDepth) {
        kWfFinish<Src, Mode><<<blocks(n), kWfThreads, 0, stream>>>(src, st, mode, live, b->counts, bounces);
        CR_LAUNCH_CHECK();
    }
    if (waveBase) {
        kWfNextWave<<<1, 1, 0, stream>>>(waveBase, n);
        CR_LAUNCH_CHECK();
    }
    return CR_OK;
}

// The plain path tracer: an ending path splats its radiance into its
// scene's film (SensorData::addSample, Core/Sensor.cu:19-43).
struct PlainMode {
    using Hooks = NoHooks;
    static constexpr bool kAllowLean = true;
    __device__ __forceinline__ Hooks hooks(const WfState&, uint32_t, const uint4&) const { return NoHooks{}; }
    __device__ __forceinline__ void keep(const WfState&, uint32_t, const Hooks&) const {}
    template <class Src>
    __device__ __forceinline__ void end(const Src& src, uint32_t item, const WfState&, uint32_t, const uint4&,
                                        const PathCtx& c, const Spec& L, float2 pix, const Hooks&) const {
        splatGlobal(src.camOf(item), pix, pathSpecToRgb(c.spec, L, src.paramsOf(item).wb), src.filmRgbOf(item),
                    src.filmWOf(item));
    }
};

// The single-scene source of a scene and its integrator parameters.
inline OneScene oneScene(cr_scene* s, const Params& p) {
    return OneScene{s->view(), s->cam, p, s->filmRgb, s->filmW, s->rayCounter, s->nMats};
}

}  // namespace
}  // namespace cr
