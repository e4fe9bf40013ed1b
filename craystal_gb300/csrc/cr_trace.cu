// cr_trace.cu -- batched closest-hit and occlusion queries
// (SceneView::intersect / intersectOcclusion, Scene/Scene.cu:5-29).

#include <cuda.h>

#include "cr_internal.cuh"
#include "cr_math.cuh"
#include "cr_traverse.cuh"

namespace cr {
namespace {

constexpr int kTraceThreads = kStackBlock;  // the top of the stack is in shared memory

// Persistent blocks with dynamic ray fetch.  The lanes of a warp take rays
// from a counter as they finish, at least kRefill lanes at a time, so that a
// warp keeps most of its lanes busy until the rays run out instead of
// waiting for its slowest ray (incoherent rays leave a one-ray-per-thread
// warp with 6 of 32 lanes busy on average).  Every ray is traversed in the
// reference's order with the reference's culling; only the lane that
// carries it changes.
//
// kSpheres: the scene also holds analytic spheres, which are tested first,
// as SceneView::intersect does (Scene/Scene.cu:5-14): a lane that takes a
// ray walks the sphere BVH to the end at once (sphere trees are small), and
// the triangle traversal then starts from the sphere hit's distance.  A
// separate instance keeps the triangle-only kernel free of the sphere code.
//
// kTwoLevel: the two-level step (travStep), chosen per scene with
// cr_scene_set_traversal.
//
// counter != nullptr: one zeroed device counter over all n rays, which
// keeps every SM busy to the end (12 % faster than one ray per thread on the
// 16M-ray cast).  nullptr: block b takes rays [b * chunk, (b + 1) * chunk)
// from a shared-memory counter, for callers that allocate nothing (4 %).
// Refilling at 4 idle lanes rather than 8 gains 0.5 % with the
// one-slot-per-step traversal.
constexpr int kRefill = 4;

template <bool kAnyHit, bool kSpheres, bool kTwoLevel>
__global__ void __launch_bounds__(kTraceThreads) kTraceDyn(const SceneView sc, const cr_ray* __restrict__ rays,
                                                           uint64_t n, cr_hit* __restrict__ hits,
                                                           uint8_t* __restrict__ occ,
                                                           unsigned long long* __restrict__ counter) {
    __shared__ SharedStackArea stk;
    __shared__ unsigned long long blockNext;
    uint64_t hi = n;
    unsigned long long* next = counter;
    if (!counter) {
        const uint64_t chunk = (n + gridDim.x - 1) / gridDim.x;
        const uint64_t lo = min(n, (uint64_t)blockIdx.x * chunk);
        hi = min(n, lo + chunk);
        if (threadIdx.x == 0) blockNext = lo;
        next = &blockNext;
    }
    __syncthreads();
    const BvhView bv{sc.pairs, sc.leaves, sc.rootRef, sc.rootFlags, sc.rootMin, sc.rootMax, sc.hasRoot};
    const TriLeaf<kAnyHit> leaf{sc.tris};
    TravStack<kSharedStack> stack;
    stack.sh = stk;
    TravState cur;
    TRay r;
    THit h{INFINITY, 0.0f, 0.0f, CR_MISS};
    uint64_t idx = 0;
    bool active = false, exhausted = false;
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    auto finish = [&](bool hit) {
        if (kAnyHit) {
            occ[idx] = hit ? 1 : 0;
        } else {
            reinterpret_cast<float4*>(hits)[idx] = hit ? make_float4(__uint_as_float(h.prim), h.t, h.u, h.v)
                                                       : make_float4(__uint_as_float(CR_MISS), INFINITY, 0.0f, 0.0f);
        }
    };
    while (true) {
        const unsigned idle = __ballot_sync(full, !active);
        if (!exhausted && __popc(idle) >= kRefill) {
            const int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(next, (unsigned long long)__popc(idle));
            base = __shfl_sync(full, base, leader);
            if (base + (unsigned)__popc(idle) >= hi) exhausted = true;
            if (!active) {
                idx = base + (unsigned)__popc(idle & ((1u << lane) - 1u));
                if (idx < hi) {
                    const float4* rp = reinterpret_cast<const float4*>(rays + idx);
                    const float4 a = __ldg(rp), b = __ldg(rp + 1);
                    r = makeTRay(mk3(a.x, a.y, a.z), a.w, mk3(b.x, b.y, b.z), b.w);
                    h.t = INFINITY;
                    h.u = h.v = 0.0f;
                    h.prim = CR_MISS;
                    bool sphereHit = false;
                    if (kSpheres) sphereHit = traverseSpheres<kAnyHit, kSharedStack>(sc, r, h, stk);
                    if (kAnyHit && sphereHit) {
                        finish(true);
                    } else if (travBegin(cur, bv, r)) {
                        cur.isHit = sphereHit;
                        active = true;
                    } else {
                        finish(sphereHit);
                    }
                }
            }
        }
        if (!__any_sync(full, active)) {
            if (exhausted) break;
            continue;  // every lane idle: the next round refills all 32
        }
        if (active && !travStep<kAnyHit, TriLeaf<kAnyHit>, TravStack<kSharedStack>, kTwoLevel>(cur, stack, bv, sc.errFlags, leaf, r, h)) {
            finish(cur.isHit);
            active = false;
        }
    }
}

// Resident blocks per SM of each kernel, per device ordinal (0 = not yet
// asked).  Host threads may call at once: each entry is an atomic, and two
// threads that both ask store the same value.
constexpr int kOccDevices = 64;
std::atomic<int> gOccupancy[kOccDevices][8];

template <bool kAnyHit, bool kSpheres, bool kTwoLevel>
int traceDynBlocks(uint64_t n) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    constexpr int kKind = (kAnyHit ? 1 : 0) + (kSpheres ? 2 : 0) + (kTwoLevel ? 4 : 0);
    int occ = 0;
    if (dev >= 0 && dev < kOccDevices) occ = gOccupancy[dev][kKind].load(std::memory_order_relaxed);
    if (!occ) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kTraceDyn<kAnyHit, kSpheres, kTwoLevel>, kTraceThreads, 0);
        occ = b > 0 ? b : 1;
        if (dev >= 0 && dev < kOccDevices) gOccupancy[dev][kKind].store(occ, std::memory_order_relaxed);
    }
    const uint64_t perThread = (n + kTraceThreads - 1) / kTraceThreads;
    return (int)std::min<uint64_t>((uint64_t)sms * occ, std::max<uint64_t>(1, perThread));
}

constexpr uint64_t kMaxRaysPerLaunch = 0x7fffffffull * kTraceThreads;

// mayAllocate: the ray counter of the dynamic fetch is a stream-ordered
// allocation (cudaMallocAsync / cudaFreeAsync on st), so that calls on
// different streams never share one; without it, per-block ranges.
template <bool kAnyHit>
int launchTrace(cr_scene* s, const cr_ray* rays, uint64_t n, cr_hit* hits, uint8_t* occ, cudaStream_t st,
                bool mayAllocate) {
    for (uint64_t off = 0; off < n; off += kMaxRaysPerLaunch) {
        const uint64_t m = std::min(n - off, kMaxRaysPerLaunch);
        unsigned long long* counter = nullptr;
        if (mayAllocate) {
            CR_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&counter), sizeof(unsigned long long), st));
            CR_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st));
        }
        cr_hit* h = hits ? hits + off : nullptr;
        uint8_t* o = occ ? occ + off : nullptr;
        const bool two = s->traversal == CR_TRAVERSAL_TWO_LEVEL && s->groupPairs;
        SceneView v = s->view();
        if (two) {
            v.pairs = s->groupPairs;
            v.rootRef = s->groupRootRef;
        }
        if (s->sphHasRoot && two)
            kTraceDyn<kAnyHit, true, true><<<traceDynBlocks<kAnyHit, true, true>(m), kTraceThreads, 0, st>>>(
                v, rays + off, m, h, o, counter);
        else if (s->sphHasRoot)
            kTraceDyn<kAnyHit, true, false><<<traceDynBlocks<kAnyHit, true, false>(m), kTraceThreads, 0, st>>>(
                v, rays + off, m, h, o, counter);
        else if (two)
            kTraceDyn<kAnyHit, false, true><<<traceDynBlocks<kAnyHit, false, true>(m), kTraceThreads, 0, st>>>(
                v, rays + off, m, h, o, counter);
        else
            kTraceDyn<kAnyHit, false, false><<<traceDynBlocks<kAnyHit, false, false>(m), kTraceThreads, 0, st>>>(
                v, rays + off, m, h, o, counter);
        CR_LAUNCH_CHECK();
        if (counter) CR_CUDA(cudaFreeAsync(counter, st));
    }
    return CR_OK;
}

}  // namespace

int traceClosestDevice(cr_scene* s, const cr_ray* rays, uint64_t n, cr_hit* hits, cudaStream_t st, bool mayAllocate) {
    return launchTrace<false>(s, rays, n, hits, nullptr, st, mayAllocate);
}

int traceOccludedDevice(cr_scene* s, const cr_ray* rays, uint64_t n, uint8_t* occ, cudaStream_t st) {
    return launchTrace<true>(s, rays, n, nullptr, occ, st, true);
}

}  // namespace cr

using namespace cr;

namespace {

constexpr uint64_t kChunk = 1ull << 21;  // rays per pipelined chunk (64 MiB of rays)

int ensureStreams(cr_scene* s) {
    for (int k = 0; k < 2; k++)
        if (!s->streams[k]) CR_CUDA(cudaStreamCreateWithFlags(&s->streams[k], cudaStreamNonBlocking));
    return CR_OK;
}

int ensureStaging(cr_scene* s) {
    if (s->stageCap) return CR_OK;
    int rc = ensureStreams(s);
    if (rc) return rc;
    for (int k = 0; k < 2; k++) {
        CR_CUDA(cudaMalloc(&s->stageRays[k], kChunk * sizeof(cr_ray)));
        CR_CUDA(cudaMalloc(&s->stageHits[k], kChunk * sizeof(cr_hit)));
        CR_CUDA(cudaMalloc(&s->stageOcc[k], kChunk));
    }
    s->stageCap = kChunk;
    return CR_OK;
}

// cuPointerGetAttribute from the driver the runtime uses (no link to libcuda).
typedef CUresult (*PointerAttributeFn)(void*, CUpointer_attribute, CUdeviceptr);

PointerAttributeFn pointerAttributeFn() {
    static const PointerAttributeFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<PointerAttributeFn>(f);
    }();
    return fn;
}

// The device address of host range [p, p + bytes) when the GPU can use it in
// place: page-locked host memory (cudaHostAlloc, cudaHostRegister, a pinned
// torch tensor) of the scene's device, mapped, with the whole range inside
// one allocation.  Anything else (pageable memory, a range that runs past its
// allocation, a driver that cannot say) gives nullptr and the staged path.
void* mappedDevicePtr(const cr_scene* s, const void* p, size_t bytes) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer || a.device != s->device) return nullptr;
    const PointerAttributeFn fn = pointerAttributeFn();
    if (!fn) return nullptr;
    unsigned long long start = 0, size = 0, mapped = 0;
    const CUdeviceptr q = (CUdeviceptr)reinterpret_cast<uintptr_t>(p);
    if (fn(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, q) != CUDA_SUCCESS ||
        fn(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, q) != CUDA_SUCCESS ||
        fn(&mapped, CU_POINTER_ATTRIBUTE_MAPPED, q) != CUDA_SUCCESS || !mapped)
        return nullptr;
    const uintptr_t lo = reinterpret_cast<uintptr_t>(p);
    if (lo < start || bytes > size || lo - start > size - bytes) return nullptr;
    return a.devicePointer;
}

// In-place query on mapped host buffers.  On GB300 the GPU reads the rays and
// writes the results over NVLink-C2C as the traversal goes: 16M rays in
// 13.97 ms against 13.87 ms on device buffers, where staging copies take
// 14.96 ms.  false: the buffers do not qualify.
template <bool kOcc>
bool traceMapped(cr_scene* s, const cr_ray* rays, uint64_t n, void* out, int& rc) {
    if (n > (~0ull >> 6)) return false;  // the byte counts below stay far from overflow
    const cr_ray* dr = static_cast<const cr_ray*>(mappedDevicePtr(s, rays, n * sizeof(cr_ray)));
    void* dout = mappedDevicePtr(s, out, n * (kOcc ? 1 : sizeof(cr_hit)));
    if (!dr || !dout) return false;
    if (reinterpret_cast<uintptr_t>(dr) & 15u) return false;
    if (!kOcc && (reinterpret_cast<uintptr_t>(dout) & 15u)) return false;
    rc = ensureStreams(s);
    if (rc) return true;
    cudaStream_t st = s->streams[0];
    rc = kOcc ? traceOccludedDevice(s, dr, n, static_cast<uint8_t*>(dout), st)
              : traceClosestDevice(s, dr, n, static_cast<cr_hit*>(dout), st);
    return true;
}

// Host-buffer query.  Mapped host buffers are used in place (traceMapped);
// otherwise chunks alternate between two streams so that the copy-in of one
// chunk overlaps the traversal and copy-out of the other.
template <bool kOcc>
int traceHost(cr_scene* s, const cr_ray* rays, uint64_t n, void* out) {
    if (!s) return fail(CR_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (n == 0) return CR_OK;
    if (!rays || !out) return fail(CR_ERR_INVALID_ARGUMENT, "rays / output is NULL");
    CR_CUDA(cudaSetDevice(s->device));
    int rc = CR_OK;
    const bool inPlace = traceMapped<kOcc>(s, rays, n, out, rc);
    if (rc) return rc;
    if (!inPlace) rc = ensureStaging(s);
    if (rc) return rc;
    for (uint64_t off = 0, k = 0; !inPlace && off < n; off += kChunk, k++) {
        const int b = (int)(k & 1);
        const uint64_t m = std::min(kChunk, n - off);
        cudaStream_t st = s->streams[b];
        CR_CUDA(cudaMemcpyAsync(s->stageRays[b], rays + off, m * sizeof(cr_ray), cudaMemcpyHostToDevice, st));
        if (kOcc) {
            rc = traceOccludedDevice(s, s->stageRays[b], m, s->stageOcc[b], st);
            if (rc) return rc;
            CR_CUDA(cudaMemcpyAsync(static_cast<uint8_t*>(out) + off, s->stageOcc[b], m, cudaMemcpyDeviceToHost, st));
        } else {
            rc = traceClosestDevice(s, s->stageRays[b], m, s->stageHits[b], st);
            if (rc) return rc;
            CR_CUDA(cudaMemcpyAsync(static_cast<cr_hit*>(out) + off, s->stageHits[b], m * sizeof(cr_hit),
                                    cudaMemcpyDeviceToHost, st));
        }
    }
    CR_CUDA(cudaStreamSynchronize(s->streams[0]));
    CR_CUDA(cudaStreamSynchronize(s->streams[1]));
    return takeDeviceErrors(s, "traversal");
}

}  // namespace

extern "C" {

int cr_trace_closest(cr_scene* scene, const cr_ray* rays, uint64_t n, cr_hit* hits) {
    clearError();
    return traceHost<false>(scene, rays, n, hits);
}

int cr_trace_closest_device(cr_scene* scene, const cr_ray* rays, uint64_t n, cr_hit* hits, void* stream) {
    clearError();
    if (!scene) return fail(CR_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (n && (!rays || !hits)) return fail(CR_ERR_INVALID_ARGUMENT, "rays / hits is NULL");
    if ((reinterpret_cast<uintptr_t>(rays) | reinterpret_cast<uintptr_t>(hits)) & 15u)
        return fail(CR_ERR_INVALID_ARGUMENT, "rays and hits must be 16-byte aligned");
    return traceClosestDevice(scene, rays, n, hits, static_cast<cudaStream_t>(stream));
}

int cr_trace_occluded(cr_scene* scene, const cr_ray* rays, uint64_t n, uint8_t* occluded) {
    clearError();
    return traceHost<true>(scene, rays, n, occluded);
}

int cr_trace_occluded_device(cr_scene* scene, const cr_ray* rays, uint64_t n, uint8_t* occluded, void* stream) {
    clearError();
    if (!scene) return fail(CR_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (n && (!rays || !occluded)) return fail(CR_ERR_INVALID_ARGUMENT, "rays / occluded is NULL");
    if (reinterpret_cast<uintptr_t>(rays) & 15u) return fail(CR_ERR_INVALID_ARGUMENT, "rays must be 16-byte aligned");
    return traceOccludedDevice(scene, rays, n, occluded, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
