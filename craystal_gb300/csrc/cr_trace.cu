// cr_trace.cu -- batched closest-hit and occlusion queries
// (SceneView::intersect / intersectOcclusion, Scene/Scene.cu:5-29).

#include "cr_internal.cuh"
#include "cr_math.cuh"
#include "cr_traverse.cuh"

namespace cr {
namespace {

constexpr int kTraceThreads = kStackBlock;  // the top of the stack is in shared memory

// One thread per ray.  (A persistent variant that refills the lanes of a
// warp from a per-warp ray range measured slower on GB300 for this
// incoherent workload: the lanes' rounds synchronise on the slowest lane.)
//
// kSpheres: the scene has analytic spheres, tested first as
// SceneView::intersect does (a separate instance keeps the triangle-only
// kernel free of the sphere code).
template <bool kAnyHit, bool kSpheres>
__global__ void __launch_bounds__(kTraceThreads) kTrace(const SceneView sc, const cr_ray* __restrict__ rays,
                                                        uint64_t n, cr_hit* __restrict__ hits,
                                                        uint8_t* __restrict__ occ) {
    __shared__ SharedStackArea stk;
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* rp = reinterpret_cast<const float4*>(rays + i);
    const float4 a = __ldg(rp), b = __ldg(rp + 1);
    const TRay r = makeTRay(mk3(a.x, a.y, a.z), a.w, mk3(b.x, b.y, b.z), b.w);
    THit h;
    h.t = INFINITY;
    h.u = h.v = 0.0f;
    h.prim = CR_MISS;
    bool hit = false;
    if (kSpheres) hit = traverseSpheres<kAnyHit, kSharedStack>(sc, r, h, stk);
    if (!(kAnyHit && hit)) hit |= traverse<kAnyHit, kSharedStack>(sc, r, h, stk);
    if (kAnyHit) {
        occ[i] = hit ? 1 : 0;
    } else {
        reinterpret_cast<float4*>(hits)[i] = hit ? make_float4(__uint_as_float(h.prim), h.t, h.u, h.v)
                                                 : make_float4(__uint_as_float(CR_MISS), INFINITY, 0.0f, 0.0f);
    }
}

constexpr uint64_t kMaxRaysPerLaunch = 0x7fffffffull * kTraceThreads;

template <bool kAnyHit>
int launchTrace(cr_scene* s, const cr_ray* rays, uint64_t n, cr_hit* hits, uint8_t* occ, cudaStream_t st) {
    const SceneView v = s->view();
    for (uint64_t off = 0; off < n; off += kMaxRaysPerLaunch) {
        const uint64_t m = std::min(n - off, kMaxRaysPerLaunch);
        const unsigned blocks = (unsigned)((m + kTraceThreads - 1) / kTraceThreads);
        if (s->sphHasRoot)
            kTrace<kAnyHit, true><<<blocks, kTraceThreads, 0, st>>>(v, rays + off, m, hits ? hits + off : nullptr,
                                                                    occ ? occ + off : nullptr);
        else
            kTrace<kAnyHit, false><<<blocks, kTraceThreads, 0, st>>>(v, rays + off, m, hits ? hits + off : nullptr,
                                                                     occ ? occ + off : nullptr);
        CR_LAUNCH_CHECK();
    }
    return CR_OK;
}

}  // namespace

int traceClosestDevice(cr_scene* s, const cr_ray* rays, uint64_t n, cr_hit* hits, cudaStream_t st) {
    return launchTrace<false>(s, rays, n, hits, nullptr, st);
}

int traceOccludedDevice(cr_scene* s, const cr_ray* rays, uint64_t n, uint8_t* occ, cudaStream_t st) {
    return launchTrace<true>(s, rays, n, nullptr, occ, st);
}

}  // namespace cr

using namespace cr;

namespace {

constexpr uint64_t kChunk = 1ull << 21;  // rays per pipelined chunk (64 MiB of rays)

int ensureStaging(cr_scene* s) {
    if (s->stageCap) return CR_OK;
    for (int k = 0; k < 2; k++) {
        CR_CUDA(cudaStreamCreateWithFlags(&s->streams[k], cudaStreamNonBlocking));
        CR_CUDA(cudaMalloc(&s->stageRays[k], kChunk * sizeof(cr_ray)));
        CR_CUDA(cudaMalloc(&s->stageHits[k], kChunk * sizeof(cr_hit)));
        CR_CUDA(cudaMalloc(&s->stageOcc[k], kChunk));
    }
    s->stageCap = kChunk;
    return CR_OK;
}

// Host-buffer query: chunks alternate between two streams so that the
// copy-in of one chunk overlaps the traversal and copy-out of the other.
template <bool kOcc>
int traceHost(cr_scene* s, const cr_ray* rays, uint64_t n, void* out) {
    if (!s) return fail(CR_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (n == 0) return CR_OK;
    if (!rays || !out) return fail(CR_ERR_INVALID_ARGUMENT, "rays / output is NULL");
    CR_CUDA(cudaSetDevice(s->device));
    int rc = ensureStaging(s);
    if (rc) return rc;
    for (uint64_t off = 0, k = 0; off < n; off += kChunk, k++) {
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
    uint32_t err = 0;
    CR_CUDA(cudaMemcpy(&err, s->errFlags, 4, cudaMemcpyDeviceToHost));
    if (err) return fail(CR_ERR_DEVICE, "traversal reported device error flags 0x%x", err);
    return CR_OK;
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
