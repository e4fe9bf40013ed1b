// cr_noalloc.cu -- closest-hit queries on host buffers without allocating
// GPU memory.
//
// cr_trace_closest stages rays and hits in device buffers that it allocates
// with cudaMalloc the first time a scene is queried.  Some callers cannot let
// a library allocate: a host application that has already committed its
// whole GPU memory budget to its own pool, a render thread that must not
// block on the implicit device synchronisation cudaMalloc / cudaFree bring,
// or a plugin whose host forbids allocations after start-up.  This entry
// point serves them: it stages through two arrays that live in the library's
// own device image (file-scope __device__ arrays), sized for at most
// kNoAllocMaxRays rays per call (3 MiB in all), and it never calls cudaMalloc,
// cudaFree or any allocating library routine.
//
// The arrays are shared by every call on a device and keep the last call's
// contents; each call overwrites every element it reads, so nothing needs
// clearing, but calls whose work overlaps on the GPU (two host threads, or
// several streams, at once) race on them and must be serialised by the
// caller.
//
// Loading.  Each translation unit of the library is its own module, and
// under CUDA's default lazy module loading a module is loaded on a device
// when it is first used there.  The first call on a device therefore makes
// the driver load this module, whose image holds the 3 MiB, and the
// traversal kernel's module: device memory that the driver, not this
// library, allocates.  A caller whose memory budget is fixed makes that first
// call at start-up, before it commits its budget (or runs with
// CUDA_MODULE_LOADING=EAGER, which loads every module when the context is
// created).  The 3 MiB then stay resident on that device until the process
// exits.

#include <cuda.h>

#include <mutex>

#include "cr_internal.cuh"

namespace cr {
namespace {

constexpr uint64_t kNoAllocMaxRays = CR_NOALLOC_MAX_RAYS;

static __device__ __align__(256) cr_ray gStageRays[kNoAllocMaxRays];
static __device__ __align__(256) cr_hit gStageHits[kNoAllocMaxRays];

// Device addresses of the two arrays, looked up per device with that device
// current.  In host code the names gStageRays / gStageHits stand for
// host-side shadows, not for device memory, so only these addresses may be
// handed to a kernel or a copy.  A module's addresses belong to the context
// it was loaded into: after cudaDeviceReset the device gets a new primary
// context, the module is loaded again and the arrays may move.  Each entry
// therefore records the unique id of the context it was looked up in
// (cuCtxGetId), and a call in another context looks the addresses up again.
constexpr int kMaxDevices = 64;
struct StageAddr {
    unsigned long long ctxId = 0;
    cr_ray* rays = nullptr;
    cr_hit* hits = nullptr;
};
StageAddr gAddr[kMaxDevices];
std::mutex gAddrMutex;

// cuCtxGetId from the driver the runtime uses (no link to libcuda).
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

CtxGetIdFn ctxGetIdFn() {
    static const CtxGetIdFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<CtxGetIdFn>(f);
    }();
    return fn;
}

// The id of the current context; 0 when it cannot be had, which makes every
// call look the addresses up afresh (cheap once the module is loaded).
unsigned long long currentContextId() {
    const CtxGetIdFn fn = ctxGetIdFn();
    unsigned long long id = 0;
    if (!fn || fn(nullptr, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Called with `device` current.
int stageAddresses(int device, StageAddr& out) {
    if (device < 0 || device >= kMaxDevices) return fail(CR_ERR_UNSUPPORTED, "device ordinal %d", device);
    const unsigned long long ctx = currentContextId();
    std::lock_guard<std::mutex> lock(gAddrMutex);
    StageAddr& a = gAddr[device];
    if (!a.rays || ctx == 0 || a.ctxId != ctx) {
        void* r = nullptr;
        void* h = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&r, gStageRays);
        if (e != cudaSuccess)
            return fail(CR_ERR_CUDA, "cudaGetSymbolAddress(staging rays) failed: %s", cudaGetErrorString(e));
        e = cudaGetSymbolAddress(&h, gStageHits);
        if (e != cudaSuccess)
            return fail(CR_ERR_CUDA, "cudaGetSymbolAddress(staging hits) failed: %s", cudaGetErrorString(e));
        a.rays = static_cast<cr_ray*>(r);
        a.hits = static_cast<cr_hit*>(h);
        a.ctxId = ctx;
    }
    out = a;
    return CR_OK;
}

}  // namespace
}  // namespace cr

using namespace cr;

extern "C" int cr_trace_closest_noalloc(cr_scene* scene, const cr_ray* rays, uint64_t n, cr_hit* hits,
                                        void* stream) {
    clearError();
    if (!scene) return fail(CR_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (n > kNoAllocMaxRays)
        return fail(CR_ERR_INVALID_ARGUMENT,
                    "cr_trace_closest_noalloc takes at most %llu rays per call (got %llu); split the batch or use "
                    "cr_trace_closest",
                    (unsigned long long)kNoAllocMaxRays, (unsigned long long)n);
    if (n == 0) return CR_OK;
    if (!rays || !hits) return fail(CR_ERR_INVALID_ARGUMENT, "rays / hits is NULL");
    CR_CUDA(cudaSetDevice(scene->device));
    StageAddr a;
    int rc = stageAddresses(scene->device, a);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CR_CUDA(cudaMemcpyAsync(a.rays, rays, n * sizeof(cr_ray), cudaMemcpyHostToDevice, st));
    rc = traceClosestDevice(scene, a.rays, n, a.hits, st, false);
    if (rc) return rc;
    CR_CUDA(cudaMemcpyAsync(hits, a.hits, n * sizeof(cr_hit), cudaMemcpyDeviceToHost, st));
    CR_CUDA(cudaStreamSynchronize(st));
    // the scene's error word is shared by all its queries: this reports (and
    // clears) whatever is set now, which includes errors of earlier device
    // queries on the scene that no call has reported yet
    return takeDeviceErrors(scene, "traversal");
}
