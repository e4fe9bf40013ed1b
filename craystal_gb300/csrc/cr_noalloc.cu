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
// caller.  Every GPU that loads the library holds the 3 MiB until the
// process exits.

#include <mutex>

#include "cr_internal.cuh"

namespace cr {
namespace {

constexpr uint64_t kNoAllocMaxRays = CR_NOALLOC_MAX_RAYS;

static __device__ __align__(256) cr_ray gStageRays[kNoAllocMaxRays];
static __device__ __align__(256) cr_hit gStageHits[kNoAllocMaxRays];

// Device addresses of the two arrays, looked up once per device with that
// device current.  In host code the names gStageRays / gStageHits stand for
// host-side shadows, not for device memory, so only these addresses may be
// handed to a kernel or a copy.
constexpr int kMaxDevices = 64;
struct StageAddr {
    cr_ray* rays = nullptr;
    cr_hit* hits = nullptr;
};
StageAddr gAddr[kMaxDevices];
std::mutex gAddrMutex;

int stageAddresses(int device, StageAddr& out) {
    if (device < 0 || device >= kMaxDevices) return fail(CR_ERR_UNSUPPORTED, "device ordinal %d", device);
    std::lock_guard<std::mutex> lock(gAddrMutex);
    StageAddr& a = gAddr[device];
    if (!a.rays) {
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
    uint32_t err = 0;
    CR_CUDA(cudaMemcpy(&err, scene->errFlags, 4, cudaMemcpyDeviceToHost));
    if (err) return fail(CR_ERR_DEVICE, "traversal reported device error flags 0x%x", err);
    return CR_OK;
}
