// cr_wavefront.cu -- the wavefront variant of pathTraceKernel<useMIS>
// (Core/Integrator.cu:142-227): paths live in HBM between bounces and each
// bounce is three launches over the live paths,
//   extend   the closest-hit query of every live path (a pure traversal
//            kernel), with the hit's material as a sort key;
//   sort     the live paths by material (CUB radix sort), so that the warps
//            of the shade stage run one BSDF and touch one material's data;
//   shade    the bounce after the query (shadeBounce, the megakernel's own
//            code: next-event estimation and MIS with their shadow and BSDF
//            rays, continuation sampling, Russian roulette); surviving paths
//            are appended to the next bounce's queue, ending paths splat
//            their radiance into the film.
// Per path the arithmetic and the sampler's sequence are the megakernel's,
// so the film equals cr_render's up to the order of the film's float adds.
//
// Path state (structure of arrays, 16-byte records):
//   ro    (origin, film x)        rd    (direction, film y)
//   beta  (throughput, depth)     rad   (radiance, 0)
//   meta  (x, y, sample index, sampler state)   inc (sampler increment)
//   hit   (prim, t, u, v) of the extend stage
// Paths run in waves of at most kWaveCap (the whole image x spp when it
// fits), 112 bytes each.

#include <cub/device/device_radix_sort.cuh>

#include "cr_internal.cuh"
#include "cr_math.cuh"
#include "cr_path.cuh"
#include "cr_shading.cuh"
#include "cr_tile.cuh"
#include "cr_traverse.cuh"

namespace cr {
namespace {

constexpr uint32_t kWaveCap = 1u << 21;
constexpr int kWfThreads = 128;

struct WfState {
    float4* ro;
    float4* rd;
    float4* beta;
    float4* rad;
    uint4* meta;
    uint32_t* inc;
    float4* hit;
};

__device__ __forceinline__ void addRays(unsigned long long* counter, uint32_t rays) {
    for (int o = 16; o > 0; o >>= 1) rays += __shfl_xor_sync(0xffffffffu, rays, o);
    if ((threadIdx.x & 31) == 0 && rays) atomicAdd(counter, (unsigned long long)rays);
}

// Camera rays of paths [base, base + n) of the wave sequence: path k is
// pixel k mod (w h) at sample p.first + k / (w h).
__global__ void __launch_bounds__(kWfThreads) kWfInit(const CameraGpu cam, const Params p, WfState st, uint64_t base,
                                                      uint32_t n, uint32_t* __restrict__ queue) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t k = base + i;
    const uint64_t area = (uint64_t)cam.width * cam.height;
    const uint32_t px = (uint32_t)(k % area);
    const uint32_t x = px % cam.width, y = px / cam.width;
    const uint32_t si = p.first + (uint32_t)(k / area);
    Sampler smp(x, y, si);
    float2 pix;
    float3 ro, rd;
    cameraRay(cam, smp, x, y, pix, ro, rd);
    st.ro[i] = make_float4(ro.x, ro.y, ro.z, pix.x);
    st.rd[i] = make_float4(rd.x, rd.y, rd.z, pix.y);
    st.beta[i] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(0u));
    st.rad[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    st.meta[i] = make_uint4(x, y, si, smp.state);
    st.inc[i] = smp.inc;
    queue[i] = i;
}

// The closest-hit query of every live path; key = the material to shade
// (nMats for a miss, nMats + 1 for a sphere light).
__global__ void __launch_bounds__(kWfThreads) kWfExtend(const SceneView sc, WfState st,
                                                        const uint32_t* __restrict__ queue, uint32_t n,
                                                        uint32_t nMats, uint32_t* __restrict__ keys,
                                                        unsigned long long* __restrict__ rayCounter) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    PathCtx c{sc, 0u, SpectralPath{}};
    if (i < n) {
        const uint32_t k = queue[i];
        const float4 o = st.ro[k], d = st.rd[k];
        THit h;
        closest(c, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), h);
        st.hit[k] = make_float4(__uint_as_float(h.prim), h.t, h.u, h.v);
        uint32_t key;
        if (h.prim == CR_MISS) key = nMats;
        else if (h.prim >= kSpherePrim) key = nMats + 1;
        else if (isSphereHit(h.prim)) key = __ldg(sc.sphMat + (h.prim & ~kSphereBit));
        else key = sc.meshes[sc.primToMesh[h.prim]].material_id;
        keys[i] = key;
    }
    addRays(rayCounter, c.rays);
}

// The bounce after the query, for the live paths in material order.
__global__ void __launch_bounds__(kWfThreads) kWfShade(const SceneView sc, const CameraGpu cam, const Params p,
                                                       WfState st, const uint32_t* __restrict__ order, uint32_t n,
                                                       uint32_t depth, uint32_t* __restrict__ next,
                                                       uint32_t* __restrict__ nextCount, float* __restrict__ filmRgb,
                                                       float* __restrict__ filmW,
                                                       unsigned long long* __restrict__ rayCounter) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    PathCtx c{sc, 0u, SpectralPath{}};
    bool push = false;
    uint32_t k = 0;
    if (i < n) {
        k = order[i];
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
        NoHooks hk;
        const bool alive = shadeBounce(c, p, smp, depth, h, ro, rd, beta, radiance, hk);
        if (alive && depth + 1 < p.maxDepth) {
            push = true;
            st.ro[k] = make_float4(ro.x, ro.y, ro.z, o.w);
            st.rd[k] = make_float4(rd.x, rd.y, rd.z, d.w);
            st.beta[k] = make_float4(beta.r, beta.g, beta.b, __uint_as_float(depth + 1));
            st.rad[k] = make_float4(radiance.r, radiance.g, radiance.b, 0.0f);
            st.meta[k] = make_uint4(meta.x, meta.y, meta.z, smp.state);
        } else {
            splatGlobal(cam, make_float2(o.w, d.w), pathSpecToRgb(c.spec, radiance, p.wb), filmRgb, filmW);
        }
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
    addRays(rayCounter, c.rays);
}

// Paths never traced (max depth 0) splat their zero radiance with its weight.
__global__ void kWfSplatAll(const CameraGpu cam, const Params p, WfState st, uint32_t n, float* __restrict__ filmRgb,
                            float* __restrict__ filmW) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    splatGlobal(cam, make_float2(st.ro[i].w, st.rd[i].w), sp(0.0f), filmRgb, filmW);
}

template <class T>
struct Buf {
    T* p = nullptr;
    ~Buf() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)); }
};

inline unsigned blocks(uint64_t n) { return (unsigned)((n + kWfThreads - 1) / kWfThreads); }

}  // namespace

// cr_render with CR_RENDER_WAVEFRONT.  Synchronises with the host once per
// bounce to read the number of live paths.
int renderWavefront(cr_scene* s, const cr_integrator_config* cfg, uint32_t spp, uint32_t first, cudaStream_t stream) {
    if (spp == 0) return CR_OK;
    Params p;
    p.maxDepth = cfg->max_depth;
    p.rrThreshold = cfg->rr_threshold;
    p.useMIS = cfg->use_mis ? 1u : 0u;
    p.spp = spp;
    p.first = first;
    p.sppPerBlock = 1;
    p.spectral = (cfg->flags & CR_RENDER_SPECTRAL) ? 1u : 0u;
    p.wb = whiteBalance();
    const uint64_t total = (uint64_t)s->cam.width * s->cam.height * spp;
    const uint32_t cap = (uint32_t)std::min<uint64_t>(total, kWaveCap);
    Buf<float4> ro, rd, beta, rad, hit;
    Buf<uint4> meta;
    Buf<uint32_t> inc, qa, qb, keysIn, keysOut, valsOut, count;
    CR_CUDA(ro.alloc(cap));
    CR_CUDA(rd.alloc(cap));
    CR_CUDA(beta.alloc(cap));
    CR_CUDA(rad.alloc(cap));
    CR_CUDA(hit.alloc(cap));
    CR_CUDA(meta.alloc(cap));
    CR_CUDA(inc.alloc(cap));
    CR_CUDA(qa.alloc(cap));
    CR_CUDA(qb.alloc(cap));
    CR_CUDA(keysIn.alloc(cap));
    CR_CUDA(keysOut.alloc(cap));
    CR_CUDA(valsOut.alloc(cap));
    CR_CUDA(count.alloc(1));
    uint32_t* countHost = nullptr;
    CR_CUDA(cudaMallocHost(&countHost, sizeof(uint32_t)));
    struct HostFree {
        uint32_t* p;
        ~HostFree() { cudaFreeHost(p); }
    } hostFree{countHost};
    int endBit = 1;
    while (endBit < 32 && (1ull << endBit) < (uint64_t)s->nMats + 2) endBit++;
    size_t sortBytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, sortBytes, keysIn.p, keysOut.p, qa.p, valsOut.p, (int)cap, 0, endBit,
                                    stream);
    Buf<uint8_t> sortTemp;
    CR_CUDA(sortTemp.alloc(sortBytes));
    const WfState st{ro.p, rd.p, beta.p, rad.p, meta.p, inc.p, hit.p};
    const SceneView v = s->view();
    for (uint64_t base = 0; base < total; base += cap) {
        uint32_t n = (uint32_t)std::min<uint64_t>(cap, total - base);
        kWfInit<<<blocks(n), kWfThreads, 0, stream>>>(s->cam, p, st, base, n, qa.p);
        CR_LAUNCH_CHECK();
        if (p.maxDepth == 0) {
            kWfSplatAll<<<blocks(n), kWfThreads, 0, stream>>>(s->cam, p, st, n, s->filmRgb, s->filmW);
            CR_LAUNCH_CHECK();
            continue;
        }
        uint32_t* live = qa.p;
        uint32_t* nextQ = qb.p;
        for (uint32_t depth = 0; depth < p.maxDepth && n > 0; depth++) {
            kWfExtend<<<blocks(n), kWfThreads, 0, stream>>>(v, st, live, n, s->nMats, keysIn.p, s->rayCounter);
            CR_LAUNCH_CHECK();
            CR_CUDA(cub::DeviceRadixSort::SortPairs(sortTemp.p, sortBytes, keysIn.p, keysOut.p, live, valsOut.p,
                                                    (int)n, 0, endBit, stream));
            countLaunch(4);
            CR_CUDA(cudaMemsetAsync(count.p, 0, sizeof(uint32_t), stream));
            kWfShade<<<blocks(n), kWfThreads, 0, stream>>>(v, s->cam, p, st, valsOut.p, n, depth, nextQ, count.p,
                                                           s->filmRgb, s->filmW, s->rayCounter);
            CR_LAUNCH_CHECK();
            CR_CUDA(cudaMemcpyAsync(countHost, count.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
            CR_CUDA(cudaStreamSynchronize(stream));
            n = *countHost;
            std::swap(live, nextQ);
        }
    }
    return CR_OK;
}

}  // namespace cr
