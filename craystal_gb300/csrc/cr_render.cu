// cr_render.cu -- the path-tracing megakernel (pathTraceKernel<useMIS>,
// Core/Integrator.cu:142-227, with sampleLight :21-72 and evalMIS :74-140)
// and the film (SensorData::addSample, Core/Sensor.cu:19-43; resolve
// Sensor::createImage, :93-112).
//
// One thread owns one pixel and loops over a run of sample indices; the
// launch covers (16 x 16 pixel tiles) x (runs of samples), so that small
// images still fill the GPU.  Film splats go to an 18 x 18 tile in shared
// memory (cr_tile.cuh) and are added to the global film once per block,
// instead of 16 global atomics per sample in the reference.

#include "cr_internal.cuh"
#include "cr_math.cuh"
#include "cr_shading.cuh"
#include "cr_traverse.cuh"
#include "cr_path.cuh"
#include "cr_tile.cuh"

namespace cr {
namespace {

constexpr int kTileW = 16;

__global__ void __launch_bounds__(kTileW* kTileW) kRender(const SceneView sc, const CameraGpu cam, const Params p,
                                                          float* __restrict__ filmRgb, float* __restrict__ filmW,
                                                          unsigned long long* __restrict__ rayCounter) {
    __shared__ TileSmem<kTileW> sm;
    const uint32_t s0 = blockIdx.z * p.sppPerBlock;
    const uint32_t s1 = min(p.spp, s0 + p.sppPerBlock);
    renderTile<kTileW>(sc, cam, p, blockIdx.x * kTileW, blockIdx.y * kTileW, s0, s1, filmRgb, filmW, rayCounter, sm);
}

__global__ void kResolve(const float* __restrict__ rgb, const float* __restrict__ w, size_t n, float* __restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float ws = w[i];
    out[3 * i + 0] = rgb[3 * i + 0] / ws;
    out[3 * i + 1] = rgb[3 * i + 1] / ws;
    out[3 * i + 2] = rgb[3 * i + 2] / ws;
}

}  // namespace

int renderDevice(cr_scene* s, const cr_integrator_config* cfg, uint32_t spp, uint32_t first, cudaStream_t st) {
    if (spp == 0) return CR_OK;
    Params p;
    p.maxDepth = cfg->max_depth;
    p.rrThreshold = cfg->rr_threshold;
    p.useMIS = cfg->use_mis ? 1u : 0u;
    p.spp = spp;
    p.first = first;
    p.spectral = (cfg->flags & CR_RENDER_SPECTRAL) ? 1u : 0u;
    p.wb = whiteBalance();
    const uint32_t tilesX = (s->cam.width + kTileW - 1) / kTileW, tilesY = (s->cam.height + kTileW - 1) / kTileW;
    // enough blocks to fill every SM several times over, at most 8 samples
    // per thread per launch run
    int dev = 0, sms = 0;
    CR_CUDA(cudaGetDevice(&dev));
    CR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const uint64_t tiles = (uint64_t)tilesX * tilesY;
    const uint64_t wantBlocks = (uint64_t)sms * 32;
    uint32_t runs = (uint32_t)std::min<uint64_t>(spp, std::max<uint64_t>(1, (wantBlocks + tiles - 1) / tiles));
    runs = std::max(runs, (spp + 7) / 8);
    runs = std::min(runs, 65535u);
    p.sppPerBlock = (spp + runs - 1) / runs;
    runs = (spp + p.sppPerBlock - 1) / p.sppPerBlock;
    dim3 grid(tilesX, tilesY, runs), block(kTileW, kTileW, 1);
    kRender<<<grid, block, 0, st>>>(s->view(), s->cam, p, s->filmRgb, s->filmW, s->rayCounter);
    CR_LAUNCH_CHECK();
    return CR_OK;
}

int resolveFilm(cr_scene* s, float* rgbHost) {
    const size_t n = (size_t)s->cam.width * s->cam.height;
    float* d = nullptr;
    CR_CUDA(cudaDeviceSynchronize());
    CR_CUDA(cudaMalloc(&d, n * 3 * sizeof(float)));
    kResolve<<<(unsigned)((n + 255) / 256), 256>>>(s->filmRgb, s->filmW, n, d);
    cudaError_t e = cudaGetLastError();
    countLaunch();
    if (e == cudaSuccess) e = cudaMemcpy(rgbHost, d, n * 3 * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(CR_ERR_CUDA, "film resolve failed: %s", cudaGetErrorString(e));
    return CR_OK;
}

}  // namespace cr

// ---------------------------------------------------------------------------
// batch entry points for single stages: camera rays and BSDF queries
// ---------------------------------------------------------------------------
namespace cr {
namespace {

__global__ void kCameraRays(const CameraGpu cam, const float2* __restrict__ sp, uint64_t n, cr_ray* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 d = cameraDir(cam, sp[i]);
    cr_ray r;
    r.o[0] = cam.pos.x;
    r.o[1] = cam.pos.y;
    r.o[2] = cam.pos.z;
    r.tmin = 0.0f;
    r.d[0] = d.x;
    r.d[1] = d.y;
    r.d[2] = d.z;
    r.tmax = INFINITY;
    out[i] = r;
}

__global__ void kBsdf(const MaterialGpu m, const float3* __restrict__ nrm, const float3* __restrict__ wo,
                      const float3* __restrict__ wi, const float2* __restrict__ u, uint64_t n, float3* __restrict__ wiOut,
                      float3* __restrict__ f, float* __restrict__ pdf) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Frame fr;
    fr.build(nrm[i]);
    Bsdf b;
    b.init(m, fr);
    Spec v;
    float p;
    if (u) {
        float3 w;
        p = 0.0f;
        v = b.sampleEvaluate(u[i], wo[i], w, p);
        wiOut[i] = w;
    } else {
        v = b.evaluate(wo[i], wi[i]);
        p = b.evaluatePdf(wo[i], wi[i]);
    }
    f[i] = mk3(v.r, v.g, v.b);
    pdf[i] = p;
}

__global__ void kTexSample(const SceneView sc, uint32_t tex, const float2* __restrict__ uv, uint64_t n,
                           float4* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = texSample(sc, tex, uv[i]);
}

template <class T>
struct Dev {
    T* p = nullptr;
    ~Dev() {
        if (p) cudaFree(p);
    }
};

}  // namespace

MaterialGpu deriveMaterialPublic(const cr_material& m);

}  // namespace cr

using namespace cr;

extern "C" int cr_camera_generate_rays(const cr_camera* cam, const float* sensor_pos, uint64_t n, cr_ray* rays) {
    clearError();
    if (!cam || (n && (!sensor_pos || !rays))) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (cam->width == 0 || cam->height == 0) return fail(CR_ERR_INVALID_ARGUMENT, "sensor size is zero");
    if (n == 0) return CR_OK;
    CameraGpu c;
    const float3 pos = mk3(cam->pos[0], cam->pos[1], cam->pos[2]);
    c.pos = pos;
    c.W = normalize(sub(mk3(cam->target[0], cam->target[1], cam->target[2]), pos));
    c.U = normalize(cross(c.W, mk3(cam->up[0], cam->up[1], cam->up[2])));
    c.V = normalize(cross(c.U, c.W));
    c.halfH = (float)std::tan(((double)cam->fov_y * 0.5) * 0.01745329251994329576923690768489);
    c.halfW = ((float)cam->width / (float)cam->height) * c.halfH;
    c.width = cam->width;
    c.height = cam->height;
    Dev<float2> dsp;
    Dev<cr_ray> dr;
    CR_CUDA(cudaMalloc(&dsp.p, n * sizeof(float2)));
    CR_CUDA(cudaMalloc(&dr.p, n * sizeof(cr_ray)));
    CR_CUDA(cudaMemcpy(dsp.p, sensor_pos, n * sizeof(float2), cudaMemcpyHostToDevice));
    kCameraRays<<<(unsigned)((n + 127) / 128), 128>>>(c, dsp.p, n, dr.p);
    CR_LAUNCH_CHECK();
    CR_CUDA(cudaMemcpy(rays, dr.p, n * sizeof(cr_ray), cudaMemcpyDeviceToHost));
    return CR_OK;
}

static int bsdfBatch(const cr_material* mat, const float* n, const float* wo, const float* wi, const float* u,
                     uint64_t count, float* wiOut, float* f, float* pdf) {
    if (!mat || (count && (!n || !wo || !f || !pdf || (!wi && !u) || (u && !wiOut))))
        return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (mat->type > CR_MATERIAL_PHONG) return fail(CR_ERR_INVALID_ARGUMENT, "material type %u", mat->type);
    if (count == 0) return CR_OK;
    const MaterialGpu m = deriveMaterialPublic(*mat);
    Dev<float3> dn, dwo, dwi, dwio, df;
    Dev<float2> du;
    Dev<float> dp;
    const size_t v3 = count * sizeof(float3);
    CR_CUDA(cudaMalloc(&dn.p, v3));
    CR_CUDA(cudaMalloc(&dwo.p, v3));
    CR_CUDA(cudaMalloc(&df.p, v3));
    CR_CUDA(cudaMalloc(&dp.p, count * sizeof(float)));
    CR_CUDA(cudaMemcpy(dn.p, n, v3, cudaMemcpyHostToDevice));
    CR_CUDA(cudaMemcpy(dwo.p, wo, v3, cudaMemcpyHostToDevice));
    if (u) {
        CR_CUDA(cudaMalloc(&du.p, count * sizeof(float2)));
        CR_CUDA(cudaMalloc(&dwio.p, v3));
        CR_CUDA(cudaMemcpy(du.p, u, count * sizeof(float2), cudaMemcpyHostToDevice));
    } else {
        CR_CUDA(cudaMalloc(&dwi.p, v3));
        CR_CUDA(cudaMemcpy(dwi.p, wi, v3, cudaMemcpyHostToDevice));
    }
    kBsdf<<<(unsigned)((count + 127) / 128), 128>>>(m, dn.p, dwo.p, dwi.p, du.p, count, dwio.p, df.p, dp.p);
    CR_LAUNCH_CHECK();
    CR_CUDA(cudaMemcpy(f, df.p, v3, cudaMemcpyDeviceToHost));
    CR_CUDA(cudaMemcpy(pdf, dp.p, count * sizeof(float), cudaMemcpyDeviceToHost));
    if (u) CR_CUDA(cudaMemcpy(wiOut, dwio.p, v3, cudaMemcpyDeviceToHost));
    return CR_OK;
}

extern "C" int cr_bsdf_evaluate(const cr_material* mat, const float* n, const float* wo, const float* wi,
                                uint64_t count, float* f, float* pdf) {
    clearError();
    return bsdfBatch(mat, n, wo, wi, nullptr, count, nullptr, f, pdf);
}

extern "C" int cr_bsdf_sample(const cr_material* mat, const float* n, const float* wo, const float* u,
                              uint64_t count, float* wi, float* f, float* pdf) {
    clearError();
    return bsdfBatch(mat, n, wo, nullptr, u, count, wi, f, pdf);
}

extern "C" int cr_texture_sample(const cr_scene* scene, uint32_t texture, const float* uv, uint64_t n, float* rgba) {
    clearError();
    if (!scene || (n && (!uv || !rgba))) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (texture >= scene->nTex) return fail(CR_ERR_INVALID_ARGUMENT, "texture %u of %u", texture, scene->nTex);
    if (n == 0) return CR_OK;
    CR_CUDA(cudaSetDevice(scene->device));
    Dev<float2> du;
    Dev<float4> dout;
    CR_CUDA(cudaMalloc(&du.p, n * sizeof(float2)));
    CR_CUDA(cudaMalloc(&dout.p, n * sizeof(float4)));
    CR_CUDA(cudaMemcpy(du.p, uv, n * sizeof(float2), cudaMemcpyHostToDevice));
    kTexSample<<<(unsigned)((n + 127) / 128), 128>>>(scene->view(), texture, du.p, n, dout.p);
    CR_LAUNCH_CHECK();
    CR_CUDA(cudaMemcpy(rgba, dout.p, n * sizeof(float4), cudaMemcpyDeviceToHost));
    return CR_OK;
}
