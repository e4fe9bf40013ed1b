// cr_cache.cu -- path tracing with an online-trained neural radiance cache.
// This integrator has no counterpart in the reference; it extends the plain
// path tracer (cr_path.cuh, the reference's estimator) as follows.
//
// One frame = one sample per pixel:
//   1. kRenderCached traces every pixel's path with the reference's
//      estimator.  A rendering path stops at the query vertex (vertex 1 =
//      the hit of the first bounce) and records a cache query: the vertex's
//      position, outgoing direction and roughness, and the path throughput
//      beta there.  A training path (one pixel in `train_every`, chosen by a
//      hash of pixel and sample index) is traced to its end by the plain
//      tracer, so its own film contribution is unbiased; every vertex v >= 1
//      of it yields a training record: inputs at v and the target
//      (L_path - L_before_v) / beta_v, the radiance the path gathered from v
//      on, as seen from v.
//   2. The network evaluates all queries (tensor-core inference).
//   3. kSplatCached adds L_before + beta * max(cache, 0) of every rendering
//      path (and the full L of every training path) into the film with the
//      reference's triangle filter.
//   4. train_steps Adam steps on the frame's training records.
// The cache learns L_o(x, w_o) of the reference estimator itself, so a
// perfect cache makes the cached image unbiased with respect to the plain
// one; its error is measured against the plain tracer's image.

#include <cstring>

#include "cr_internal.cuh"
#include "cr_mlp.cuh"
#include "cr_path.cuh"
#include "cr_wavefront.cuh"

namespace cr {
namespace {

constexpr int kMaxRecords = 16;
constexpr float kMaxTarget = 1e4f;

struct CacheParams {
    float3 sceneMin, sceneInvExtent;
    uint32_t queryVertex;
    uint32_t trainEvery;
    uint32_t trainCap;
};

struct SampleRec {
    float4 a;  // radiance before the query (or the full path radiance), film x
    float4 b;  // film y, query index (bits; CR_MISS = none), 0, 0
};

__device__ __forceinline__ float roughnessOf(const MaterialGpu& m) {
    if (m.type == CR_MATERIAL_PRINCIPLED) return m.rough;
    if (m.type == CR_MATERIAL_PHONG) return fminf(sqrtf(2.0f / (m.shininess + 2.0f)), 1.0f);
    return 1.0f;
}

__device__ __forceinline__ void features(const CacheParams& cp, const Isect& it, const MaterialGpu& m, float f[7]) {
    const float3 p = mul(sub(it.posW, cp.sceneMin), 1.0f);
    f[0] = fminf(fmaxf(p.x * cp.sceneInvExtent.x, 0.0f), 1.0f);
    f[1] = fminf(fmaxf(p.y * cp.sceneInvExtent.y, 0.0f), 1.0f);
    f[2] = fminf(fmaxf(p.z * cp.sceneInvExtent.z, 0.0f), 1.0f);
    f[3] = (it.viewW.x + 1.0f) * 0.5f;
    f[4] = (it.viewW.y + 1.0f) * 0.5f;
    f[5] = (it.viewW.z + 1.0f) * 0.5f;
    f[6] = roughnessOf(m);
}

struct QueryHooks {
    const CacheParams* cp;
    bool queried;
    float f[7];
    Spec beta;
    __device__ __forceinline__ bool atVertex(uint32_t depth, const Isect& it, const MaterialGpu& m, const Spec& b,
                                             const Spec&) {
        if (depth != cp->queryVertex) return false;
        features(*cp, it, m, f);
        beta = b;
        queried = true;
        return true;
    }
};

struct TrainHooks {
    const CacheParams* cp;
    int n;
    float f[kMaxRecords][7];
    Spec beta[kMaxRecords];
    Spec before[kMaxRecords];
    __device__ __forceinline__ bool atVertex(uint32_t depth, const Isect& it, const MaterialGpu& m, const Spec& b,
                                             const Spec& radiance) {
        if (depth >= 1 && n < kMaxRecords) {
            features(*cp, it, m, f[n]);
            beta[n] = b;
            before[n] = radiance;
            n++;
        }
        return false;
    }
};

__device__ __forceinline__ uint32_t hash3(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t h = a * 0x8da6b343u ^ b * 0xd8163841u ^ c * 0xcb1ab31fu;
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    h *= 0x846ca68bu;
    h ^= h >> 16;
    return h;
}

__device__ __forceinline__ bool finite3(Spec s) { return isfinite(s.r) && isfinite(s.g) && isfinite(s.b); }

__global__ void __launch_bounds__(256) kRenderCached(const SceneView sc, const CameraGpu cam, const Params p,
                                                     const CacheParams cp, SampleRec* __restrict__ samples,
                                                     float* __restrict__ qIn, float* __restrict__ qBeta,
                                                     uint32_t* __restrict__ qCount, float* __restrict__ tIn,
                                                     float* __restrict__ tTarget, uint32_t* __restrict__ tCount,
                                                     unsigned long long* __restrict__ rayCounter) {
    const uint32_t x = blockIdx.x * 16 + threadIdx.x, y = blockIdx.y * 16 + threadIdx.y;
    PathCtx c{sc, 0u, SpectralPath{}};
    if (x < cam.width && y < cam.height) {
        const uint32_t si = p.first;
        const bool train = cp.trainEvery > 0 && hash3(x, y, si) % cp.trainEvery == 0;
        float2 pix;
        Spec L;
        uint32_t q = CR_MISS;
        if (train) {
            TrainHooks hk;
            hk.cp = &cp;
            hk.n = 0;
            L = tracePath(c, cam, p, x, y, si, pix, hk);
            for (int r = 0; r < hk.n; r++) {
                const Spec be = hk.beta[r];
                const Spec d = sub(L, hk.before[r]);
                const Spec t = Spec{be.r > 0.0f ? d.r / be.r : 0.0f, be.g > 0.0f ? d.g / be.g : 0.0f,
                                    be.b > 0.0f ? d.b / be.b : 0.0f};
                // targets beyond kMaxTarget come from near-zero throughputs,
                // not from the scene's radiance; they are left out
                if (!finite3(t) || maxValue(be) <= 0.0f || maxValue(t) > kMaxTarget) continue;
                const uint32_t idx = atomicAdd(tCount, 1u);  // counts records beyond the cap too
                if (idx >= cp.trainCap) continue;
                for (int k = 0; k < 7; k++) tIn[(size_t)idx * 7 + k] = hk.f[r][k];
                tTarget[(size_t)idx * 3 + 0] = t.r;
                tTarget[(size_t)idx * 3 + 1] = t.g;
                tTarget[(size_t)idx * 3 + 2] = t.b;
            }
        } else {
            QueryHooks hk;
            hk.cp = &cp;
            hk.queried = false;
            L = tracePath(c, cam, p, x, y, si, pix, hk);
            if (hk.queried && finite3(hk.beta) && maxValue(hk.beta) > 0.0f) {
                q = atomicAdd(qCount, 1u);
                for (int k = 0; k < 7; k++) qIn[(size_t)q * 7 + k] = hk.f[k];
                qBeta[(size_t)q * 3 + 0] = hk.beta.r;
                qBeta[(size_t)q * 3 + 1] = hk.beta.g;
                qBeta[(size_t)q * 3 + 2] = hk.beta.b;
            }
        }
        SampleRec rec;
        rec.a = make_float4(L.r, L.g, L.b, pix.x);
        rec.b = make_float4(pix.y, __uint_as_float(q), 0.0f, 0.0f);
        samples[(size_t)y * cam.width + x] = rec;
    }
    uint32_t r = c.rays;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if (((threadIdx.y * 16 + threadIdx.x) & 31) == 0) atomicAdd(rayCounter, (unsigned long long)r);
}

// SensorData::addSample (Core/Sensor.cu:19-43) of each pixel's final sample.
__global__ void kSplatCached(const SampleRec* __restrict__ samples, const float* __restrict__ qBeta,
                             const float* __restrict__ qOut, uint64_t count, uint32_t W, uint32_t H,
                             float* __restrict__ filmRgb, float* __restrict__ filmW) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const SampleRec s = samples[i];
    Spec L = sp(s.a.x, s.a.y, s.a.z);
    const uint32_t q = __float_as_uint(s.b.y);
    if (q != CR_MISS) {
        const Spec c = sp(fmaxf(qOut[(size_t)q * 3 + 0], 0.0f), fmaxf(qOut[(size_t)q * 3 + 1], 0.0f),
                          fmaxf(qOut[(size_t)q * 3 + 2], 0.0f));
        L = add(L, mul(sp(qBeta[(size_t)q * 3 + 0], qBeta[(size_t)q * 3 + 1], qBeta[(size_t)q * 3 + 2]), c));
    }
    if (!finite3(L)) return;
    const float px = s.a.w, py = s.b.x;
    int xa = max((int)floorf(px - 1.0f), 0), ya = max((int)floorf(py - 1.0f), 0);
    int xb = min((int)ceilf(px + 1.0f), (int)W - 1), yb = min((int)ceilf(py + 1.0f), (int)H - 1);
    for (int yy = ya; yy <= yb; yy++) {
        for (int xx = xa; xx <= xb; xx++) {
            const float dx = px - ((float)xx + 0.5f), dy = py - ((float)yy + 0.5f);
            const float w = smax(0.0f, 1.0f - fabsf(dx)) * smax(0.0f, 1.0f - fabsf(dy));
            if (w == 0.0f) continue;
            const size_t pi = (size_t)yy * W + xx;
            atomicAdd(filmRgb + 3 * pi + 0, L.r * w);
            atomicAdd(filmRgb + 3 * pi + 1, L.g * w);
            atomicAdd(filmRgb + 3 * pi + 2, L.b * w);
            atomicAdd(filmW + pi, w);
        }
    }
}

// The cached integrator on the wavefront schedule (cr_wavefront.cuh).  The
// megakernel form above keeps a warp busy until its slowest path ends, and
// one training path in `train_every` runs to full depth, so nearly every
// warp of rendering paths (which stop at the query vertex) waits for one;
// here the short paths leave the queue after their query and only the
// training paths keep bouncing.  Per path the estimator, the sampler
// sequence, the queries and the training records are the megakernel's.
struct CachedMode;

struct WfCacheHooks {
    const CachedMode* m;
    bool train;
    uint32_t q, slot, nRec;
    __device__ __forceinline__ bool atVertex(uint32_t depth, const Isect& it, const MaterialGpu& mat, const Spec& b,
                                             const Spec& radiance);
};

struct CachedMode {
    using Hooks = WfCacheHooks;
    CacheParams cp;
    uint32_t width, height;
    uint32_t first;    // sample index of the wave's first frame

    float* qIn;
    float* qBeta;
    uint32_t* qCount;
    float* recIn;      // per training path slot: kMaxRecords x 7 inputs
    float* recBeta;    // kMaxRecords x 3
    float* recBefore;  // kMaxRecords x 3
    uint32_t* slotCount;
    uint32_t slotCap;
    float* tIn;
    float* tTarget;
    uint32_t* tCount;
    SampleRec* samples;

    __device__ __forceinline__ Hooks hooks(const WfState& st, uint32_t k, const uint4& meta) const {
        const uint4 a = st.aux[k];
        return Hooks{this, cp.trainEvery > 0 && hash3(meta.x, meta.y, meta.z) % cp.trainEvery == 0, a.x, a.y, a.z};
    }
    __device__ __forceinline__ void keep(const WfState& st, uint32_t k, const Hooks& h) const {
        st.aux[k] = make_uint4(h.q, h.slot, h.nRec, 0u);
    }
    template <class Src>
    __device__ __forceinline__ void end(const Src&, uint32_t, const WfState&, uint32_t, const uint4& meta,
                                        const PathCtx&, const Spec& L, float2 pix, const Hooks& h) const {
        SampleRec rec;
        rec.a = make_float4(L.r, L.g, L.b, pix.x);
        rec.b = make_float4(pix.y, __uint_as_float(h.q), 0.0f, 0.0f);
        samples[((size_t)(meta.z - first) * height + meta.y) * width + meta.x] = rec;
        if (!h.train || h.slot >= slotCap) return;
        const size_t r0 = (size_t)h.slot * kMaxRecords;
        for (uint32_t r = 0; r < h.nRec; r++) {
            const size_t ri = r0 + r;
            const Spec be = sp(recBeta[ri * 3 + 0], recBeta[ri * 3 + 1], recBeta[ri * 3 + 2]);
            const Spec d = sub(L, sp(recBefore[ri * 3 + 0], recBefore[ri * 3 + 1], recBefore[ri * 3 + 2]));
            const Spec t = Spec{be.r > 0.0f ? d.r / be.r : 0.0f, be.g > 0.0f ? d.g / be.g : 0.0f,
                                be.b > 0.0f ? d.b / be.b : 0.0f};
            if (!finite3(t) || maxValue(be) <= 0.0f || maxValue(t) > kMaxTarget) continue;
            const uint32_t idx = atomicAdd(tCount, 1u);  // counts records beyond the cap too
            if (idx >= cp.trainCap) continue;
            for (int j = 0; j < 7; j++) tIn[(size_t)idx * 7 + j] = recIn[ri * 7 + j];
            tTarget[(size_t)idx * 3 + 0] = t.r;
            tTarget[(size_t)idx * 3 + 1] = t.g;
            tTarget[(size_t)idx * 3 + 2] = t.b;
        }
    }
};

// TrainHooks / QueryHooks with their state in the path's aux record.
__device__ __forceinline__ bool WfCacheHooks::atVertex(uint32_t depth, const Isect& it, const MaterialGpu& mat,
                                                       const Spec& b, const Spec& radiance) {
    if (train) {
        if (depth >= 1 && nRec < kMaxRecords) {
            if (slot == CR_MISS) slot = atomicAdd(m->slotCount, 1u);
            if (slot < m->slotCap) {
                const size_t ri = (size_t)slot * kMaxRecords + nRec;
                float f[7];
                features(m->cp, it, mat, f);
                for (int j = 0; j < 7; j++) m->recIn[ri * 7 + j] = f[j];
                m->recBeta[ri * 3 + 0] = b.r;
                m->recBeta[ri * 3 + 1] = b.g;
                m->recBeta[ri * 3 + 2] = b.b;
                m->recBefore[ri * 3 + 0] = radiance.r;
                m->recBefore[ri * 3 + 1] = radiance.g;
                m->recBefore[ri * 3 + 2] = radiance.b;
                nRec++;
            }
        }
        return false;
    }
    if (depth != m->cp.queryVertex) return false;
    if (finite3(b) && maxValue(b) > 0.0f) {
        float f[7];
        features(m->cp, it, mat, f);
        q = atomicAdd(m->qCount, 1u);
        for (int j = 0; j < 7; j++) m->qIn[(size_t)q * 7 + j] = f[j];
        m->qBeta[(size_t)q * 3 + 0] = b.r;
        m->qBeta[(size_t)q * 3 + 1] = b.g;
        m->qBeta[(size_t)q * 3 + 2] = b.b;
    }
    return true;
}

}  // namespace

// Per-scene buffers of the cached integrator (sized for the film).
struct CacheBuffers {
    uint64_t pixels = 0;
    uint32_t frames = 0;  // frames per wave the per-path buffers hold
    uint32_t trainCap = 0;
    SampleRec* samples = nullptr;
    float* qIn = nullptr;
    float* qBeta = nullptr;
    float* qOut = nullptr;
    float* tIn = nullptr;
    float* tTarget = nullptr;
    uint32_t* counters = nullptr;  // [0] queries, [1] training records, [2] training path slots
    uint32_t slotCap = 0;          // training paths with records (wavefront form)
    float* recIn = nullptr;
    float* recBeta = nullptr;
    float* recBefore = nullptr;
    // adaptive training-path spacing carried from one call to the next (a
    // renderer dispatching one frame per call still converges)
    uint32_t teStart = 0;    // the start value it was adapted from
    uint32_t teAdapted = 0;  // the spacing for the next frame
};

void freeCacheBuffers(void* p) {
    CacheBuffers* b = static_cast<CacheBuffers*>(p);
    if (!b) return;
    void* ptrs[] = {b->samples, b->qIn, b->qBeta, b->qOut, b->tIn, b->tTarget, b->counters, b->recIn, b->recBeta,
                    b->recBefore};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    delete b;
}

namespace {

// frames: frames per wave; the sample and query buffers hold px x frames
// entries, the training buffers trainCap records (all frames of a wave).
int ensureCacheBuffers(cr_scene* s, uint32_t frames, uint32_t trainCap, uint32_t slotCap, CacheBuffers** out) {
    const uint64_t px = (uint64_t)s->cam.width * s->cam.height;
    CacheBuffers* b = static_cast<CacheBuffers*>(s->cacheBuffers);
    if (b && b->pixels == px && b->frames >= frames && b->trainCap >= trainCap && b->slotCap >= slotCap) {
        *out = b;
        return CR_OK;
    }
    CR_CUDA(cudaDeviceSynchronize());  // earlier renders may still use the old buffers
    freeCacheBuffers(b);
    s->cacheBuffers = nullptr;
    b = new CacheBuffers();
    s->cacheBuffers = b;
    b->pixels = px;
    b->frames = frames;
    b->trainCap = trainCap;
    const uint64_t n = px * frames;
    CR_CUDA(cudaMalloc(&b->samples, n * sizeof(SampleRec)));
    CR_CUDA(cudaMalloc(&b->qIn, n * kMlpInputs * sizeof(float)));
    CR_CUDA(cudaMalloc(&b->qBeta, n * 3 * sizeof(float)));
    CR_CUDA(cudaMalloc(&b->qOut, n * 3 * sizeof(float)));
    CR_CUDA(cudaMalloc(&b->tIn, (size_t)trainCap * kMlpInputs * sizeof(float)));
    CR_CUDA(cudaMalloc(&b->tTarget, (size_t)trainCap * 3 * sizeof(float)));
    CR_CUDA(cudaMalloc(&b->counters, 3 * sizeof(uint32_t)));
    b->slotCap = slotCap;
    if (slotCap) {
        CR_CUDA(cudaMalloc(&b->recIn, (size_t)slotCap * kMaxRecords * kMlpInputs * sizeof(float)));
        CR_CUDA(cudaMalloc(&b->recBeta, (size_t)slotCap * kMaxRecords * 3 * sizeof(float)));
        CR_CUDA(cudaMalloc(&b->recBefore, (size_t)slotCap * kMaxRecords * 3 * sizeof(float)));
    }
    *out = b;
    return CR_OK;
}

}  // namespace

int renderCached(cr_scene* s, const cr_integrator_config* cfg, const cr_cache_config* cc, MlpState* mlp,
                 uint32_t frames, uint32_t first, cudaStream_t st, cr_cache_stats* stats) {
    const uint32_t trainCap = cc->train_samples ? cc->train_samples : 8192u;
    const bool wavefront = !(cfg->flags & CR_RENDER_MEGAKERNEL);
    CacheParams cp;
    float3 mn = s->rootMin, mx = s->rootMax;
    if (cc->scene_max[0] > cc->scene_min[0]) {
        mn = mk3(cc->scene_min[0], cc->scene_min[1], cc->scene_min[2]);
        mx = mk3(cc->scene_max[0], cc->scene_max[1], cc->scene_max[2]);
    }
    const float3 ext = sub(mx, mn);
    cp.sceneMin = mn;
    cp.sceneInvExtent = mk3(ext.x > 0 ? 1.0f / ext.x : 0.0f, ext.y > 0 ? 1.0f / ext.y : 0.0f,
                            ext.z > 0 ? 1.0f / ext.z : 0.0f);
    cp.queryVertex = cc->query_vertex;
    // train_every 0 (adaptive): start at about train_samples records per
    // frame for ~3 records per training path, then after every frame scale the
    // spacing of the training paths by (records produced / train_samples),
    // by at most 2x per frame and never below half the start.  Training paths
    // run to full depth, so more of them than the batch can use only cost time.
    const uint64_t px = (uint64_t)s->cam.width * s->cam.height;
    const bool adaptive = cc->train_every == 0;
    const uint32_t te0 = adaptive ? (uint32_t)std::max<uint64_t>(1, (px * 3 + trainCap / 2) / trainCap)
                                  : cc->train_every;
    const uint32_t teMin = adaptive ? std::max(1u, te0 / 2) : te0;
    const uint32_t teMax = (uint32_t)std::max<uint64_t>(te0, std::min<uint64_t>(px, 1u << 24));
    cp.trainEvery = te0;
    cp.trainCap = trainCap;
    // training paths of a frame: px / trainEvery on average (the hash picks
    // them); room for four times that at the smallest spacing, beyond which a
    // path keeps no records
    //
    // Frames per wave (wavefront form).  After the query vertex only the
    // training paths are live, and kWfFinish runs their remaining bounces as
    // one serial chain per path, which a frame alone would wait for; a wave
    // of several frames waits for it once.  Up to 8 frames, or 2^23 paths.
    // Each frame of a wave still gets its own Adam steps, on its share of the
    // wave's records; the frames of a wave share the network they start with.
    WfBuffers* wb = nullptr;
    uint32_t waveCap = 0;
    uint32_t F = 1;
    if (wavefront) {
        F = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(std::min<uint64_t>(8, frames), (1ull << 23) / px));
        int rcw = ensureWavefrontWave(s->wfBuffers, px * F, s->nMats + 2, wb, waveCap);
        if (rcw) return rcw;
        clearError();
        F = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(F, waveCap / px));
    }
    const uint32_t slotCap =
        wavefront ? (uint32_t)std::min<uint64_t>(px * F, 4 * (px * F / teMin) + 4096) : 0u;
    CacheBuffers* b = nullptr;
    int rc = ensureCacheBuffers(s, F, trainCap * F, slotCap, &b);
    if (rc) return rc;
    if (adaptive && b->teStart == te0 && b->teAdapted) cp.trainEvery = b->teAdapted;
    Params p;
    p.maxDepth = cfg->max_depth;
    p.rrThreshold = cfg->rr_threshold;
    p.useMIS = cfg->use_mis ? 1u : 0u;
    p.spp = 1;
    p.sppPerBlock = 1;
    p.spectral = 0;
    p.wb = mk3(1.0f, 1.0f, 1.0f);
    const uint32_t W = s->cam.width, H = s->cam.height;
    dim3 grid((W + 15) / 16, (H + 15) / 16), block(16, 16);
    const uint32_t steps = cc->train_steps ? cc->train_steps : 1u;
    uint32_t lastTrain = 0;
    for (uint32_t f = 0; f < frames;) {
        const uint32_t fw = std::min(F, frames - f);  // frames in this wave
        p.first = first + f;
        p.spp = fw;
        cp.trainCap = trainCap * fw;
        CR_CUDA(cudaMemsetAsync(b->counters, 0, 3 * sizeof(uint32_t), st));
        if (wavefront) {
            const CachedMode mode{cp,          W,          H,         p.first,        b->qIn,
                                  b->qBeta,    b->counters, b->recIn, b->recBeta,     b->recBefore,
                                  b->counters + 2, slotCap, b->tIn,   b->tTarget,     b->counters + 1,
                                  b->samples};
            const uint64_t paths = px * fw;
            for (uint64_t base = 0; base < paths; base += waveCap) {
                // after the query vertex only training paths are live: one
                // launch finishes them
                rc = runWave(oneScene(s, p), mode, wb, base, (uint32_t)std::min<uint64_t>(waveCap, paths - base),
                             p.maxDepth, s->nMats + 2, st, nullptr, 0, cp.queryVertex + 1);
                if (rc) return rc;
            }
        } else {
            kRenderCached<<<grid, block, 0, st>>>(s->view(), s->cam, p, cp, b->samples, b->qIn, b->qBeta,
                                                  b->counters, b->tIn, b->tTarget, b->counters + 1, s->rayCounter);
            CR_LAUNCH_CHECK();
        }
        uint32_t cnt[2];
        CR_CUDA(cudaMemcpyAsync(cnt, b->counters, sizeof(cnt), cudaMemcpyDeviceToHost, st));
        CR_CUDA(cudaStreamSynchronize(st));
        const uint32_t nq = cnt[0], nt = std::min(cnt[1], trainCap * fw);
        const uint32_t teUsed = cp.trainEvery;
        if (adaptive) {
            const double ratio = std::min(2.0, std::max(0.5, (double)cnt[1] / ((double)trainCap * fw)));
            const double te = std::min((double)teMax, std::max((double)teMin, (double)cp.trainEvery * ratio));
            cp.trainEvery = (uint32_t)(te + 0.5);
            b->teStart = te0;
            b->teAdapted = cp.trainEvery;
        }
        rc = mlpInferDevice(mlp, b->qIn, nq, b->qOut, true, st);
        if (rc) return rc;
        const uint64_t nSamples = px * fw;
        kSplatCached<<<(unsigned)((nSamples + 255) / 256), 256, 0, st>>>(b->samples, b->qBeta, b->qOut, nSamples, W,
                                                                       H, s->filmRgb, s->filmW);
        CR_LAUNCH_CHECK();
        if (nt > 0 && !cc->freeze) {
            // train_steps Adam steps per frame, each frame on its share of the
            // wave's records
            for (uint32_t k = 0; k < fw; k++) {
                const uint32_t r0 = (uint32_t)((uint64_t)nt * k / fw), r1 = (uint32_t)((uint64_t)nt * (k + 1) / fw);
                if (r1 <= r0) continue;
                lastTrain = r1 - r0;
                for (uint32_t j = 0; j < steps; j++) {
                    rc = mlpGradDevice(mlp, b->tIn + (size_t)r0 * kMlpInputs, b->tTarget + (size_t)r0 * 3, r1 - r0, st);
                    if (rc) return rc;
                    rc = mlpAdamDevice(mlp, st);
                    if (rc) return rc;
                }
            }
        }
        if (stats) {
            stats->queries += nq;
            stats->train_records += nt;
            stats->frames += fw;
            stats->last_train_every = teUsed;
        }
        f += fw;
    }
    rc = mlpCheck(mlp);
    if (rc) return rc;
    if (stats && lastTrain) {
        float l = 0;
        CR_CUDA(cudaMemcpyAsync(&l, mlpLossPtr(mlp), sizeof(float), cudaMemcpyDeviceToHost, st));
        CR_CUDA(cudaStreamSynchronize(st));
        stats->last_loss = l / (3.0f * (float)lastTrain);
    }
    return CR_OK;
}

}  // namespace cr

using namespace cr;

extern "C" int cr_render_cached(cr_scene* scene, const cr_integrator_config* cfg, const cr_cache_config* cc,
                                cr_mlp* mlp, uint32_t frames, uint32_t first_sample, void* stream,
                                cr_cache_stats* stats) {
    clearError();
    if (!scene || !cfg || !cc || !mlp) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!scene->hasCamera) return fail(CR_ERR_INVALID_ARGUMENT, "scene has no camera; call cr_scene_set_camera");
    if (cfg->max_depth > 1024) return fail(CR_ERR_INVALID_ARGUMENT, "max_depth %u", cfg->max_depth);
    if (cfg->flags & CR_RENDER_SPECTRAL)
        return fail(CR_ERR_UNSUPPORTED, "the radiance cache learns RGB radiance; spectral rendering is not cached");
    if (cfg->flags & ~(CR_RENDER_WAVEFRONT | CR_RENDER_MEGAKERNEL))
        return fail(CR_ERR_INVALID_ARGUMENT, "unknown render flags 0x%x", cfg->flags);
    if ((cfg->flags & CR_RENDER_WAVEFRONT) && (cfg->flags & CR_RENDER_MEGAKERNEL))
        return fail(CR_ERR_INVALID_ARGUMENT, "CR_RENDER_WAVEFRONT and CR_RENDER_MEGAKERNEL exclude each other");
    if (cc->query_vertex == 0 || cc->query_vertex >= cfg->max_depth)
        return fail(CR_ERR_INVALID_ARGUMENT, "query_vertex %u must be in [1, max_depth)", cc->query_vertex);
    CR_CUDA(cudaSetDevice(scene->device));
    return renderCached(scene, cfg, cc, mlp->s, frames, first_sample, static_cast<cudaStream_t>(stream), stats);
}
