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
    static constexpr bool kAllowLean = false;
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

// One cached render in progress: its configuration and the state kept
// between waves.
struct CachedJob {
    cr_scene* s = nullptr;
    cr_integrator_config cfg{};
    cr_cache_config cc{};
    MlpState* mlp = nullptr;
    uint32_t frames = 0, first = 0;
    cr_cache_stats* stats = nullptr;
    uint32_t* cnt = nullptr;  // the wave's query and record counts, read back (page-locked when batched)
    // derived by cachedSetup
    bool wavefront = true, adaptive = true;
    uint64_t px = 0;
    uint32_t trainCap = 0, te0 = 0, teMin = 0, teMax = 0, F = 1, waveCap = 0, slotCap = 0, steps = 1;
    uint32_t lastTrain = 0, f = 0, fw = 0;
    CacheParams cp{};
    Params p{};
    WfBuffers* wb = nullptr;
    CacheBuffers* b = nullptr;
};

// Sets up a cached render of j.frames frames: the network input
// normalisation, the training-path spacing, the frames per wave and the
// buffers.
int cachedSetup(CachedJob& j) {
    cr_scene* s = j.s;
    const cr_cache_config* cc = &j.cc;
    j.trainCap = cc->train_samples ? cc->train_samples : 8192u;
    j.wavefront = !(j.cfg.flags & CR_RENDER_MEGAKERNEL);
    CacheParams& cp = j.cp;
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
    j.px = (uint64_t)s->cam.width * s->cam.height;
    j.adaptive = cc->train_every == 0;
    j.te0 = j.adaptive ? (uint32_t)std::max<uint64_t>(1, (j.px * 3 + j.trainCap / 2) / j.trainCap) : cc->train_every;
    j.teMin = j.adaptive ? std::max(1u, j.te0 / 2) : j.te0;
    j.teMax = (uint32_t)std::max<uint64_t>(j.te0, std::min<uint64_t>(j.px, 1u << 24));
    cp.trainEvery = j.te0;
    cp.trainCap = j.trainCap;
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
    j.F = 1;
    if (j.wavefront) {
        j.F = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(std::min<uint64_t>(8, j.frames), (1ull << 23) / j.px));
        int rcw = ensureWavefrontWave(s->wfBuffers, j.px * j.F, s->nMats + 2, j.wb, j.waveCap);
        if (rcw) return rcw;
        clearError();
        j.F = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(j.F, j.waveCap / j.px));
    }
    j.slotCap = j.wavefront ? (uint32_t)std::min<uint64_t>(j.px * j.F, 4 * (j.px * j.F / j.teMin) + 4096) : 0u;
    int rc = ensureCacheBuffers(s, j.F, j.trainCap * j.F, j.slotCap, &j.b);
    if (rc) return rc;
    if (j.adaptive && j.b->teStart == j.te0 && j.b->teAdapted) cp.trainEvery = j.b->teAdapted;
    Params& p = j.p;
    p.maxDepth = j.cfg.max_depth;
    p.rrThreshold = j.cfg.rr_threshold;
    p.useMIS = j.cfg.use_mis ? 1u : 0u;
    p.spp = 1;
    p.sppPerBlock = 1;
    p.spectral = 0;
    p.wb = mk3(1.0f, 1.0f, 1.0f);
    j.steps = cc->train_steps ? cc->train_steps : 1u;
    j.lastTrain = 0;
    j.f = 0;
    return CR_OK;
}

// Issues the next wave of frames on st (the paths up to their query vertex,
// the training paths to their end) and the copy of its two record counters
// to j.cnt; the caller waits for st before cachedFinishWave.
int cachedIssueWave(CachedJob& j, cudaStream_t st) {
    cr_scene* s = j.s;
    CacheBuffers* b = j.b;
    CacheParams& cp = j.cp;
    Params& p = j.p;
    j.fw = std::min(j.F, j.frames - j.f);  // frames in this wave
    p.first = j.first + j.f;
    p.spp = j.fw;
    cp.trainCap = j.trainCap * j.fw;
    CR_CUDA(cudaMemsetAsync(b->counters, 0, 3 * sizeof(uint32_t), st));
    const uint32_t W = s->cam.width, H = s->cam.height;
    if (j.wavefront) {
        const CachedMode mode{cp,          W,          H,         p.first,        b->qIn,
                              b->qBeta,    b->counters, b->recIn, b->recBeta,     b->recBefore,
                              b->counters + 2, j.slotCap, b->tIn,   b->tTarget,     b->counters + 1,
                              b->samples};
        const uint64_t paths = j.px * j.fw;
        for (uint64_t base = 0; base < paths; base += j.waveCap) {
            // after the query vertex only training paths are live: one
            // launch finishes them
            int rc = runWave(oneScene(s, p), mode, j.wb, base, (uint32_t)std::min<uint64_t>(j.waveCap, paths - base),
                             p.maxDepth, s->nMats + 2, st, nullptr, 0, cp.queryVertex + 1);
            if (rc) return rc;
        }
    } else {
        dim3 grid((W + 15) / 16, (H + 15) / 16), block(16, 16);
        kRenderCached<<<grid, block, 0, st>>>(s->view(), s->cam, p, cp, b->samples, b->qIn, b->qBeta, b->counters,
                                              b->tIn, b->tTarget, b->counters + 1, s->rayCounter);
        CR_LAUNCH_CHECK();
    }
    CR_CUDA(cudaMemcpyAsync(j.cnt, b->counters, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    return CR_OK;
}

// After the wave's counters are in j.cnt: adapts the training-path spacing,
// then issues on st the inference of the wave's queries, the film splat and
// the frames' training steps.
int cachedFinishWave(CachedJob& j, cudaStream_t st) {
    cr_scene* s = j.s;
    CacheBuffers* b = j.b;
    CacheParams& cp = j.cp;
    const uint32_t fw = j.fw;
    const uint32_t nq = j.cnt[0], nt = std::min(j.cnt[1], j.trainCap * fw);
    const uint32_t teUsed = cp.trainEvery;
    if (j.adaptive) {
        const double ratio = std::min(2.0, std::max(0.5, (double)j.cnt[1] / ((double)j.trainCap * fw)));
        const double te = std::min((double)j.teMax, std::max((double)j.teMin, (double)cp.trainEvery * ratio));
        cp.trainEvery = (uint32_t)(te + 0.5);
        b->teStart = j.te0;
        b->teAdapted = cp.trainEvery;
    }
    int rc = mlpInferDevice(j.mlp, b->qIn, nq, b->qOut, true, st);
    if (rc) return rc;
    const uint64_t nSamples = j.px * fw;
    kSplatCached<<<(unsigned)((nSamples + 255) / 256), 256, 0, st>>>(b->samples, b->qBeta, b->qOut, nSamples,
                                                                   s->cam.width, s->cam.height, s->filmRgb, s->filmW);
    CR_LAUNCH_CHECK();
    if (nt > 0 && !j.cc.freeze) {
        // train_steps Adam steps per frame, each frame on its share of the
        // wave's records
        for (uint32_t k = 0; k < fw; k++) {
            const uint32_t r0 = (uint32_t)((uint64_t)nt * k / fw), r1 = (uint32_t)((uint64_t)nt * (k + 1) / fw);
            if (r1 <= r0) continue;
            j.lastTrain = r1 - r0;
            for (uint32_t q = 0; q < j.steps; q++) {
                rc = mlpTrainStepDevice(j.mlp, b->tIn + (size_t)r0 * kMlpInputs, b->tTarget + (size_t)r0 * 3,
                                        r1 - r0, st);
                if (rc) return rc;
            }
        }
    }
    if (j.stats) {
        j.stats->queries += nq;
        j.stats->train_records += nt;
        j.stats->frames += fw;
        j.stats->last_train_every = teUsed;
    }
    j.f += fw;
    return CR_OK;
}

// Reports a tensor-core wait that ran out and the last training loss
// (synchronises st).
int cachedEnd(CachedJob& j, cudaStream_t st) {
    CR_CUDA(cudaStreamSynchronize(st));
    int rc = mlpCheck(j.mlp);
    if (rc) return rc;
    if (j.stats && j.lastTrain) {
        float l = 0;
        CR_CUDA(cudaMemcpyAsync(&l, mlpLossPtr(j.mlp), sizeof(float), cudaMemcpyDeviceToHost, st));
        CR_CUDA(cudaStreamSynchronize(st));
        j.stats->last_loss = l / (3.0f * (float)j.lastTrain);
    }
    return CR_OK;
}

}  // namespace

int renderCached(cr_scene* s, const cr_integrator_config* cfg, const cr_cache_config* cc, MlpState* mlp,
                 uint32_t frames, uint32_t first, cudaStream_t st, cr_cache_stats* stats) {
    CachedJob j;
    j.s = s;
    j.cfg = *cfg;
    j.cc = *cc;
    j.mlp = mlp;
    j.frames = frames;
    j.first = first;
    j.stats = stats;
    uint32_t cnt[2] = {0, 0};
    j.cnt = cnt;
    int rc = cachedSetup(j);
    if (rc) return rc;
    while (j.f < j.frames) {
        rc = cachedIssueWave(j, st);
        if (rc) return rc;
        CR_CUDA(cudaStreamSynchronize(st));
        rc = cachedFinishWave(j, st);
        if (rc) return rc;
    }
    return cachedEnd(j, st);
}

// Cached renders of n scenes, interleaved wave by wave: every round issues
// the next wave of each unfinished scene on that scene's stream, then, as
// each stream's counters arrive, that scene's inference, splat and training.
// A scene's renders follow the same sequence as renderCached, so its film
// receives the same samples; the scenes' work overlaps on the GPU.
// cnt: 2 x n page-locked words for the counters.
int renderCachedMany(cr_scene* const* scenes, const cr_integrator_config* cfgs, const uint32_t* frames,
                     const uint32_t* firsts, MlpState* const* mlps, const cr_cache_config* cc,
                     const cudaStream_t* streams, uint32_t n, cr_cache_stats* stats, uint32_t* cnt) {
    std::vector<CachedJob> jobs(n);
    for (uint32_t i = 0; i < n; i++) {
        CachedJob& j = jobs[i];
        j.s = scenes[i];
        j.cfg = cfgs[i];
        j.cc = *cc;
        j.mlp = mlps[i];
        j.frames = frames[i];
        j.first = firsts[i];
        j.stats = stats ? stats + i : nullptr;
        j.cnt = cnt + 2 * i;
        int rc = cachedSetup(j);
        if (rc) return rc;
    }
    for (bool more = true; more;) {
        more = false;
        for (uint32_t i = 0; i < n; i++) {
            if (jobs[i].f >= jobs[i].frames) continue;
            int rc = cachedIssueWave(jobs[i], streams[i]);
            if (rc) return rc;
            more = true;
        }
        for (uint32_t i = 0; more && i < n; i++) {
            if (jobs[i].f >= jobs[i].frames) continue;
            CR_CUDA(cudaStreamSynchronize(streams[i]));
            int rc = cachedFinishWave(jobs[i], streams[i]);
            if (rc) return rc;
        }
    }
    for (uint32_t i = 0; i < n; i++) {
        int rc = cachedEnd(jobs[i], streams[i]);
        if (rc) return rc;
    }
    return CR_OK;
}

// Validates a cached-render configuration (the checks of cr_render_cached).
int checkCachedConfig(const cr_integrator_config* cfg, const cr_cache_config* cc) {
    if (cfg->max_depth > 1024) return fail(CR_ERR_INVALID_ARGUMENT, "max_depth %u", cfg->max_depth);
    if (cfg->flags & CR_RENDER_SPECTRAL)
        return fail(CR_ERR_UNSUPPORTED, "the radiance cache learns RGB radiance; spectral rendering is not cached");
    if (cfg->flags & ~(CR_RENDER_WAVEFRONT | CR_RENDER_MEGAKERNEL))
        return fail(CR_ERR_INVALID_ARGUMENT, "unknown render flags 0x%x", cfg->flags);
    if ((cfg->flags & CR_RENDER_WAVEFRONT) && (cfg->flags & CR_RENDER_MEGAKERNEL))
        return fail(CR_ERR_INVALID_ARGUMENT, "CR_RENDER_WAVEFRONT and CR_RENDER_MEGAKERNEL exclude each other");
    if (cc->query_vertex == 0 || cc->query_vertex >= cfg->max_depth)
        return fail(CR_ERR_INVALID_ARGUMENT, "query_vertex %u must be in [1, max_depth)", cc->query_vertex);
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
    int rc = checkCachedConfig(cfg, cc);
    if (rc) return rc;
    CR_CUDA(cudaSetDevice(scene->device));
    return renderCached(scene, cfg, cc, mlp->s, frames, first_sample, static_cast<cudaStream_t>(stream), stats);
}
