// cr_batch.cu -- many scenes of uneven size, resolution and sample count
// rendered by one persistent launch, replayed from a captured CUDA graph,
// with tile size and work granularity picked by an autotuner.  (No
// counterpart in the reference, which renders one scene per dispatch with a
// launch and a device synchronisation per sample, Core/Integrator.cu:246-259.)
//
// Work is a flat list of items (scene, tile, run of sample indices), ordered
// by scene cost, largest first.  Every block of the persistent kernel takes
// the next item from a global counter (one atomicAdd per item; no block
// ever waits for another), copies the item's scene descriptor to shared
// memory and renders the tile with the same code as the per-image launch
// (cr_tile.cuh), so each scene's film receives exactly the samples a
// cr_render of that scene would add.

#include <algorithm>
#include <cstring>
#include <vector>

#include "cr_internal.cuh"
#include "cr_mlp.cuh"
#include "cr_tile.cuh"
#include "cr_wavefront.cuh"

namespace cr {
namespace {

struct __align__(16) BatchScene {
    SceneView view;
    CameraGpu cam;
    Params p;
    float* filmRgb;
    float* filmW;
    unsigned long long* rayCounter;
    uint32_t tilesX, pad[3];
};

struct __align__(16) BatchItem {
    uint32_t scene, tile, s0, s1;
};

template <int TW>
__global__ void __launch_bounds__(TW* TW) kBatch(const BatchScene* __restrict__ scenes,
                                                 const BatchItem* __restrict__ items, uint32_t nItems,
                                                 uint32_t* __restrict__ queue) {
    __shared__ TileSmem<TW> sm;
    __shared__ BatchScene bs;
    __shared__ BatchItem item;
    const int tid = threadIdx.y * TW + threadIdx.x;
    while (true) {
        __syncthreads();  // everyone is done with the previous item's bs / item
        if (tid == 0) {
            const uint32_t i = atomicAdd(queue, 1u);
            item = i < nItems ? items[i] : BatchItem{0xffffffffu, 0, 0, 0};
        }
        __syncthreads();
        if (item.scene == 0xffffffffu) break;
        constexpr int kWords = sizeof(BatchScene) / 16;
        for (int k = tid; k < kWords; k += TW * TW)
            reinterpret_cast<uint4*>(&bs)[k] = reinterpret_cast<const uint4*>(scenes + item.scene)[k];
        __syncthreads();
        const int tx0 = (int)(item.tile % bs.tilesX) * TW, ty0 = (int)(item.tile / bs.tilesX) * TW;
        renderTile<TW>(bs.view, bs.cam, bs.p, tx0, ty0, item.s0, item.s1, bs.filmRgb, bs.filmW, bs.rayCounter, sm);
    }
}

}  // namespace
}  // namespace cr

using namespace cr;

struct cr_batch {
    int device = 0;
    std::vector<cr_scene*> scenes;
    std::vector<cr_batch_item> items;
    cr_batch_tuning tuning{16, 4, 0, 0};
    BatchScene* dScenes = nullptr;
    // wavefront schedule
    WfScene* dWf = nullptr;
    void* wfBuffers = nullptr;
    uint64_t* dWaveBase = nullptr;
    uint64_t wfTotal = 0;
    uint32_t wfKeys = 0, wfMaxDepth = 0, wfWaves = 0;
    BatchItem* dItems = nullptr;
    uint32_t nItems = 0;
    uint32_t* dQueue = nullptr;
    cudaStream_t stream = nullptr;  // capture / launch stream when the caller passes none
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool built = false;
    uint64_t replays = 0;
    // cached renders: one stream per scene and the page-locked counters
    std::vector<cudaStream_t> sceneStreams;
    uint32_t* cnt = nullptr;
};

namespace {

void releaseGraph(cr_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

int blocksPerSm(int tw, int* out) {
    int per = 0;
    if (tw == 8) CR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kBatch<8>, 64, 0));
    else CR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kBatch<16>, 256, 0));
    *out = std::max(per, 1);
    return CR_OK;
}

// On the wavefront schedule a scene with at least one whole wave of paths
// renders on its own single-scene wavefront (waves of up to kWaveCap paths,
// cr_render's form), and only the smaller scenes share the captured
// many-scene waves: sharing a wave pays only for scenes smaller than one.
bool ownWaves(const cr_batch* b, size_t i) {
    const cr_scene* s = b->scenes[i];
    return b->tuning.wave_log2 &&
           (uint64_t)s->cam.width * s->cam.height * b->items[i].spp >= (1ull << b->tuning.wave_log2);
}

// Descriptors (re-uploaded on every render, so that sample indices can
// advance between replays) and the work list plus graph (rebuilt when the
// tuning changes).
int uploadDescriptors(cr_batch* b, cudaStream_t st) {
    const int tw = b->tuning.tile;
    std::vector<BatchScene> d(b->scenes.size());
    for (size_t i = 0; i < b->scenes.size(); i++) {
        cr_scene* s = b->scenes[i];
        const cr_batch_item& it = b->items[i];
        std::memset(&d[i], 0, sizeof(BatchScene));
        d[i].view = s->view();
        d[i].cam = s->cam;
        Params& p = d[i].p;
        p.maxDepth = it.config.max_depth;
        p.rrThreshold = it.config.rr_threshold;
        p.useMIS = it.config.use_mis ? 1u : 0u;
        p.spp = it.spp;
        p.first = it.first_sample + (uint32_t)(b->replays * it.spp);
        p.sppPerBlock = b->tuning.spp_per_item;
        p.spectral = (it.config.flags & CR_RENDER_SPECTRAL) ? 1u : 0u;
        p.wb = whiteBalance();
        d[i].filmRgb = s->filmRgb;
        d[i].filmW = s->filmW;
        d[i].rayCounter = s->rayCounter;
        d[i].tilesX = (s->cam.width + tw - 1) / tw;
    }
    CR_CUDA(cudaMemcpyAsync(b->dScenes, d.data(), d.size() * sizeof(BatchScene), cudaMemcpyHostToDevice, st));
    if (b->tuning.wave_log2) {
        // the wavefront's scene table: the same descriptors plus each scene's
        // range of the path sequence and of the sort keys
        std::vector<WfScene> w(b->scenes.size());
        uint64_t path = 0;
        uint32_t key = 0;
        for (size_t i = 0; i < w.size(); i++) {
            cr_scene* s = b->scenes[i];
            std::memset(&w[i], 0, sizeof(WfScene));
            w[i].view = d[i].view;
            w[i].cam = d[i].cam;
            w[i].p = d[i].p;
            w[i].p.sppPerBlock = 1;
            w[i].filmRgb = d[i].filmRgb;
            w[i].filmW = d[i].filmW;
            w[i].rayCounter = d[i].rayCounter;
            w[i].pathBase = path;
            w[i].keyBase = key;
            w[i].nMats = s->nMats;
            // a scene on its own waves holds an empty range of the shared sequence
            if (!ownWaves(b, i)) path += (uint64_t)s->cam.width * s->cam.height * b->items[i].spp;
            key += s->nMats + 2;
        }
        CR_CUDA(cudaMemcpyAsync(b->dWf, w.data(), w.size() * sizeof(WfScene), cudaMemcpyHostToDevice, st));
    }
    return CR_OK;
}

// The wavefront schedule: one wave of the batch's path sequence captured as
// a graph; renderOnce replays it until the sequence is done.
int buildWavefront(cr_batch* b, cudaStream_t st) {
    uint64_t total = 0;
    uint32_t keys = 0, maxDepth = 0;
    for (size_t i = 0; i < b->scenes.size(); i++) {
        const cr_scene* s = b->scenes[i];
        keys += s->nMats + 2;
        if (ownWaves(b, i)) continue;
        total += (uint64_t)s->cam.width * s->cam.height * b->items[i].spp;
        maxDepth = std::max(maxDepth, b->items[i].config.max_depth);
    }
    if (!b->dWf) CR_CUDA(cudaMalloc(&b->dWf, b->scenes.size() * sizeof(WfScene)));
    if (!b->dWaveBase) CR_CUDA(cudaMalloc(&b->dWaveBase, sizeof(uint64_t)));
    b->wfTotal = total;
    b->wfKeys = keys;
    b->wfMaxDepth = maxDepth;
    if (total == 0) {  // every scene renders on its own waves
        b->wfWaves = 0;
        b->built = true;
        return CR_OK;
    }
    const uint32_t cap = (uint32_t)std::min<uint64_t>(total, 1ull << b->tuning.wave_log2);
    WfBuffers* wb = nullptr;
    int rc = ensureWavefrontBuffers(b->wfBuffers, cap, keys, wb);
    if (rc) return rc;
    b->wfWaves = (uint32_t)((total + cap - 1) / cap);
    const ManyScenes src{b->dWf, (uint32_t)b->scenes.size()};
    CR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    // the shared waves finish their tails in one launch as single-scene
    // waves of at least 2M paths do (renderWavefront)
    rc = runWave(src, PlainMode{}, wb, 0, cap, maxDepth, keys, st, b->dWaveBase, total, 0xffffffffu,
                 cap >= (1u << 21) ? 65536u : 0u);
    cudaError_t e = cudaStreamEndCapture(st, &b->graph);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(CR_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
    CR_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    b->built = true;
    return CR_OK;
}

int buildWork(cr_batch* b, cudaStream_t st) {
    releaseGraph(b);
    if (b->dItems) cudaFree(b->dItems);
    b->dItems = nullptr;
    if (b->tuning.wave_log2) return buildWavefront(b, st);
    const int tw = b->tuning.tile;
    const uint32_t run = std::max(1u, b->tuning.spp_per_item);
    // scenes by estimated cost (pixels * spp * depth), largest first
    std::vector<size_t> order(b->scenes.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = i;
    auto cost = [&](size_t i) {
        const cr_scene* s = b->scenes[i];
        return (double)s->cam.width * s->cam.height * b->items[i].spp * b->items[i].config.max_depth;
    };
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t c) { return cost(a) > cost(c); });
    std::vector<BatchItem> items;
    for (size_t i : order) {
        const cr_scene* s = b->scenes[i];
        const uint32_t tx = (s->cam.width + tw - 1) / tw, ty = (s->cam.height + tw - 1) / tw;
        const uint32_t spp = b->items[i].spp;
        for (uint32_t s0 = 0; s0 < spp; s0 += run)
            for (uint32_t t = 0; t < tx * ty; t++) items.push_back(BatchItem{(uint32_t)i, t, s0, std::min(spp, s0 + run)});
    }
    b->nItems = (uint32_t)items.size();
    CR_CUDA(cudaMalloc(&b->dItems, std::max<size_t>(items.size(), 1) * sizeof(BatchItem)));
    CR_CUDA(cudaMemcpy(b->dItems, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice));
    // capture: reset the queue, one persistent launch
    int sms = 0, per = 0;
    CR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
    int rc = blocksPerSm(tw, &per);
    if (rc) return rc;
    const uint32_t bpsm = b->tuning.blocks_per_sm ? std::min<uint32_t>(b->tuning.blocks_per_sm, per) : per;
    const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sms * bpsm, b->nItems));
    CR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(b->dQueue, 0, sizeof(uint32_t), st);
    if (tw == 8) kBatch<8><<<blocks, dim3(8, 8), 0, st>>>(b->dScenes, b->dItems, b->nItems, b->dQueue);
    else kBatch<16><<<blocks, dim3(16, 16), 0, st>>>(b->dScenes, b->dItems, b->nItems, b->dQueue);
    cudaError_t launchErr = cudaGetLastError();
    cudaError_t e = cudaStreamEndCapture(st, &b->graph);
    if (launchErr != cudaSuccess) return fail(CR_ERR_CUDA, "batch capture launch: %s", cudaGetErrorString(launchErr));
    if (e != cudaSuccess) return fail(CR_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
    CR_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    b->built = true;
    return CR_OK;
}

int renderOnce(cr_batch* b, cudaStream_t st) {
    if (!b->built) {
        int rc = buildWork(b, st);
        if (rc) return rc;
    }
    int rc = uploadDescriptors(b, st);
    if (rc) return rc;
    if (b->tuning.wave_log2) {
        if (b->wfWaves) {
            CR_CUDA(cudaMemsetAsync(b->dWaveBase, 0, sizeof(uint64_t), st));
            for (uint32_t w = 0; w < b->wfWaves; w++) CR_CUDA(cudaGraphLaunch(b->exec, st));
            countLaunch(b->wfWaves);
        }
        for (size_t i = 0; i < b->scenes.size(); i++) {
            if (!ownWaves(b, i)) continue;
            const cr_batch_item& it = b->items[i];
            rc = renderWavefront(b->scenes[i], &it.config, it.spp, it.first_sample + (uint32_t)(b->replays * it.spp),
                                 st);
            if (rc) return rc;
        }
    } else {
        CR_CUDA(cudaGraphLaunch(b->exec, st));
        countLaunch();
    }
    b->replays++;
    return CR_OK;
}

}  // namespace

extern "C" {

int cr_batch_create(cr_scene* const* scenes, const cr_batch_item* items, uint32_t n, cr_batch** out) {
    clearError();
    if (!out || (n && (!scenes || !items))) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0) return fail(CR_ERR_INVALID_ARGUMENT, "a batch needs at least one scene");
    *out = nullptr;
    for (uint32_t i = 0; i < n; i++) {
        if (!scenes[i] || !scenes[i]->hasCamera)
            return fail(CR_ERR_INVALID_ARGUMENT, "scene %u is NULL or has no camera", i);
        if (items[i].config.max_depth > 1024) return fail(CR_ERR_INVALID_ARGUMENT, "scene %u max_depth", i);
        if (i && scenes[i]->device != scenes[0]->device)
            return fail(CR_ERR_INVALID_ARGUMENT, "all scenes of a batch must live on one device");
    }
    cr_batch* b = new cr_batch();
    b->device = scenes[0]->device;
    b->scenes.assign(scenes, scenes + n);
    b->items.assign(items, items + n);
    CR_CUDA(cudaSetDevice(b->device));
    CR_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CR_CUDA(cudaMalloc(&b->dScenes, n * sizeof(BatchScene)));
    CR_CUDA(cudaMalloc(&b->dQueue, sizeof(uint32_t)));
    *out = b;
    return CR_OK;
}

int cr_batch_destroy(cr_batch* b) {
    clearError();
    if (!b) return CR_OK;
    cudaSetDevice(b->device);
    releaseGraph(b);
    if (b->dItems) cudaFree(b->dItems);
    if (b->dScenes) cudaFree(b->dScenes);
    if (b->dQueue) cudaFree(b->dQueue);
    if (b->dWf) cudaFree(b->dWf);
    if (b->dWaveBase) cudaFree(b->dWaveBase);
    freeWavefrontBuffers(b->wfBuffers);
    if (b->stream) cudaStreamDestroy(b->stream);
    for (cudaStream_t st : b->sceneStreams) cudaStreamDestroy(st);
    if (b->cnt) cudaFreeHost(b->cnt);
    delete b;
    return CR_OK;
}

int cr_batch_set_tuning(cr_batch* b, const cr_batch_tuning* t) {
    clearError();
    if (!b || !t) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (t->wave_log2 && (t->wave_log2 < 16 || t->wave_log2 > 25))
        return fail(CR_ERR_INVALID_ARGUMENT, "wave_log2 must be 0 or 16..25");
    if (!t->wave_log2 && t->tile != 8 && t->tile != 16) return fail(CR_ERR_INVALID_ARGUMENT, "tile must be 8 or 16");
    if (!t->wave_log2 && t->spp_per_item == 0) return fail(CR_ERR_INVALID_ARGUMENT, "spp_per_item must be positive");
    b->tuning = *t;
    b->built = false;
    return CR_OK;
}

int cr_batch_get_tuning(const cr_batch* b, cr_batch_tuning* t) {
    clearError();
    if (!b || !t) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    *t = b->tuning;
    return CR_OK;
}

int cr_batch_render(cr_batch* b, void* stream) {
    clearError();
    if (!b) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    CR_CUDA(cudaSetDevice(b->device));
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : b->stream;
    int rc = renderOnce(b, st);
    if (rc) return rc;
    if (!stream) CR_CUDA(cudaStreamSynchronize(st));
    return CR_OK;
}

int cr_batch_render_cached(cr_batch* b, cr_mlp* const* mlps, const cr_cache_config* cache, cr_cache_stats* stats) {
    clearError();
    if (!b || !mlps || !cache) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    const uint32_t n = (uint32_t)b->scenes.size();
    std::vector<MlpState*> nets(n);
    std::vector<cr_integrator_config> cfgs(n);
    std::vector<uint32_t> frames(n), firsts(n);
    for (uint32_t i = 0; i < n; i++) {
        if (!mlps[i]) return fail(CR_ERR_INVALID_ARGUMENT, "network %u is NULL", i);
        for (uint32_t k = 0; k < i; k++)
            if (mlps[k] == mlps[i]) return fail(CR_ERR_INVALID_ARGUMENT, "scenes %u and %u share a network", k, i);
        int rc = checkCachedConfig(&b->items[i].config, cache);
        if (rc) return rc;
        nets[i] = mlps[i]->s;
        cfgs[i] = b->items[i].config;
        frames[i] = b->items[i].spp;
        firsts[i] = b->items[i].first_sample + (uint32_t)(b->replays * b->items[i].spp);
    }
    CR_CUDA(cudaSetDevice(b->device));
    if (b->sceneStreams.size() != n) {
        for (uint32_t i = (uint32_t)b->sceneStreams.size(); i < n; i++) {
            cudaStream_t st = nullptr;
            CR_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            b->sceneStreams.push_back(st);
        }
    }
    if (!b->cnt) CR_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&b->cnt), 2 * n * sizeof(uint32_t), cudaHostAllocDefault));
    CR_CUDA(cudaStreamSynchronize(b->stream));  // plain renders of the batch on its own stream come first
    int rc = renderCachedMany(b->scenes.data(), cfgs.data(), frames.data(), firsts.data(), nets.data(), cache,
                              b->sceneStreams.data(), n, stats, b->cnt);
    if (rc) return rc;
    b->replays++;
    return CR_OK;
}

int cr_batch_autotune(cr_batch* b, cr_batch_tuning* best, cr_batch_tuning_result* results, uint32_t max_results,
                      uint32_t* n_results) {
    clearError();
    if (!b) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    CR_CUDA(cudaSetDevice(b->device));
    std::vector<cr_batch_tuning> cands;
    for (uint32_t tw : {8u, 16u})
        for (uint32_t r : {1u, 2u, 4u, 8u, 16u}) cands.push_back(cr_batch_tuning{tw, r, 0, 0});
    for (uint32_t w : {20u, 22u, 23u, 24u, 25u}) cands.push_back(cr_batch_tuning{16, 4, 0, w});
    cudaEvent_t e0, e1;
    CR_CUDA(cudaEventCreate(&e0));
    CR_CUDA(cudaEventCreate(&e1));
    float bestMs = INFINITY;
    cr_batch_tuning bestT = b->tuning;
    uint32_t k = 0;
    {
        for (const cr_batch_tuning& t : cands) {
            b->tuning = t;
            b->built = false;
            int rc = buildWork(b, b->stream);
            if (rc) return rc;
            rc = renderOnce(b, b->stream);  // warm-up replay
            if (rc) return rc;
            CR_CUDA(cudaEventRecord(e0, b->stream));
            rc = renderOnce(b, b->stream);
            if (rc) return rc;
            CR_CUDA(cudaEventRecord(e1, b->stream));
            CR_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            CR_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (results && k < max_results) results[k] = cr_batch_tuning_result{t, ms};
            k++;
            if (ms < bestMs) {
                bestMs = ms;
                bestT = t;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (n_results) *n_results = k;
    b->tuning = bestT;
    b->built = false;
    b->replays = 0;
    if (best) *best = bestT;
    // the tuning renders added samples: clear the films
    for (cr_scene* s : b->scenes) {
        const size_t px = (size_t)s->cam.width * s->cam.height;
        CR_CUDA(cudaMemsetAsync(s->filmRgb, 0, px * 3 * sizeof(float), b->stream));
        CR_CUDA(cudaMemsetAsync(s->filmW, 0, px * sizeof(float), b->stream));
        CR_CUDA(cudaMemsetAsync(s->rayCounter, 0, sizeof(unsigned long long), b->stream));
    }
    CR_CUDA(cudaStreamSynchronize(b->stream));
    return CR_OK;
}

}  // extern "C"
