// cr_wavefront.cu -- the plain path tracer on the wavefront schedule
// (cr_wavefront.cuh): ending paths splat their radiance into the film, as
// the megakernel's SensorData::addSample does (Core/Sensor.cu:19-43).

#include "cr_wavefront.cuh"

namespace cr {

void freeWavefrontBuffers(void* p) {
    if (!p) return;
    WfBuffers* b = static_cast<WfBuffers*>(p);
    b->release();
    delete b;
}

// The tail of a wave of at least kFewMinWave paths finishes in one launch
// once at most kFewPaths paths are live.  Measured on GB300 against no tail
// launch: 1080p x 64 spp (2^26-path waves) 0.1337 -> 0.1316 s, the 4M-path
// box clutter 29.1 -> 28.5 ms; on the 1M-path Cornell box the two extra
// launches per bounce and the megakernel-form finish cost 2 %, so waves that
// small keep their bounce-by-bounce tail.
constexpr uint32_t kFewPaths = 65536;
constexpr uint32_t kFewMinWave = 1u << 21;

// cr_render with the wavefront schedule, in waves of at most kWaveCap paths.
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
    WfBuffers* b = nullptr;
    uint32_t cap = 0;
    int rc = ensureWavefrontWave(s->wfBuffers, total, s->nMats + 2, b, cap);
    if (rc) return rc;
    clearError();
    const OneScene src = oneScene(s, p);
    // the lean shade stage when the scene needs neither Principled lobes,
    // diffuse textures nor analytic spheres
    const bool lean = !s->hasPrincipled && !s->hasTextures && !s->sphHasRoot;
    for (uint64_t base = 0; base < total; base += cap) {
        rc = runWave(src, PlainMode{}, b, base, (uint32_t)std::min<uint64_t>(cap, total - base), p.maxDepth,
                     s->nMats + 2, stream, nullptr, 0, 0xffffffffu, cap >= kFewMinWave ? kFewPaths : 0u, lean);
        if (rc) return rc;
    }
    return CR_OK;
}

}  // namespace cr
