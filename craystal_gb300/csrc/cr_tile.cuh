// cr_tile.cuh -- one block renders a TW x TW pixel tile for a run of sample
// indices: pathTraceKernel<useMIS> per pixel (cr_path.cuh) and
// SensorData::addSample (Core/Sensor.cu:19-43) into a (TW+2)^2 film tile in
// shared memory (the tile plus the one-pixel apron the radius-1 triangle
// filter reaches), added to the global film once per call.  Shared by the
// per-image launch (cr_render.cu) and the batched persistent launch
// (cr_batch.cu).
#pragma once

#include "cr_path.cuh"

namespace cr {

// SensorData::addSample (Core/Sensor.cu:19-43) straight into the global
// film: the radius-1 triangle filter around the film position pix.
__device__ __forceinline__ void splatGlobal(const CameraGpu& cam, float2 pix, const Spec& L, float* __restrict__ filmRgb,
                                            float* __restrict__ filmW) {
    if (isnan(L.r) || isnan(L.g) || isnan(L.b) || isinf(L.r) || isinf(L.g) || isinf(L.b)) return;
    int xa = (int)floorf(pix.x - 1.0f), ya = (int)floorf(pix.y - 1.0f);
    int xb = (int)ceilf(pix.x + 1.0f), yb = (int)ceilf(pix.y + 1.0f);
    xa = max(xa, 0);
    ya = max(ya, 0);
    xb = min(xb, (int)cam.width - 1);
    yb = min(yb, (int)cam.height - 1);
    for (int yy = ya; yy <= yb; yy++)
        for (int xx = xa; xx <= xb; xx++) {
            const float dx = pix.x - ((float)xx + 0.5f), dy = pix.y - ((float)yy + 0.5f);
            const float w = smax(0.0f, 1.0f - fabsf(dx)) * smax(0.0f, 1.0f - fabsf(dy));
            if (w == 0.0f) continue;
            const size_t pi = (size_t)yy * cam.width + xx;
            atomicAdd(filmRgb + 3 * pi + 0, L.r * w);
            atomicAdd(filmRgb + 3 * pi + 1, L.g * w);
            atomicAdd(filmRgb + 3 * pi + 2, L.b * w);
            atomicAdd(filmW + pi, w);
        }
}

template <int TW>
struct TileSmem {
    float film[(TW + 2) * (TW + 2) * 4];
    uint32_t warpRays[(TW * TW + 31) / 32];
};

template <int TW>
__device__ __forceinline__ void renderTile(const SceneView& sc, const CameraGpu& cam, const Params& p, int tx0,
                                           int ty0, uint32_t s0, uint32_t s1, float* __restrict__ filmRgb,
                                           float* __restrict__ filmW, unsigned long long* __restrict__ rayCounter,
                                           TileSmem<TW>& sm) {
    constexpr int kApronW = TW + 2;
    const int tid = threadIdx.y * TW + threadIdx.x;
    __syncthreads();  // the previous tile's flush is done
    for (int i = tid; i < kApronW * kApronW * 4; i += TW * TW) sm.film[i] = 0.0f;
    __syncthreads();
    const uint32_t x = tx0 + threadIdx.x, y = ty0 + threadIdx.y;
    PathCtx c{sc, 0u, SpectralPath{}};
    if (x < cam.width && y < cam.height) {
        for (uint32_t s = s0; s < s1; s++) {
            float2 pix;
            NoHooks hk;
            const Spec L = pathSpecToRgb(c.spec, tracePath(c, cam, p, x, y, p.first + s, pix, hk), p.wb);
            if (isnan(L.r) || isnan(L.g) || isnan(L.b) || isinf(L.r) || isinf(L.g) || isinf(L.b)) continue;
            int xa = (int)floorf(pix.x - 1.0f), ya = (int)floorf(pix.y - 1.0f);
            int xb = (int)ceilf(pix.x + 1.0f), yb = (int)ceilf(pix.y + 1.0f);
            xa = max(xa, 0);
            ya = max(ya, 0);
            xb = min(xb, (int)cam.width - 1);
            yb = min(yb, (int)cam.height - 1);
            for (int yy = ya; yy <= yb; yy++) {
                for (int xx = xa; xx <= xb; xx++) {
                    const float dx = pix.x - ((float)xx + 0.5f), dy = pix.y - ((float)yy + 0.5f);
                    const float w = smax(0.0f, 1.0f - fabsf(dx)) * smax(0.0f, 1.0f - fabsf(dy));
                    if (w == 0.0f) continue;  // adding +0 leaves the film unchanged
                    const int lx = xx - tx0 + 1, ly = yy - ty0 + 1;
                    if (lx >= 0 && lx < kApronW && ly >= 0 && ly < kApronW) {
                        float* cell = sm.film + (ly * kApronW + lx) * 4;
                        atomicAdd(cell + 0, L.r * w);
                        atomicAdd(cell + 1, L.g * w);
                        atomicAdd(cell + 2, L.b * w);
                        atomicAdd(cell + 3, w);
                    } else {
                        const size_t pi = (size_t)yy * cam.width + xx;
                        atomicAdd(filmRgb + 3 * pi + 0, L.r * w);
                        atomicAdd(filmRgb + 3 * pi + 1, L.g * w);
                        atomicAdd(filmRgb + 3 * pi + 2, L.b * w);
                        atomicAdd(filmW + pi, w);
                    }
                }
            }
        }
    }
    uint32_t r = c.rays;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if ((tid & 31) == 0) sm.warpRays[tid >> 5] = r;
    __syncthreads();
    if (tid == 0) {
        unsigned long long t = 0;
        for (int k = 0; k < (TW * TW + 31) / 32; k++) t += sm.warpRays[k];
        atomicAdd(rayCounter, t);
    }
    for (int i = tid; i < kApronW * kApronW; i += TW * TW) {
        const float* cell = sm.film + i * 4;
        if (cell[3] == 0.0f && cell[0] == 0.0f && cell[1] == 0.0f && cell[2] == 0.0f) continue;
        const int gx = tx0 - 1 + i % kApronW, gy = ty0 - 1 + i / kApronW;
        if (gx < 0 || gy < 0 || gx >= (int)cam.width || gy >= (int)cam.height) continue;
        const size_t pi = (size_t)gy * cam.width + gx;
        atomicAdd(filmRgb + 3 * pi + 0, cell[0]);
        atomicAdd(filmRgb + 3 * pi + 1, cell[1]);
        atomicAdd(filmRgb + 3 * pi + 2, cell[2]);
        atomicAdd(filmW + pi, cell[3]);
    }
}

}  // namespace cr
