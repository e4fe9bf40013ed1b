// cr_mlp.cu -- the radiance-cache network: a 7-input MLP with a 12-frequency
// sin / cos encoding (168 features, padded to 176), five hidden layers of 64
// ReLU units and 3 linear outputs (RGB radiance), FP16 weights and
// activations with FP32 accumulation on the tensor cores (mma.sync
// m16n8k16), trained online with Adam on a relative L2 loss.
//
// This part has no counterpart in the reference; it is the cache that ends
// paths early (see cr_cache.cu).
//
// Kernels
//   kInfer     fused forward: one warp carries 16 queries through all six
//              layers; each layer's accumulator fragments are the next
//              layer's A fragments (the m16n8k16 C layout of two adjacent
//              n-tiles is the A layout of one k-tile), so activations never
//              leave registers.  Weights live in shared memory.
//   kTrainFwdBwd  the same forward, storing every layer's input activations,
//              then the loss gradient and the backward pass for the data
//              gradients, storing every layer's output gradient dY.
//   kWeightGrad   dW_l = X_l^T dY_l over the batch (split over CTAs,
//              accumulated with atomics in FP32).
//   kAdam      Adam on FP32 master weights; refreshes the two FP16 copies
//              (n-major for the forward B operand, k-major for the backward).

#include <cstring>
#include <vector>

#include <cuda_fp16.h>

#include "cr_internal.cuh"
#include "cr_mlp.cuh"

namespace cr {
namespace {

// ---------------------------------------------------------------------------
// sizes and layouts
// ---------------------------------------------------------------------------
constexpr int kIn = 7;          // network inputs
constexpr int kFreq = 12;       // frequencies per input
constexpr int kFeat = 176;      // encoded features: 7 * 12 * 2 = 168, padded
constexpr int kHid = 64;
constexpr int kLayers = 6;      // 5 hidden + output
constexpr int kOutPad = 8;      // 3 outputs padded to one n8 tile
// (K, N) of each layer's weight matrix
__host__ __device__ constexpr int layerK(int l) { return l == 0 ? kFeat : kHid; }
__host__ __device__ constexpr int layerN(int l) { return l == kLayers - 1 ? 3 : kHid; }
// offsets in the flat FP32 parameter vector (k-major: W[k][n] at k * N + n)
__host__ __device__ constexpr int paramOffset(int l) { return l == 0 ? 0 : kFeat * kHid + (l - 1) * kHid * kHid; }
constexpr int kParams = kFeat * kHid + 4 * kHid * kHid + kHid * 3;  // 27,840

// FP16 forward copy (n-major, padded rows): WT_l[n][k], row stride K + 8
// halves (the pad spreads the 8 rows a fragment load touches over distinct
// shared-memory banks).  The output layer has 8 rows (3 real).
__host__ __device__ constexpr int fwdStride(int l) { return layerK(l) + 8; }
__host__ __device__ constexpr int fwdRows(int l) { return l == kLayers - 1 ? kOutPad : kHid; }
__host__ __device__ constexpr int fwdOffset(int l) {
    int o = 0;
    for (int i = 0; i < l; i++) o += fwdRows(i) * fwdStride(i);
    return o;
}
constexpr int kFwdHalves = fwdOffset(kLayers);
// FP16 backward copy (k-major): W_l[k][n], row stride Npad + 8 with the
// output layer's N padded to 16 (it is the K dimension of the backward MMA).
__host__ __device__ constexpr int bwdCols(int l) { return l == kLayers - 1 ? 16 : kHid; }
__host__ __device__ constexpr int bwdStride(int l) { return bwdCols(l) + 8; }
__host__ __device__ constexpr int bwdOffset(int l) {
    int o = 0;
    for (int i = 0; i < l; i++) o += layerK(i) * bwdStride(i);
    return o;
}
constexpr int kBwdHalves = bwdOffset(kLayers);

constexpr int kWarps = 4;
constexpr float kGradClip = 256.0f;  // |dL/dy| per sample and channel
constexpr int kThreads = kWarps * 32;

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ float2 unpack2(uint32_t v) {
    __half2 h = *reinterpret_cast<__half2*>(&v);
    return __half22float2(h);
}

// Encoded features of one query row for the columns a thread owns in k-tile
// kt: (c, c+1) and (c+8, c+9) with c = kt*16 + tig*2.  Feature j = d*24 +
// 2f + {0: sin, 1: cos} of sin / cos(pi * 2^f * x_d).
__device__ __forceinline__ uint32_t featurePair(const float* x, int j) {
    if (j >= kIn * kFreq * 2) return 0u;
    const int d = j / (kFreq * 2), f = (j % (kFreq * 2)) >> 1;
    // pi * 2^f * x, reduced exactly: 2^f * x is exact, fmod by 2 is exact
    float y = ldexpf(x[d], f);
    y = y - 2.0f * floorf(y * 0.5f);
    float s, c;
    sincospif(y, &s, &c);
    return pack2(s, c);
}

// A fragments of the encoded input for the 16 rows of a warp tile.
__device__ __forceinline__ void encodeTile(const float xr0[kIn], const float xr1[kIn], uint32_t a[11][4]) {
    const int tig = threadIdx.x & 3;
#pragma unroll
    for (int kt = 0; kt < 11; kt++) {
        const int c = kt * 16 + tig * 2;
        a[kt][0] = featurePair(xr0, c);
        a[kt][1] = featurePair(xr1, c);
        a[kt][2] = featurePair(xr0, c + 8);
        a[kt][3] = featurePair(xr1, c + 8);
    }
}

// One hidden / output layer: acc[nt] += A(16 x K) * W(K x N) for nTiles n-tiles.
template <int KT, int NT>
__device__ __forceinline__ void layerFwd(const __half* wt, int stride, const uint32_t (*a)[4], float acc[][4]) {
    const int g = (threadIdx.x & 31) >> 2, tig = threadIdx.x & 3;
#pragma unroll
    for (int nt = 0; nt < NT; nt++) {
        acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
        const __half* row = wt + (nt * 8 + g) * stride + tig * 2;
#pragma unroll
        for (int kt = 0; kt < KT; kt++) {
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(row + kt * 16);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(row + kt * 16 + 8);
            mma16816(acc[nt], a[kt], b0, b1);
        }
    }
}

// ReLU of 8 n-tiles of accumulators into the A fragments of 4 k-tiles.
__device__ __forceinline__ void reluToA(const float acc[8][4], uint32_t a[4][4]) {
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        a[kt][0] = pack2(fmaxf(acc[2 * kt][0], 0.0f), fmaxf(acc[2 * kt][1], 0.0f));
        a[kt][1] = pack2(fmaxf(acc[2 * kt][2], 0.0f), fmaxf(acc[2 * kt][3], 0.0f));
        a[kt][2] = pack2(fmaxf(acc[2 * kt + 1][0], 0.0f), fmaxf(acc[2 * kt + 1][1], 0.0f));
        a[kt][3] = pack2(fmaxf(acc[2 * kt + 1][2], 0.0f), fmaxf(acc[2 * kt + 1][3], 0.0f));
    }
}

__device__ void loadFwdWeights(const __half* __restrict__ g, __half* s) {
    const int n = kFwdHalves / 8;  // 16-byte chunks
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        reinterpret_cast<uint4*>(s)[i] = reinterpret_cast<const uint4*>(g)[i];
}

// Stores the A fragments of a layer input (16 rows x 16*KT halves) at rows
// [row0, row0+16) of a row-major FP16 matrix with the given stride.
template <int KT>
__device__ __forceinline__ void storeA(const uint32_t (*a)[4], __half* m, int stride, uint64_t row0, uint64_t n) {
    const int g = (threadIdx.x & 31) >> 2, tig = threadIdx.x & 3;
    const uint64_t r0 = row0 + g, r1 = row0 + g + 8;
#pragma unroll
    for (int kt = 0; kt < KT; kt++) {
        const int c = kt * 16 + tig * 2;
        if (r0 < n) {
            *reinterpret_cast<uint32_t*>(m + r0 * stride + c) = a[kt][0];
            *reinterpret_cast<uint32_t*>(m + r0 * stride + c + 8) = a[kt][2];
        }
        if (r1 < n) {
            *reinterpret_cast<uint32_t*>(m + r1 * stride + c) = a[kt][1];
            *reinterpret_cast<uint32_t*>(m + r1 * stride + c + 8) = a[kt][3];
        }
    }
}

__device__ __forceinline__ void loadInputs(const float* __restrict__ in, uint64_t n, uint64_t row, float x[kIn]) {
#pragma unroll
    for (int d = 0; d < kIn; d++) x[d] = row < n ? in[row * kIn + d] : 0.0f;
}

// Full forward for the warp's 16 rows; returns the output accumulators
// (16 x 8; columns 0..2 are RGB).  When act != nullptr the input of every
// layer is stored (layer 0: kFeat halves per row, others kHid).
__device__ void forwardTile(const __half* sw, const float* __restrict__ in, uint64_t n, uint64_t row0,
                            float out[4], __half* const* act) {
    const int g = (threadIdx.x & 31) >> 2;
    float x0[kIn], x1[kIn];
    loadInputs(in, n, row0 + g, x0);
    loadInputs(in, n, row0 + g + 8, x1);
    uint32_t a0[11][4];
    encodeTile(x0, x1, a0);
    if (act) storeA<11>(a0, act[0], kFeat, row0, n);
    float acc[8][4];
    layerFwd<11, 8>(sw + fwdOffset(0), fwdStride(0), a0, acc);
    uint32_t a[4][4];
    reluToA(acc, a);
#pragma unroll 1
    for (int l = 1; l < kLayers - 1; l++) {
        if (act) storeA<4>(a, act[l], kHid, row0, n);
        layerFwd<4, 8>(sw + fwdOffset(l), fwdStride(l), a, acc);
        reluToA(acc, a);
    }
    if (act) storeA<4>(a, act[kLayers - 1], kHid, row0, n);
    float o[1][4];
    layerFwd<4, 1>(sw + fwdOffset(kLayers - 1), fwdStride(kLayers - 1), a, o);
    out[0] = o[0][0];
    out[1] = o[0][1];
    out[2] = o[0][2];
    out[3] = o[0][3];
}

// Writes the 3 real output columns of a tile; thread (g, tig) holds columns
// tig*2, tig*2+1 of rows g and g+8.
__device__ __forceinline__ void storeOut(const float o[4], float* __restrict__ out, uint64_t n, uint64_t row0,
                                         bool clampNonNeg) {
    const int g = (threadIdx.x & 31) >> 2, tig = threadIdx.x & 3;
    const uint64_t r0 = row0 + g, r1 = row0 + g + 8;
    for (int k = 0; k < 2; k++) {
        const int col = tig * 2 + k;
        if (col >= 3) continue;
        if (r0 < n) out[r0 * 3 + col] = clampNonNeg ? fmaxf(o[k], 0.0f) : o[k];
        if (r1 < n) out[r1 * 3 + col] = clampNonNeg ? fmaxf(o[2 + k], 0.0f) : o[2 + k];
    }
}

__global__ void __launch_bounds__(kThreads) kInfer(const __half* __restrict__ wFwd, const float* __restrict__ in,
                                                   uint64_t n, float* __restrict__ out, int clampNonNeg) {
    extern __shared__ __align__(16) __half smem[];
    loadFwdWeights(wFwd, smem);
    __syncthreads();
    const uint64_t warpsTotal = (uint64_t)gridDim.x * kWarps;
    const uint64_t w = (uint64_t)blockIdx.x * kWarps + (threadIdx.x >> 5);
    for (uint64_t row0 = w * 16; row0 < n; row0 += warpsTotal * 16) {
        float o[4];
        forwardTile(smem, in, n, row0, o, nullptr);
        storeOut(o, out, n, row0, clampNonNeg != 0);
    }
}

struct Acts {
    __half* act[kLayers];   // inputs of each layer: [n][K_l]
    __half* dy[kLayers];    // output gradients of each layer: [n][Npad_l] (Npad = 64, or 16 for the output)
};

// dX (16 x K) = dY (16 x N) * W^T, with W k-major [K][Npad] in shared memory;
// KT_N = k-tiles over N, NT_K = n-tiles over K.
template <int KT_N, int NT_K>
__device__ __forceinline__ void layerBwd(const __half* wk, int stride, const uint32_t (*dy)[4], float acc[][4]) {
    const int g = (threadIdx.x & 31) >> 2, tig = threadIdx.x & 3;
#pragma unroll
    for (int nt = 0; nt < NT_K; nt++) {
        acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
        const __half* row = wk + (nt * 8 + g) * stride + tig * 2;
#pragma unroll
        for (int kt = 0; kt < KT_N; kt++) {
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(row + kt * 16);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(row + kt * 16 + 8);
            mma16816(acc[nt], dy[kt], b0, b1);
        }
    }
}

// Loads the A fragments (16 rows x 64) of a stored activation.
__device__ __forceinline__ void loadA4(const __half* m, uint64_t row0, uint64_t n, uint32_t a[4][4]) {
    const int g = (threadIdx.x & 31) >> 2, tig = threadIdx.x & 3;
    const uint64_t r0 = row0 + g, r1 = row0 + g + 8;
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        const int c = kt * 16 + tig * 2;
        a[kt][0] = r0 < n ? *reinterpret_cast<const uint32_t*>(m + r0 * kHid + c) : 0u;
        a[kt][2] = r0 < n ? *reinterpret_cast<const uint32_t*>(m + r0 * kHid + c + 8) : 0u;
        a[kt][1] = r1 < n ? *reinterpret_cast<const uint32_t*>(m + r1 * kHid + c) : 0u;
        a[kt][3] = r1 < n ? *reinterpret_cast<const uint32_t*>(m + r1 * kHid + c + 8) : 0u;
    }
}

// dY of the layer below: dX masked by the ReLU of that layer's output (the
// stored input of this layer), packed as A fragments.
__device__ __forceinline__ void maskToA(const float acc[8][4], const uint32_t act[4][4], uint32_t dy[4][4]) {
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float2 av = unpack2(act[kt][q]);
            const int nt = 2 * kt + (q >> 1), e = (q & 1) * 2;
            dy[kt][q] = pack2(av.x > 0.0f ? acc[nt][e] : 0.0f, av.y > 0.0f ? acc[nt][e + 1] : 0.0f);
        }
    }
}

__global__ void __launch_bounds__(kThreads) kTrainFwdBwd(const __half* __restrict__ wFwd,
                                                         const __half* __restrict__ wBwd,
                                                         const float* __restrict__ in,
                                                         const float* __restrict__ target, uint64_t n, Acts acts,
                                                         float* __restrict__ lossSum) {
    extern __shared__ __align__(16) __half smem[];
    __half* sf = smem;
    __half* sb = smem + kFwdHalves;
    loadFwdWeights(wFwd, sf);
    for (int i = threadIdx.x; i < kBwdHalves / 8; i += blockDim.x)
        reinterpret_cast<uint4*>(sb)[i] = reinterpret_cast<const uint4*>(wBwd)[i];
    __syncthreads();
    const int g = (threadIdx.x & 31) >> 2, tig = threadIdx.x & 3;
    const uint64_t warpsTotal = (uint64_t)gridDim.x * kWarps;
    const uint64_t w = (uint64_t)blockIdx.x * kWarps + (threadIdx.x >> 5);
    float lossLocal = 0.0f;
    for (uint64_t row0 = w * 16; row0 < n; row0 += warpsTotal * 16) {
        float o[4];
        forwardTile(sf, in, n, row0, o, acts.act);
        // relative L2 loss (y - t)^2 / (sg(y)^2 + 0.01) and its gradient
        // 2 (y - t) / (y^2 + 0.01); the 1 / (3 n) of the mean is applied to dW
        uint32_t dy[1][4];
        float d[4];
        for (int q = 0; q < 4; q++) {
            const uint64_t r = row0 + g + (q >= 2 ? 8 : 0);
            const int col = tig * 2 + (q & 1);
            d[q] = 0.0f;
            if (r < n && col < 3) {
                const float y = o[q], t = target[r * 3 + col];
                const float den = y * y + 0.01f;
                // per-sample gradient clipped to +-kGradClip: the relative loss
                // gradient of a far-off prediction (y ~ 0, t large) would
                // otherwise overflow the FP16 gradient path
                d[q] = fminf(fmaxf(2.0f * (y - t) / den, -kGradClip), kGradClip);
                lossLocal += (y - t) * (y - t) / den;
            }
        }
        // output dY (16 x 8) as the A fragment of a 16 x 16 k-tile (cols 8..15 zero)
        dy[0][0] = pack2(d[0], d[1]);
        dy[0][1] = pack2(d[2], d[3]);
        dy[0][2] = 0u;
        dy[0][3] = 0u;
        {
            const uint64_t r0 = row0 + g, r1 = row0 + g + 8;
            if (r0 < n) *reinterpret_cast<uint32_t*>(acts.dy[kLayers - 1] + r0 * 16 + tig * 2) = dy[0][0];
            if (r1 < n) *reinterpret_cast<uint32_t*>(acts.dy[kLayers - 1] + r1 * 16 + tig * 2) = dy[0][1];
            if (r0 < n) *reinterpret_cast<uint32_t*>(acts.dy[kLayers - 1] + r0 * 16 + 8 + tig * 2) = 0u;
            if (r1 < n) *reinterpret_cast<uint32_t*>(acts.dy[kLayers - 1] + r1 * 16 + 8 + tig * 2) = 0u;
        }
        float acc[8][4];
        layerBwd<1, 8>(sb + bwdOffset(kLayers - 1), bwdStride(kLayers - 1), dy, acc);
        uint32_t a[4][4], g4[4][4];
        loadA4(acts.act[kLayers - 1], row0, n, a);
        maskToA(acc, a, g4);
#pragma unroll 1
        for (int l = kLayers - 2; l >= 1; l--) {
            storeA<4>(g4, acts.dy[l], kHid, row0, n);
            layerBwd<4, 8>(sb + bwdOffset(l), bwdStride(l), g4, acc);
            loadA4(acts.act[l], row0, n, a);
            maskToA(acc, a, g4);
        }
        storeA<4>(g4, acts.dy[0], kHid, row0, n);
    }
    for (int o = 16; o > 0; o >>= 1) lossLocal += __shfl_xor_sync(0xffffffffu, lossLocal, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(lossSum, lossLocal);
}

// dW_l[k][n] += scale * sum_b act_l[b][k] * dY_l[b][n] over a chunk of rows.
constexpr int kGradRows = 64;
template <int K, int NP>
__global__ void __launch_bounds__(256) kWeightGrad(const __half* __restrict__ act, const __half* __restrict__ dy,
                                                   uint64_t n, int nReal, float scale, float* __restrict__ dW) {
    __shared__ __align__(16) __half sa[kGradRows][K + 8];
    __shared__ __align__(16) __half sd[kGradRows][NP + 8];
    const uint64_t row0 = (uint64_t)blockIdx.x * kGradRows;
    for (int i = threadIdx.x; i < kGradRows * K / 2; i += blockDim.x) {
        const int r = i / (K / 2), c = (i % (K / 2)) * 2;
        const uint64_t gr = row0 + r;
        *reinterpret_cast<uint32_t*>(&sa[r][c]) = gr < n ? *reinterpret_cast<const uint32_t*>(act + gr * K + c) : 0u;
    }
    for (int i = threadIdx.x; i < kGradRows * NP / 2; i += blockDim.x) {
        const int r = i / (NP / 2), c = (i % (NP / 2)) * 2;
        const uint64_t gr = row0 + r;
        *reinterpret_cast<uint32_t*>(&sd[r][c]) = gr < n ? *reinterpret_cast<const uint32_t*>(dy + gr * NP + c) : 0u;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, g = (threadIdx.x & 31) >> 2, tig = threadIdx.x & 3;
    constexpr int MT = K / 16, NT = (NP + 7) / 8;
    for (int tile = warp; tile < MT * NT; tile += 8) {
        const int mt = tile / NT, nt = tile % NT;
        float c[4] = {0, 0, 0, 0};
        for (int kb = 0; kb < kGradRows; kb += 16) {
            // A = act^T (m = feature, k = batch row); B = dY (k = batch row, n)
            uint32_t a[4];
            const int m0 = mt * 16 + g, kr = kb + tig * 2;
            auto pk = [&](int m, int r) {
                __half2 h;
                h.x = sa[r][m];
                h.y = sa[r + 1][m];
                return *reinterpret_cast<uint32_t*>(&h);
            };
            a[0] = pk(m0, kr);
            a[1] = pk(m0 + 8, kr);
            a[2] = pk(m0, kr + 8);
            a[3] = pk(m0 + 8, kr + 8);
            const int nn = nt * 8 + g;
            __half2 h0, h1;
            h0.x = sd[kr][nn];
            h0.y = sd[kr + 1][nn];
            h1.x = sd[kr + 8][nn];
            h1.y = sd[kr + 9][nn];
            mma16816(c, a, *reinterpret_cast<uint32_t*>(&h0), *reinterpret_cast<uint32_t*>(&h1));
        }
        // c: rows (m = mt*16 + g, +8), cols (n = nt*8 + tig*2, +1)
        for (int q = 0; q < 4; q++) {
            const int m = mt * 16 + g + (q >= 2 ? 8 : 0), col = nt * 8 + tig * 2 + (q & 1);
            if (col < nReal) atomicAdd(dW + m * nReal + col, c[q] * scale);
        }
    }
}

__global__ void kAdam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v, float* __restrict__ grad,
                      int count, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gr = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gr;
    const float vi = b2 * v[i] + (1.0f - b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    grad[i] = 0.0f;
}

// Refreshes the FP16 forward (n-major) and backward (k-major) copies.
__global__ void kPackWeights(const float* __restrict__ w, __half* __restrict__ fwd, __half* __restrict__ bwd) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    int l = 0;
    while (l < kLayers - 1 && i >= paramOffset(l + 1)) l++;
    const int K = layerK(l), N = layerN(l);
    const int local = i - paramOffset(l), k = local / N, n = local % N;
    const __half h = __float2half_rn(w[i]);
    fwd[fwdOffset(l) + n * fwdStride(l) + k] = h;
    bwd[bwdOffset(l) + k * bwdStride(l) + n] = h;
    (void)K;
}

inline unsigned cdiv(uint64_t a, uint64_t b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct MlpState {
    int device = 0;
    cr_mlp_config cfg{};
    float* w = nullptr;     // FP32 master weights
    float* m = nullptr;
    float* v = nullptr;
    float* grad = nullptr;
    float* loss = nullptr;
    __half* wFwd = nullptr;
    __half* wBwd = nullptr;
    uint64_t cap = 0;       // rows of the training buffers
    __half* act[kLayers] = {};
    __half* dy[kLayers] = {};
    float* stageIn = nullptr;
    float* stageOut = nullptr;
    uint64_t stageCap = 0;
    uint32_t step = 0;
    int sms = 0;
};

namespace {

int ensureTrainCap(MlpState* s, uint64_t n) {
    if (n <= s->cap) return CR_OK;
    for (int l = 0; l < kLayers; l++) {
        if (s->act[l]) cudaFree(s->act[l]);
        if (s->dy[l]) cudaFree(s->dy[l]);
        s->act[l] = s->dy[l] = nullptr;
    }
    for (int l = 0; l < kLayers; l++) {
        CR_CUDA(cudaMalloc(&s->act[l], n * layerK(l) * sizeof(__half)));
        CR_CUDA(cudaMalloc(&s->dy[l], n * (l == kLayers - 1 ? 16 : kHid) * sizeof(__half)));
    }
    s->cap = n;
    return CR_OK;
}

int ensureStage(MlpState* s, uint64_t n) {
    if (n <= s->stageCap) return CR_OK;
    if (s->stageIn) cudaFree(s->stageIn);
    if (s->stageOut) cudaFree(s->stageOut);
    s->stageIn = s->stageOut = nullptr;
    CR_CUDA(cudaMalloc(&s->stageIn, n * kIn * sizeof(float)));
    CR_CUDA(cudaMalloc(&s->stageOut, n * 3 * sizeof(float)));
    s->stageCap = n;
    return CR_OK;
}

int pack(MlpState* s, cudaStream_t st) {
    kPackWeights<<<cdiv(kParams, 256), 256, 0, st>>>(s->w, s->wFwd, s->wBwd);
    CR_LAUNCH_CHECK();
    return CR_OK;
}

constexpr size_t kInferSmem = (size_t)kFwdHalves * sizeof(__half);
constexpr size_t kTrainSmem = (size_t)(kFwdHalves + kBwdHalves) * sizeof(__half);

}  // namespace

int mlpCreate(const cr_mlp_config* cfg, MlpState** out) {
    MlpState* s = new MlpState();
    s->cfg = *cfg;
    CR_CUDA(cudaGetDevice(&s->device));
    CR_CUDA(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device));
    CR_CUDA(cudaMalloc(&s->w, kParams * sizeof(float)));
    CR_CUDA(cudaMalloc(&s->m, kParams * sizeof(float)));
    CR_CUDA(cudaMalloc(&s->v, kParams * sizeof(float)));
    CR_CUDA(cudaMalloc(&s->grad, kParams * sizeof(float)));
    CR_CUDA(cudaMalloc(&s->loss, sizeof(float)));
    CR_CUDA(cudaMalloc(&s->wFwd, kFwdHalves * sizeof(__half)));
    CR_CUDA(cudaMalloc(&s->wBwd, kBwdHalves * sizeof(__half)));
    CR_CUDA(cudaMemset(s->wFwd, 0, kFwdHalves * sizeof(__half)));
    CR_CUDA(cudaMemset(s->wBwd, 0, kBwdHalves * sizeof(__half)));
    CR_CUDA(cudaMemset(s->m, 0, kParams * sizeof(float)));
    CR_CUDA(cudaMemset(s->v, 0, kParams * sizeof(float)));
    CR_CUDA(cudaMemset(s->grad, 0, kParams * sizeof(float)));
    // uniform(-a, a) with a = sqrt(6 / (fan_in + fan_out)) from a 64-bit LCG
    std::vector<float> w(kParams);
    uint64_t x = 0x9E3779B97F4A7C15ull ^ ((uint64_t)cfg->seed * 0xD1B54A32D192ED03ull);
    for (int l = 0; l < kLayers; l++) {
        const float a = std::sqrt(6.0f / (float)(layerK(l) + layerN(l)));
        for (int i = 0; i < layerK(l) * layerN(l); i++) {
            x = x * 6364136223846793005ull + 1442695040888963407ull;
            const float u = (float)((x >> 40) & 0xffffff) / 16777216.0f;
            w[paramOffset(l) + i] = (2.0f * u - 1.0f) * a;
        }
    }
    CR_CUDA(cudaMemcpy(s->w, w.data(), kParams * sizeof(float), cudaMemcpyHostToDevice));
    CR_CUDA(cudaFuncSetAttribute(kInfer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem));
    CR_CUDA(cudaFuncSetAttribute(kTrainFwdBwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem));
    int rc = pack(s, 0);
    if (rc) return rc;
    CR_CUDA(cudaDeviceSynchronize());
    *out = s;
    return CR_OK;
}

void mlpDestroy(MlpState* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    void* p[] = {s->w, s->m, s->v, s->grad, s->loss, s->wFwd, s->wBwd, s->stageIn, s->stageOut};
    for (void* q : p)
        if (q) cudaFree(q);
    for (int l = 0; l < kLayers; l++) {
        if (s->act[l]) cudaFree(s->act[l]);
        if (s->dy[l]) cudaFree(s->dy[l]);
    }
    delete s;
}

int mlpInferDevice(MlpState* s, const float* in, uint64_t n, float* out, bool clampNonNeg, cudaStream_t st) {
    if (n == 0) return CR_OK;
    const unsigned blocks = std::min<unsigned>(cdiv(n, kWarps * 16), (unsigned)s->sms * 2);
    kInfer<<<blocks, kThreads, kInferSmem, st>>>(s->wFwd, in, n, out, clampNonNeg ? 1 : 0);
    CR_LAUNCH_CHECK();
    return CR_OK;
}

// Accumulates dW of the mean relative L2 loss over n samples into s->grad.
int mlpGradDevice(MlpState* s, const float* in, const float* target, uint64_t n, cudaStream_t st) {
    if (n == 0) return CR_OK;
    int rc = ensureTrainCap(s, n);
    if (rc) return rc;
    CR_CUDA(cudaMemsetAsync(s->loss, 0, sizeof(float), st));
    Acts acts;
    for (int l = 0; l < kLayers; l++) {
        acts.act[l] = s->act[l];
        acts.dy[l] = s->dy[l];
    }
    const unsigned blocks = std::min<unsigned>(cdiv(n, kWarps * 16), (unsigned)s->sms * 2);
    kTrainFwdBwd<<<blocks, kThreads, kTrainSmem, st>>>(s->wFwd, s->wBwd, in, target, n, acts, s->loss);
    CR_LAUNCH_CHECK();
    const float scale = 1.0f / (3.0f * (float)n);
    const unsigned gb = cdiv(n, kGradRows);
    kWeightGrad<kFeat, kHid><<<gb, 256, 0, st>>>(s->act[0], s->dy[0], n, kHid, scale, s->grad + paramOffset(0));
    CR_LAUNCH_CHECK();
    for (int l = 1; l < kLayers - 1; l++) {
        kWeightGrad<kHid, kHid><<<gb, 256, 0, st>>>(s->act[l], s->dy[l], n, kHid, scale, s->grad + paramOffset(l));
        CR_LAUNCH_CHECK();
    }
    kWeightGrad<kHid, 16><<<gb, 256, 0, st>>>(s->act[kLayers - 1], s->dy[kLayers - 1], n, 3, scale,
                                             s->grad + paramOffset(kLayers - 1));
    CR_LAUNCH_CHECK();
    return CR_OK;
}

int mlpAdamDevice(MlpState* s, cudaStream_t st) {
    s->step++;
    const float c1 = 1.0f - std::pow(s->cfg.beta1, (float)s->step);
    const float c2 = 1.0f - std::pow(s->cfg.beta2, (float)s->step);
    kAdam<<<cdiv(kParams, 256), 256, 0, st>>>(s->w, s->m, s->v, s->grad, kParams, s->cfg.lr, s->cfg.beta1,
                                               s->cfg.beta2, s->cfg.eps, c1, c2);
    CR_LAUNCH_CHECK();
    return pack(s, st);
}

float* mlpLossPtr(MlpState* s) { return s->loss; }

}  // namespace cr

using namespace cr;

extern "C" {

uint64_t cr_mlp_param_count(void) { return kParams; }

int cr_mlp_create(const cr_mlp_config* cfg, cr_mlp** out) {
    clearError();
    if (!cfg || !out) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    MlpState* s = nullptr;
    int rc = mlpCreate(cfg, &s);
    if (rc) return rc;
    *out = new cr_mlp{s};
    return CR_OK;
}

int cr_mlp_destroy(cr_mlp* m) {
    clearError();
    if (m) {
        mlpDestroy(m->s);
        delete m;
    }
    return CR_OK;
}

int cr_mlp_get_params(cr_mlp* m, float* out) {
    clearError();
    if (!m || !out) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    CR_CUDA(cudaDeviceSynchronize());
    CR_CUDA(cudaMemcpy(out, m->s->w, kParams * sizeof(float), cudaMemcpyDeviceToHost));
    return CR_OK;
}

int cr_mlp_set_params(cr_mlp* m, const float* in) {
    clearError();
    if (!m || !in) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    CR_CUDA(cudaMemcpy(m->s->w, in, kParams * sizeof(float), cudaMemcpyHostToDevice));
    int rc = pack(m->s, 0);
    if (rc) return rc;
    CR_CUDA(cudaDeviceSynchronize());
    return CR_OK;
}

int cr_mlp_infer(cr_mlp* m, const float* inputs, uint64_t n, float* outputs) {
    clearError();
    if (!m || (n && (!inputs || !outputs))) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0) return CR_OK;
    int rc = ensureStage(m->s, n);
    if (rc) return rc;
    CR_CUDA(cudaMemcpy(m->s->stageIn, inputs, n * kIn * sizeof(float), cudaMemcpyHostToDevice));
    rc = mlpInferDevice(m->s, m->s->stageIn, n, m->s->stageOut, false, 0);
    if (rc) return rc;
    CR_CUDA(cudaMemcpy(outputs, m->s->stageOut, n * 3 * sizeof(float), cudaMemcpyDeviceToHost));
    return CR_OK;
}

static int gradOrTrain(cr_mlp* m, const float* inputs, const float* targets, uint64_t n, float* grads, float* loss,
                       bool step) {
    clearError();
    if (!m || (n && (!inputs || !targets))) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0) return CR_OK;
    MlpState* s = m->s;
    int rc = ensureStage(s, n);
    if (rc) return rc;
    CR_CUDA(cudaMemcpy(s->stageIn, inputs, n * kIn * sizeof(float), cudaMemcpyHostToDevice));
    CR_CUDA(cudaMemcpy(s->stageOut, targets, n * 3 * sizeof(float), cudaMemcpyHostToDevice));
    CR_CUDA(cudaMemset(s->grad, 0, kParams * sizeof(float)));
    rc = mlpGradDevice(s, s->stageIn, s->stageOut, n, 0);
    if (rc) return rc;
    if (grads) CR_CUDA(cudaMemcpy(grads, s->grad, kParams * sizeof(float), cudaMemcpyDeviceToHost));
    if (loss) {
        float l = 0;
        CR_CUDA(cudaMemcpy(&l, s->loss, sizeof(float), cudaMemcpyDeviceToHost));
        *loss = l / (3.0f * (float)n);
    }
    if (step) {
        rc = mlpAdamDevice(s, 0);
        if (rc) return rc;
    } else {
        CR_CUDA(cudaMemset(s->grad, 0, kParams * sizeof(float)));
    }
    CR_CUDA(cudaDeviceSynchronize());
    return CR_OK;
}

int cr_mlp_gradients(cr_mlp* m, const float* inputs, const float* targets, uint64_t n, float* grads, float* loss) {
    return gradOrTrain(m, inputs, targets, n, grads, loss, false);
}

int cr_mlp_train_step(cr_mlp* m, const float* inputs, const float* targets, uint64_t n, float* loss) {
    return gradOrTrain(m, inputs, targets, n, nullptr, loss, true);
}

}  // extern "C"
