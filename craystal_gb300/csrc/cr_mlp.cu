// cr_mlp.cu -- the radiance-cache network: a 7-input MLP with a 12-frequency
// sin / cos encoding (168 features, padded to 176), five hidden layers of 64
// ReLU units and 3 linear outputs (RGB radiance), FP16 weights and
// activations with FP32 accumulation on the tensor cores, trained online
// with Adam on a relative L2 loss.
//
// This part has no counterpart in the reference; it is the cache that ends
// paths early (see cr_cache.cu).
//
// Kernels
//   kInferTc   fused forward on the 5th-generation tensor cores: each of
//              three warpgroups of a persistent CTA carries a tile of 128
//              queries through all six layers.  The weights are brought into
//              shared memory once per CTA by bulk asynchronous copies; each
//              layer is tcgen05.mma (M 128, N 64 or 16, K 16 per instruction)
//              from shared-memory operands into a 64-column TMEM accumulator
//              per warpgroup, read back with tcgen05.ld, ReLU'd and written as
//              the next layer's FP16 operand.  Three tiles in flight per SM
//              overlap one warpgroup's encoding and epilogue with another's
//              MMAs.
//   kTrainFwdBwd  training forward (mma.sync m16n8k16; one warp carries 16
//              rows, activations in registers, every layer's input stored),
//              then the loss gradient and the backward pass for the data
//              gradients, storing every layer's output gradient dY.
//   kWeightGrad   dW_l = X_l^T dY_l over the batch (split over CTAs,
//              accumulated with atomics in FP32).
//   kAdam      Adam on FP32 master weights; kPackWeights refreshes the three
//              FP16 copies (n-major and k-major for training, core-matrix
//              tiles for the tensor-core inference).

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

// The encoding: feature j = d*24 + 2f + {0: sin, 1: cos} of pi * 2^f * x_d.
// For f = 4q the angle is reduced exactly (2^f x is exact, and so is taking
// it modulo 2) and sincospif evaluates it; f = 4q+1 .. 4q+3 follow by the
// double-angle formulas sin 2a = 2 sin a cos a, cos 2a = (cos a - sin a)
// (cos a + sin a).  Three doublings at most keep the error below 1e-6, far
// under the FP16 rounding of the features, at a quarter of the sincospif
// calls.  Training and inference evaluate the same operations.
__device__ __forceinline__ void sincosBase(float x, int f, float& s, float& c) {
    float y = ldexpf(x, f);
    y = y - 2.0f * floorf(y * 0.5f);
    sincospif(y, &s, &c);
}
__device__ __forceinline__ void doubleAngle(float& s, float& c) {
    const float s2 = 2.0f * s * c;
    const float c2 = (c - s) * (c + s);
    s = s2;
    c = c2;
}

// Encoded features j, j+1 (j even) of one query row.
__device__ __forceinline__ uint32_t featurePair(const float* x, int j) {
    if (j >= kIn * kFreq * 2) return 0u;
    const int d = j / (kFreq * 2), f = (j % (kFreq * 2)) >> 1;
    float s, c;
    sincosBase(x[d], f & ~3, s, c);
    for (int r = 0; r < (f & 3); r++) doubleAngle(s, c);
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

// ---------------------------------------------------------------------------
// inference on the tensor cores (tcgen05)
// ---------------------------------------------------------------------------
// Operands sit in shared memory in the canonical K-major layout without
// swizzle: 8 x 8 FP16 core matrices of 128 contiguous bytes (8 rows of 16 B).
//   A (a tile's layer input, 128 rows x K): core (m/8, k/8) at
//     (k/8) * 2048 + (m/8) * 128, so row m's 16-byte chunk k/8 is at
//     (k/8) * 2048 + m * 16 and a warp's 32 rows write 512 contiguous bytes;
//     leading-dimension (K) stride 2048 B, stride-dimension (M) stride 128 B.
//   B (layer l's weights as N x K, K-major): core (n/8, k/8) at
//     ((k/8) * (Npad/8) + n/8) * 128; K stride Npad * 16 B, N stride 128 B.
constexpr int kTile = 128;                     // queries per tile (the MMA's M)
constexpr int kSlots = 3;                      // warpgroups per CTA, one tile each
__host__ __device__ constexpr int layerNpad(int l) { return l == kLayers - 1 ? 16 : kHid; }
__host__ __device__ constexpr int tcBytes(int l) { return layerK(l) * layerNpad(l) * 2; }
__host__ __device__ constexpr int tcOffset(int l) {
    int o = 0;
    for (int i = 0; i < l; i++) o += tcBytes(i);
    return o;
}
constexpr int kTcWeightBytes = tcOffset(kLayers);        // 57,344
constexpr int kTcABytes = kTile * kFeat * 2;             // 45,056 per slot
constexpr int kTcSmemW = kSlots * kTcABytes;             // the A buffers come first
constexpr int kTcSmemBar = kTcSmemW + kTcWeightBytes;    // 192,512: mbarriers, TMEM address
// The allocation extends 4 KB past the barriers, so that every operand read
// stays inside it even under the other assignment of the two descriptor
// strides.
constexpr int kTcSmem = 196608;
constexpr uint32_t kTcCols = 256;                        // 64 per slot, a power of two
constexpr uint32_t kTcSpin = 1u << 20;                   // bounded waits (try_wait rounds)
static_assert(kTcSmemBar + 8 + 8 * kSlots + 4 <= kTcSmem, "tensor-core inference shared memory");

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start, leading- and stride-dimension byte
// offsets (each >> 4), the fixed version bit 46, no swizzle.
__device__ __forceinline__ uint64_t tcDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), FP16
// A and B, both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t tcInstr(int m, int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mbarInit(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
// Waits for phase `phase` of the barrier; false after kTcSpin rounds.
__device__ __forceinline__ bool mbarWait(uint32_t bar, uint32_t phase) {
    for (uint32_t i = 0; i < kTcSpin; i++) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void tcBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tcAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// makes this thread's shared-memory stores visible to the tensor core's reads
__device__ __forceinline__ void proxyFence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void stShared4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1,%2,%3,%4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

__device__ __forceinline__ void tcMma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tcCommit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tcLoad32(uint32_t taddr, uint32_t* v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
        "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tcLoad4(uint32_t taddr, uint32_t* v) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                 : "r"(taddr));
}
__device__ __forceinline__ void tcLoadWait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Barrier and AND vote over the 128 threads of warpgroup g (named barrier g + 1).
__device__ __forceinline__ void wgSync(int g) { asm volatile("bar.sync %0, 128;" ::"r"(g + 1) : "memory"); }
__device__ __forceinline__ bool wgAnd(int g, bool v) {
    uint32_t r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.and.pred p, %2, 128, q;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(g + 1)
        : "memory");
    return r != 0;
}

// Persistent: CTA b's warpgroup g takes tiles b * kSlots + g, stepping by
// gridDim.x * kSlots.  A wait that runs out (it should never) sets bit 0 of
// *err, ends the warpgroup's loop and still frees the TMEM.
__global__ void __launch_bounds__(kTile * kSlots, 1) kInferTc(const uint8_t* __restrict__ wTc,
                                                              const float* __restrict__ in, uint64_t n,
                                                              float* __restrict__ out, int clampNonNeg,
                                                              uint32_t* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    const int tid = threadIdx.x, g = tid / kTile, lt = tid % kTile, warp = tid >> 5, quarter = warp & 3;
    const uint32_t sA = smemAddr(sm + g * kTcABytes), sW = smemAddr(sm + kTcSmemW);
    const uint32_t barW = smemAddr(sm + kTcSmemBar), barM = barW + 8 + 8 * g, slot = barW + 8 + 8 * kSlots;
    if (tid == 0) {
        mbarInit(barW, 1);
        for (int i = 0; i < kSlots; i++) mbarInit(barW + 8 + 8 * i, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tcBefore();
    __syncthreads();
    tcAfter();
    const uint32_t tmemBase = *reinterpret_cast<volatile uint32_t*>(sm + kTcSmemBar + 8 + 8 * kSlots);
    const uint32_t tmem = tmemBase + (uint32_t)(g * 64);               // this warpgroup's accumulator
    const uint32_t tq = tmem + ((uint32_t)(quarter * 32) << 16);        // the lanes (rows) this warp reads
    if (tid == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(barW), "r"((uint32_t)kTcWeightBytes)
                     : "memory");
        for (int off = 0; off < kTcWeightBytes; off += 8192) {
            const uint32_t bytes = (uint32_t)(kTcWeightBytes - off < 8192 ? kTcWeightBytes - off : 8192);
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(sW + off),
                "l"(wTc + off), "r"(bytes), "r"(barW)
                : "memory");
        }
    }
    bool ok = wgAnd(g, mbarWait(barW, 0));
    uint32_t phase = 0;
    const uint64_t tiles = (n + kTile - 1) / kTile;
    for (uint64_t tile = (uint64_t)blockIdx.x * kSlots + g; ok && tile < tiles; tile += (uint64_t)gridDim.x * kSlots) {
        // encode this thread's row: chunk 3d + q holds f = 4q .. 4q+3 of input d
        const uint64_t row = tile * kTile + lt;
#pragma unroll 1
        for (int d = 0; d < kIn; d++) {
            const float xd = row < n ? in[row * kIn + d] : 0.0f;
#pragma unroll
            for (int q = 0; q < kFreq / 4; q++) {
                float sn, cs;
                sincosBase(xd, 4 * q, sn, cs);
                uint32_t v[4];
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    if (r) doubleAngle(sn, cs);
                    v[r] = pack2(sn, cs);
                }
                stShared4(sA + (d * 3 + q) * 2048 + lt * 16, v[0], v[1], v[2], v[3]);
            }
        }
        stShared4(sA + (kFeat / 8 - 1) * 2048 + lt * 16, 0u, 0u, 0u, 0u);  // features 168..175
        proxyFence();
        tcBefore();
        wgSync(g);
#pragma unroll 1
        for (int l = 0; l < kLayers; l++) {
            if (lt == 0) {
                tcAfter();
                const int K = layerK(l), Np = layerNpad(l);
                const uint32_t idesc = tcInstr(kTile, Np), wl = sW + tcOffset(l);
                for (int k = 0; k < K / 16; k++)
                    tcMma(tmem, tcDesc(sA + k * 2 * 2048, 2048, 128), tcDesc(wl + k * 2 * (Np * 16), Np * 16, 128),
                          idesc, k > 0 ? 1u : 0u);
                tcCommit(barM);
            }
            ok = wgAnd(g, mbarWait(barM, phase));
            phase ^= 1u;
            tcAfter();
            if (!ok) break;
            if (l < kLayers - 1) {
                // ReLU, FP16, and into A as the next layer's input (chunks 0..7)
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    uint32_t v[32];
                    tcLoad32(tq + h * 32, v);
                    tcLoadWait();
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        uint32_t q[4];
#pragma unroll
                        for (int e = 0; e < 4; e++)
                            q[e] = pack2(fmaxf(__uint_as_float(v[c * 8 + 2 * e]), 0.0f),
                                         fmaxf(__uint_as_float(v[c * 8 + 2 * e + 1]), 0.0f));
                        stShared4(sA + (h * 4 + c) * 2048 + lt * 16, q[0], q[1], q[2], q[3]);
                    }
                }
                proxyFence();
            } else {
                uint32_t v[4];
                tcLoad4(tq, v);
                tcLoadWait();
                if (row < n) {
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float o = __uint_as_float(v[c]);
                        out[row * 3 + c] = clampNonNeg ? fmaxf(o, 0.0f) : o;
                    }
                }
            }
            // the next MMAs overwrite the accumulator and read A: all loads and stores first
            tcBefore();
            wgSync(g);
        }
    }
    tcBefore();
    __syncthreads();
    tcAfter();
    if (!ok && lt == 0) atomicOr(err, 1u);
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmemBase), "r"(kTcCols) : "memory");
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

// Refreshes the FP16 copies: forward (n-major) and backward (k-major) for
// training, core-matrix tiles for the tensor-core inference (its padding,
// zeroed once, is never written).
__global__ void kPackWeights(const float* __restrict__ w, __half* __restrict__ fwd, __half* __restrict__ bwd,
                             __half* __restrict__ tc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    int l = 0;
    while (l < kLayers - 1 && i >= paramOffset(l + 1)) l++;
    const int N = layerN(l);
    const int local = i - paramOffset(l), k = local / N, n = local % N;
    const __half h = __float2half_rn(w[i]);
    fwd[fwdOffset(l) + n * fwdStride(l) + k] = h;
    bwd[bwdOffset(l) + k * bwdStride(l) + n] = h;
    tc[(tcOffset(l) + ((k >> 3) * (layerNpad(l) >> 3) + (n >> 3)) * 128 + (n & 7) * 16 + (k & 7) * 2) / 2] = h;
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
    __half* wTc = nullptr;      // inference operand tiles (kTcWeightBytes)
    uint32_t* err = nullptr;    // bit 0: a tensor-core wait ran out
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
    kPackWeights<<<cdiv(kParams, 256), 256, 0, st>>>(s->w, s->wFwd, s->wBwd, s->wTc);
    CR_LAUNCH_CHECK();
    return CR_OK;
}

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
    CR_CUDA(cudaMalloc(&s->wTc, kTcWeightBytes));
    CR_CUDA(cudaMemset(s->wTc, 0, kTcWeightBytes));
    CR_CUDA(cudaMalloc(&s->err, sizeof(uint32_t)));
    CR_CUDA(cudaMemset(s->err, 0, sizeof(uint32_t)));
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
    CR_CUDA(cudaFuncSetAttribute(kInferTc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
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
    void* p[] = {s->w, s->m, s->v, s->grad, s->loss, s->wFwd, s->wBwd, s->wTc, s->err, s->stageIn, s->stageOut};
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
    // one persistent CTA per SM (its shared memory admits one), fewer for small batches
    const unsigned blocks = std::min<unsigned>(cdiv(cdiv(n, kTile), kSlots), (unsigned)s->sms);
    kInferTc<<<blocks, kTile * kSlots, kTcSmem, st>>>(reinterpret_cast<const uint8_t*>(s->wTc), in, n, out,
                                                        clampNonNeg ? 1 : 0, s->err);
    CR_LAUNCH_CHECK();
    return CR_OK;
}

// Reports (and clears) a tensor-core wait that ran out; synchronises.
int mlpCheck(MlpState* s) {
    uint32_t e = 0;
    CR_CUDA(cudaMemcpy(&e, s->err, sizeof(e), cudaMemcpyDeviceToHost));
    if (e) {
        CR_CUDA(cudaMemset(s->err, 0, sizeof(uint32_t)));
        return fail(CR_ERR_CUDA, "radiance-cache inference: a tensor-core wait timed out");
    }
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
    return mlpCheck(m->s);
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

int cr_mlp_infer_device(cr_mlp* m, const float* inputs, uint64_t n, float* outputs, void* stream) {
    clearError();
    if (!m || (n && (!inputs || !outputs))) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    CR_CUDA(cudaSetDevice(m->s->device));
    return mlpInferDevice(m->s, inputs, n, outputs, false, (cudaStream_t)stream);
}

int cr_mlp_train_step_device(cr_mlp* m, const float* inputs, const float* targets, uint64_t n, void* stream) {
    clearError();
    if (!m || (n && (!inputs || !targets))) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0) return CR_OK;
    CR_CUDA(cudaSetDevice(m->s->device));
    // kAdam leaves the gradient zeroed, so every step starts from zero
    const cudaStream_t st = (cudaStream_t)stream;
    int rc = mlpGradDevice(m->s, inputs, targets, n, st);
    if (rc) return rc;
    return mlpAdamDevice(m->s, st);
}

int cr_mlp_gradients(cr_mlp* m, const float* inputs, const float* targets, uint64_t n, float* grads, float* loss) {
    return gradOrTrain(m, inputs, targets, n, grads, loss, false);
}

int cr_mlp_train_step(cr_mlp* m, const float* inputs, const float* targets, uint64_t n, float* loss) {
    return gradOrTrain(m, inputs, targets, n, nullptr, loss, true);
}

}  // extern "C"
