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
//              seven warpgroups of a persistent CTA carries a tile of 128
//              queries through all six layers.  The weights are brought into
//              shared memory once per CTA by bulk asynchronous copies; each
//              layer is tcgen05.mma (M 128, N 64 or 16, K 16 per instruction)
//              from shared-memory operands into a 64-column TMEM accumulator
//              per warpgroup, read back with tcgen05.ld, ReLU'd and written as
//              the next layer's FP16 operand.  Seven tiles in flight per SM
//              overlap some warpgroups' encoding and epilogues with the
//              others' MMAs.
//   kTrainTc   one training pass on the 5th-generation tensor cores: a
//              persistent CTA per SM carries tiles of 128 records through the
//              forward, the loss gradient, the backward data gradients and
//              the weight gradients (the last accumulated in TMEM over all
//              the CTA's tiles).
//   kReduceAdam the rest of a training step in one launch: the CTAs'
//              partials summed, Adam on the FP32 master weights and the
//              FP16 core-matrix tiles of the weights refreshed (W_l for the
//              forward, W_l^T for the backward data gradients).
//              kReduceGrad sums the partials alone (gradient queries);
//              kPackWeights refreshes every tile (weights set by the caller).

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
// (K, N) of each layer's weight matrix
__host__ __device__ constexpr int layerK(int l) { return l == 0 ? kFeat : kHid; }
__host__ __device__ constexpr int layerN(int l) { return l == kLayers - 1 ? 3 : kHid; }
// offsets in the flat FP32 parameter vector (k-major: W[k][n] at k * N + n)
__host__ __device__ constexpr int paramOffset(int l) { return l == 0 ? 0 : kFeat * kHid + (l - 1) * kHid * kHid; }
constexpr int kParams = kFeat * kHid + 4 * kHid * kHid + kHid * 3;  // 27,840

constexpr float kGradClip = 256.0f;  // |dL/dy| per sample and channel

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
constexpr int kSlots = 7;                      // warpgroups per CTA, one tile each
__host__ __device__ constexpr int layerNpad(int l) { return l == kLayers - 1 ? 16 : kHid; }
__host__ __device__ constexpr int tcBytes(int l) { return layerK(l) * layerNpad(l) * 2; }
__host__ __device__ constexpr int tcOffset(int l) {
    int o = 0;
    for (int i = 0; i < l; i++) o += tcBytes(i);
    return o;
}
constexpr int kTcWeightBytes = tcOffset(kLayers);        // 57,344
// A slot's operand buffer holds one part of layer 0's input (chunks 0..11,
// inputs 0..3, or chunks 12..21, inputs 4..6 and the zero chunk) or a hidden
// layer's input (8 chunks): 12 chunks of 2048 B.  Layer 0 runs as two MMA
// groups, K = 96 then K = 80, accumulating into the same TMEM columns, so
// that seven tiles fit in flight per SM instead of three with whole 176-wide
// layer-0 operands.
constexpr int kTcPart0Chunks = 12;
constexpr int kTcPart0Steps = kTcPart0Chunks / 2;        // K16 steps of the first group
constexpr int kTcABytes = kTcPart0Chunks * 2048;         // 24,576 per slot
constexpr int kTcSmemW = kSlots * kTcABytes;             // the A buffers come first
constexpr int kTcSmemBar = kTcSmemW + kTcWeightBytes;    // 204,800: mbarriers, TMEM address
// The allocation extends to the per-block maximum, about 3 KB past the
// barriers.
constexpr int kTcSmem = 232448;
constexpr uint32_t kTcCols = 512;                        // 64 per slot, a power of two
constexpr uint32_t kTcSpin = 1u << 20;                   // bounded waits (try_wait rounds)
static_assert(kTcSmemBar + 8 + 8 * kSlots + 4 <= kTcSmem, "tensor-core inference shared memory");
static_assert(kTcSmem <= 232448, "tensor-core inference shared memory");
static_assert(64u * kSlots <= kTcCols, "TMEM columns");
static_assert(kFeat / 8 - kTcPart0Chunks <= kTcPart0Chunks, "layer-0 parts");

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

// Encodes row `row` of the inputs (zeros past n) into row lt of a layer-0
// operand at sA: chunk 3d + q holds f = 4q .. 4q+3 of input d; chunk 21
// (features 168..175) is zero.  part -1 writes all 22 chunks; part 0 only
// chunks 0..11 (inputs 0..3) and part 1 chunks 12..21 (inputs 4..6, then the
// zero chunk), each part to chunk positions 0.. of sA.
__device__ __forceinline__ void encodeRowTc(const float* __restrict__ in, uint64_t n, uint64_t row, uint32_t sA,
                                            int lt, int part = -1) {
    const int d0 = part == 1 ? kTcPart0Chunks / 3 : 0, d1 = part == 0 ? kTcPart0Chunks / 3 : kIn;
    const int shift = part == 1 ? kTcPart0Chunks : 0;
#pragma unroll 1
    for (int d = d0; d < d1; d++) {
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
            stShared4(sA + (d * 3 + q - shift) * 2048 + lt * 16, v[0], v[1], v[2], v[3]);
        }
    }
    if (part != 0) stShared4(sA + (kFeat / 8 - 1 - shift) * 2048 + lt * 16, 0u, 0u, 0u, 0u);
}

// Persistent: CTA b's warpgroup g takes tiles b * kSlots + g, stepping by
// gridDim.x * kSlots.  A tile runs seven MMA groups: layer 0 in two parts
// (its operand encoded part by part into the slot's buffer), then layers
// 1..5.  A wait that runs out (it should never) sets bit 0 of *err, ends the
// warpgroup's loop and still frees the TMEM.
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
        const uint64_t row = tile * kTile + lt;
        encodeRowTc(in, n, row, sA, lt, 0);
        proxyFence();
        tcBefore();
        wgSync(g);
#pragma unroll 1
        for (int grp = 0; grp <= kLayers; grp++) {
            const int l = grp == 0 ? 0 : grp - 1;  // groups 0 and 1 are layer 0's two parts
            if (lt == 0) {
                tcAfter();
                const int Np = layerNpad(l);
                const int k0 = grp == 1 ? kTcPart0Steps : 0, k1 = grp == 0 ? kTcPart0Steps : layerK(l) / 16;
                const uint32_t idesc = tcInstr(kTile, Np), wl = sW + tcOffset(l);
                for (int k = k0; k < k1; k++)
                    tcMma(tmem, tcDesc(sA + (k - k0) * 2 * 2048, 2048, 128),
                          tcDesc(wl + k * 2 * (Np * 16), Np * 16, 128), idesc, k > 0 ? 1u : 0u);
                tcCommit(barM);
            }
            ok = wgAnd(g, mbarWait(barM, phase));
            phase ^= 1u;
            tcAfter();
            if (!ok) break;
            if (grp == 0) {
                // the first part is consumed: the second part into the same buffer
                encodeRowTc(in, n, row, sA, lt, 1);
                proxyFence();
            } else if (l < kLayers - 1) {
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

// ---------------------------------------------------------------------------
// training on the tensor cores (tcgen05)
// ---------------------------------------------------------------------------
// One persistent CTA per SM with one warpgroup; thread t owns record t of
// the current tile of 128.  Per tile:
//   forward   Y_l = A_l W_l for l = 0..5 (M 128 records, N 64 / 16, K the
//             layer's inputs), ReLU into A_{l+1}; all six inputs stay in
//             shared memory in the inference kernel's core-matrix layout;
//   loss      dY_5 = clip(2 (y - t) / (y^2 + 0.01)) (FP16, 16 columns);
//   backward  for l = 5..1: dW_l += A_l^T dY_l and dA_l = dY_l W_l^T, then
//             dY_{l-1} = dA_l * (A_l > 0) is written over A_l, which the
//             weight-gradient MMA no longer needs; finally dW_0 += A_0^T dY_0.
// The weight gradients are MMAs with M = 128 input features (layers with 64
// read 64 features of the next buffer into rows that are never used), N =
// the layer's outputs and K = 128 records.  Their operands are the same
// tiles read MN-major: a core matrix of the record-major layout holds 8
// records x 8 features, which is the MN-major core matrix of the transpose.
// For these MN-major operands the descriptor's leading-dimension offset is
// the stride between core matrices along K (8 records, 128 B) and its
// stride-dimension offset the stride along M or N (8 features, 2048 B), the
// same roles the two offsets have for K-major operands (found on GB300: the
// other assignment gives wrong gradients; both stay inside the allocation).
// The dW accumulators stay in TMEM across all the CTA's tiles (400 of its
// 512 columns) and are written once per CTA as FP32 partials; kReduceGrad
// sums the partials of all CTAs.  Every wait is bounded: one that runs out
// sets bit 1 of *err, ends the loop, and the TMEM is still freed.
constexpr int kTrThreads = 128;
constexpr int kTrChunk = kTile * 16;  // 8 features of 128 records: 2048 B
// backward-data weights, B = W_l^T as N = 64 inputs x K = outputs (16 for the
// output layer), K-major core matrices; layer 0 needs none
__host__ __device__ constexpr int bwdKpad(int l) { return l == kLayers - 1 ? 16 : kHid; }
__host__ __device__ constexpr int tcBwdBytes(int l) { return l == 0 ? 0 : kHid * bwdKpad(l) * 2; }
__host__ __device__ constexpr int tcBwdOffset(int l) {
    int o = 0;
    for (int i = 1; i < l; i++) o += tcBwdBytes(i);
    return o;
}
constexpr int kTcBwdBytes = tcBwdOffset(kLayers);  // 34,816
// shared memory: layer inputs (A_0: 22 chunks, A_1..A_5: 8 chunks each), the
// output layer's dY (2 chunks), forward and backward weights, barriers
__host__ __device__ constexpr int trA(int l) { return l == 0 ? 0 : (kFeat / 8) * kTrChunk + (l - 1) * 8 * kTrChunk; }
constexpr int kTrDy5 = trA(kLayers);
constexpr int kTrWf = kTrDy5 + 2 * kTrChunk;
constexpr int kTrWb = kTrWf + kTcWeightBytes;
constexpr int kTrBar = kTrWb + kTcBwdBytes;
// 4 KB past the barriers, as for inference: operand reads stay inside the
// allocation under either reading of the descriptors' two strides
constexpr int kTrSmem = kTrBar + 64 + 4096;
static_assert(kTrSmem <= 232448, "tensor-core training shared memory");
// TMEM columns: the forward / backward-data accumulator, then dW per layer
// (layer 0 in two groups of 128 input features)
constexpr uint32_t kTrCols = 512;
__host__ __device__ constexpr uint32_t trDwCol(int l, int grp) {
    return l == 0 ? 64u + 64u * (uint32_t)grp : (l < kLayers - 1 ? 192u + 64u * (uint32_t)(l - 1) : 448u);
}
static_assert(trDwCol(kLayers - 1, 0) + 16 <= kTrCols, "TMEM columns");
constexpr uint32_t kTcMnA = 1u << 15, kTcMnB = 1u << 16;  // MN-major A / B in the instruction descriptor

__device__ __forceinline__ void ldShared4(uint32_t addr, uint32_t v[4]) {
    asm volatile("ld.shared.v4.b32 {%0,%1,%2,%3}, [%4];" : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]) : "r"(addr)
                 : "memory");
}

__global__ void __launch_bounds__(kTrThreads, 1) kTrainTc(const uint8_t* __restrict__ wTc,
                                                          const uint8_t* __restrict__ wTcT,
                                                          const float* __restrict__ in,
                                                          const float* __restrict__ target, uint64_t n,
                                                          float* __restrict__ part, float* __restrict__ lossSum,
                                                          uint32_t* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t base = smemAddr(sm);
    const uint32_t barW = base + kTrBar, barM = barW + 8, slot = barW + 16;
    if (tid == 0) {
        mbarInit(barW, 1);
        mbarInit(barM, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(kTrCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tcBefore();
    __syncthreads();
    tcAfter();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + kTrBar + 16);
    const uint32_t tq = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's lanes (records, or features for dW)
    if (tid == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(barW),
                     "r"((uint32_t)(kTcWeightBytes + kTcBwdBytes))
                     : "memory");
        for (int off = 0; off < kTcWeightBytes; off += 8192) {
            const uint32_t bytes = (uint32_t)(kTcWeightBytes - off < 8192 ? kTcWeightBytes - off : 8192);
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    base + kTrWf + off),
                "l"(wTc + off), "r"(bytes), "r"(barW)
                : "memory");
        }
        for (int off = 0; off < kTcBwdBytes; off += 8192) {
            const uint32_t bytes = (uint32_t)(kTcBwdBytes - off < 8192 ? kTcBwdBytes - off : 8192);
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    base + kTrWb + off),
                "l"(wTcT + off), "r"(bytes), "r"(barW)
                : "memory");
        }
    }
    bool ok = __syncthreads_and(mbarWait(barW, 0));
    uint32_t phase = 0;
    float lossLocal = 0.0f;
    // waits for the MMAs committed so far; false when the wait runs out.  Each
    // thread waits for itself: the barrier at the end of the phase that
    // follows makes the outcome uniform (one barrier per phase instead of two,
    // 2 % of a step)
    auto waitMma = [&]() {
        const bool done = mbarWait(barM, phase);
        phase ^= 1u;
        tcAfter();
        return done;
    };
    const uint64_t tiles = (n + kTile - 1) / kTile;
    bool first = true;
    for (uint64_t tile = blockIdx.x; ok && tile < tiles; tile += gridDim.x) {
        const uint64_t row = tile * kTile + tid;
        encodeRowTc(in, n, row, base + trA(0), tid);
        proxyFence();
        tcBefore();
        __syncthreads();
        // forward
#pragma unroll 1
        for (int l = 0; ok && l < kLayers; l++) {
            if (tid == 0) {
                tcAfter();
                const int K = layerK(l), Np = layerNpad(l);
                const uint32_t idesc = tcInstr(kTile, Np), wl = base + kTrWf + tcOffset(l);
                for (int k = 0; k < K / 16; k++)
                    tcMma(tmem, tcDesc(base + trA(l) + k * 2 * kTrChunk, kTrChunk, 128),
                          tcDesc(wl + k * 2 * (Np * 16), Np * 16, 128), idesc, k > 0 ? 1u : 0u);
                tcCommit(barM);
            }
            const bool done = waitMma();
            if (l < kLayers - 1) {
                const uint32_t dst = base + trA(l + 1) + tid * 16;
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
                        stShared4(dst + (h * 4 + c) * kTrChunk, q[0], q[1], q[2], q[3]);
                    }
                }
            } else {
                // relative L2 loss (y - t)^2 / (sg(y)^2 + 0.01) and its gradient
                // 2 (y - t) / (y^2 + 0.01), clipped to +-kGradClip so that the FP16
                // gradient path stays finite; the 1 / (3 n) of the mean is applied
                // when the partials are summed
                uint32_t v[4];
                tcLoad4(tq, v);
                tcLoadWait();
                float d[3] = {0.0f, 0.0f, 0.0f};
                if (row < n) {
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float y = __uint_as_float(v[c]), t = target[row * 3 + c];
                        const float den = y * y + 0.01f;
                        d[c] = fminf(fmaxf(2.0f * (y - t) / den, -kGradClip), kGradClip);
                        lossLocal += (y - t) * (y - t) / den;
                    }
                }
                stShared4(base + kTrDy5 + tid * 16, pack2(d[0], d[1]), pack2(d[2], 0.0f), 0u, 0u);
                stShared4(base + kTrDy5 + kTrChunk + tid * 16, 0u, 0u, 0u, 0u);
            }
            proxyFence();
            tcBefore();
            ok = __syncthreads_and(done);
        }
        // backward: weight and data gradients, layers 5..1
#pragma unroll 1
        for (int l = kLayers - 1; ok && l >= 1; l--) {
            const uint32_t dy = l == kLayers - 1 ? base + kTrDy5 : base + trA(l + 1);  // dY_l
            const int Nl = bwdKpad(l);
            if (tid == 0) {
                tcAfter();
                const uint32_t idw = tcInstr(kTile, Nl) | kTcMnA | kTcMnB;
                for (int k = 0; k < kTile / 16; k++)
                    tcMma(tmem + trDwCol(l, 0), tcDesc(base + trA(l) + k * 256, 128, kTrChunk),
                          tcDesc(dy + k * 256, 128, kTrChunk), idw, (first && k == 0) ? 0u : 1u);
                const uint32_t wb = base + kTrWb + tcBwdOffset(l);
                for (int k = 0; k < Nl / 16; k++)
                    tcMma(tmem, tcDesc(dy + k * 2 * kTrChunk, kTrChunk, 128), tcDesc(wb + k * 2 * 1024, 1024, 128),
                          tcInstr(kTile, kHid), k > 0 ? 1u : 0u);
                tcCommit(barM);
            }
            const bool done = waitMma();
            const uint32_t a = base + trA(l) + tid * 16;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                uint32_t v[32];
                tcLoad32(tq + h * 32, v);
                tcLoadWait();
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    uint32_t act[4], q[4];
                    ldShared4(a + (h * 4 + c) * kTrChunk, act);
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const float2 av = unpack2(act[e]);
                        q[e] = pack2(av.x > 0.0f ? __uint_as_float(v[c * 8 + 2 * e]) : 0.0f,
                                     av.y > 0.0f ? __uint_as_float(v[c * 8 + 2 * e + 1]) : 0.0f);
                    }
                    stShared4(a + (h * 4 + c) * kTrChunk, q[0], q[1], q[2], q[3]);
                }
            }
            proxyFence();
            tcBefore();
            ok = __syncthreads_and(done);
        }
        if (!ok) break;
        // dW_0 += A_0^T dY_0 (dY_0 is over A_1), input features in two groups of 128
        if (tid == 0) {
            tcAfter();
            const uint32_t idw = tcInstr(kTile, kHid) | kTcMnA | kTcMnB;
            for (int grp = 0; grp < 2; grp++)
                for (int k = 0; k < kTile / 16; k++)
                    tcMma(tmem + trDwCol(0, grp), tcDesc(base + trA(0) + grp * 16 * kTrChunk + k * 256, 128, kTrChunk),
                          tcDesc(base + trA(1) + k * 256, 128, kTrChunk), idw, (first && k == 0) ? 0u : 1u);
            tcCommit(barM);
        }
        {
            const bool done = waitMma();
            tcBefore();
            ok = __syncthreads_and(done);
        }
        first = false;
    }
    tcBefore();
    __syncthreads();
    tcAfter();
    // this CTA's dW partials: lane = input feature k, column = output n,
    // stored output-major (slot paramOffset(l) + n K_l + k, partialSlotParam)
    // so that a warp's 32 lanes write 128 contiguous bytes per column
    if (ok) {
        float* p = part + (size_t)blockIdx.x * kParams;
        const int lane = tid & 31;
#pragma unroll 1
        for (int l = 0; l < kLayers; l++) {
            const int groups = l == 0 ? 2 : 1, K = layerK(l);
            for (int grp = 0; grp < groups; grp++) {
                const int k = grp * 128 + warp * 32 + lane;
                const bool valid = k < K;
                const uint32_t col = tq + trDwCol(l, grp);
                if (l < kLayers - 1) {
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        uint32_t v[32];
                        tcLoad32(col + h * 32, v);
                        tcLoadWait();
                        if (valid) {
                            float* dst = p + paramOffset(l) + h * 32 * K + k;
#pragma unroll
                            for (int j = 0; j < 32; j++) dst[j * K] = __uint_as_float(v[j]);
                        }
                    }
                } else {
                    uint32_t v[4];
                    tcLoad4(col, v);
                    tcLoadWait();
                    if (valid)
                        for (int j = 0; j < 3; j++) p[paramOffset(l) + j * K + k] = __uint_as_float(v[j]);
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) lossLocal += __shfl_xor_sync(0xffffffffu, lossLocal, o);
    if ((tid & 31) == 0) atomicAdd(lossSum, lossLocal);
    tcBefore();
    __syncthreads();
    tcAfter();
    if (!ok && tid == 0) atomicOr(err, 2u);
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTrCols) : "memory");
}

// The parameter (k-major index paramOffset(l) + k N_l + n) of partial slot
// paramOffset(l) + n K_l + k.  Every layer's slots start on a multiple of 32,
// so a warp's 32 slots lie in one layer.
__device__ __forceinline__ int partialSlotParam(int slot) {
    int l = 0;
    while (l < kLayers - 1 && slot >= paramOffset(l + 1)) l++;
    const int K = layerK(l), local = slot - paramOffset(l);
    return paramOffset(l) + (local % K) * layerN(l) + local / K;
}
static_assert(paramOffset(1) % 32 == 0 && paramOffset(kLayers - 1) % 32 == 0 && kParams % 32 == 0,
              "whole warps of partial slots per layer");

// Sum over the CTAs' weight-gradient partials for slots 32 b .. 32 b + 31
// (block b of kRedThreads): warp w adds partials w, w + kRedWarps, ..., the
// lanes one 128-byte row each, and warp 0 adds the warps' sums in a fixed
// order (so the result depends only on the partials).  Valid in warp 0.
constexpr int kRedWarps = 8;  // 16 measured 4 % slower
constexpr int kRedThreads = kRedWarps * 32;

__device__ __forceinline__ float sumPartials(const float* __restrict__ part, int parts, int i) {
    __shared__ float red[kRedWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float s = 0.0f;
#pragma unroll 4
    for (int b = w; b < parts; b += kRedWarps) s += part[(size_t)b * kParams + i];
    red[w][lane] = s;
    __syncthreads();
    float t = 0.0f;
    if (w == 0)
        for (int k = 0; k < kRedWarps; k++) t += red[k][lane];
    return t;
}

// FP16 core-matrix tiles of parameter i: W_l for inference and the training
// forward, W_l^T for the training backward (the padding, zeroed once, is
// never written).
__device__ __forceinline__ void packParam(int i, float wi, __half* __restrict__ tc, __half* __restrict__ tcT) {
    int l = 0;
    while (l < kLayers - 1 && i >= paramOffset(l + 1)) l++;
    const int N = layerN(l);
    const int local = i - paramOffset(l), k = local / N, n = local % N;
    const __half h = __float2half_rn(wi);
    tc[(tcOffset(l) + ((k >> 3) * (layerNpad(l) >> 3) + (n >> 3)) * 128 + (n & 7) * 16 + (k & 7) * 2) / 2] = h;
    // backward-data operand W_l^T: N = input k, K = output n
    if (l > 0) tcT[(tcBwdOffset(l) + ((n >> 3) * (kHid >> 3) + (k >> 3)) * 128 + (k & 7) * 16 + (n & 7) * 2) / 2] = h;
}

// grad += scale * (sum of the CTAs' partials)
__global__ void __launch_bounds__(kRedThreads) kReduceGrad(const float* __restrict__ part, int parts, float scale,
                                                           float* __restrict__ grad) {
    const int slot = blockIdx.x * 32 + (threadIdx.x & 31);
    const float t = sumPartials(part, parts, slot);
    if (threadIdx.x < 32) grad[partialSlotParam(slot)] += t * scale;
}

struct AdamArgs {
    float lr, b1, b2, eps, c1, c2;  // c1, c2: the bias corrections 1 - beta^step
};

// One training step's tail in one launch: the gradient (grad + scale * the
// partials' sum), Adam on the FP32 master weights, the gradient cleared for
// the next step and the weight's FP16 tiles refreshed.
__global__ void __launch_bounds__(kRedThreads) kReduceAdam(const float* __restrict__ part, int parts, float scale,
                                                           float* __restrict__ grad, float* __restrict__ w,
                                                           float* __restrict__ m, float* __restrict__ v,
                                                           const AdamArgs a, __half* __restrict__ tc,
                                                           __half* __restrict__ tcT) {
    const int slot = blockIdx.x * 32 + (threadIdx.x & 31);
    const float t = sumPartials(part, parts, slot);
    if (threadIdx.x >= 32) return;
    const int i = partialSlotParam(slot);
    const float gr = grad[i] + t * scale;
    const float mi = a.b1 * m[i] + (1.0f - a.b1) * gr;
    const float vi = a.b2 * v[i] + (1.0f - a.b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - a.lr * (mi / a.c1) / (sqrtf(vi / a.c2) + a.eps);
    w[i] = wi;
    grad[i] = 0.0f;
    packParam(i, wi, tc, tcT);
}

// Refreshes the FP16 tiles of every weight (after the weights are set).
__global__ void kPackWeights(const float* __restrict__ w, __half* __restrict__ tc, __half* __restrict__ tcT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    packParam(i, w[i], tc, tcT);
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
    __half* wTc = nullptr;      // inference and training forward operand tiles (kTcWeightBytes)
    __half* wTcT = nullptr;     // training backward-data operand tiles (kTcBwdBytes)
    float* part = nullptr;      // per-CTA weight-gradient partials of the training kernel (sms x kParams)
    uint32_t* err = nullptr;    // bit 0: a tensor-core wait ran out
    float* stageIn = nullptr;
    float* stageOut = nullptr;
    uint64_t stageCap = 0;
    uint32_t step = 0;
    int sms = 0;
};

namespace {

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
    kPackWeights<<<cdiv(kParams, 256), 256, 0, st>>>(s->w, s->wTc, s->wTcT);
    CR_LAUNCH_CHECK();
    return CR_OK;
}

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
    CR_CUDA(cudaMalloc(&s->wTc, kTcWeightBytes));
    CR_CUDA(cudaMemset(s->wTc, 0, kTcWeightBytes));
    CR_CUDA(cudaMalloc(&s->wTcT, kTcBwdBytes));
    CR_CUDA(cudaMemset(s->wTcT, 0, kTcBwdBytes));
    CR_CUDA(cudaMalloc(&s->part, (size_t)s->sms * kParams * sizeof(float)));
    CR_CUDA(cudaMalloc(&s->err, sizeof(uint32_t)));
    CR_CUDA(cudaMemset(s->err, 0, sizeof(uint32_t)));
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
    CR_CUDA(cudaFuncSetAttribute(kTrainTc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrSmem));
    int rc = pack(s, 0);
    if (rc) return rc;
    CR_CUDA(cudaDeviceSynchronize());
    *out = s;
    return CR_OK;
}

void mlpDestroy(MlpState* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    void* p[] = {s->w, s->m, s->v, s->grad, s->loss, s->wTc, s->wTcT, s->err, s->part, s->stageIn, s->stageOut};
    for (void* q : p)
        if (q) cudaFree(q);
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
        return fail(CR_ERR_CUDA, "radiance-cache network: a tensor-core wait timed out (%s)",
                    (e & 2u) ? ((e & 1u) ? "inference and training" : "training") : "inference");
    }
    return CR_OK;
}

// kTrainTc over n samples: the CTAs' weight-gradient partials of the mean
// relative L2 loss in s->part (returns the CTA count), the loss sum in s->loss.
int trainPartials(MlpState* s, const float* in, const float* target, uint64_t n, cudaStream_t st,
                  unsigned& blocks) {
    CR_CUDA(cudaMemsetAsync(s->loss, 0, sizeof(float), st));
    // one persistent CTA per SM at most (its shared memory admits one), every
    // CTA with the same number of tiles: the slowest CTA's tile count is the
    // same as with one CTA per SM, and fewer CTAs leave fewer partials to sum
    // (65,536 records: 128 CTAs of 4 tiles instead of 152 of 3 or 4, 0.055
    // against 0.056-0.057 ms per step)
    const unsigned tiles = std::max(1u, cdiv(n, kTile)), perCta = cdiv(tiles, (unsigned)s->sms);
    blocks = cdiv(tiles, perCta);
    kTrainTc<<<blocks, kTrThreads, kTrSmem, st>>>(reinterpret_cast<const uint8_t*>(s->wTc),
                                                 reinterpret_cast<const uint8_t*>(s->wTcT), in, target, n, s->part,
                                                 s->loss, s->err);
    CR_LAUNCH_CHECK();
    return CR_OK;
}

// Accumulates dW of the mean relative L2 loss over n samples into s->grad.
int mlpGradDevice(MlpState* s, const float* in, const float* target, uint64_t n, cudaStream_t st) {
    if (n == 0) return CR_OK;
    unsigned blocks = 0;
    int rc = trainPartials(s, in, target, n, st, blocks);
    if (rc) return rc;
    kReduceGrad<<<kParams / 32, kRedThreads, 0, st>>>(s->part, (int)blocks, 1.0f / (3.0f * (float)n), s->grad);
    CR_LAUNCH_CHECK();
    return CR_OK;
}

// One Adam step on s->grad + dW of n samples (n may be 0): two launches,
// kTrainTc and kReduceAdam.  Leaves s->grad zeroed.
int mlpTrainStepDevice(MlpState* s, const float* in, const float* target, uint64_t n, cudaStream_t st) {
    unsigned blocks = 0;
    if (n) {
        int rc = trainPartials(s, in, target, n, st, blocks);
        if (rc) return rc;
    }
    s->step++;
    const AdamArgs a{s->cfg.lr, s->cfg.beta1, s->cfg.beta2, s->cfg.eps,
                     1.0f - std::pow(s->cfg.beta1, (float)s->step), 1.0f - std::pow(s->cfg.beta2, (float)s->step)};
    kReduceAdam<<<kParams / 32, kRedThreads, 0, st>>>(s->part, (int)blocks, n ? 1.0f / (3.0f * (float)n) : 0.0f,
                                                       s->grad, s->w, s->m, s->v, a, s->wTc, s->wTcT);
    CR_LAUNCH_CHECK();
    return CR_OK;
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
    rc = step ? mlpTrainStepDevice(s, s->stageIn, s->stageOut, n, 0) : mlpGradDevice(s, s->stageIn, s->stageOut, n, 0);
    if (rc) return rc;
    if (grads) CR_CUDA(cudaMemcpy(grads, s->grad, kParams * sizeof(float), cudaMemcpyDeviceToHost));
    if (loss) {
        float l = 0;
        CR_CUDA(cudaMemcpy(&l, s->loss, sizeof(float), cudaMemcpyDeviceToHost));
        *loss = l / (3.0f * (float)n);
    }
    if (!step) CR_CUDA(cudaMemset(s->grad, 0, kParams * sizeof(float)));
    CR_CUDA(cudaDeviceSynchronize());
    return mlpCheck(s);
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
    // each step leaves the gradient zeroed, so every step starts from zero
    return mlpTrainStepDevice(m->s, inputs, targets, n, (cudaStream_t)stream);
}

int cr_mlp_gradients(cr_mlp* m, const float* inputs, const float* targets, uint64_t n, float* grads, float* loss) {
    return gradOrTrain(m, inputs, targets, n, grads, loss, false);
}

int cr_mlp_train_step(cr_mlp* m, const float* inputs, const float* targets, uint64_t n, float* loss) {
    return gradOrTrain(m, inputs, targets, n, nullptr, loss, true);
}

}  // extern "C"
