// cr_math.cuh -- float3 arithmetic in glm 1.0.1's evaluation order.
// The translation units that include this are compiled with -fmad=false,
// so each product and sum below is rounded separately, as written.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace cr {

__host__ __device__ __forceinline__ float3 mk3(float x, float y, float z) {
    float3 r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
__host__ __device__ __forceinline__ float3 add(float3 a, float3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ float3 sub(float3 a, float3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ float3 neg(float3 a) { return mk3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ float3 mul(float3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 mul(float s, float3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ __forceinline__ float3 divs(float3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
// glm compute_dot<vec3>: (a.x*b.x + a.y*b.y) + a.z*b.z
__host__ __device__ __forceinline__ float dot(float3 a, float3 b) {
    float x = a.x * b.x, y = a.y * b.y, z = a.z * b.z;
    return (x + y) + z;
}
__host__ __device__ __forceinline__ float absDot(float3 a, float3 b) { return fabsf(dot(a, b)); }
// glm compute_cross
__host__ __device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return mk3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
// glm normalize: v * (1 / sqrt(dot(v, v)))
__host__ __device__ __forceinline__ float3 normalize(float3 a) {
    float inv = 1.0f / sqrtf(dot(a, a));
    return mul(a, inv);
}
__host__ __device__ __forceinline__ float length(float3 a) { return sqrtf(dot(a, a)); }
// glm reflect: I - N * dot(N, I) * 2
__host__ __device__ __forceinline__ float3 reflect(float3 I, float3 N) {
    return sub(I, mul(mul(N, dot(N, I)), 2.0f));
}
// std::max / std::min (first argument kept unless the second compares
// strictly greater / smaller; NaN in the second argument is ignored)
__host__ __device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }
__host__ __device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
// glm scalar min / max / clamp
__host__ __device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__host__ __device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }
__host__ __device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }

// float -> int with x86 cvttss2si semantics (NaN / out of range -> INT_MIN),
// the conversion the reference's host build performs.
__host__ __device__ __forceinline__ int f2iX86(float f) {
    if (!(f > -2147483904.0f && f < 2147483648.0f)) return (int)0x80000000;
    return (int)f;
}

// Order-preserving float <-> uint32 encoding for atomic min / max.
__host__ __device__ __forceinline__ uint32_t fenc(float f) {
#ifdef __CUDA_ARCH__
    uint32_t u = __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
#endif
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float fdec(uint32_t u) {
    uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    memcpy(&f, &b, 4);
    return f;
#endif
}

// RGB spectrum (Core/Spectrum.h:237-273), component-wise.
struct Spec {
    float r, g, b;
};
__host__ __device__ __forceinline__ Spec sp(float a) { return Spec{a, a, a}; }
__host__ __device__ __forceinline__ Spec sp(float r, float g, float b) { return Spec{r, g, b}; }
__host__ __device__ __forceinline__ Spec add(Spec a, Spec b) { return Spec{a.r + b.r, a.g + b.g, a.b + b.b}; }
__host__ __device__ __forceinline__ Spec sub(Spec a, Spec b) { return Spec{a.r - b.r, a.g - b.g, a.b - b.b}; }
__host__ __device__ __forceinline__ Spec mul(Spec a, Spec b) { return Spec{a.r * b.r, a.g * b.g, a.b * b.b}; }
__host__ __device__ __forceinline__ Spec mul(Spec a, float s) { return Spec{a.r * s, a.g * s, a.b * s}; }
__host__ __device__ __forceinline__ Spec mul(float s, Spec a) { return Spec{s * a.r, s * a.g, s * a.b}; }
__host__ __device__ __forceinline__ Spec divs(Spec a, float s) { return Spec{a.r / s, a.g / s, a.b / s}; }
__host__ __device__ __forceinline__ float maxValue(Spec a) { return smax(smax(a.r, a.g), a.b); }
__host__ __device__ __forceinline__ float averageValue(Spec a) {
    float v = 0.0f;
    v += a.r;
    v += a.g;
    v += a.b;
    return v / 3.0f;
}

// PhongBRDF::PhongBRDF lobe-selection probabilities (Material/PhongBRDF.cu:10-19)
__host__ __device__ __forceinline__ void phongLobeProbs(Spec kd, Spec ks, float eps, float& dProb, float& sProb) {
    const float d = smax(averageValue(kd), 0.0f);
    const float s = smax(averageValue(ks), 0.0f);
    const float sum = gmax(d + s, eps);
    dProb = d / sum;
    sProb = s / sum;
}

}  // namespace cr
