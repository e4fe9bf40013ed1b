// cr_spectral.cuh -- hero-wavelength spectral rendering (an extension: the
// reference's Spectrum is RGB, Core/Spectrum.h:326, and its 95-bin
// BroadSpectrum is never used).
//
// A path carries three wavelengths in the three channels of Spec: a hero
// wavelength lambda_0 ~ U[360, 830) nm and its two rotations by 470/3 nm
// (hero-wavelength sampling, Wilkie et al. 2014, with three wavelengths).
// The hero wavelength comes from a hash of (pixel, sample index), so the
// path's own random sequence is the RGB integrator's.
//
// Reflectance and emission spectra are upsampled from RGB with a smooth
// partition of unity: s(lambda) = r B_r + g B_g + b B_b with
//   B_b = 1 - S((lambda - 490) / 15), B_r = S((lambda - 590) / 15),
//   B_g = 1 - B_b - B_r  (S = logistic sigmoid),
// so a grey (a, a, a) is the flat spectrum a.  Radiance reaching the film is
// turned into XYZ with the analytic multi-lobe fit of the CIE 1931 colour
// matching functions of Wyman, Sloan and Shirley (JCGT 2(2), 2013) and into
// linear sRGB with the IEC 61966-2-1 matrix, white-balanced to equal energy
// (divided by the RGB of the flat unit spectrum), so a flat spectrum renders
// as the RGB integrator does, in expectation.
#pragma once

#include "cr_math.cuh"

namespace cr {

constexpr float kLambdaMin = 360.0f;
constexpr float kLambdaRange = 470.0f;

__host__ __device__ __forceinline__ float sigmoid(float x) { return 1.0f / (1.0f + expf(-x)); }

__host__ __device__ __forceinline__ void upsampleBasis(float lambda, float& br, float& bg, float& bb) {
    bb = 1.0f - sigmoid((lambda - 490.0f) / 15.0f);
    br = sigmoid((lambda - 590.0f) / 15.0f);
    bg = 1.0f - bb - br;
}

// piecewise Gaussian of the multi-lobe CMF fit
__host__ __device__ __forceinline__ float lobe(float l, float mu, float s1, float s2) {
    const float t = (l - mu) / (l < mu ? s1 : s2);
    return expf(-0.5f * t * t);
}

__host__ __device__ __forceinline__ float3 cieXYZ(float l) {
    const float x = 1.056f * lobe(l, 599.8f, 37.9f, 31.0f) + 0.362f * lobe(l, 442.0f, 16.0f, 26.7f) -
                    0.065f * lobe(l, 501.1f, 20.4f, 26.2f);
    const float y = 0.821f * lobe(l, 568.8f, 46.9f, 40.5f) + 0.286f * lobe(l, 530.9f, 16.3f, 31.1f);
    const float z = 1.217f * lobe(l, 437.0f, 11.8f, 36.0f) + 0.681f * lobe(l, 459.0f, 26.0f, 13.8f);
    return mk3(x, y, z);
}

__host__ __device__ __forceinline__ float3 xyzToLinearSrgb(float3 c) {
    return mk3(3.2404542f * c.x - 1.5371385f * c.y - 0.4985314f * c.z,
               -0.9692660f * c.x + 1.8760108f * c.y + 0.0415560f * c.z,
               0.0556434f * c.x - 0.2040259f * c.y + 1.0572252f * c.z);
}

// Per-path spectral state: the three wavelengths and the upsampling basis at
// each of them.
struct SpectralPath {
    bool on;
    float lambda[3];
    float br[3], bg[3], bb[3];
};

__host__ __device__ __forceinline__ uint32_t spectralHash(uint32_t x, uint32_t y, uint32_t s) {
    uint32_t h = x * 0x9E3779B1u ^ (y + 0x7F4A7C15u) * 0x85EBCA77u ^ (s + 0x165667B1u) * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h;
}

__host__ __device__ __forceinline__ SpectralPath makeSpectralPath(bool on, uint32_t x, uint32_t y, uint32_t s) {
    SpectralPath p;
    p.on = on;
    if (!on) return p;
    const float u = (float)(spectralHash(x, y, s) >> 8) * (1.0f / 16777216.0f);
    for (int i = 0; i < 3; i++) {
        float t = u + (float)i / 3.0f;
        t = t >= 1.0f ? t - 1.0f : t;
        p.lambda[i] = kLambdaMin + kLambdaRange * t;
        upsampleBasis(p.lambda[i], p.br[i], p.bg[i], p.bb[i]);
    }
    return p;
}

// RGB material colour -> the path's spectral triple (or the RGB itself).
__host__ __device__ __forceinline__ Spec toPathSpec(const SpectralPath& p, float r, float g, float b) {
    if (!p.on) return sp(r, g, b);
    return Spec{(r * p.br[0] + g * p.bg[0]) + b * p.bb[0], (r * p.br[1] + g * p.bg[1]) + b * p.bb[1],
                (r * p.br[2] + g * p.bg[2]) + b * p.bb[2]};
}

// Radiance at the path's wavelengths -> linear sRGB (white-balanced with the
// per-channel scale `wb` = 1 / RGB of the flat unit spectrum).
__host__ __device__ __forceinline__ Spec pathSpecToRgb(const SpectralPath& p, Spec L, float3 wb) {
    if (!p.on) return L;
    const float v[3] = {L.r, L.g, L.b};
    float3 xyz = mk3(0.0f, 0.0f, 0.0f);
    for (int i = 0; i < 3; i++) xyz = add(xyz, mul(cieXYZ(p.lambda[i]), v[i]));
    xyz = mul(xyz, kLambdaRange / 3.0f);  // Monte Carlo weight of 3 uniform wavelengths
    const float3 rgb = xyzToLinearSrgb(xyz);
    return sp(rgb.x * wb.x, rgb.y * wb.y, rgb.z * wb.z);
}

// 1 / (linear sRGB of the flat unit spectrum), by midpoint integration.
inline float3 whiteBalance() {
    float3 xyz = mk3(0.0f, 0.0f, 0.0f);
    const int n = 4700;
    const double dl = kLambdaRange / n;
    double acc[3] = {0, 0, 0};
    for (int i = 0; i < n; i++) {
        const float3 c = cieXYZ((float)(kLambdaMin + (i + 0.5) * dl));
        acc[0] += c.x * dl;
        acc[1] += c.y * dl;
        acc[2] += c.z * dl;
    }
    xyz = mk3((float)acc[0], (float)acc[1], (float)acc[2]);
    const float3 rgb = xyzToLinearSrgb(xyz);
    return mk3(1.0f / rgb.x, 1.0f / rgb.y, 1.0f / rgb.z);
}

}  // namespace cr
