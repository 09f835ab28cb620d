// ntp_device.cuh -- device-side building blocks of the photon step law.
//
// Each function restates one piece of the reference (chrhck/NeutrinoTelescopes,
// file:line given) for sm_103a in single precision.  Where the reference's
// float arithmetic is ill-conditioned (sin of a scattering angle near the
// forward pole computed as sqrt(1 - cos^2)), the same quantity is evaluated
// in an algebraically identical, well-conditioned form; results agree with
// the double-precision oracle instead of inheriting float cancellation.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/ntp.h"

namespace ntp {

constexpr float kCVac = 0.299792458f;        // m/ns
constexpr float kInvCVac = 3.3356409519815204f;  // ns/m
constexpr unsigned kFull = 0xffffffffu;

// Philox block indices (the "draw" word of the counter).  Photon k of source
// s uses counter (draw, k_lo, k_hi, s) under key = seed.
constexpr uint32_t kDrawInitA = 0;   // x: wavelength, y: azimuth, z: polar (isotropic), w: time / track position
constexpr uint32_t kDrawInitB = 1;   // x: track-direction cos, y: track-direction azimuth
constexpr uint32_t kDrawGamma0 = 2;  // attempt k of the gamma sampler: x, y -> normal, z -> accept
constexpr int kGammaAttempts = 32;
constexpr uint32_t kDrawStep0 = 64;  // step j: x: length, y: scatter cos, z: scatter azimuth, w: Rayleigh select

// Philox4x32-10 (Salmon et al., SC'11).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k.x += 0x9E3779B9u;
            k.y += 0xBB67AE85u;
        }
        // one 32x32->64 wide multiply each
        const unsigned long long p0 = static_cast<unsigned long long>(0xD2511F53u) * c.x;
        const unsigned long long p1 = static_cast<unsigned long long>(0xCD9E8D57u) * c.z;
        c = make_uint4(static_cast<uint32_t>(p1 >> 32) ^ c.y ^ k.x, static_cast<uint32_t>(p1),
                       static_cast<uint32_t>(p0 >> 32) ^ c.w ^ k.y, static_cast<uint32_t>(p0));
    }
    return c;
}

// The same generator with the round keys precomputed: rk[2r], rk[2r + 1] =
// key + r (0x9E3779B9, 0xBB67AE85).  With rk in a kernel's parameters each
// round's key is an operand of the XOR rather than two additions.
__device__ __forceinline__ uint4 philox4x32_10_rk(uint4 c, const uint32_t (&rk)[20]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const unsigned long long p0 = static_cast<unsigned long long>(0xD2511F53u) * c.x;
        const unsigned long long p1 = static_cast<unsigned long long>(0xCD9E8D57u) * c.z;
        c = make_uint4(static_cast<uint32_t>(p1 >> 32) ^ c.y ^ rk[2 * r], static_cast<uint32_t>(p1),
                       static_cast<uint32_t>(p0 >> 32) ^ c.w ^ rk[2 * r + 1], static_cast<uint32_t>(p0));
    }
    return c;
}

// Top 23 bits plus one half, times 2^-23: uniform on the open interval (0, 1),
// exact in float; 1 - u01(w) is exact too.  Formed from the bit pattern: the
// float 1.m (m the top 23 bits) minus 1 - 2^-24 is exact (both lie within a
// factor 2 of each other) and equals (m + 1/2) 2^-23, with no
// integer-to-float conversion.
__device__ __forceinline__ float u01(uint32_t w) {
    return __uint_as_float((w >> 9) | 0x3F800000u) - 0.999999940395355224609375f;
}

// 53 random bits from two Philox words: a double on the open interval (0, 1).
__device__ __forceinline__ double u01_53(uint32_t a, uint32_t b) {
    const unsigned long long m = (static_cast<unsigned long long>(a) << 21) ^ (b >> 11);
    return (static_cast<double>(m & ((1ull << 53) - 1)) + 0.5) * (1.0 / 9007199254740992.0);
}

constexpr uint32_t kDrawPoisson = 0x504F4953u;  // "POIS": Poisson counts
constexpr int kPoissonAttempts = 64;

// Poisson(lam) from the Philox stream (kDrawPoisson, lo, attempt, hi) under
// key: inversion below a mean of 30, above the transformed rejection of
// Hormann (1993, "PTRS") with at most kPoissonAttempts tries (then the
// rounded mean).
__device__ __forceinline__ double poisson_draw(double lam, uint2 key, uint32_t lo, uint32_t hi) {
    if (!(lam > 0.0)) return 0.0;
    if (lam < 30.0) {
        const uint4 r = philox4x32_10(make_uint4(kDrawPoisson, lo, 0u, hi), key);
        const double u = u01_53(r.x, r.y);
        double p = exp(-lam), F = p, k = 0.0;
        while (u > F && k < 1000.0) {
            k += 1.0;
            p *= lam / k;
            F += p;
        }
        return k;
    }
    const double slam = sqrt(lam), loglam = log(lam);
    const double b = 0.931 + 2.53 * slam, a = -0.059 + 0.02483 * b;
    const double invalpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2.0);
    for (int t = 0; t < kPoissonAttempts; ++t) {
        const uint4 r = philox4x32_10(make_uint4(kDrawPoisson, lo, static_cast<uint32_t>(t) + 1u, hi), key);
        const double U = u01_53(r.x, r.y) - 0.5, V = u01_53(r.z, r.w);
        const double us = 0.5 - fabs(U);
        const double k = floor((2.0 * a / us + b) * U + lam + 0.43);
        if (us >= 0.07 && V <= vr) return k;
        if (k < 0.0 || (us < 0.013 && V > us)) continue;
        if (log(V) + log(invalpha) - log(a / (us * us) + b) <= -lam + k * loglam - lgamma(k + 1.0)) return k;
    }
    return floor(lam + 0.5);
}

// Approximate instructions with subnormal results and inputs flushed to 0,
// for arguments known to be normal
__device__ __forceinline__ float log2_ftz(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rcp_ftz(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sin_ftz(float x) {
    float r;
    asm("sin.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float cos_ftz(float x) {
    float r;
    asm("cos.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

struct V3 {
    float x, y, z;
};

// rot_from_ez_fast, utils.jl:228-243: the rotation taking e_z to a, applied
// to o.  At a = +-e_z the reference returns (o1, copysign(o2,a3),
// copysign(o3,a3)); exact_pole switches to the true rotation there.
// The reference tests |a3| == 1; here the pole is a1^2 + a2^2 below the
// smallest normal float (a direction within 1e-19 of the axis, where the
// two forms agree to that order).  The two agree for every exact +-e_z, but
// a scattered direction whose z component rounds to 1.0f in single
// precision while x, y are not tiny keeps its transverse part here (the
// general formula stays bounded: a_i^2 fact <= 1 - a3), as the same step in
// double precision does.
__device__ __forceinline__ V3 rot_from_ez(V3 a, V3 o, bool exact_pole) {
    const float a1sq = a.x * a.x, a2sq = a.y * a.y;
    const float t = a1sq + a2sq;
    if (t < 1.17549435e-38f) {
        if (exact_pole) return V3{o.x, copysignf(1.0f, a.z) * o.y, copysignf(1.0f, a.z) * o.z};
        return V3{o.x, copysignf(o.y, a.z), copysignf(o.z, a.z)};
    }
    const float fact = (1.0f - a.z) * rcp_ftz(t);
    const float a1a2 = a.x * a.y;
    V3 r;
    r.x = fmaf(-a1sq, fact, 1.0f) * o.x - a1a2 * fact * o.y + a.x * o.z;
    r.y = -a1a2 * fact * o.x + fmaf(-a2sq, fact, 1.0f) * o.y + a.y * o.z;
    r.z = -a.x * o.x - a.y * o.y + a.z * o.z;
    return r;
}

// Linear interpolation in a uniform table of float4 knots.
__device__ __forceinline__ float4 interp_table(const float4* t, int n, float x0, float scale, float x) {
    float pos = fminf(fmaxf((x - x0) * scale, 0.0f), static_cast<float>(n - 1));
    int i = min(static_cast<int>(pos), n - 2);
    const float f = pos - static_cast<float>(i);
    const float4 a = t[i], b = t[i + 1];
    return make_float4(fmaf(f, b.x - a.x, a.x), fmaf(f, b.y - a.y, a.y), fmaf(f, b.z - a.z, a.z),
                       fmaf(f, b.w - a.w, a.w));
}

struct SpectrumView {
    int kind;
    int n;
    const float* knots;  // shared memory
    float p0, p1;        // INV_SQUARE: 1/wl_min, 1/wl_min - 1/wl_max ; MONOCHROMATIC: p0 = wavelength
};

// initialize_wavelength, photon_prop_cuda.jl:128-130 (the texture fetch of
// spectrum.jl:102-103 is emulated in NTP_SPEC_TABLE_TEXTURE).
__device__ __forceinline__ float sample_wavelength(const SpectrumView& s, float u) {
    switch (s.kind) {
    case NTP_SPEC_MONOCHROMATIC:
        return s.p0;
    case NTP_SPEC_TABLE_LINEAR: {
        const float x = u * static_cast<float>(s.n - 1);
        const int i = min(static_cast<int>(x), s.n - 2);
        const float f = x - static_cast<float>(i);
        const float k0 = s.knots[i], k1 = s.knots[i + 1];
        return fmaf(f, k1 - k0, k0);
    }
    case NTP_SPEC_TABLE_TEXTURE: {
        const float xb = fmaf(u, static_cast<float>(s.n), -0.5f);
        const float fl = floorf(xb);
        const int i = static_cast<int>(fl);
        const float a = rintf((xb - fl) * 256.0f) * (1.0f / 256.0f);
        const int i0 = min(max(i, 0), s.n - 1), i1 = min(max(i + 1, 0), s.n - 1);
        return (1.0f - a) * s.knots[i0] + a * s.knots[i1];
    }
    default:  // NTP_SPEC_INV_SQUARE
        return 1.0f / fmaf(-u, s.p1, s.p0);
}
}

// Fast single-precision helpers for the per-step arithmetic.  Their errors
// (a few ulp relative, or ~4e-7 absolute for the sine and cosine) are far
// below the 1e-4 per-photon agreement the propagation is held to.
__device__ __forceinline__ float fast_rcp(float x) { return __fdividef(1.0f, x); }

// sqrt(max(x, 0)) by the approximate square-root instruction (relative error
// within 2^-23 over the normal range; exact 0 at 0)
__device__ __forceinline__ float fast_sqrt(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(fmaxf(x, 0.0f)));
    return r;
}

// 2^x by the approximate base-2 exponential instruction (relative error
// about 2^-22; results below the normal range flush to 0)
__device__ __forceinline__ float fast_exp2(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// (sin, cos)(2 pi u) for u in (0, 1): the hardware sine / cosine on the
// argument moved to [-pi, pi), where their absolute error is below 2^-21.
__device__ __forceinline__ void sincos_2pi(float u, float* s, float* c) {
    const float x = fmaf(u, 6.283185307179586f, -3.141592653589793f);
    *s = -sin_ftz(x);
    *c = -cos_ftz(x);
}

// One minus the Henyey-Greenstein cosine (cuda_hg_scattering_func,
// photon_prop_cuda.jl:70-77).  With D = 1 + g(2 eta - 1), t = (1 - g^2)/D:
//   cos = (1 + g^2 - t^2) / 2g    and    1 - cos = (1-g)(1-eta)(t + 1 - g) / D,
// the second form keeps full relative precision for forward scatters.
__device__ __forceinline__ float hg_one_minus_cos(float g, float one_m_g, float one_m_g2, float eta) {
    const float D = fmaf(g, fmaf(2.0f, eta, -1.0f), 1.0f);
    const float invD = rcp_ftz(D);
    const float t = one_m_g2 * invD;
    const float omc = one_m_g * (1.0f - eta) * (t + one_m_g) * invD;
    return fminf(fmaxf(omc, 0.0f), 2.0f);
}

// Rayleigh (3/8)(1 + mu^2): exact CDF inverse, mu^3 + 3 mu = 8u - 4, by
// Cardano in the form mu = sign(q)(A - 1/A), A = cbrt(|q| + sqrt(q^2 + 1)),
// the cube root as 2^(log2(x)/3) on x in [1, 2 + sqrt 5].
__device__ __forceinline__ float rayleigh_cos(float u) {
    const float q = fmaf(4.0f, u, -2.0f);
    const float x = fabsf(q) + fast_sqrt(fmaf(q, q, 1.0f));
    const float A = fast_exp2(log2_ftz(x) * (1.0f / 3.0f));
    const float mu = A - rcp_ftz(A);
    return copysignf(mu, q);
}

// Direction from (1 - cos theta) and an azimuth uniform, as
// sph_to_cart (utils.jl:105-115) with sin theta = sqrt(omc (2 - omc)).
__device__ __forceinline__ V3 dir_from_omc(float omc, float u_phi) {
    float sp, cp;
    sincos_2pi(u_phi, &sp, &cp);
    const float st = fast_sqrt(omc * (2.0f - omc));
    return V3{cp * st, sp * st, 1.0f - omc};
}

}  // namespace ntp
