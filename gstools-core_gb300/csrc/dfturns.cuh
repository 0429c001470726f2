// dfturns.cuh -- sine and cosine of phases held in turns as FP32 pairs.
//
// A phase k.x is carried as theta = kappa.x turns, kappa = k / 2 pi, with
// kappa and x each split into FP32 hi + lo parts (48 significant bits).
// Whole turns drop out exactly, so the reduced phase of one product keeps
// about |theta| * 2^-46 turns of absolute accuracy (2^-29 turns at |k.x| =
// 1e6) with FP32 instructions only (GB300 runs FP64 at 1/64 of the FP32
// rate); summing the fractions of several products in FP32 adds up to 2^-24
// turns where one product is under a turn (mixed.cu).  sin(2 pi f), cos(2 pi f) on
// |f| <= 1/8 come from polynomials fitted for this project (FP32
// coefficients, max error 8.6e-8 / 5.8e-8 over the interval), corrected to
// first order for the low part of the phase (the mixed summators,
// mixed.cu).  The factor tables of the separable tensor-core form
// (separable_tc.cu) take the same phase reduction and sincosf for the last
// step (cis_turns_acc).
#pragma once

#include <cuda_runtime.h>

namespace gsc {

constexpr double kInv2Pi = 0.15915494309189535;   // fl(1 / (2 pi))
constexpr float kTwoPiF = 6.2831854820251465f;     // fl32(2 pi)
constexpr float kRoundF = 12582912.0f;             // 1.5 * 2^23: x + kRoundF rounds x

// sin(2 pi f) = f * S(f^2), cos(2 pi f) = C(f^2) on |f| <= 1/8 (fitted here)
constexpr float kS0 = 6.2831854820251465f, kS1 = -41.34170150756836f, kS2 = 81.60517883300781f,
                kS3 = -76.6958236694336f, kS4 = 41.41468811035156f;
constexpr float kC0 = 1.0f, kC1 = -19.739208221435547f, kC2 = 64.93931579589844f,
                kC3 = -85.44285583496094f, kC4 = 59.220428466796875f;

// sin and cos of 2 pi (th - q/4 + tl) for the quarter-turn count q nearest
// 4 th (returned, as an integer whose low two bits are q mod 4): the caller
// rotates by q quarter turns.  th within a few turns of zero, tl tiny.
__device__ __forceinline__ int sincos_turns_reduced(float th, float tl, float &s1, float &c1) {
    const float qf = fmaf(th, 4.0f, kRoundF);
    const float q = qf - kRoundF;
    const float f = fmaf(q, -0.25f, th);                     // exact, |f| <= 1/8
    const float f2 = f * f;
    const float s = fmaf(fmaf(fmaf(fmaf(kS4, f2, kS3), f2, kS2), f2, kS1), f2, kS0) * f;
    const float c = fmaf(fmaf(fmaf(fmaf(kC4, f2, kC3), f2, kC2), f2, kC1), f2, kC0);
    const float tw = tl * kTwoPiF;                           // first-order low-part correction
    s1 = fmaf(tw, c, s);
    c1 = fmaf(-tw, s, c);
    return __float_as_int(qf);
}

// (cos, sin) of 2 pi (kh + kl)(xh + xl) to about the accuracy of CUDA's
// sincosf: the product split exactly into its rounded value and error,
// whole turns dropped, small terms added in FP32; the reduced phase less
// its quarter turns turned into radians as an FP32 pair, sincosf of the
// high part, first-order correction for the low part, rotation by the
// quarter turns.  Valid while |kh * xh| stays below 2^22 turns (the caller
// checks).  For factor tables, where accuracy counts more than speed.
__device__ __forceinline__ float2 cis_turns_acc(float kh, float kl, float xh, float xl) {
    const float pr = kh * xh;
    const float e = fmaf(kh, xh, -pr);                       // exact
    const float a = pr - rintf(pr);                          // exact
    const float b = fmaf(kh, xl, fmaf(kl, xh, e));
    const float th = a + b;
    const float tl = b - (th - a);
    // quarter turns taken out exactly, so sincosf sees |rh| <= pi / 4
    const float qf = fmaf(th, 4.0f, kRoundF);
    const float f = fmaf(qf - kRoundF, -0.25f, th);          // exact, |f| <= 1/8
    constexpr float kTwoPiLo = -1.7484555e-07f;              // 2 pi - fl32(2 pi)
    const float rh = f * kTwoPiF;
    const float rl = fmaf(f, kTwoPiF, -rh) + fmaf(f, kTwoPiLo, tl * kTwoPiF);
    float sn, cs;
    sincosf(rh, &sn, &cs);
    const float s = fmaf(rl, cs, sn), c = fmaf(-rl, sn, cs);
    switch (__float_as_int(qf) & 3) {
        case 0: return make_float2(c, s);
        case 1: return make_float2(-s, c);
        case 2: return make_float2(-c, -s);
        default: return make_float2(s, -c);
    }
}

}  // namespace gsc
