// Test infrastructure (oracle side): the project's own single-precision sine/cosine,
// used by the glm shim's rotate() so that the model-matrix rebuild of the reference's
// render code (code/nans.cpp:1870-1881, 1913-1942) is reproducible bit for bit on any
// IEEE-754 machine. The device kernels carry an independent copy of the same method;
// a GPU test compares the two over a sweep of arguments.
//
// Method: Cody-Waite argument reduction by pi/2 with a three-part split of pi/2
// (8 + 12 significant bits + a float remainder, derived from pi in extended precision),
// then the Taylor series of sin (to r^9) and cos (to r^10) on |r| <= pi/4, evaluated by
// Horner's rule. Truncation error is below 3e-9, well under half a float ulp.
// Every operation is a single IEEE float operation; compile without FP contraction.
#ifndef NANS_TRIG_H
#define NANS_TRIG_H

#include <math.h>

static inline void nans_trig_sincosf(float x, float *s_out, float *c_out)
{
    const float two_over_pi = 0.636619746685028076171875f;
    const float pio2_hi = 1.5703125f;                  // 8 significant bits
    const float pio2_mid = 4.838705062866210938e-04f;  // next 12 bits
    const float pio2_lo = -4.371138828673792886e-08f;  // float remainder
    float q = floorf(x * two_over_pi + 0.5f);
    float r = x - q * pio2_hi;
    r = r - q * pio2_mid;
    r = r - q * pio2_lo;
    float r2 = r * r;
    // sin(r) = r + r^3 * (-1/3! + r^2 * (1/5! + r^2 * (-1/7! + r^2 * (1/9!))))
    float ps = 2.7557319223985891e-06f;
    ps = ps * r2 + -1.9841269841269841e-04f;
    ps = ps * r2 + 8.3333333333333332e-03f;
    ps = ps * r2 + -1.6666666666666666e-01f;
    float sr = r + (r * r2) * ps;
    // cos(r) = 1 + r^2 * (-1/2! + r^2 * (1/4! + r^2 * (-1/6! + r^2 * (1/8! + r^2 * (-1/10!)))))
    float pc = -2.7557319223985888e-07f;
    pc = pc * r2 + 2.4801587301587302e-05f;
    pc = pc * r2 + -1.3888888888888889e-03f;
    pc = pc * r2 + 4.1666666666666664e-02f;
    pc = pc * r2 + -0.5f;
    float cr = 1.0f + r2 * pc;
    int quadrant = 0;
    if (fabsf(q) < 16777216.0f)
        quadrant = ((int)q) & 3;
    float s, c;
    switch (quadrant)
    {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = -sr; break;
    case 2: s = -sr; c = -cr; break;
    default: s = -cr; c = sr; break;
    }
    *s_out = s;
    *c_out = c;
}

static inline float nans_trig_sinf(float x)
{
    float s, c;
    nans_trig_sincosf(x, &s, &c);
    return s;
}

static inline float nans_trig_cosf(float x)
{
    float s, c;
    nans_trig_sincosf(x, &s, &c);
    return c;
}

#endif
