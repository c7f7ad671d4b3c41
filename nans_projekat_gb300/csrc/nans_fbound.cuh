// The friction bound of the sequential-impulse loop without the FP64 pipe.
//
// Constraint (code/nans.cpp:1199, 1214) clamps each tangent impulse to sqrt(2) * Cf * Sum, the
// product taken in double (sqrt(2) is a double literal) and the result stored to float: with
// c2 = sqrt(2) * Cf (a double, fixed per scene) the bound is (float)(c2 * (double)Sum), two
// roundings: to 53 bits, then to 24. On a GB300 a warp's double-precision instruction holds the
// FP64 pipe for tens of cycles and the multiply and its two conversions sit on the loop's
// critical path. fbound_mul computes the same float in single precision and certifies it:
//
//   c2 = ch + cm + cl exactly (ch = (float)c2, cm = (float)(c2 - ch), |cl| <= 2^-48 |ch|)
//   p1 = fl(s ch), e1 = fma(s, ch, -p1)           s ch = p1 + e1 exactly (TwoProd)
//   t  = fma(s, cm, e1)                            s c = p1 + t + d, |d| < 2^-46 |p1|
//   r  = fl(p1 + t), err = t - fl(r - p1)          p1 + t = r + err exactly (FastTwoSum)
//
// so x = s c = r + err + d. If |err| < ulp(r) (1/2 - 2^-20), then x and its double rounding
// (within 2^-53 |x| of x) lie strictly between the midpoints around r, |err| + |d| + 2^-53 |r|
// being below ulp(r) / 2 since ulp(r) 2^-20 >= 2^-44 |r|; both roundings then give r. The
// certificate is refused (and the caller computes the product in double) for s subnormal,
// infinite, NaN or -0, r outside [2^-99, 2^124) in magnitude, r a power of two (the spacing
// below it is half), or err too close to the half ulp: about two products in a million of those
// in range. Sum = +0 is certified with bound +0. The code is plain IEEE single arithmetic with explicit
// fused multiply-adds, compiled for the device (the solver) and for the host (the CPU check
// against the double computation, tests/fbound_check.cpp).
#pragma once
#include <cmath>
#include <cstring>
#ifdef __CUDACC__
#define NANS_FB_FN __host__ __device__ __forceinline__
#else
#define NANS_FB_FN inline
#endif

namespace nans
{

struct FBound
{
    float ch, cm; // c2 = ch + cm + (|cl| <= 2^-48 |ch|)
    bool ok;      // c2 is a positive normal double of a range where the split is exact
};

NANS_FB_FN unsigned fb_bits(float x)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    unsigned u;
    std::memcpy(&u, &x, 4);
    return u;
#endif
}

NANS_FB_FN float fb_float(unsigned u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, 4);
    return x;
#endif
}

NANS_FB_FN float fb_fma(float a, float b, float c)
{
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}

NANS_FB_FN FBound fbound_split(double c2)
{
    FBound f;
    // 2^-60 <= c2 < 2^60: ch, cm and cl are normal floats (or cm = cl = 0)
    f.ok = c2 >= 0x1p-60 && c2 < 0x1p60;
    f.ch = (float)c2;
    f.cm = (float)(c2 - (double)f.ch);
    if (!f.ok)
        f.ch = f.cm = 0.0f;
    return f;
}

// (float)(c2 * (double)s) where *certified comes back true.
NANS_FB_FN float fbound_mul(const FBound &f, float s, bool *certified)
{
    const float p1 = s * f.ch;
    const float e1 = fb_fma(s, f.ch, -p1);
    const float t = fb_fma(s, f.cm, e1);
    const float r = p1 + t;
    const float err = t - (r - p1);
    const unsigned rb = fb_bits(r), ex = rb & 0x7f800000u;
    const float lim = fb_float(ex - (23u << 23)) * 0x1.ffffcp-2f; // ulp(r) (1/2 - 2^-20)
    const bool zero = fb_bits(s) == 0u;
    const bool in_range = ex >= (28u << 23) && ex < (251u << 23) && (rb & 0x7fffffu) != 0u;
    *certified = f.ok && (zero || (in_range && (err < lim && -err < lim)));
    return zero ? 0.0f : r;
}

} // namespace nans
