// Device vector arithmetic for the physics step.
//
// Every operation is one IEEE-754 single-precision operation in a fixed order, so that
// the kernels reproduce the reference step (code/nans.cpp) bit for bit when compiled with
// -fmad=false and IEEE division / square root (no --use_fast_math):
//   dot(a,b)     = (a.x*b.x + a.y*b.y) + a.z*b.z
//   cross(a,b)   = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x)
//   normalize(v) = v * (1/sqrt(dot(v,v)))
//   length(v)    = sqrt(dot(v,v))
// These are the formulations of the glm functions the reference calls (glm is header-only,
// unvendored and unpinned in the reference; this order is the project's definition).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define NANS_HD __host__ __device__ __forceinline__

struct v3
{
    float x, y, z;
};

NANS_HD v3 mk3(float x, float y, float z)
{
    v3 r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
NANS_HD v3 operator+(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
NANS_HD v3 operator-(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
NANS_HD v3 operator-(v3 a) { return mk3(-a.x, -a.y, -a.z); }
NANS_HD v3 operator*(float s, v3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
NANS_HD v3 div3(v3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
NANS_HD float dot3(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
NANS_HD v3 cross3(v3 a, v3 b)
{
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
NANS_HD float len3(v3 a) { return sqrtf(dot3(a, a)); }
NANS_HD v3 normalize3(v3 a)
{
    float inv = 1.0f / sqrtf(dot3(a, a));
    return mk3(a.x * inv, a.y * inv, a.z * inv);
}
NANS_HD bool eq3(v3 a, v3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
NANS_HD v3 xyz(float4 f) { return mk3(f.x, f.y, f.z); }
NANS_HD float4 f4(v3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

// ------------------------------------------------------------------------------------
// Sine and cosine for the model-matrix rebuild (angles are degrees in the reference,
// converted by glm::radians, code/nans.cpp:1915-1920).
//
// The project's own method, identical in every operation to the host copy used by the
// oracle: Cody-Waite reduction by pi/2 with a three-part split of pi/2 (8 + 12 significant
// bits + a float remainder), then the Taylor series of sin (to r^9) and cos (to r^10) on
// |r| <= pi/4 in Horner form. Truncation error < 3e-9 (below half a float ulp).
// ------------------------------------------------------------------------------------
NANS_HD void nans_sincos(float x, float *s_out, float *c_out)
{
    const float two_over_pi = 0.636619746685028076171875f;
    const float pio2_hi = 1.5703125f;
    const float pio2_mid = 4.838705062866210938e-04f;
    const float pio2_lo = -4.371138828673792886e-08f;
    float q = floorf(x * two_over_pi + 0.5f);
    float r = x - q * pio2_hi;
    r = r - q * pio2_mid;
    r = r - q * pio2_lo;
    float r2 = r * r;
    float ps = 2.7557319223985891e-06f;
    ps = ps * r2 + -1.9841269841269841e-04f;
    ps = ps * r2 + 8.3333333333333332e-03f;
    ps = ps * r2 + -1.6666666666666666e-01f;
    float sr = r + (r * r2) * ps;
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
    if (quadrant == 0)
    {
        s = sr;
        c = cr;
    }
    else if (quadrant == 1)
    {
        s = cr;
        c = -sr;
    }
    else if (quadrant == 2)
    {
        s = -sr;
        c = -cr;
    }
    else
    {
        s = -cr;
        c = sr;
    }
    *s_out = s;
    *c_out = c;
}

// ------------------------------------------------------------------------------------
// 3x4 affine part of the model matrix Model = T(P) * Rx * Ry * Rz * S, built with the same
// sequence of glm calls as the reference's render code (code/nans.cpp:1913-1923): each
// call right-multiplies, with columns combined as ((m0*a + m1*b) + m2*c) [+ m3].
// The fourth row of every intermediate matrix is kept too, because translate() mixes it
// into column 3 (with the identity start it stays (0,0,0,1) up to signed zeros, which the
// arithmetic reproduces exactly).
// ------------------------------------------------------------------------------------
struct m4
{
    float c[4][4]; // column-major: c[col][row]
};

NANS_HD void col_lin3(const m4 &m, float a, float b, float cc, float out[4])
{
#pragma unroll
    for (int r = 0; r < 4; ++r)
        out[r] = (m.c[0][r] * a + m.c[1][r] * b) + m.c[2][r] * cc;
}

NANS_HD void m4_rotate(m4 &m, float angle, float ax, float ay, float az)
{
    float s, c;
    nans_sincos(angle, &s, &c);
    v3 a = normalize3(mk3(ax, ay, az));
    v3 t = (1.0f - c) * a;
    v3 r0 = mk3(c + t.x * a.x, t.x * a.y + s * a.z, t.x * a.z - s * a.y);
    v3 r1 = mk3(t.y * a.x - s * a.z, c + t.y * a.y, t.y * a.z + s * a.x);
    v3 r2 = mk3(t.z * a.x + s * a.y, t.z * a.y - s * a.x, c + t.z * a.z);
    m4 r;
    col_lin3(m, r0.x, r0.y, r0.z, r.c[0]);
    col_lin3(m, r1.x, r1.y, r1.z, r.c[1]);
    col_lin3(m, r2.x, r2.y, r2.z, r.c[2]);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        r.c[3][k] = m.c[3][k];
    m = r;
}

NANS_HD float nans_radians(float deg) { return deg * 0.0174532925199432957692f; }

NANS_HD m4 model_of(v3 P, v3 A, v3 S)
{
    m4 m;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int r = 0; r < 4; ++r)
            m.c[j][r] = (j == r) ? 1.0f : 0.0f;
    // translate
    float t[4];
    col_lin3(m, P.x, P.y, P.z, t);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        m.c[3][k] = t[k] + m.c[3][k];
    m4_rotate(m, nans_radians(A.x), 1.0f, 0.0f, 0.0f);
    m4_rotate(m, nans_radians(A.y), 0.0f, 1.0f, 0.0f);
    m4_rotate(m, nans_radians(A.z), 0.0f, 0.0f, 1.0f);
    // scale
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        m.c[0][k] = m.c[0][k] * S.x;
        m.c[1][k] = m.c[1][k] * S.y;
        m.c[2][k] = m.c[2][k] * S.z;
    }
    return m;
}

// Model * (p, 1), xyz: ((m0*x + m1*y) + m2*z) + m3*1
NANS_HD v3 xform(const m4 &m, v3 p)
{
    float o[4];
    col_lin3(m, p.x, p.y, p.z, o);
    return mk3(o[0] + m.c[3][0] * 1.0f, o[1] + m.c[3][1] * 1.0f, o[2] + m.c[3][2] * 1.0f);
}
