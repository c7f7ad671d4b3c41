// Test infrastructure: a minimal glm API subset used only to compile the reference
// physics step (code/nans.cpp, code/utilities.cpp) headless for the oracle. It is not
// part of the product and is never linked into the CUDA library.
//
// glm itself is a header-only third-party dependency that the reference does not vendor
// and does not pin (code/nans.h:6-10 only #include it). This file is written from the
// mathematics; its operation order IS the pinned definition of every vector operation the
// oracle and the device kernels reproduce:
//   dot(a,b)        = (a.x*b.x + a.y*b.y) + a.z*b.z
//   cross(a,b)      = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x)
//   length(v)       = sqrt(dot(v,v))
//   normalize(v)    = v * (1/sqrt(dot(v,v)))
//   M*v (mat4,vec4) = ((M[0]*v.x + M[1]*v.y) + M[2]*v.z) + M[3]*v.w   (column major)
//   translate/rotate/scale: right-multiplication, rotate via the Rodrigues matrix with
//   cos/sin from nans_trig.h (a project-written Cody-Waite + Taylor sincos), so that the
//   model-matrix rebuild is bit-identical on x86, aarch64 and the GPU.
#ifndef NANS_SHIM_GLM_HPP
#define NANS_SHIM_GLM_HPP

#include <cmath>
#include <cfloat>
#include "nans_trig.h"

namespace glm
{

struct vec4;

struct vec3
{
    float x, y, z;
    vec3() = default;
    template <class S> explicit vec3(S s) : x((float)s), y((float)s), z((float)s) {}
    template <class A, class B, class C>
    vec3(A a, B b, C c) : x((float)a), y((float)b), z((float)c) {}
    explicit vec3(const vec4 &v);

    float &operator[](int i) { return (&x)[i]; }
    const float &operator[](int i) const { return (&x)[i]; }

    vec3 &operator+=(const vec3 &o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3 &operator-=(const vec3 &o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
    template <class S> vec3 &operator*=(S s)
    {
        float f = (float)s;
        x = x * f; y = y * f; z = z * f;
        return *this;
    }
};

struct vec4
{
    float x, y, z, w;
    vec4() = default;
    template <class S> explicit vec4(S s) : x((float)s), y((float)s), z((float)s), w((float)s) {}
    template <class A, class B, class C, class D>
    vec4(A a, B b, C c, D d) : x((float)a), y((float)b), z((float)c), w((float)d) {}
    vec4(const vec3 &v, float w_) : x(v.x), y(v.y), z(v.z), w(w_) {}

    float &operator[](int i) { return (&x)[i]; }
    const float &operator[](int i) const { return (&x)[i]; }
};

inline vec3::vec3(const vec4 &v) : x(v.x), y(v.y), z(v.z) {}

struct ivec2
{
    int x, y;
};

// Column-major 4x4 matrix: c[j] is column j.
struct mat4
{
    vec4 c[4];
    mat4() = default;
    template <class S> explicit mat4(S s)
    {
        float f = (float)s;
        c[0] = vec4(f, 0.0f, 0.0f, 0.0f);
        c[1] = vec4(0.0f, f, 0.0f, 0.0f);
        c[2] = vec4(0.0f, 0.0f, f, 0.0f);
        c[3] = vec4(0.0f, 0.0f, 0.0f, f);
    }
    vec4 &operator[](int i) { return c[i]; }
    const vec4 &operator[](int i) const { return c[i]; }
};

// ---- vec3 arithmetic (component-wise, single rounding per component) ----
inline vec3 operator+(const vec3 &a, const vec3 &b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3 &a, const vec3 &b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(const vec3 &a) { return vec3(-a.x, -a.y, -a.z); }
template <class S> inline vec3 operator*(S s, const vec3 &v)
{
    float f = (float)s;
    return vec3(f * v.x, f * v.y, f * v.z);
}
template <class S> inline vec3 operator*(const vec3 &v, S s)
{
    float f = (float)s;
    return vec3(v.x * f, v.y * f, v.z * f);
}
template <class S> inline vec3 operator/(const vec3 &v, S s)
{
    float f = (float)s;
    return vec3(v.x / f, v.y / f, v.z / f);
}
inline bool operator==(const vec3 &a, const vec3 &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(const vec3 &a, const vec3 &b) { return !(a == b); }

// ---- vec4 arithmetic ----
inline vec4 operator+(const vec4 &a, const vec4 &b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator-(const vec4 &a, const vec4 &b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline vec4 operator*(const vec4 &v, float f) { return vec4(v.x * f, v.y * f, v.z * f, v.w * f); }
inline vec4 operator*(float f, const vec4 &v) { return vec4(f * v.x, f * v.y, f * v.z, f * v.w); }

inline vec4 operator*(const mat4 &m, const vec4 &v)
{
    return ((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3] * v.w;
}

inline mat4 operator*(const mat4 &a, const mat4 &b)
{
    mat4 r;
    for (int j = 0; j < 4; ++j)
        r[j] = ((a[0] * b[j].x + a[1] * b[j].y) + a[2] * b[j].z) + a[3] * b[j].w;
    return r;
}

// ---- geometric functions ----
inline float dot(const vec3 &a, const vec3 &b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 cross(const vec3 &a, const vec3 &b)
{
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(const vec3 &v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(const vec3 &v)
{
    float inv = 1.0f / std::sqrt(dot(v, v));
    return v * inv;
}
inline float abs(float f) { return std::fabs(f); }
inline float radians(float deg) { return deg * 0.0174532925199432957692f; }

// ---- transforms (right-multiplication, as the reference's render code expects) ----
inline mat4 translate(const mat4 &m, const vec3 &v)
{
    mat4 r = m;
    r[3] = ((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3];
    return r;
}

inline mat4 rotate(const mat4 &m, float angle, const vec3 &axis_in)
{
    float c = nans_trig_cosf(angle);
    float s = nans_trig_sinf(angle);
    vec3 a = normalize(axis_in);
    vec3 t = (1.0f - c) * a;
    // Rodrigues rotation matrix, columns.
    vec3 r0(c + t.x * a.x, t.x * a.y + s * a.z, t.x * a.z - s * a.y);
    vec3 r1(t.y * a.x - s * a.z, c + t.y * a.y, t.y * a.z + s * a.x);
    vec3 r2(t.z * a.x + s * a.y, t.z * a.y - s * a.x, c + t.z * a.z);
    mat4 r;
    r[0] = (m[0] * r0.x + m[1] * r0.y) + m[2] * r0.z;
    r[1] = (m[0] * r1.x + m[1] * r1.y) + m[2] * r1.z;
    r[2] = (m[0] * r2.x + m[1] * r2.y) + m[2] * r2.z;
    r[3] = m[3];
    return r;
}

inline mat4 scale(const mat4 &m, const vec3 &v)
{
    mat4 r;
    r[0] = m[0] * v.x;
    r[1] = m[1] * v.y;
    r[2] = m[2] * v.z;
    r[3] = m[3];
    return r;
}

// Camera helpers used only by the (GL-less) render code; never on the physics path.
inline mat4 perspective(float fovy, float aspect, float znear, float zfar)
{
    float t = std::tan(fovy / 2.0f);
    mat4 r(0.0f);
    r[0][0] = 1.0f / (aspect * t);
    r[1][1] = 1.0f / t;
    r[2][2] = -(zfar + znear) / (zfar - znear);
    r[2][3] = -1.0f;
    r[3][2] = -(2.0f * zfar * znear) / (zfar - znear);
    return r;
}

inline mat4 lookAt(const vec3 &eye, const vec3 &center, const vec3 &up)
{
    vec3 f = normalize(center - eye);
    vec3 s = normalize(cross(f, up));
    vec3 u = cross(s, f);
    mat4 r(1.0f);
    r[0][0] = s.x; r[1][0] = s.y; r[2][0] = s.z;
    r[0][1] = u.x; r[1][1] = u.y; r[2][1] = u.z;
    r[0][2] = -f.x; r[1][2] = -f.y; r[2][2] = -f.z;
    r[3][0] = -dot(s, eye);
    r[3][1] = -dot(u, eye);
    r[3][2] = dot(f, eye);
    return r;
}

} // namespace glm

#endif
