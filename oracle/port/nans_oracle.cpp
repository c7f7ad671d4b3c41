// Test infrastructure: the oracle. A CPU restatement of the reference physics step
// (code/nans.cpp, L4v/nans_projekat) templated on the scalar type:
//   * float  -- must reproduce the reference bit for bit (checked against the reference
//               compiled headless from its own sources, and against committed fixtures);
//   * double -- the FP64 run of the same method, used as the error and gradient reference.
// It is the checker for the CUDA library and the CPU baseline that bench.py times; the
// product never links or calls it.
//
// Vector arithmetic follows the operation order pinned by the glm shim
// (oracle/shim/glm/glm.hpp): dot = (x*x'+y*y')+z*z', normalize = v*(1/sqrt(dot(v,v))).
// Build without FP contraction (-ffp-contract=off).
//
// Scenes are independent; nanso_step runs them on a pool of host threads.
#include <cmath>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <vector>
#include <thread>
#include <atomic>
#include <algorithm>
#include <string>
#include <array>
#include <map>
#include <cstdio>
#include <cstdlib>

#include "nans_trig.h"  // the project sincos (oracle/shim/glm/nans_trig.h)

namespace
{

// ---------------------------------------------------------------------------------
// scalar traits: the literal constants of the reference in each precision
// ---------------------------------------------------------------------------------
template <class T> struct K;
template <> struct K<float>
{
    static float gravity() { return 9.81f; }            // code/nans.cpp:68 (9.81f)
    static float damping() { return 1.5f; }             // GLOBAL_FRICTION code/nans.h:46
    static float sixth() { return 1.0f / 6.0f; }        // code/nans.cpp:59
    static float epa_tol() { return 0.001f; }           // MAX_EPA_ERROR code/nans.h:55
    static float dir_eps() { return 0.0001f; }          // code/nans.cpp:755
    static float tangent_switch() { return 0.57735f; }  // code/nans.cpp:1125
    static float beta() { return 0.3f; }                // code/nans.cpp:1152
    static float neg_flt_max() { return -FLT_MAX; }     // code/nans.cpp:412
    // (real32)(1.0 / Mass): the reciprocal is taken in double, then rounded (code/nans.cpp:68)
    static float inv_mass_rk(float m) { return (float)(1.0 / (double)m); }
    static float inv_f(float m) { return 1.0f / m; }
    // sqrt(2) * Cf * Sum is evaluated in double and stored to real32 (code/nans.cpp:1199)
    static float friction_bound(float cf, float sum)
    {
        return (float)(std::sqrt(2.0) * (double)cf * (double)sum);
    }
    static float radians(float d) { return d * 0.0174532925199432957692f; }
    static void sincos(float x, float *s, float *c) { nans_trig_sincosf(x, s, c); }
};
template <> struct K<double>
{
    static double gravity() { return 9.81; }
    static double damping() { return 1.5; }
    static double sixth() { return 1.0 / 6.0; }
    static double epa_tol() { return 0.001; }
    static double dir_eps() { return 0.0001; }
    static double tangent_switch() { return 0.57735; }
    static double beta() { return 0.3; }
    static double neg_flt_max() { return -DBL_MAX; }
    static double inv_mass_rk(double m) { return 1.0 / m; }
    static double inv_f(double m) { return 1.0 / m; }
    static double friction_bound(double cf, double sum) { return std::sqrt(2.0) * cf * sum; }
    static double radians(double d) { return d * 0.017453292519943295769; }
    static void sincos(double x, double *s, double *c)
    {
        *s = std::sin(x);
        *c = std::cos(x);
    }
};

template <class T> struct V3
{
    T x, y, z;
};
template <class T> static inline V3<T> mk(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> static inline V3<T> add(V3<T> a, V3<T> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> static inline V3<T> sub(V3<T> a, V3<T> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> static inline V3<T> neg(V3<T> a) { return mk(-a.x, -a.y, -a.z); }
template <class T> static inline V3<T> mul(T s, V3<T> a) { return mk(s * a.x, s * a.y, s * a.z); }
template <class T> static inline V3<T> divs(V3<T> a, T s) { return mk(a.x / s, a.y / s, a.z / s); }
template <class T> static inline T dot(V3<T> a, V3<T> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class T> static inline V3<T> cross(V3<T> a, V3<T> b)
{
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T> static inline T len(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> static inline V3<T> normalize(V3<T> a)
{
    T inv = T(1) / std::sqrt(dot(a, a));
    return mk(a.x * inv, a.y * inv, a.z * inv);
}
template <class T> static inline bool eq(V3<T> a, V3<T> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// 4x4 column-major matrix: c[j] = column j (4 entries).
template <class T> struct M4
{
    T c[4][4];
};
template <class T> static inline void col_lin3(const M4<T> &m, T a, T b, T cc, T out[4])
{
    // ((m0*a + m1*b) + m2*c)
    for (int r = 0; r < 4; ++r)
        out[r] = (m.c[0][r] * a + m.c[1][r] * b) + m.c[2][r] * cc;
}
template <class T> static M4<T> ident()
{
    M4<T> m;
    for (int j = 0; j < 4; ++j)
        for (int r = 0; r < 4; ++r)
            m.c[j][r] = (j == r) ? T(1) : T(0);
    return m;
}
template <class T> static M4<T> translate(const M4<T> &m, V3<T> v)
{
    M4<T> r = m;
    T t[4];
    col_lin3(m, v.x, v.y, v.z, t);
    for (int k = 0; k < 4; ++k)
        r.c[3][k] = t[k] + m.c[3][k];
    return r;
}
template <class T> static M4<T> rotate(const M4<T> &m, T angle, V3<T> axis)
{
    T s, c;
    K<T>::sincos(angle, &s, &c);
    V3<T> a = normalize(axis);
    V3<T> t = mul(T(1) - c, a);
    V3<T> r0 = mk(c + t.x * a.x, t.x * a.y + s * a.z, t.x * a.z - s * a.y);
    V3<T> r1 = mk(t.y * a.x - s * a.z, c + t.y * a.y, t.y * a.z + s * a.x);
    V3<T> r2 = mk(t.z * a.x + s * a.y, t.z * a.y - s * a.x, c + t.z * a.z);
    M4<T> r;
    col_lin3(m, r0.x, r0.y, r0.z, r.c[0]);
    col_lin3(m, r1.x, r1.y, r1.z, r.c[1]);
    col_lin3(m, r2.x, r2.y, r2.z, r.c[2]);
    for (int k = 0; k < 4; ++k)
        r.c[3][k] = m.c[3][k];
    return r;
}
template <class T> static M4<T> scale(const M4<T> &m, V3<T> v)
{
    M4<T> r;
    for (int k = 0; k < 4; ++k)
    {
        r.c[0][k] = m.c[0][k] * v.x;
        r.c[1][k] = m.c[1][k] * v.y;
        r.c[2][k] = m.c[2][k] * v.z;
        r.c[3][k] = m.c[3][k];
    }
    return r;
}
// M * (p, 1), keeping xyz: ((m0*x + m1*y) + m2*z) + m3*1
template <class T> static inline V3<T> xform(const M4<T> &m, V3<T> p)
{
    T o[4];
    col_lin3(m, p.x, p.y, p.z, o);
    return mk(o[0] + m.c[3][0] * T(1), o[1] + m.c[3][1] * T(1), o[2] + m.c[3][2] * T(1));
}

// Model = T(P) * Rx * Ry * Rz * S, angles in degrees (code/nans.cpp:1913-1923)
template <class T> static M4<T> model_of(V3<T> P, V3<T> A, V3<T> S)
{
    M4<T> m = ident<T>();
    m = translate(m, P);
    m = rotate(m, K<T>::radians(A.x), mk(T(1), T(0), T(0)));
    m = rotate(m, K<T>::radians(A.y), mk(T(0), T(1), T(0)));
    m = rotate(m, K<T>::radians(A.z), mk(T(0), T(0), T(1)));
    m = scale(m, S);
    return m;
}

// Unit-cube corners in the order of UpdateVertices (code/nans.cpp:399-406).
static const float kCorner[8][3] = {
    {0.5f, 0.5f, 0.5f}, {0.5f, 0.5f, -0.5f}, {-0.5f, 0.5f, 0.5f}, {-0.5f, 0.5f, -0.5f},
    {0.5f, -0.5f, 0.5f}, {0.5f, -0.5f, -0.5f}, {-0.5f, -0.5f, 0.5f}, {-0.5f, -0.5f, -0.5f}};

enum { TCC = 0, TCS = 1, TCF = 2, TSS = 3, TSF = 4 };

template <class T> struct Body
{
    V3<T> P, V, F, A, W, Tq;
    T mass, moi, radius;
    V3<T> scl;             // model scale (cubes / hulls / floor)
    M4<T> model;           // current model (built after each step)
    int npts;              // local hull points (8 = reference cube corners)
    std::vector<V3<T>> local;
    std::vector<V3<T>> verts;
};

template <class T> struct Vx
{
    V3<T> P, SupA, SupB;
};

template <class T> struct Contact
{
    int type, a, b;
    V3<T> pa, pb, n;
    T sn, st1, st2; // accumulated impulses: initial values (warm start), then final values
    bool held = false;   // replayed contact: the solve takes the bodies' positions from pos_a / pos_b
    V3<T> pos_a, pos_b;  // (replayed contacts only) the two bodies' positions at the recorded solve
};

struct Consts
{
    float cr, cf;
    int iters;
};

template <class T> struct Scene
{
    std::vector<Body<T>> cubes, spheres;
    Body<T> floor;
    std::vector<Contact<T>> pairs;
    Consts k;
    bool warm = false;                // warm starting: accumulators carried across steps
    std::vector<Contact<T>> prev;     // the last solve's contacts with their accumulators
    // Held contacts (test infrastructure for gradient checks): when replay is non-empty, the
    // detect stage of the k-th step does not run GJK/EPA but takes replay[k], the contact list
    // and contact geometry recorded from another run, and the solve computes its
    // velocity-independent constants (lever arms, depth) from the recorded body positions. The
    // step is then the rollout with its contact set and geometry held fixed.
    std::vector<std::vector<Contact<T>>> replay;
    size_t replay_step = 0;
};

// ---------------------------------------------------------------------------------
// integration (code/nans.cpp:50-78, 974-1018, 1331-1349)
// ---------------------------------------------------------------------------------
// MovementFunction (code/nans.cpp:63-70): (1/m)(F + m g (0,-1,0) - 1.5 v), 1/m in double
template <class T> static V3<T> movement(V3<T> v, V3<T> f, T m, T invm)
{
    T s = m * K<T>::gravity();
    V3<T> g = mk(s * T(0), s * T(-1), s * T(0));
    V3<T> t = sub(add(f, g), mul(K<T>::damping(), v));
    return mul(invm, t);
}
// RotationFunction (code/nans.cpp:72-78)
template <class T> static V3<T> rotation(V3<T> w, V3<T> tq, T invi)
{
    return mul(invi, sub(tq, mul(K<T>::damping(), w)));
}
// RK4 (code/nans.cpp:50-61): Y0 + (1/6)(((K1 + 2 K2) + 2 K3) + K4)
template <class T, class Fn> static V3<T> rk4(Fn f, T dt, V3<T> y0)
{
    V3<T> k1 = mul(dt, f(y0));
    V3<T> k2 = mul(dt, f(add(y0, divs(k1, T(2)))));
    V3<T> k3 = mul(dt, f(add(y0, divs(k2, T(2)))));
    V3<T> k4 = mul(dt, f(add(y0, k3)));
    V3<T> s = add(add(add(k1, mul(T(2), k2)), mul(T(2), k3)), k4);
    return add(y0, mul(K<T>::sixth(), s));
}

// UpdateVertices / FloorUpdateVertices (code/nans.cpp:379-407): Model times each local point
template <class T> static void update_vertices(Body<T> &b)
{
    b.verts.resize(b.npts);
    for (int k = 0; k < b.npts; ++k)
        b.verts[k] = xform(b.model, b.local[k]);
}

// the two RK4 calls of IntegrateForces for one body (code/nans.cpp:974-1018)
template <class T> static void integrate_body(Body<T> &b, T dt)
{
    T invm = K<T>::inv_mass_rk(b.mass);
    T m = b.mass;
    V3<T> f = b.F;
    b.V = rk4([&](V3<T> y) { return movement(y, f, m, invm); }, dt, b.V);
    T invi = K<T>::inv_f(b.moi);
    V3<T> tq = b.Tq;
    b.W = rk4([&](V3<T> y) { return rotation(y, tq, invi); }, dt, b.W);
}

// IntegrateForces (code/nans.cpp:974-1018)
template <class T> static void integrate_forces(Scene<T> &s, T dt)
{
    for (auto &b : s.cubes)
    {
        integrate_body(b, dt);
        update_vertices(b);
        b.F = mk(T(0), T(0), T(0));
        b.Tq = mk(T(0), T(0), T(0));
    }
    for (auto &b : s.spheres)
    {
        integrate_body(b, dt);
        b.F = mk(T(0), T(0), T(0));
        b.Tq = mk(T(0), T(0), T(0));
    }
    update_vertices(s.floor);
}

// IntegrateVelocities (code/nans.cpp:1331-1349)
template <class T> static void integrate_velocities(Scene<T> &s, T dt)
{
    for (auto &b : s.cubes)
    {
        b.P = add(b.P, mul(dt, b.V));
        b.A = add(b.A, mul(dt, b.W));
    }
    for (auto &b : s.spheres)
    {
        b.P = add(b.P, mul(dt, b.V));
        b.A = add(b.A, mul(dt, b.W));
    }
}

// the render code's Model rebuild after the step (code/nans.cpp:1870-1881, 1909-1942)
template <class T> static void rebuild(Scene<T> &s)
{
    for (auto &b : s.cubes)
        b.model = model_of(b.P, b.A, b.scl);
    s.floor.model = model_of(s.floor.P, s.floor.A, s.floor.scl);
}

// ---------------------------------------------------------------------------------
// support maps (code/nans.cpp:409-537)
// ---------------------------------------------------------------------------------
// GetCubeSupport / GetFloorSupport (code/nans.cpp:409-430, 440-461): first maximum from -FLT_MAX
template <class T> static V3<T> hull_support(const Body<T> &b, V3<T> d)
{
    T best = K<T>::neg_flt_max();
    V3<T> r = mk(T(0), T(0), T(0));
    for (int k = 0; k < b.npts; ++k)
    {
        T dist = dot(b.verts[k], d);
        if (dist > best)
        {
            best = dist;
            r = b.verts[k];
        }
    }
    return r;
}
// GetSphereSupport (code/nans.cpp:432-438)
template <class T> static V3<T> sphere_support(const Body<T> &b, V3<T> d)
{
    return add(b.P, mul(b.radius, normalize(d)));
}

template <class T> struct PairCtx
{
    const Body<T> *A;
    const Body<T> *B;
    bool a_sphere, b_sphere;
};

// CalculateSupport (code/nans.cpp:463-519): SupA(d) - SupB(-d) by pair type
template <class T> static Vx<T> support(const PairCtx<T> &p, V3<T> d)
{
    V3<T> nd = mul(T(-1), d);
    V3<T> sa = p.a_sphere ? sphere_support(*p.A, d) : hull_support(*p.A, d);
    V3<T> sb = p.b_sphere ? sphere_support(*p.B, nd) : hull_support(*p.B, nd);
    return Vx<T>{sub(sa, sb), sa, sb};
}

// ---------------------------------------------------------------------------------
// GJK (code/nans.cpp:539-769, 906-966)
// ---------------------------------------------------------------------------------
enum { NoHit = 0, Found = 1, Evolving = 2 };

// EvolveSimplex (code/nans.cpp:571-769) with ClosestPointOnLine / TripleCross (:539-569)
template <class T> static int evolve(const PairCtx<T> &p, std::vector<Vx<T>> &S)
{
    V3<T> dir = normalize(sub(p.B->P, p.A->P));
    switch (S.size())
    {
    case 0:
        break;
    case 1:
        dir = mul(T(-1), dir);
        break;
    case 2:
    {
        // ClosestPointOnLine (code/nans.cpp:539-562) with A=S0, B=S1
        V3<T> a = S[0].P, b = S[1].P;
        V3<T> l = normalize(sub(b, a));
        T ln = len(l);
        T v = dot(neg(a), l) / ln;
        T u = dot(b, l) / ln;
        V3<T> cp;
        if (u <= T(0))
            cp = b;
        else if (v <= T(0))
            cp = a;
        else
            cp = add(mul(u, a), mul(v, b));
        if (v <= T(0))
            S.erase(S.begin() + 1);
        else if (u <= T(0))
            S.erase(S.begin());
        dir = neg(cp);
        break;
    }
    case 3:
    {
        V3<T> a0 = neg(S[0].P);
        V3<T> e1 = sub(S[1].P, S[0].P);
        V3<T> e2 = sub(S[2].P, S[0].P);
        V3<T> tn = cross(e1, e2);
        V3<T> e1n = cross(e1, tn);
        V3<T> e2n = cross(tn, e2);
        auto triple = [](V3<T> a, V3<T> b, V3<T> c) { return sub(mul(dot(c, a), b), mul(dot(c, b), a)); };
        if (dot(e2n, a0) > T(0))
        {
            if (dot(e2, a0) > T(0))
            {
                dir = triple(e2, a0, e2);
                S.erase(S.begin() + 1);
            }
            else if (dot(e1, a0) > T(0))
            {
                dir = triple(e1, a0, e1);
                S.erase(S.begin() + 2);
            }
            else
            {
                dir = a0;
                S.erase(S.begin() + 2);
                S.erase(S.begin() + 1);
            }
        }
        else if (dot(e1n, a0) > T(0))
        {
            if (dot(e1, a0) > T(0))
            {
                dir = triple(e1, a0, e1);
                S.erase(S.begin() + 2);
            }
            else
            {
                dir = a0;
                S.erase(S.begin() + 2);
                S.erase(S.begin() + 1);
            }
        }
        else if (dot(tn, a0) > T(0))
        {
            dir = tn;
        }
        else
        {
            dir = neg(tn);
            std::swap(S[1], S[2]);
        }
        break;
    }
    case 4:
    {
        V3<T> da = sub(S[0].P, S[3].P);
        V3<T> db = sub(S[1].P, S[3].P);
        V3<T> dc = sub(S[2].P, S[3].P);
        V3<T> d0 = mul(T(-1), S[3].P);
        V3<T> abd = cross(da, db);
        V3<T> bcd = cross(db, dc);
        V3<T> cad = cross(dc, da);
        if (dot(abd, d0) > T(0))
        {
            S.erase(S.begin() + 2);
            dir = abd;
        }
        else if (dot(bcd, d0) > T(0))
        {
            S.erase(S.begin());
            dir = bcd;
        }
        else if (dot(cad, d0) > T(0))
        {
            S.erase(S.begin() + 1);
            dir = cad;
        }
        else
            return Found;
        break;
    }
    default:
        break;
    }
    if (len(dir) <= K<T>::dir_eps())
        return NoHit;
    Vx<T> nv = support(p, dir);
    S.push_back(nv);
    return dot(dir, nv.P) >= T(0) ? Evolving : NoHit;
}

// ---------------------------------------------------------------------------------
// EPA (code/nans.cpp:217-328, 771-904)
// ---------------------------------------------------------------------------------
template <class T> struct Face
{
    Vx<T> a, b, c;
    V3<T> n;
};
template <class T> struct Edge
{
    Vx<T> a, b;
};

// PushTriangle (code/nans.cpp:292-328): normal flipped away from the origin
template <class T> static void push_face(std::vector<Face<T>> &F, const Vx<T> &a, const Vx<T> &b, const Vx<T> &c)
{
    Face<T> f{a, b, c, normalize(cross(sub(b.P, a.P), sub(c.P, a.P)))};
    if (dot(a.P, f.n) < T(0))
        f.n = mul(T(-1), f.n);
    F.push_back(f);
}

// PushEdge (code/nans.cpp:232-266): cancels the first stored reverse edge, else appends
template <class T> static void push_edge(std::vector<Edge<T>> &E, const Vx<T> &a, const Vx<T> &b)
{
    for (size_t i = 0; i < E.size(); ++i)
        if (eq(E[i].a.P, b.P) && eq(E[i].b.P, a.P))
        {
            E.erase(E.begin() + i);
            return;
        }
    E.push_back(Edge<T>{a, b});
}

// Barycentric (code/nans.cpp:771-785)
template <class T> static void barycentric(V3<T> p, V3<T> a, V3<T> b, V3<T> c, T *u, T *v, T *w)
{
    V3<T> v0 = sub(b, a), v1 = sub(c, a), v2 = sub(p, a);
    T d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1);
    T d20 = dot(v2, v0), d21 = dot(v2, v1);
    T den = d00 * d11 - d01 * d01;
    *v = (d11 * d20 - d01 * d21) / den;
    *w = (d00 * d21 - d01 * d20) / den;
    *u = T(1) - *v - *w;
}

// IsValid (code/nans.cpp:3-17)
template <class T> static bool finite(T x) { return !(std::isnan(x) || std::isinf(x)); }

// EPA size statistics (max faces, max horizon edges, max iterations), for sizing the
// device's shared-memory buffers.
// Statistics are off unless nanso_stats_enable(1) is called: the shared counters would
// otherwise serialise the host threads of a timed run.
static bool g_stats = false;
static std::atomic<int> g_epa_max_faces(0), g_epa_max_edges(0), g_epa_max_iters(0);
static std::atomic<long long> g_epa_calls(0);
static std::atomic<long long> g_epa_big[4]; // EPAs whose face list exceeded 128, 256, 1024, 4096
static std::atomic<long long> g_epa_big_nan0(0); // of those above 128: face 0 had a NaN distance
static std::atomic<long long> g_epa_stale(0);     // EPAs that read the emptied face list
static std::atomic<long long> g_epa_big_contact(0); // EPAs above 1024 faces that returned a contact
static std::atomic<long long> g_epa_iter_hist[5];  // EPAs ending after 1-4, 5-8, 9-16, 17-64, 65 iterations
static std::atomic<long long> g_gjk_iters(0), g_gjk_calls(0);
static std::atomic<long long> g_epa_tiny_fit[4]; // EPAs that fit (V<=12,F<=20,E<=12), exceed V, F, E
static std::atomic<int> g_epa_hist_faces[64];
static std::atomic<long long> g_gjk_hist[8]; // GJK runs by evolve calls: 1,2,3-4,5-8,9-16,17-32,33-64,65 + result
static void atomic_max(std::atomic<int> &a, int v)
{
    int cur = a.load();
    while (v > cur && !a.compare_exchange_weak(cur, v))
    {
    }
}

// ResolveCollision (code/nans.cpp:787-904)
template <class T> static bool epa(const PairCtx<T> &p, const std::vector<Vx<T>> &S, Contact<T> &out)
{
    if (g_stats)
        g_epa_calls.fetch_add(1);
    struct BigCount
    {
        size_t peak = 0;
        size_t peak_edges = 0;
        bool contact = false;
        int iters = 65;
        ~BigCount()
        {
            if (!g_stats)
                return;
            int verts = 4 + iters - 1; // supports added before the final iteration
            bool v_ok = verts <= 12, f_ok = peak <= 20, e_ok = peak_edges <= 12;
            if (v_ok && f_ok && e_ok) g_epa_tiny_fit[0].fetch_add(1);
            if (!v_ok) g_epa_tiny_fit[1].fetch_add(1);
            if (!f_ok) g_epa_tiny_fit[2].fetch_add(1);
            if (!e_ok) g_epa_tiny_fit[3].fetch_add(1);
            g_epa_hist_faces[peak < 63 ? peak : 63].fetch_add(1);
            int b = iters <= 4 ? 0 : iters <= 8 ? 1 : iters <= 16 ? 2 : iters <= 64 ? 3 : 4;
            g_epa_iter_hist[b].fetch_add(1);
            if (peak > 1024 && contact) g_epa_big_contact.fetch_add(1);
            if (peak > 128) g_epa_big[0].fetch_add(1);
            if (peak > 256) g_epa_big[1].fetch_add(1);
            if (peak > 1024) g_epa_big[2].fetch_add(1);
            if (peak > 4096) g_epa_big[3].fetch_add(1);
        }
    } big;
    std::vector<Face<T>> F;
    std::vector<Edge<T>> E;
    F.reserve(64);
    push_face(F, S[0], S[1], S[2]);
    push_face(F, S[0], S[2], S[3]);
    push_face(F, S[0], S[3], S[1]);
    push_face(F, S[1], S[3], S[2]);
#ifdef NANS_EPA_TRACE
    std::vector<std::string> trace;
#endif
    // When every face was removed and the horizon cancelled out, the reference reads
    // Triangle[0] of an empty vector (code/nans.cpp:807, 824). With libstdc++ that slot
    // still holds the face erased last (erase shifts trivially copyable elements down and
    // leaves the old slot contents), which is the last face of the list before removal.
    // `stale` models exactly that read.
    bool has_stale = false;
    Face<T> stale{};
    for (int it = 0; it <= 64; ++it)
    {
        if (F.empty())
        {
            if (!has_stale)
                return false;
            T cur = std::fabs(dot(stale.n, stale.a.P));
            Vx<T> ns = support(p, stale.n);
            if (!(dot(stale.n, ns.P) - cur < K<T>::epa_tol()))
                return false; // every remaining iteration repeats this one
            T u, v, w;
            barycentric(mul(cur, stale.n), stale.a.P, stale.b.P, stale.c.P, &u, &v, &w);
            if (std::fabs(u) > T(1) || std::fabs(v) > T(1) || std::fabs(w) > T(1))
                return false;
            if (!finite(u) || !finite(v) || !finite(w))
                return false;
            out.pa = add(add(mul(u, stale.a.SupA), mul(v, stale.b.SupA)), mul(w, stale.c.SupA));
            out.n = mul(T(-1), stale.n);
            out.pb = add(add(mul(u, stale.a.SupB), mul(v, stale.b.SupB)), mul(w, stale.c.SupB));
            return true;
        }
        if (g_stats)
        {
            atomic_max(g_epa_max_faces, (int)F.size());
            if (F.size() > 128 && big.peak <= 128 && std::isnan(std::fabs(dot(F[0].n, F[0].a.P))))
                g_epa_big_nan0.fetch_add(1);
            atomic_max(g_epa_max_iters, it);
        }
        big.peak = std::max(big.peak, F.size());
        big.iters = it + 1;
        T cur = std::fabs(dot(F[0].n, F[0].a.P));
        size_t ci = 0;
        for (size_t i = 0; i < F.size(); ++i)
        {
            V3<T> nrm = normalize(cross(sub(F[i].b.P, F[i].a.P), sub(F[i].c.P, F[i].a.P)));
            T d = std::fabs(dot(nrm, F[i].a.P));
            if (d < cur)
            {
                cur = d;
                ci = i;
            }
        }
        Face<T> cf = F[ci];
        Vx<T> ns = support(p, cf.n);
#ifdef NANS_EPA_TRACE
        {
            int nanf = 0, vis = 0, dup = 0;
            for (auto &f : F)
            {
                if (std::isnan(std::fabs(dot(f.n, f.a.P))))
                    ++nanf;
                if (dot(f.n, sub(ns.P, f.a.P)) > T(0))
                    ++vis;
            }
            for (auto &f : F)
                if (eq(f.a.P, ns.P) || eq(f.b.P, ns.P) || eq(f.c.P, ns.P))
                {
                    dup = 1;
                    break;
                }
            char buf[256];
            snprintf(buf, sizeof(buf), "it %d faces %zu nan %d visible %d closest %zu cur %.9g gap %.9g dupS %d",
                     it, F.size(), nanf, vis, ci, (double)cur, (double)(dot(cf.n, ns.P) - cur), dup);
            trace.push_back(buf);
            if (F.size() > 50000)
            {
                // group sizes of the horizon pushes by undirected P-edge key
                std::vector<std::pair<std::array<float, 6>, int>> keys;
                for (auto &f : F)
                    if (dot(f.n, sub(ns.P, f.a.P)) > T(0))
                    {
                        const Vx<T> *vv[4] = {&f.a, &f.b, &f.c, &f.a};
                        for (int k = 0; k < 3; ++k)
                        {
                            std::array<float, 6> a = {(float)vv[k]->P.x, (float)vv[k]->P.y, (float)vv[k]->P.z,
                                                      (float)vv[k + 1]->P.x, (float)vv[k + 1]->P.y, (float)vv[k + 1]->P.z};
                            std::array<float, 6> b = {a[3], a[4], a[5], a[0], a[1], a[2]};
                            keys.push_back({std::min(a, b), 0});
                        }
                    }
                std::sort(keys.begin(), keys.end());
                std::map<int, long> hist;
                for (size_t i = 0; i < keys.size();)
                {
                    size_t j = i;
                    while (j < keys.size() && keys[j].first == keys[i].first)
                        ++j;
                    hist[(int)std::min<size_t>(j - i, 64)]++;
                    i = j;
                }
                fprintf(stderr, "it %d faces %zu pushes %zu groups:", it, F.size(), keys.size());
                for (auto &h : hist)
                    fprintf(stderr, " %d:%ld", h.first, h.second);
                fprintf(stderr, "\n");
                static int printed = 0;
                if (++printed >= 4)
                    abort();
            }
        }
#endif
        if (dot(cf.n, ns.P) - cur < K<T>::epa_tol())
        {
            T u, v, w;
            barycentric(mul(cur, cf.n), cf.a.P, cf.b.P, cf.c.P, &u, &v, &w);
            if (std::fabs(u) > T(1) || std::fabs(v) > T(1) || std::fabs(w) > T(1))
                return false;
            if (!finite(u) || !finite(v) || !finite(w))
                return false;
            out.pa = add(add(mul(u, cf.a.SupA), mul(v, cf.b.SupA)), mul(w, cf.c.SupA));
            out.n = mul(T(-1), cf.n);
            out.pb = add(add(mul(u, cf.a.SupB), mul(v, cf.b.SupB)), mul(w, cf.c.SupB));
            big.contact = true;
            return true;
        }
        const Face<T> last_face = F.back();
        for (size_t i = 0; i < F.size();)
        {
            V3<T> tmp = sub(ns.P, F[i].a.P);
            V3<T> nrm = normalize(cross(sub(F[i].b.P, F[i].a.P), sub(F[i].c.P, F[i].a.P)));
            if (dot(nrm, F[i].a.P) < T(0))
                nrm = mul(T(-1), nrm);
            if (dot(nrm, tmp) > T(0))
            {
                push_edge(E, F[i].a, F[i].b);
                push_edge(E, F[i].b, F[i].c);
                push_edge(E, F[i].c, F[i].a);
                F.erase(F.begin() + i);
                continue;
            }
            ++i;
        }
        if (g_stats)
            atomic_max(g_epa_max_edges, (int)E.size());
        big.peak_edges = std::max(big.peak_edges, E.size());
        big.peak = std::max(big.peak, F.size() + E.size());
        if (F.empty() && E.empty())
        {
            if (g_stats)
                g_epa_stale.fetch_add(1);
            has_stale = true;
            stale = last_face;
        }
        for (size_t i = 0; i < E.size(); ++i)
            push_face(F, ns, E[i].a, E[i].b);
        E.clear();
    }
    return false;
}

// CheckCollision (code/nans.cpp:906-966)
template <class T> static bool check_collision(const PairCtx<T> &p, Contact<T> &c)
{
    std::vector<Vx<T>> S;
    S.reserve(8);
    int r = Evolving;
    int it = 0;
    for (; r == Evolving && it <= 64; ++it)
        r = evolve(p, S);
    if (g_stats)
    {
        g_gjk_iters.fetch_add(it);
        g_gjk_calls.fetch_add(1);
        int b = it <= 1 ? 0 : it <= 2 ? 1 : it <= 4 ? 2 : it <= 8 ? 3 : it <= 16 ? 4 : it <= 32 ? 5 : it <= 64 ? 6 : 7;
        g_gjk_hist[b].fetch_add(1);
    }
    if (r == Found)
        return epa(p, S, c);
    return false;
}

// ---------------------------------------------------------------------------------
// narrowphase driver: pair order CC, CF, SF, CS, SS (code/nans.cpp:1351-1536)
// ---------------------------------------------------------------------------------
// DetectCollisions (code/nans.cpp:1351-1536)
template <class T> static void detect(Scene<T> &s)
{
    if (!s.replay.empty())
    {
        if (s.replay_step < s.replay.size())
            s.pairs = s.replay[s.replay_step++];
        else
            s.pairs.clear();
        return;
    }
    s.pairs.clear();
    const int nc = (int)s.cubes.size(), ns = (int)s.spheres.size();
    auto run = [&](int type, int ia, int ib, const Body<T> *A, const Body<T> *B, bool as, bool bs) {
        Contact<T> c{type, ia, ib, mk(T(0), T(0), T(0)), mk(T(0), T(0), T(0)), mk(T(0), T(0), T(0)), T(0), T(0),
                     T(0)};
        PairCtx<T> p{A, B, as, bs};
        if (check_collision(p, c))
            s.pairs.push_back(c);
    };
    for (int i = 0; i < nc; ++i)
        for (int j = i + 1; j < nc; ++j)
            run(TCC, i, j, &s.cubes[i], &s.cubes[j], false, false);
    for (int i = 0; i < nc; ++i)
        run(TCF, i, i, &s.cubes[i], &s.floor, false, false);
    for (int i = 0; i < ns; ++i)
        run(TSF, i, i, &s.spheres[i], &s.floor, true, false);
    for (int i = 0; i < nc; ++i)
        for (int j = 0; j < ns; ++j)
            run(TCS, i, j, &s.cubes[i], &s.spheres[j], false, true);
    for (int i = 0; i < ns; ++i)
        for (int j = i + 1; j < ns; ++j)
            run(TSS, i, j, &s.spheres[i], &s.spheres[j], true, true);
}

// ---------------------------------------------------------------------------------
// sequential impulses (code/nans.cpp:1020-1329, 1538-1548)
// ---------------------------------------------------------------------------------
// Constraint (code/nans.cpp:1020-1329)
template <class T> static void constraint(Scene<T> &s, Contact<T> &c, T dt)
{
    Body<T> *A, *B;
    switch (c.type)
    {
    case TCC: A = &s.cubes[c.a]; B = &s.cubes[c.b]; break;
    case TCS: A = &s.cubes[c.a]; B = &s.spheres[c.b]; break;
    case TCF: A = &s.cubes[c.a]; B = &s.floor; break;
    case TSS: A = &s.spheres[c.a]; B = &s.spheres[c.b]; break;
    default: A = &s.spheres[c.a]; B = &s.floor; break;
    }
    const bool writes_b = (c.type != TCF && c.type != TSF);
    V3<T> n = normalize(c.n);
    V3<T> pa = c.held ? c.pos_a : A->P, pb = c.held ? c.pos_b : B->P;
    T invi1 = T(1) / A->moi, invi2 = T(1) / B->moi;
    T invm1 = T(1) / A->mass, invm2 = T(1) / B->mass;
    V3<T> v1 = A->V, v2 = B->V, w1 = A->W, w2 = B->W;
    if (eq(n, mk(T(0), T(0), T(0))))
        n = normalize(sub(pb, pa));
    V3<T> r1 = sub(c.pa, pa);
    V3<T> r2 = sub(c.pb, pb);
    V3<T> t1 = (n.x >= K<T>::tangent_switch()) ? mk(n.y, -n.x, T(0)) : mk(T(0), n.z, -n.y);
    V3<T> t2 = cross(n, t1);
    T depth = dot(sub(add(pa, r1), add(pb, r2)), n);
    V3<T> rn1 = cross(r1, n);
    V3<T> rn2 = cross(r2, n);
    T jn = invm1 + invm2;
    jn = jn + (invi1 * dot(rn1, rn1) - invi2 * dot(neg(rn2), neg(rn2)));
    jn = T(1) / jn;
    V3<T> dvn = sub(sub(add(v1, cross(w1, n)), v2), cross(w2, n));
    T jdvn = dot(dvn, n);
    T cr = (T)s.k.cr, cf = (T)s.k.cf;
    T bias = (-K<T>::beta()) / dt * depth + cr * jdvn;
    V3<T> r1t1 = cross(r1, t1), r2t1 = cross(r2, t1), r1t2 = cross(r1, t2), r2t2 = cross(r2, t2);
    T jt1 = invm1 + invm2;
    jt1 = jt1 + (invi1 * dot(r1t1, r1t1) - invi2 * dot(neg(r2t1), neg(r2t1)));
    jt1 = T(1) / jt1;
    T jt2 = invm1 + invm2;
    jt2 = jt2 + (invi1 * dot(r1t2, r1t2) - invi2 * dot(neg(r2t2), neg(r2t2)));
    jt2 = T(1) / jt2;
    T jdvt1 = dot(sub(sub(add(v1, cross(w1, t1)), v2), cross(w2, t1)), t1);
    T jdvt2 = dot(sub(sub(add(v1, cross(w1, t2)), v2), cross(w2, t2)), t2);

    T sn = c.sn, st1 = c.st1, st2 = c.st2, dn = 0, dt1 = 0, dt2 = 0;
    for (int it = 0; it < s.k.iters; ++it)
    {
        T ln = (-jdvn + bias) * jn;
        T old = sn;
        sn = sn + ln;
        if (sn < T(0))
            sn = T(0);
        dn = sn - old;
        T lt1 = (-jdvt1) * jt1;
        old = st1;
        st1 = st1 + lt1;
        T m1 = K<T>::friction_bound(cf, sn);
        if (st1 < -m1)
            st1 = -m1;
        if (st1 > m1)
            st1 = m1;
        dt1 = st1 - old;
        T lt2 = (-jdvt2) * jt2;
        old = st2;
        st2 = st2 + lt2;
        T m2 = K<T>::friction_bound(cf, sn);
        if (st2 < -m2)
            st2 = -m2;
        if (st2 > m2)
            st2 = m2;
        dt2 = st2 - old;
    }
    c.sn = sn;
    c.st1 = st1;
    c.st2 = st2;
    V3<T> li = mul(dn, n), lt1 = mul(dt1, t1), lt2 = mul(dt2, t2);
    V3<T> ai1 = mul(dn, rn1), ai2 = mul(dn, rn2);
    V3<T> ai1t1 = mul(dt1, r1t1), ai2t1 = mul(dt1, r2t1);
    V3<T> ai1t2 = mul(dt2, r1t2), ai2t2 = mul(dt2, r2t2);
    // three sequential updates per body: normal, tangent 1, tangent 2 (code/nans.cpp:1244-1257)
    A->V = add(A->V, mul(invm1, li));
    if (writes_b) B->V = sub(B->V, mul(invm2, li));
    A->W = add(A->W, mul(invi1, ai1));
    if (writes_b) B->W = sub(B->W, mul(invi2, ai2));
    A->V = add(A->V, mul(invm1, lt1));
    if (writes_b) B->V = sub(B->V, mul(invm2, lt1));
    A->W = add(A->W, mul(invi1, ai1t1));
    if (writes_b) B->W = sub(B->W, mul(invi2, ai2t1));
    A->V = add(A->V, mul(invm1, lt2));
    if (writes_b) B->V = sub(B->V, mul(invm2, lt2));
    A->W = add(A->W, mul(invi1, ai1t2));
    if (writes_b) B->W = sub(B->W, mul(invi2, ai2t2));
}

// With warm starting (the reference's TODO at its pair dedupe, code/nans.cpp:1386-1389) a
// contact whose pair (type, IndexA, IndexB) was in contact at the previous solve starts its
// accumulators from that solve's final values instead of zero.
// SolveConstraints (code/nans.cpp:1538-1548)
template <class T> static void solve(Scene<T> &s, T dt)
{
    for (auto &c : s.pairs)
    {
        c.sn = c.st1 = c.st2 = T(0);
        if (s.warm)
            for (const auto &p : s.prev)
                if (p.type == c.type && p.a == c.a && p.b == c.b)
                {
                    c.sn = p.sn;
                    c.st1 = p.st1;
                    c.st2 = p.st2;
                    break;
                }
        constraint(s, c, dt);
    }
    if (s.warm)
        s.prev = s.pairs;
}

template <class T> static void stage(Scene<T> &s, int st, T dt)
{
    switch (st)
    {
    case 0: integrate_forces(s, dt); break;
    case 1: detect(s); break;
    case 2: solve(s, dt); break;
    case 3: integrate_velocities(s, dt); break;
    case 4: rebuild(s); break;
    }
}

// ---------------------------------------------------------------------------------
// record layouts of the reference (code/nans.h:303-372)
// ---------------------------------------------------------------------------------
struct RCube
{
    float Model[16];
    float Vertices[8][3];
    float Position[3], V[3], Forces[3], Angles[3], W[3], Torque[3];
    float Size, Mass, MOI;
};
struct RSphere
{
    float Model[16];
    float Position[3], V[3], Forces[3], Angles[3], W[3], Torque[3];
    float Radius, Mass, MOI;
};
struct RPair
{
    int32_t Type;
    float DLNormal, DLNormalSum, DLTangent1, DLTangent1Sum, DLTangent2, DLTangent2Sum;
    float PointA[3], PointB[3], N[3], T1[3], T2[3];
    int32_t IndexA, IndexB;
};
static_assert(sizeof(RCube) == 244, "cube layout");
static_assert(sizeof(RSphere) == 148, "sphere layout");
static_assert(sizeof(RPair) == 96, "contact_pair layout");

template <class T> static V3<T> v3(const float *f) { return mk((T)f[0], (T)f[1], (T)f[2]); }
template <class T> static void put(float *o, V3<T> v)
{
    o[0] = (float)v.x;
    o[1] = (float)v.y;
    o[2] = (float)v.z;
}

template <class T> static void load_cube(Body<T> &b, const RCube &r, const float *scl, int npts, const float *pts)
{
    b.P = v3<T>(r.Position);
    b.V = v3<T>(r.V);
    b.F = v3<T>(r.Forces);
    b.A = v3<T>(r.Angles);
    b.W = v3<T>(r.W);
    b.Tq = v3<T>(r.Torque);
    b.mass = (T)r.Mass;
    b.moi = (T)r.MOI;
    b.radius = 0;
    b.scl = scl ? v3<T>(scl) : mk((T)r.Size, (T)r.Size, (T)r.Size);
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 4; ++k)
            b.model.c[j][k] = (T)r.Model[4 * j + k];
    if (pts && npts > 0)
    {
        b.npts = npts;
        b.local.resize(npts);
        for (int k = 0; k < npts; ++k)
            b.local[k] = v3<T>(pts + 3 * k);
    }
    else
    {
        b.npts = 8;
        b.local.resize(8);
        for (int k = 0; k < 8; ++k)
            b.local[k] = v3<T>(kCorner[k]);
    }
    b.verts.resize(b.npts);
    for (int k = 0; k < b.npts; ++k)
        b.verts[k] = (k < 8) ? v3<T>(r.Vertices[k]) : mk(T(0), T(0), T(0));
}

template <class T> static void load_sphere(Body<T> &b, const RSphere &r)
{
    b.P = v3<T>(r.Position);
    b.V = v3<T>(r.V);
    b.F = v3<T>(r.Forces);
    b.A = v3<T>(r.Angles);
    b.W = v3<T>(r.W);
    b.Tq = v3<T>(r.Torque);
    b.mass = (T)r.Mass;
    b.moi = (T)r.MOI;
    b.radius = (T)r.Radius;
    b.npts = 0;
    b.scl = mk(T(1), T(1), T(1));
    b.model = ident<T>();
}

template <class T> static void store_cube(const Body<T> &b, RCube &r, float size)
{
    std::memset(&r, 0, sizeof(r));
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 4; ++k)
            r.Model[4 * j + k] = (float)b.model.c[j][k];
    for (int k = 0; k < 8 && k < (int)b.verts.size(); ++k)
        put(r.Vertices[k], b.verts[k]);
    put(r.Position, b.P);
    put(r.V, b.V);
    put(r.Forces, b.F);
    put(r.Angles, b.A);
    put(r.W, b.W);
    put(r.Torque, b.Tq);
    r.Size = size;
    r.Mass = (float)b.mass;
    r.MOI = (float)b.moi;
}

template <class T> static void store_sphere(const Body<T> &b, RSphere &r)
{
    std::memset(&r, 0, sizeof(r));
    for (int k = 0; k < 16; ++k)
        r.Model[k] = (k % 5 == 0) ? 1.0f : 0.0f;
    put(r.Position, b.P);
    put(r.V, b.V);
    put(r.Forces, b.F);
    put(r.Angles, b.A);
    put(r.W, b.W);
    put(r.Torque, b.Tq);
    r.Radius = (float)b.radius;
    r.Mass = (float)b.mass;
    r.MOI = (float)b.moi;
}

struct World
{
    int fp64;
    std::vector<Scene<float>> sf;
    std::vector<Scene<double>> sd;
    std::vector<std::vector<float>> sizes; // per scene: cube Size fields (kept for store)
    std::vector<float> floor_size;
};

template <class T>
static void run_scenes(std::vector<Scene<T>> &scenes, int st_lo, int st_hi, T dt, int nsteps, int nthreads)
{
    std::atomic<size_t> next(0);
    auto worker = [&]() {
        for (;;)
        {
            size_t i = next.fetch_add(1);
            if (i >= scenes.size())
                break;
            for (int s = 0; s < nsteps; ++s)
                for (int st = st_lo; st <= st_hi; ++st)
                    stage(scenes[i], st, dt);
        }
    };
    int nt = std::max(1, std::min<int>(nthreads, (int)scenes.size()));
    if (nt == 1)
    {
        worker();
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back(worker);
    for (auto &t : th)
        t.join();
}

} // namespace

extern "C" {

void *nanso_create(int fp64)
{
    World *w = new World();
    w->fp64 = fp64 ? 1 : 0;
    return w;
}

void nanso_destroy(void *h) { delete (World *)h; }

int nanso_num_scenes(void *h)
{
    World *w = (World *)h;
    return w->fp64 ? (int)w->sd.size() : (int)w->sf.size();
}

// Adds one scene. cube_scale: ncubes*3 model scales or NULL (Size on every axis).
// hull_npts / hull_pts: per cube local point count and packed points (NULL = unit cube
// corners). rebuild != 0 rebuilds every model from Position/Angles/scale before the first
// step; otherwise the Model fields of the records are used as given.
int nanso_add_scene(void *h, const void *cubes, uint32_t nc, const void *spheres, uint32_t ns,
                    const void *floor, const float *cube_scale, const float *floor_scale,
                    const int32_t *hull_npts, const float *hull_pts, float cr, float cf, int iters,
                    int rebuild_models)
{
    World *w = (World *)h;
    const RCube *rc = (const RCube *)cubes;
    const RSphere *rs = (const RSphere *)spheres;
    const RCube *rf = (const RCube *)floor;
    auto fill = [&](auto &sc) {
        sc.cubes.resize(nc);
        sc.spheres.resize(ns);
        size_t off = 0;
        for (uint32_t i = 0; i < nc; ++i)
        {
            int np = hull_npts ? hull_npts[i] : 0;
            load_cube(sc.cubes[i], rc[i], cube_scale ? cube_scale + 3 * i : nullptr, np,
                      (hull_pts && np > 0) ? hull_pts + 3 * off : nullptr);
            off += (size_t)(np > 0 ? np : 0);
        }
        for (uint32_t i = 0; i < ns; ++i)
            load_sphere(sc.spheres[i], rs[i]);
        float fs3[3] = {rf->Size, 1.0f, rf->Size};
        load_cube(sc.floor, *rf, floor_scale ? floor_scale : fs3, 0, nullptr);
        sc.k = Consts{cr, cf, iters};
        if (rebuild_models)
            rebuild(sc);
    };
    if (w->fp64)
    {
        w->sd.emplace_back();
        fill(w->sd.back());
    }
    else
    {
        w->sf.emplace_back();
        fill(w->sf.back());
    }
    std::vector<float> sz(nc);
    for (uint32_t i = 0; i < nc; ++i)
        sz[i] = rc[i].Size;
    w->sizes.push_back(sz);
    w->floor_size.push_back(rf->Size);
    return (int)w->sizes.size() - 1;
}

// Runs nsteps full steps (stages 0..4) on every scene.
void nanso_step(void *h, float dt, int nsteps, int nthreads)
{
    World *w = (World *)h;
    if (w->fp64)
        run_scenes(w->sd, 0, 4, (double)dt, nsteps, nthreads);
    else
        run_scenes(w->sf, 0, 4, dt, nsteps, nthreads);
}

// Runs a single stage on every scene (0 forces, 1 detect, 2 solve, 3 velocities, 4 rebuild).
void nanso_stage(void *h, int st, float dt, int nthreads)
{
    World *w = (World *)h;
    if (w->fp64)
        run_scenes(w->sd, st, st, (double)dt, 1, nthreads);
    else
        run_scenes(w->sf, st, st, dt, 1, nthreads);
}

// Runs nsteps full steps on scenes [lo, hi) only (used for bounded CPU-baseline samples).
void nanso_step_range(void *h, int lo, int hi, float dt, int nsteps, int nthreads)
{
    World *w = (World *)h;
    if (w->fp64)
    {
        std::vector<Scene<double>> part(w->sd.begin() + lo, w->sd.begin() + hi);
        run_scenes(part, 0, 4, (double)dt, nsteps, nthreads);
        std::copy(part.begin(), part.end(), w->sd.begin() + lo);
    }
    else
    {
        std::vector<Scene<float>> part(w->sf.begin() + lo, w->sf.begin() + hi);
        run_scenes(part, 0, 4, dt, nsteps, nthreads);
        std::copy(part.begin(), part.end(), w->sf.begin() + lo);
    }
}

// Copies a scene's bodies out in the reference record layouts (FP64 runs are rounded).
int nanso_store(void *h, int scene, void *cubes, void *spheres, void *floor)
{
    World *w = (World *)h;
    auto out = [&](auto &sc) {
        for (size_t i = 0; i < sc.cubes.size(); ++i)
            if (cubes)
                store_cube(sc.cubes[i], ((RCube *)cubes)[i], w->sizes[scene][i]);
        for (size_t i = 0; i < sc.spheres.size(); ++i)
            if (spheres)
                store_sphere(sc.spheres[i], ((RSphere *)spheres)[i]);
        if (floor)
            store_cube(sc.floor, *(RCube *)floor, w->floor_size[scene]);
    };
    if (w->fp64)
        out(w->sd[scene]);
    else
        out(w->sf[scene]);
    return 0;
}

// Full-precision body state: per body (cubes then spheres) P, V, A, W as 12 doubles.
int nanso_state_f64(void *h, int scene, double *out)
{
    World *w = (World *)h;
    auto emit = [&](auto &sc) {
        size_t k = 0;
        auto one = [&](auto &b) {
            double v[12] = {(double)b.P.x, (double)b.P.y, (double)b.P.z, (double)b.V.x, (double)b.V.y,
                            (double)b.V.z, (double)b.A.x, (double)b.A.y, (double)b.A.z, (double)b.W.x,
                            (double)b.W.y, (double)b.W.z};
            std::memcpy(out + 12 * k, v, sizeof(v));
            ++k;
        };
        for (auto &b : sc.cubes)
            one(b);
        for (auto &b : sc.spheres)
            one(b);
    };
    if (w->fp64)
        emit(w->sd[scene]);
    else
        emit(w->sf[scene]);
    return 0;
}

// The contact list of the scene's last detect stage, in the reference record layout.
uint32_t nanso_pairs(void *h, int scene, void *outp, uint32_t cap)
{
    World *w = (World *)h;
    auto emit = [&](auto &sc) -> uint32_t {
        uint32_t n = (uint32_t)sc.pairs.size();
        RPair *o = (RPair *)outp;
        for (uint32_t i = 0; o && i < n && i < cap; ++i)
        {
            std::memset(&o[i], 0, sizeof(RPair));
            o[i].Type = sc.pairs[i].type;
            o[i].IndexA = sc.pairs[i].a;
            o[i].IndexB = sc.pairs[i].b;
            put(o[i].PointA, sc.pairs[i].pa);
            put(o[i].PointB, sc.pairs[i].pb);
            put(o[i].N, sc.pairs[i].n);
        }
        return n;
    };
    return w->fp64 ? emit(w->sd[scene]) : emit(w->sf[scene]);
}

// Sets the per-scene solver constants (restitution, friction, iterations).
// Holds the contacts of one scene for its next nsteps steps (see Scene::replay): counts[k]
// contact records (the reference's contact_pair layout) for step k, concatenated in `pairs`,
// with the two bodies' positions at that step's solve in pos_a / pos_b (3 floats per contact).
// nsteps = 0 turns the replay off (GJK/EPA again).
void nanso_set_replay(void *h, int scene, int nsteps, const int32_t *counts, const void *pairs, const float *pos_a,
                      const float *pos_b)
{
    World *w = (World *)h;
    const RPair *rp = (const RPair *)pairs;
    auto fill = [&](auto &sc) {
        using T = decltype(sc.floor.mass);
        sc.replay.assign((size_t)std::max(0, nsteps), {});
        sc.replay_step = 0;
        size_t q = 0;
        for (int k = 0; k < nsteps; ++k)
            for (int i = 0; i < counts[k]; ++i, ++q)
            {
                const RPair &r = rp[q];
                Contact<T> c{};
                c.type = r.Type;
                c.a = r.IndexA;
                c.b = r.IndexB;
                c.pa = v3<T>(r.PointA);
                c.pb = v3<T>(r.PointB);
                c.n = v3<T>(r.N);
                c.sn = c.st1 = c.st2 = T(0);
                c.held = true;
                c.pos_a = v3<T>(pos_a + 3 * q);
                c.pos_b = v3<T>(pos_b + 3 * q);
                sc.replay[k].push_back(c);
            }
    };
    if (w->fp64)
        fill(w->sd[scene]);
    else
        fill(w->sf[scene]);
}

void nanso_set_constants(void *h, int scene, float cr, float cf, int iters)
{
    World *w = (World *)h;
    if (w->fp64)
        w->sd[scene].k = Consts{cr, cf, iters};
    else
        w->sf[scene].k = Consts{cr, cf, iters};
}

// Turns the EPA / GJK statistics on or off (off by default).
void nanso_stats_enable(int on) { g_stats = on != 0; }

// Warm starting for every scene of the world (off by default: the reference's behaviour).
void nanso_set_warm(void *h, int on)
{
    World *w = (World *)h;
    for (auto &s : w->sf)
    {
        s.warm = on != 0;
        s.prev.clear();
    }
    for (auto &s : w->sd)
    {
        s.warm = on != 0;
        s.prev.clear();
    }
}

// EPA size statistics since the last reset: out[0] max faces, [1] max edges,
// [2] max iteration index, [3] EPA calls, [4..7] EPAs whose face list exceeded
// 128, 256, 1024, 4096 faces, [8] of those above 128 with a NaN face 0, [9] EPAs whose
// face list emptied, [10] EPAs above 1024 faces that returned a contact, [11..15] EPAs that
// ended after 1-4, 5-8, 9-16, 17-64, 65 iterations, [16] GJK evolve calls, [17] GJK runs,
// [18..21] EPAs fitting 12 vertices / 20 faces / 12 edges, exceeding each, [22..85] EPAs by
// peak face count (after removal plus new faces), [86..93] GJK runs by evolve calls
// (1, 2, 3-4, 5-8, 9-16, 17-32, 33-64, 65).
void nanso_epa_stats(long long *out, int reset)
{
    out[0] = g_epa_max_faces.load();
    out[1] = g_epa_max_edges.load();
    out[2] = g_epa_max_iters.load();
    out[3] = g_epa_calls.load();
    for (int i = 0; i < 4; ++i)
        out[4 + i] = g_epa_big[i].load();
    out[8] = g_epa_big_nan0.load();
    out[9] = g_epa_stale.load();
    out[10] = g_epa_big_contact.load();
    for (int i = 0; i < 5; ++i)
        out[11 + i] = g_epa_iter_hist[i].load();
    out[16] = g_gjk_iters.load();
    out[17] = g_gjk_calls.load();
    for (int i = 0; i < 4; ++i)
        out[18 + i] = g_epa_tiny_fit[i].load();
    for (int i = 0; i < 64; ++i)
        out[22 + i] = g_epa_hist_faces[i].load();
    for (int i = 0; i < 8; ++i)
        out[86 + i] = g_gjk_hist[i].load();
    if (reset)
    {
        g_epa_big_contact = 0;
        for (int i = 0; i < 5; ++i)
            g_epa_iter_hist[i] = 0;
        g_gjk_iters = 0;
        g_gjk_calls = 0;
        for (int i = 0; i < 4; ++i)
            g_epa_tiny_fit[i] = 0;
        for (int i = 0; i < 64; ++i)
            g_epa_hist_faces[i] = 0;
        for (int i = 0; i < 8; ++i)
            g_gjk_hist[i] = 0;
        g_epa_stale = 0;
        g_epa_big_nan0 = 0;
        for (int i = 0; i < 4; ++i)
            g_epa_big[i] = 0;
        g_epa_max_faces = 0;
        g_epa_max_edges = 0;
        g_epa_max_iters = 0;
        g_epa_calls = 0;
    }
}

// Project sincos, exported so tests can compare it with the device copy.
void nanso_sincosf(const float *x, float *s, float *c, int n)
{
    for (int i = 0; i < n; ++i)
        nans_trig_sincosf(x[i], s + i, c + i);
}

} // extern "C"
