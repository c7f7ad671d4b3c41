// GJK (CheckCollision / EvolveSimplex) and the result write shared by the narrowphase tiers.
#pragma once
#include "nans_kernels.cuh"

namespace nans
{

enum
{
    G_NOHIT = 0,
    G_FOUND = 1,
    G_EVOLVING = 2,
    G_BUDGET = 3 // still evolving after the caller's budget of EvolveSimplex calls
};

// TripleCross (code/nans.cpp:564-569): (A x B) x C = B * dot(C, A) - A * dot(C, B)
__device__ __forceinline__ v3 triple_cross(v3 a, v3 b, v3 c) { return (dot3(c, a) * b) - (dot3(c, b) * a); }

// CheckCollision's GJK loop (at most 65 EvolveSimplex calls) from call `it` with the simplex
// (s0..s3, n points). With budget < 65 it stops before call `budget` and returns G_BUDGET if
// the simplex is still evolving; (simplex, n, it) then resume it exactly.
template <class Support>
__device__ __forceinline__ int gjk_from_with(const Support &support, const Shape &A, const Shape &B, GV &s0, GV &s1,
                                             GV &s2, GV &s3, int &n, int &it, int budget)
{
    const v3 dir0 = normalize3(B.p - A.p);
    int res = G_EVOLVING;
    for (; it <= 64; ++it)
    {
        if (it >= budget)
            return G_BUDGET;
        v3 dir = dir0;
        if (n == 1)
        {
            dir = -1.0f * dir;
        }
        else if (n == 2)
        {
            // ClosestPointOnLine (code/nans.cpp:539-562)
            v3 a = s0.p, b = s1.p;
            v3 l = normalize3(b - a);
            float ln = len3(l);
            float v = dot3(-a, l) / ln;
            float u = dot3(b, l) / ln;
            v3 cp;
            if (u <= 0.0f)
                cp = b;
            else if (v <= 0.0f)
                cp = a;
            else
                cp = (u * a) + (v * b);
            if (v <= 0.0f)
                n = 1;
            else if (u <= 0.0f)
            {
                s0 = s1;
                n = 1;
            }
            dir = -cp;
        }
        else if (n == 3)
        {
            v3 a0 = -s0.p;
            v3 e1 = s1.p - s0.p;
            v3 e2 = s2.p - s0.p;
            v3 tn = cross3(e1, e2);
            v3 e1n = cross3(e1, tn);
            v3 e2n = cross3(tn, e2);
            if (dot3(e2n, a0) > 0.0f)
            {
                if (dot3(e2, a0) > 0.0f)
                {
                    dir = triple_cross(e2, a0, e2);
                    s1 = s2;
                    n = 2;
                }
                else if (dot3(e1, a0) > 0.0f)
                {
                    dir = triple_cross(e1, a0, e1);
                    n = 2;
                }
                else
                {
                    dir = a0;
                    n = 1;
                }
            }
            else if (dot3(e1n, a0) > 0.0f)
            {
                if (dot3(e1, a0) > 0.0f)
                {
                    dir = triple_cross(e1, a0, e1);
                    n = 2;
                }
                else
                {
                    dir = a0;
                    n = 1;
                }
            }
            else if (dot3(tn, a0) > 0.0f)
            {
                dir = tn;
            }
            else
            {
                dir = -tn;
                GV t = s1;
                s1 = s2;
                s2 = t;
            }
        }
        else if (n == 4)
        {
            v3 da = s0.p - s3.p;
            v3 db = s1.p - s3.p;
            v3 dc = s2.p - s3.p;
            v3 d0 = -1.0f * s3.p;
            v3 abd = cross3(da, db);
            v3 bcd = cross3(db, dc);
            v3 cad = cross3(dc, da);
            if (dot3(abd, d0) > 0.0f)
            {
                s2 = s3;
                n = 3;
                dir = abd;
            }
            else if (dot3(bcd, d0) > 0.0f)
            {
                s0 = s1;
                s1 = s2;
                s2 = s3;
                n = 3;
                dir = bcd;
            }
            else if (dot3(cad, d0) > 0.0f)
            {
                s1 = s2;
                s2 = s3;
                n = 3;
                dir = cad;
            }
            else
                return G_FOUND;
        }
        if (len3(dir) <= 0.0001f)
            return G_NOHIT;
        GV nv = support(dir);
        if (n == 0)
            s0 = nv;
        else if (n == 1)
            s1 = nv;
        else if (n == 2)
            s2 = nv;
        else
            s3 = nv;
        ++n;
        res = (dot3(dir, nv.p) >= 0.0f) ? G_EVOLVING : G_NOHIT;
        if (res != G_EVOLVING)
            return res;
    }
    return G_NOHIT; // iteration cap reached while still evolving: no collision
}

// The support of one thread: minkowski_support over the shapes' vertices in global memory.
struct ThreadSupport
{
    const float *verts;
    const Shape &A, &B;
    __device__ __forceinline__ GV operator()(v3 d) const { return minkowski_support(verts, A, B, d); }
};

__device__ __forceinline__ int gjk_from(const float *verts, const Shape &A, const Shape &B, GV &s0, GV &s1, GV &s2,
                                        GV &s3, int &n, int &it, int budget)
{
    return gjk_from_with(ThreadSupport{verts, A, B}, A, B, s0, s1, s2, s3, n, it, budget);
}

__device__ __forceinline__ int gjk(const float *verts, const Shape &A, const Shape &B, GV &s0, GV &s1, GV &s2,
                                   GV &s3, int budget = 65)
{
    int n = 0, it = 0;
    return gjk_from(verts, A, B, s0, s1, s2, s3, n, it, budget);
}

enum
{
    EPA_NONE = 0,
    EPA_CONTACT = 1,
    EPA_OVERFLOW = -1
};

__device__ __forceinline__ void write_result(const DevWorld &w, int cc, int res, v3 pa, v3 pb, v3 nn)
{
    w.hit[cc] = (res == EPA_CONTACT) ? 1 : 0;
    if (res == EPA_CONTACT)
    {
        w.c_pa[cc] = f4(pa, 0.0f);
        w.c_pb[cc] = f4(pb, 0.0f);
        w.c_n[cc] = f4(nn, 0.0f);
    }
}

} // namespace nans
