// Pair space of one scene, numbered in the reference's enumeration order.
//
// DetectCollisions (code/nans.cpp:1355-1535) visits a scene's pairs in the fixed order
//   CC  cube i < cube j            nc(nc-1)/2 pairs, row-major in i
//   CF  cube i with the floor      nc
//   SF  sphere i with the floor    ns
//   CS  cube i with sphere j       nc*ns, row-major in i
//   SS  sphere i < sphere j        ns(ns-1)/2, row-major in i
// and appends contacts in that order, which the solver's result depends on. A pair's
// scene-local index k is its position in this list. These helpers are plain index arithmetic,
// compiled for the device (the cull) and for the host (the exhaustive CPU check of the decode).
#pragma once
#ifdef __CUDACC__
#define NANS_PAIRS_FN __host__ __device__ __forceinline__
#else
#include <math.h>
#define NANS_PAIRS_FN inline
#endif

namespace nans
{

// collision_type values (code/nans.h:73-89)
enum PairType
{
    T_CC = 0,
    T_CS = 1,
    T_CF = 2,
    T_SS = 3,
    T_SF = 4
};

NANS_PAIRS_FN bool type_b_is_floor(int t) { return t == T_CF || t == T_SF; }
NANS_PAIRS_FN bool type_a_is_sphere(int t) { return t == T_SS || t == T_SF; }
NANS_PAIRS_FN bool type_b_is_sphere(int t) { return t == T_CS || t == T_SS; }

NANS_PAIRS_FN long long scene_pair_count(long long nc, long long ns)
{
    return nc * (nc - 1) / 2 + nc + ns + nc * ns + ns * (ns - 1) / 2;
}

// Largest i with row_start(i) = i*n - i*(i+1)/2 <= k, for pairs i < j < n: a single-precision
// first guess from the quadratic's root, corrected exactly in integers (the guess only sets
// how many correction steps run).
NANS_PAIRS_FN void tri_decode_fast(long long k, long long n, int &i, int &j)
{
    const float a = 2.0f * (float)n - 1.0f;
    const float disc = a * a - 8.0f * (float)k;
    long long ii = (long long)floorf((a - sqrtf(disc > 0.0f ? disc : 0.0f)) * 0.5f);
    if (ii < 0)
        ii = 0;
    if (ii > n - 2)
        ii = n - 2;
    while (ii > 0 && ii * n - ii * (ii + 1) / 2 > k)
        --ii;
    while (ii + 1 <= n - 2 && (ii + 1) * n - (ii + 1) * (ii + 2) / 2 <= k)
        ++ii;
    const long long rs = ii * n - ii * (ii + 1) / 2;
    i = (int)ii;
    j = (int)(ii + 1 + (k - rs));
}

// Scene-local pair index k (0 <= k < scene_pair_count(nc, ns)) -> (type, i, j).
NANS_PAIRS_FN void decode_pair(long long k, int nc, int ns, int &type, int &i, int &j)
{
    const long long ncc = (long long)nc * (nc - 1) / 2;
    if (k < ncc)
    {
        type = T_CC;
        tri_decode_fast(k, nc, i, j);
        return;
    }
    k -= ncc;
    if (k < nc)
    {
        type = T_CF;
        i = j = (int)k;
        return;
    }
    k -= nc;
    if (k < ns)
    {
        type = T_SF;
        i = j = (int)k;
        return;
    }
    k -= ns;
    const long long ncs = (long long)nc * ns;
    if (k < ncs)
    {
        type = T_CS;
        i = (int)(k / ns);
        j = (int)(k % ns);
        return;
    }
    k -= ncs;
    type = T_SS;
    tri_decode_fast(k, ns, i, j);
}

// (type, i, j) of the pair `off` places after (type0, i0, j0), the pair at scene-local index
// p0: for cube-cube pairs the same row or the next one directly, otherwise a full decode.
NANS_PAIRS_FN void pair_after(long long p0, int nc, int ns, int type0, int i0, int j0, int off, int &type,
                              int &i, int &j)
{
    if (type0 == T_CC)
    {
        const int r0 = nc - j0; // pairs (i0, j0 .. nc-1)
        if (off < r0)
        {
            type = T_CC;
            i = i0;
            j = j0 + off;
            return;
        }
        if (off - r0 < nc - i0 - 2) // pairs (i0+1, i0+2 .. nc-1)
        {
            type = T_CC;
            i = i0 + 1;
            j = i0 + 2 + (off - r0);
            return;
        }
    }
    decode_pair(p0 + off, nc, ns, type, i, j);
}

} // namespace nans
