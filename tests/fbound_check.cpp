// CPU check of the solver's single-precision friction bound (nans_projekat_gb300/csrc/
// nans_fbound.cuh) against the double computation it replaces, (float)(c2 * (double)s)
// (code/nans.cpp:1199, 1214 with c2 = sqrt(2) * Cf).
//
//   fbound_check            seeded sample: 1,000 values of c2 (the friction coefficients of the
//                           workloads, random coefficients, random doubles, doubles of few
//                           significant bits) x 40,000 values of s (random bit patterns over
//                           the floats, mantissas of few bits, the range edges); then products
//                           built to land on each rounding's half and the carry between them
//   fbound_check all <cf>   every non-negative float s (2^31 bit patterns) for c2 = sqrt(2) cf
//
// Prints "ok <checked> <refused> <refused in range> [<constructed products>]" or the first
// mismatch. Wherever fbound_mul certifies a value it must equal the double computation bit for
// bit. Refusals are counted: all of them, and those of products the certificate covers in
// principle (s a positive normal, c2 in the split's range, a normal result in [2^-98, 2^123)).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "nans_fbound.cuh"

static unsigned f2u(float x)
{
    unsigned u;
    std::memcpy(&u, &x, 4);
    return u;
}
static float u2f(unsigned u)
{
    float x;
    std::memcpy(&x, &u, 4);
    return x;
}
static uint64_t d2u(double x)
{
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
}
static double u2d(uint64_t u)
{
    double x;
    std::memcpy(&x, &u, 8);
    return x;
}

struct Rng
{
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
};

static long long checked = 0, refused = 0, refused_in_range = 0;

static bool check_one(double c2, unsigned sb)
{
    const nans::FBound f = nans::fbound_split(c2);
    const float ref = (float)(c2 * (double)u2f(sb));
    bool cert = false;
    const float got = nans::fbound_mul(f, u2f(sb), &cert);
    ++checked;
    if (cert)
    {
        if (f2u(got) != f2u(ref))
        {
            std::printf("mismatch c2=%a (%016llx) s=%a (%08x): got %08x want %08x\n", c2,
                        (unsigned long long)d2u(c2), (double)u2f(sb), sb, f2u(got), f2u(ref));
            return false;
        }
        return true;
    }
    ++refused;
    const unsigned es = sb >> 23, re = (f2u(ref) >> 23) & 0xffu;
    if (f.ok && es >= 1u && es <= 254u && re >= 29u && re <= 249u)
        ++refused_in_range;
    return true;
}

static double friction_scale(float cf) { return 1.4142135623730951 * (double)cf; }

// Products with chosen low bits. For an odd float mantissa ms, mc = pattern * ms^-1 modulo
// 2^(d1 + 29) makes the exact product's low d1 + 29 bits equal to pattern = R1 | R2 << d1:
// R1 is what the double product drops (d1 = 23 or 24 bits, by the product's size) and R2 the
// low 29 bits of the double product's mantissa before its rounding, which the conversion to
// float drops. Halves, off-by-ones and all-ones in both fields exercise the two ties, the
// double-rounding corner (a first rounding up onto the second half) and the carry out of R2.
static bool check_constructed(Rng &r, long long *hits)
{
    for (unsigned d1 = 23; d1 <= 24; ++d1)
    {
        const uint64_t h1 = 1ull << (d1 - 1);
        const uint64_t r1s[] = {h1, h1 - 1, h1 + 1, 0, (1ull << d1) - 1};
        const uint64_t r2s[] = {(1u << 28) - 1, 1u << 28, (1u << 28) + 1, (1u << 29) - 1, 0, (1u << 28) - 2,
                                (1u << 29) - 2};
        const uint64_t mask = (1ull << (d1 + 29)) - 1;
        for (uint64_t R1 : r1s)
            for (uint64_t R2 : r2s)
                for (int rep = 0; rep < 64; ++rep)
                    for (int tries = 0; tries < 64; ++tries)
                    {
                        const unsigned ms = 0x800001u | ((unsigned)r.next() & 0x7ffffeu); // odd
                        uint64_t inv = ms;                                              // ms^-1 mod 2^64
                        for (int i = 0; i < 6; ++i)
                            inv *= 2 - (uint64_t)ms * inv;
                        uint64_t mc = ((R1 | (R2 << d1)) * inv) & mask;
                        if (d1 == 23)
                            mc |= 1ull << 52;
                        if (!(mc >> 52))
                            continue;
                        const unsigned __int128 P = (unsigned __int128)ms * mc;
                        if ((unsigned)(P >> 76) != d1 - 23u)
                            continue;
                        const uint64_t e = 1023 - 3 + r.next() % 7;
                        const double c2 = u2d((e << 52) | (mc & 0xfffffffffffffull));
                        const unsigned sb = ((127u - 3u + (unsigned)(r.next() % 7)) << 23) | (ms & 0x7fffffu);
                        if (!check_one(c2, sb))
                            return false;
                        ++*hits;
                        break;
                    }
    }
    return true;
}

int main(int argc, char **argv)
{
    if (argc == 3 && std::strcmp(argv[1], "all") == 0)
    {
        const double c2 = friction_scale((float)std::atof(argv[2]));
        for (uint64_t u = 0; u < (1ull << 31); ++u)
            if (!check_one(c2, (unsigned)u))
                return 1;
        std::printf("ok %lld %lld %lld\n", checked, refused, refused_in_range);
        return 0;
    }
    Rng r{20261204};
    std::vector<double> c2s;
    const float cfs[] = {0.5f, 0.3f, 1.0f, 0.1f, 0.7f, 0.25f, 2.0f, 0.05f, 0.9f, 1.5f};
    for (float cf : cfs)
        c2s.push_back(friction_scale(cf));
    while (c2s.size() < 400)
        c2s.push_back(friction_scale((float)((r.next() >> 40) * 0x1p-24 * 4.0)));
    // random normal doubles over a wide exponent range
    while (c2s.size() < 700)
    {
        const uint64_t e = 1023 - 60 + r.next() % 121;
        c2s.push_back(u2d((e << 52) | (r.next() & 0xfffffffffffffull)));
    }
    // doubles with few significant bits (the products' low bits then hit the rounding halves)
    while (c2s.size() < 1000)
    {
        const int k = 1 + (int)(r.next() % 52);
        uint64_t m = (r.next() & 0xfffffffffffffull) & ~((1ull << (52 - k)) - 1ull);
        m |= 1ull << (52 - k); // lowest set bit at 52 - k
        const uint64_t e = 1023 - 4 + r.next() % 9;
        c2s.push_back(u2d((e << 52) | m));
    }
    c2s.push_back(0.0);
    c2s.push_back(-0.5);
    c2s.push_back(INFINITY);
    c2s.push_back(u2d(1)); // subnormal
    for (double c2 : c2s)
    {
        for (int i = 0; i < 20000; ++i)
        {
            const unsigned u = (unsigned)(r.next() % 0x7f800001ull); // +0 .. +inf
            if (!check_one(c2, u))
                return 1;
        }
        for (int i = 0; i < 19000; ++i)
        {
            // mantissas with few significant bits near 1, where products of a few-bit c2 tie
            const int k = (int)(r.next() % 24);
            unsigned m = (unsigned)(r.next() & 0x7fffffu) & ~((1u << k) - 1u);
            const unsigned e = 127 - 20 + (unsigned)(r.next() % 41);
            if (!check_one(c2, (e << 23) | m))
                return 1;
        }
        const unsigned edges[] = {0x00000000u, 0x00000001u, 0x007fffffu, 0x00800000u, 0x00800001u, 0x3f800000u,
                                  0x3f7fffffu, 0x7f7fffffu, 0x7f000000u, 0x7f800000u, 0x7fc00000u, 0x80000000u,
                                  0xbf800000u, 0xff800000u, 0x01000000u, 0x0c000000u, 0x33800000u, 0x4b800000u};
        for (int i = 0; i < 1000; ++i)
            if (!check_one(c2, edges[i % (sizeof(edges) / sizeof(edges[0]))] + (i >= 18 ? (unsigned)(i / 18) : 0u)))
                return 1;
    }
    long long hits = 0;
    if (!check_constructed(r, &hits))
        return 1;
    std::printf("ok %lld %lld %lld %lld\n", checked, refused, refused_in_range, hits);
    return 0;
}
