// Host-side check of the cull's pair-space decode (nans_pairs.cuh, the same source the cull
// kernels compile): every scene-local index of every scene shape up to 48 cubes x 24 spheres
// against a brute-force walk of the reference's pair order (code/nans.cpp:1355-1535), the
// pair_after shortcut for every start index and every offset of a 32-pair mask word, and the
// triangle decode on row boundaries of large triangles. Prints "ok <counts>" or the first
// mismatch and exits 1.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "nans_pairs.cuh"

using namespace nans;

struct P
{
    int t, i, j;
};

static std::vector<P> walk(int nc, int ns)
{
    std::vector<P> v;
    for (int i = 0; i < nc; ++i)
        for (int j = i + 1; j < nc; ++j)
            v.push_back({T_CC, i, j});
    for (int i = 0; i < nc; ++i)
        v.push_back({T_CF, i, i});
    for (int i = 0; i < ns; ++i)
        v.push_back({T_SF, i, i});
    for (int i = 0; i < nc; ++i)
        for (int j = 0; j < ns; ++j)
            v.push_back({T_CS, i, j});
    for (int i = 0; i < ns; ++i)
        for (int j = i + 1; j < ns; ++j)
            v.push_back({T_SS, i, j});
    return v;
}

static int fail(const char *what, long long a, long long b, long long c, long long d)
{
    std::printf("mismatch %s %lld %lld %lld %lld\n", what, a, b, c, d);
    return 1;
}

int main()
{
    long long decodes = 0, afters = 0, rows = 0;
    for (int nc = 0; nc <= 48; ++nc)
        for (int ns = 0; ns <= 24; ++ns)
        {
            const std::vector<P> v = walk(nc, ns);
            if ((long long)v.size() != scene_pair_count(nc, ns))
                return fail("count", nc, ns, (long long)v.size(), scene_pair_count(nc, ns));
            for (long long k = 0; k < (long long)v.size(); ++k)
            {
                int t, i, j;
                decode_pair(k, nc, ns, t, i, j);
                if (t != v[k].t || i != v[k].i || j != v[k].j)
                    return fail("decode", nc, ns, k, t * 1000000LL + i * 1000 + j);
                ++decodes;
                for (int off = 0; off < 32 && k + off < (long long)v.size(); ++off)
                {
                    int t2, i2, j2;
                    pair_after(k, nc, ns, t, i, j, off, t2, i2, j2);
                    const P &q = v[k + off];
                    if (t2 != q.t || i2 != q.i || j2 != q.j)
                        return fail("after", nc, ns, k, off);
                    ++afters;
                }
            }
        }
    // large triangles: the first and last pair of every row, and the pairs next to them
    const long long ns_big[] = {2, 3, 4096, 4608, 16384, 65536, 131072};
    for (long long n : ns_big)
    {
        for (long long r = 0; r <= n - 2; ++r)
        {
            const long long rs = r * n - r * (r + 1) / 2, len = n - 1 - r;
            const long long ks[4] = {rs, rs + 1, rs + len - 1, rs + len / 2};
            for (long long k : ks)
            {
                if (k < rs || k >= rs + len)
                    continue;
                int i, j;
                tri_decode_fast(k, n, i, j);
                if (i != r || j != r + 1 + (k - rs))
                    return fail("tri", n, k, i, j);
                ++rows;
            }
        }
    }
    std::printf("ok %lld %lld %lld\n", decodes, afters, rows);
    return 0;
}
