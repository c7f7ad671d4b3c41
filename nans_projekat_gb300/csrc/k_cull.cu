// Conservative AABB pair cull, in the reference's pair enumeration order.
//
// The reference has no broadphase: DetectCollisions runs GJK on every pair of a scene in the
// fixed order CC (i<j), CF, SF, CS, SS (code/nans.cpp:1355-1535) and appends hits in that order.
// Here a scene's pairs are numbered in that order and grouped in 32-pair mask words; a scene's
// words are contiguous and start on a word boundary (scene s owns words [sc_word0[s],
// sc_word0[s+1]); word_scene maps a word back to its scene). Three passes keep the order while
// skipping pairs whose inflated AABBs are disjoint:
//   k_cull_mask   one thread per word: the word's bits, a count per block
//   k_cull_scan   exclusive scan of the block counts -> candidate offsets, total, capacity
//   k_cull_write  each thread writes its word's pairs at its prefix position
// all_pairs != 0 keeps every pair (the reference's exact all-pairs behaviour).
#include "nans_kernels.cuh"

namespace nans
{

// Largest i with row_start(i) = i*n - i*(i+1)/2 <= k, for pairs i < j < n: a single-precision
// first guess corrected exactly in integers.
__device__ __forceinline__ void tri_decode_fast(long long k, long long n, int &i, int &j)
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

// Scene-local pair index k -> (type, i, j), as decode_local with the fast triangle decode.
__device__ __forceinline__ void decode_pair(long long k, int nc, int ns, int &type, int &i, int &j)
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

__device__ __forceinline__ int block_sum(int v, int *sh)
{
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0)
        sh[wid] = v;
    __syncthreads();
    int t = 0;
    for (int q = 0; q < nw; ++q)
        t += sh[q];
    __syncthreads();
    return t;
}

// Exclusive block scan of v; returns the prefix, writes the block total to *total.
__device__ __forceinline__ int block_exclusive_scan(int v, int *sh, int *total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1)
    {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        sh[wid] = x;
    __syncthreads();
    if (wid == 0)
    {
        const int nw = blockDim.x >> 5;
        int t = (lane < nw) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1)
        {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o)
                t += y;
        }
        if (lane < nw)
            sh[lane] = t;
    }
    __syncthreads();
    const int warp_prefix = (wid > 0) ? sh[wid - 1] : 0;
    *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

// Box test of the pairs of one mask word: word wi of scene s covers the scene's pairs
// 32*(wi - sc_word0[s]) onward. Body ids are global (pair_bodies); the box of body a is kept in
// registers while consecutive pairs share it.
__device__ __forceinline__ unsigned word_mask(const DevWorld &w, int wi, int all_pairs)
{
    const int s = w.word_scene[wi];
    const int nc = __ldg(w.sc_nc + s), ns = __ldg(w.sc_ns + s);
    const long long npair = scene_pair_count(nc, ns);
    const long long p0 = (long long)(wi - __ldg(w.sc_word0 + s)) * 32;
    const int cnt = (int)min(32ll, npair - p0);
    int type, i, j;
    decode_pair(p0, nc, ns, type, i, j);
    unsigned mask = 0u;
    int last_a = -1;
    float4 la = make_float4(0.f, 0.f, 0.f, 0.f), ha = la;
    for (int bit = 0; bit < cnt; ++bit)
    {
        int a, b;
        pair_bodies(w, s, type, i, j, a, b);
        if (all_pairs)
            mask |= 1u << bit;
        else
        {
            if (a != last_a)
            {
                la = __ldg(w.box_lo + a);
                ha = __ldg(w.box_hi + a);
                last_a = a;
            }
            const float4 lb = __ldg(w.box_lo + b), hb = __ldg(w.box_hi + b);
            if (la.x <= hb.x && lb.x <= ha.x && la.y <= hb.y && lb.y <= ha.y && la.z <= hb.z && lb.z <= ha.z)
                mask |= 1u << bit;
        }
        advance_local(nc, ns, type, i, j);
    }
    return mask;
}

// One thread per mask word; per block, the number of culled pairs.
__global__ void __launch_bounds__(kCullThreads) k_cull_mask(DevWorld w, int all_pairs)
{
    __shared__ int sh[32];
    const int wi = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned mask = 0u;
    if (wi < w.n_words)
    {
        mask = word_mask(w, wi, all_pairs);
        w.pair_mask[wi] = mask;
    }
    const int total = block_sum(__popc(mask), sh);
    if (threadIdx.x == 0)
        w.block_hits[blockIdx.x] = total;
}

// One block of 1024 threads: exclusive scan of the per-block counts in place; the total and
// the capacity check.
__global__ void __launch_bounds__(1024) k_cull_scan(DevWorld w, int nblocks)
{
    __shared__ int sh[32];
    __shared__ long long carry;
    if (threadIdx.x == 0)
        carry = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += blockDim.x)
    {
        const int i = base + threadIdx.x;
        const int v = (i < nblocks) ? w.block_hits[i] : 0;
        int total;
        const int pre = block_exclusive_scan(v, sh, &total);
        if (i < nblocks)
            w.block_hits[i] = (int)min(carry + pre, (long long)INT32_MAX);
        __syncthreads();
        if (threadIdx.x == 0)
            carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        long long n = carry;
        *w.cull_total = (int)min(n, (long long)INT32_MAX);
        if (n > w.cand_cap)
        {
            atomicOr(w.status, (unsigned)ST_CANDIDATES);
            n = w.cand_cap;
        }
        *w.n_cand = (int)n;
    }
}

// Each thread writes its word's culled pairs at its prefix position (scene-major order).
__global__ void __launch_bounds__(kCullThreads) k_cull_write(DevWorld w)
{
    __shared__ int sh[32];
    const int wi = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned mask = (wi < w.n_words) ? w.pair_mask[wi] : 0u;
    int total;
    int pos = w.block_hits[blockIdx.x] + block_exclusive_scan(__popc(mask), sh, &total);
    if (mask == 0u)
        return;
    const int s = w.word_scene[wi];
    const int nc = __ldg(w.sc_nc + s), ns = __ldg(w.sc_ns + s);
    const long long p0 = (long long)(wi - __ldg(w.sc_word0 + s)) * 32;
    int type, i, j;
    decode_pair(p0, nc, ns, type, i, j);
    const int cap = w.cand_cap;
    for (int bit = 0; bit < 32; ++bit)
    {
        if (mask & (1u << bit))
        {
            if (pos < cap)
            {
                int a, b;
                pair_bodies(w, s, type, i, j, a, b);
                w.cand_a[pos] = a;
                w.cand_b[pos] = b;
                w.cand_meta[pos] = (s << 3) | type;
                if (w.cand_pidx)
                    w.cand_pidx[pos] = wi * 32 + bit;
            }
            ++pos;
        }
        if ((mask >> bit) <= 1u)
            break;
        advance_local(nc, ns, type, i, j);
    }
}


} // namespace nans
