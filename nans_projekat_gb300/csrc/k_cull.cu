// Conservative AABB pair cull, in the reference's pair enumeration order.
//
// The reference has no broadphase: DetectCollisions runs GJK on every pair of a scene in the
// fixed order CC (i<j), CF, SF, CS, SS (code/nans.cpp:1355-1535) and appends hits in that order.
// Here every pair of every scene has an index in one "pair space" (scene-major, then that
// order). Three passes keep the order while skipping pairs whose inflated AABBs are disjoint:
//   k_cull_mask   one bit per pair (32 consecutive pairs per thread), hit count per block
//   k_scan_blocks exclusive scan of the block counts -> candidate offsets and total
//   k_cull_write  each thread writes its set bits' pairs at its prefix position
// all_pairs != 0 keeps every pair (the reference's exact all-pairs behaviour).
#include "nans_kernels.cuh"

namespace nans
{

__device__ __forceinline__ int find_scene(const DevWorld &w, long long p)
{
    // last scene s with sc_pair0[s] <= p (sc_pair0 has n_scenes + 1 entries)
    int lo = 0, hi = w.n_scenes - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(w.sc_pair0 + mid) <= p)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ bool boxes_overlap(const DevWorld &w, int a, int b)
{
    float4 la = __ldg(w.box_lo + a), ha = __ldg(w.box_hi + a);
    float4 lb = __ldg(w.box_lo + b), hb = __ldg(w.box_hi + b);
    return la.x <= hb.x && lb.x <= ha.x && la.y <= hb.y && lb.y <= ha.y && la.z <= hb.z && lb.z <= ha.z;
}

// Walks `count` consecutive pairs starting at global pair index p0, calling fn(bit, scene,
// type, i, j) for each.
template <class Fn> __device__ __forceinline__ void walk_pairs(const DevWorld &w, long long p0, int count, Fn fn)
{
    if (p0 >= w.pair_total)
        return;
    int s = find_scene(w, p0);
    int nc = __ldg(w.sc_nc + s), ns = __ldg(w.sc_ns + s);
    int type, i, j;
    decode_local(p0 - __ldg(w.sc_pair0 + s), nc, ns, type, i, j);
    for (int bit = 0; bit < count; ++bit)
    {
        if (p0 + bit >= w.pair_total)
            break;
        fn(bit, s, type, i, j);
        if (!advance_local(nc, ns, type, i, j))
        {
            // next scene with at least one pair
            do
            {
                ++s;
                if (s >= w.n_scenes)
                    return;
                nc = __ldg(w.sc_nc + s);
                ns = __ldg(w.sc_ns + s);
            } while (!start_region(nc, ns, T_CC, type, i, j));
        }
    }
}

__device__ __forceinline__ int block_reduce_sum(int v, int *sh)
{
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        sh[wid] = v;
    __syncthreads();
    int nw = blockDim.x >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0;
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Exclusive block scan of v; returns the prefix, writes the block total to *total.
__device__ __forceinline__ int block_exclusive_scan(int v, int *sh, int *total)
{
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1)
    {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        sh[wid] = x;
    __syncthreads();
    if (wid == 0)
    {
        int nw = blockDim.x >> 5;
        int t = (lane < nw) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1)
        {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o)
                t += y;
        }
        if (lane < nw)
            sh[lane] = t;
    }
    __syncthreads();
    int warp_prefix = (wid > 0) ? sh[wid - 1] : 0;
    *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

__global__ void __launch_bounds__(kCullThreads) k_cull_mask(DevWorld w, int all_pairs)
{
    __shared__ int sh[32];
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long p0 = t * kPairsPerThread;
    unsigned mask = 0u;
    walk_pairs(w, p0, kPairsPerThread, [&](int bit, int s, int type, int i, int j) {
        int a, b;
        pair_bodies(w, s, type, i, j, a, b);
        if (all_pairs || boxes_overlap(w, a, b))
            mask |= 1u << bit;
    });
    if (p0 < w.pair_total)
        w.pair_mask[t] = mask;
    int total = block_reduce_sum(__popc(mask), sh);
    if (threadIdx.x == 0)
        w.block_hits[blockIdx.x] = total;
}

// One block of 1024 threads: exclusive scan of the per-block hit counts in place.
__global__ void __launch_bounds__(1024) k_scan_blocks(DevWorld w, int nblocks)
{
    __shared__ int sh[32];
    __shared__ int carry;
    if (threadIdx.x == 0)
        carry = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += blockDim.x)
    {
        int i = base + threadIdx.x;
        int v = (i < nblocks) ? w.block_hits[i] : 0;
        int total;
        int pre = block_exclusive_scan(v, sh, &total);
        if (i < nblocks)
            w.block_hits[i] = carry + pre;
        __syncthreads();
        if (threadIdx.x == 0)
            carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        int n = carry;
        if (n > w.cand_cap)
        {
            atomicOr(w.status, (unsigned)ST_CANDIDATES);
            n = w.cand_cap;
        }
        *w.n_cand = n;
    }
}

__global__ void __launch_bounds__(kCullThreads) k_cull_write(DevWorld w)
{
    __shared__ int sh[32];
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long p0 = t * kPairsPerThread;
    unsigned mask = (p0 < w.pair_total) ? w.pair_mask[t] : 0u;
    int total;
    int pre = block_exclusive_scan(__popc(mask), sh, &total);
    if (mask == 0u)
        return;
    int pos = w.block_hits[blockIdx.x] + pre;
    const int cap = w.cand_cap;
    walk_pairs(w, p0, kPairsPerThread, [&](int bit, int s, int type, int i, int j) {
        if (mask & (1u << bit))
        {
            if (pos < cap)
            {
                int a, b;
                pair_bodies(w, s, type, i, j, a, b);
                w.cand_a[pos] = a;
                w.cand_b[pos] = b;
                w.cand_meta[pos] = (s << 3) | type;
            }
            ++pos;
        }
    });
}

} // namespace nans
