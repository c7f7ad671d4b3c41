// Conservative AABB pair cull, in the reference's pair enumeration order.
//
// The reference has no broadphase: DetectCollisions runs GJK on every pair of a scene in the
// fixed order CC (i<j), CF, SF, CS, SS (code/nans.cpp:1355-1535) and appends hits in that order.
// Here a scene's pairs are numbered in that order and grouped in 32-pair mask words; a scene's
// words are contiguous and start on a word boundary (scene s owns words [sc_word0[s],
// sc_word0[s+1]); word_scene maps a word back to its scene). Three passes keep the order while
// skipping pairs whose inflated AABBs are disjoint:
//   k_cull_mask   one warp per word, one lane per pair: the word's bits, a count per block
//   k_cull_scan   exclusive scan of the block counts -> candidate offsets, total, capacity
//   k_cull_write  the pairs of each word at its prefix position, one lane per word
// all_pairs != 0 keeps every pair (the reference's exact all-pairs behaviour).
#include "nans_kernels.cuh" // pair-space decode: nans_pairs.cuh

namespace nans
{

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

// One warp per mask word, one lane per pair (bit = lane): the pairs' second boxes are read
// coalesced and the word is a ballot. Lane q first loads the scene data of word w0 + q and
// decodes its first pair (32 decodes side by side); the warp then walks the 32 words with
// that data broadcast by shuffles. A block covers kCullThreads words, as the scan and the
// write expect. Per block, the number of culled pairs.
__global__ void __launch_bounds__(kCullThreads) k_cull_mask(DevWorld w, int all_pairs)
{
    __shared__ int sh[32];
    const int lane = threadIdx.x & 31;
    const int wo = blockIdx.x * kCullThreads + threadIdx.x;
    const int w0 = wo - lane;
    int s = 0, nc = 0, ns = 0, c0 = 0, t0 = 0, i0 = 0, j0 = 0, cnt = 0;
    long long p0 = 0;
    if (wo < w.n_words)
    {
        s = __ldg(w.word_scene + wo);
        nc = __ldg(w.sc_nc + s);
        ns = __ldg(w.sc_ns + s);
        c0 = __ldg(w.sc_cube0 + s);
        p0 = (long long)(wo - __ldg(w.sc_word0 + s)) * 32;
        cnt = (int)min(32ll, scene_pair_count(nc, ns) - p0);
        decode_pair(p0, nc, ns, t0, i0, j0);
    }
    unsigned keep = 0u; // lane q keeps word w0 + q
    const int nq = min(32, w.n_words - w0);
    for (int q = 0; q < nq; ++q)
    {
        const int qcnt = __shfl_sync(0xffffffffu, cnt, q);
        const int qs = __shfl_sync(0xffffffffu, s, q);
        const int qnc = __shfl_sync(0xffffffffu, nc, q), qns = __shfl_sync(0xffffffffu, ns, q);
        const int qc0 = __shfl_sync(0xffffffffu, c0, q);
        const int qt = __shfl_sync(0xffffffffu, t0, q), qi = __shfl_sync(0xffffffffu, i0, q);
        const int qj = __shfl_sync(0xffffffffu, j0, q);
        const long long qp0 = __shfl_sync(0xffffffffu, p0, q);
        bool hit = false;
        if (lane < qcnt)
        {
            if (all_pairs)
                hit = true;
            else
            {
                int type, i, j, a, b;
                pair_after(qp0, qnc, qns, qt, qi, qj, lane, type, i, j);
                pair_ids(w, qs, qc0, qnc, type, i, j, a, b);
                const float4 la = __ldg(w.box_lo + a), ha = __ldg(w.box_hi + a);
                const float4 lb = __ldg(w.box_lo + b), hb = __ldg(w.box_hi + b);
                hit = la.x <= hb.x && lb.x <= ha.x && la.y <= hb.y && lb.y <= ha.y && la.z <= hb.z && lb.z <= ha.z;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (lane == q)
            keep = m;
    }
    if (wo < w.n_words)
        w.pair_mask[wo] = keep;
    const int total = block_sum(__popc(keep), sh);
    if (threadIdx.x == 0)
        w.block_hits[blockIdx.x] = total;
}

// ---------------------------------------------------------------------------------------
// The culled pair mask by tiles (the default; k_cull_mask serves the all-pairs mode). The mask
// is cleared, then:
//   k_cull_tiles  cube-cube pairs of a scene in 32 x 32 tiles (rows i, columns j > i), one warp
//                 per tile: each lane holds one column's box, the rows' boxes are broadcast by
//                 shuffles, a row's 32 tests are one ballot, and the row's bits are ORed into the
//                 mask at the row's pair indices (row i of the triangle is contiguous in j)
//   k_cull_rest   the other pairs (CF, SF, CS, SS), one warp per task of up to 64 chunks of 32
//                 consecutive pairs of a scene
//   k_cull_count  per block of kCullThreads mask words, the number of culled pairs (the scan and
//                 the write pass use the same blocks as with k_cull_mask)
// The box test and the pair numbering are k_cull_mask's, so the mask is the same bit for bit.
// ---------------------------------------------------------------------------------------

// ORs the row bits m (bit c = pair index base + c of the scene starting at bit wbit0) into the
// mask, from the first set bit on (so that no word before the scene's first is touched).
__device__ __forceinline__ void or_bits(unsigned *mask, long long wbit0, long long base, unsigned m)
{
    if (!m)
        return;
    const int c = __ffs(m) - 1;
    const long long b = wbit0 + base + c;
    m >>= c;
    const long long word = b >> 5;
    const int sh = (int)(b & 31);
    atomicOr(mask + word, m << sh);
    if (sh && (m >> (32 - sh)))
        atomicOr(mask + word + 1, m >> (32 - sh));
}

__global__ void __launch_bounds__(kCullTileThreads) k_cull_tiles(DevWorld w)
{
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < w.n_tiles; t += nwarps)
    {
        const int4 tile = __ldg(w.tiles + t); // scene, row block, column block
        const int s = tile.x, r0 = 32 * tile.y, k0 = 32 * tile.z;
        const int nc = __ldg(w.sc_nc + s), c0 = __ldg(w.sc_cube0 + s);
        const long long wbit0 = (long long)__ldg(w.sc_word0 + s) * 32;
        const int j = k0 + lane, ir = r0 + lane;
        float4 cl = make_float4(0.f, 0.f, 0.f, 0.f), ch = cl, rl = cl, rh = cl;
        if (j < nc)
        {
            cl = __ldg(w.box_lo + c0 + j);
            ch = __ldg(w.box_hi + c0 + j);
        }
        if (ir < nc)
        {
            rl = __ldg(w.box_lo + c0 + ir);
            rh = __ldg(w.box_hi + c0 + ir);
        }
        const int rows = min(32, nc - r0);
        unsigned mine = 0u; // lane r: the bits of row r0 + r
        for (int r = 0; r < rows; ++r)
        {
            const int i = r0 + r;
            const float lx = __shfl_sync(0xffffffffu, rl.x, r), ly = __shfl_sync(0xffffffffu, rl.y, r),
                        lz = __shfl_sync(0xffffffffu, rl.z, r);
            const float hx = __shfl_sync(0xffffffffu, rh.x, r), hy = __shfl_sync(0xffffffffu, rh.y, r),
                        hz = __shfl_sync(0xffffffffu, rh.z, r);
            const bool hit = j < nc && j > i && lx <= ch.x && cl.x <= hx && ly <= ch.y && cl.y <= hy &&
                             lz <= ch.z && cl.z <= hz;
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (lane == r)
                mine = m;
        }
        if (lane < rows && mine)
        {
            const long long i = ir;
            // pair index of (i, k0): row i starts at i*nc - i*(i+1)/2 with column i + 1
            or_bits(w.pair_mask, wbit0, i * nc - i * (i + 1) / 2 + (k0 - i - 1), mine);
        }
    }
}

// The pairs that are not cube-cube, in chunks of 32 consecutive pair indices of one scene: one
// warp per task of at most kRestChunksPerTask chunks (rest_tasks: scene, first chunk, chunks),
// so that a scene of many spheres (millions of cube-sphere pairs) spreads over the grid while a
// small scene is one task.
__global__ void __launch_bounds__(kCullTileThreads) k_cull_rest(DevWorld w)
{
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < w.n_rest_tasks; g += nwarps)
    {
        const int4 task = __ldg(w.rest_tasks + g);
        const int s = task.x;
        const int nc = __ldg(w.sc_nc + s), ns = __ldg(w.sc_ns + s), c0 = __ldg(w.sc_cube0 + s);
        const long long wbit0 = (long long)__ldg(w.sc_word0 + s) * 32;
        const long long np = scene_pair_count(nc, ns);
        const long long ncc = (long long)nc * (nc - 1) / 2;
        for (int q = 0; q < task.z; ++q)
        {
            const long long k0 = ncc + 32LL * (task.y + q);
            const long long k = k0 + lane;
            bool hit = false;
            if (k < np)
            {
                int type, i, j, a, b;
                decode_pair(k, nc, ns, type, i, j);
                pair_ids(w, s, c0, nc, type, i, j, a, b);
                const float4 la = __ldg(w.box_lo + a), ha = __ldg(w.box_hi + a);
                const float4 lb = __ldg(w.box_lo + b), hb = __ldg(w.box_hi + b);
                hit = la.x <= hb.x && lb.x <= ha.x && la.y <= hb.y && lb.y <= ha.y && la.z <= hb.z &&
                      lb.z <= ha.z;
            }
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (lane == 0)
                or_bits(w.pair_mask, wbit0, k0, m);
        }
    }
}

__global__ void __launch_bounds__(kCullThreads) k_cull_count(DevWorld w)
{
    __shared__ int sh[32];
    const int wo = blockIdx.x * kCullThreads + threadIdx.x;
    const unsigned m = (wo < w.n_words) ? w.pair_mask[wo] : 0u;
    const int total = block_sum(__popc(m), sh);
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
        *w.cull_max = max(*w.cull_max, *w.cull_total);
        if (n > w.cand_cap)
        {
            atomicOr(w.status, (unsigned)ST_CANDIDATES);
            n = w.cand_cap;
        }
        *w.n_cand = (int)n;
    }
}

// The culled pairs at their prefix positions (scene-major order). Thread t of the block owns
// word blockIdx.x * kCullThreads + t: its scan position, scene data and first pair, then
// writes the word's pairs in bit order. (A warp walking its non-empty words one lane per pair
// spent ten shuffles a word on words of two or three pairs.)
__global__ void __launch_bounds__(kCullThreads) k_cull_write(DevWorld w)
{
    __shared__ int sh[32];
    const int wo = blockIdx.x * kCullThreads + threadIdx.x;
    const unsigned own = (wo < w.n_words) ? w.pair_mask[wo] : 0u;
    int total;
    const int own_pos = w.block_hits[blockIdx.x] + block_exclusive_scan(__popc(own), sh, &total);
    int s = 0, nc = 0, ns = 0, c0 = 0, t0 = 0, i0 = 0, j0 = 0;
    long long p0 = 0;
    if (own)
    {
        s = __ldg(w.word_scene + wo);
        nc = __ldg(w.sc_nc + s);
        ns = __ldg(w.sc_ns + s);
        c0 = __ldg(w.sc_cube0 + s);
        p0 = (long long)(wo - __ldg(w.sc_word0 + s)) * 32;
        decode_pair(p0, nc, ns, t0, i0, j0);
    }
    const int cap = w.cand_cap;
    // each lane writes its own word's pairs, in bit order, at its prefix position (the warp's 32
    // words' positions are contiguous, so the stores stay within a few lines)
    unsigned m = own;
    int pos = own_pos;
    while (m)
    {
        const int bit = __ffs(m) - 1;
        m &= m - 1u;
        if (pos >= cap)
            break;
        int type, i, j, a, b;
        pair_after(p0, nc, ns, t0, i0, j0, bit, type, i, j);
        pair_ids(w, s, c0, nc, type, i, j, a, b);
        w.cand_a[pos] = a;
        w.cand_b[pos] = b;
        w.cand_meta[pos] = (s << 3) | type;
        if (w.cand_pidx)
            w.cand_pidx[pos] = wo * 32 + bit;
        ++pos;
    }
}

} // namespace nans
