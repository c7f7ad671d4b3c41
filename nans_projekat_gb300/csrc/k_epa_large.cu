// Tiers 3 and 4 of the narrowphase: EPA on polytopes beyond the warp tier's 256 faces.
//
// ResolveCollision (code/nans.cpp:787-904) with the polytope in global memory, run by a team
// of threads: one block per EPA in tier 3 (arenas of 32,768 faces, two blocks per SM), the
// whole grid per EPA in tier 4 (a cooperative launch; one arena of 8,388,608 faces). Every
// step of an iteration is a parallel pass over the face list or the horizon pushes, so a
// polytope of millions of faces (the reference's EPA can grow geometrically on degenerate
// input) is processed at memory speed by the whole GPU instead of one SM. Each tier resumes
// the polytope the previous tier left at the start of the iteration that outgrew it (the warp
// tier's through a handover buffer, tier 3's in its block arena), so no iteration runs twice.
//
// Per iteration:
//   closest face      argmin of the cached distances, first minimum; a NaN face 0 is chosen
//   support, test     every thread evaluates the same support and the same convergence test
//   remove / push     warp-range passes: each warp owns a contiguous range of faces; a count
//                     pass and a team-wide prefix give every visible face its rank (its three
//                     edges are pushed at 3*rank) and every other face its slot in the other
//                     face bank (stable compaction into a double buffer)
//   horizon           PushEdge (code/nans.cpp:232-266) cancels the FIRST stored edge that is
//                     the reverse of the pushed one (vertex equality compares P) and otherwise
//                     appends. Group pushes by their undirected key {P(u), P(v)}: a push only
//                     cancels an edge of its own group and a group's live edges always run in
//                     one direction, so the survivors of a group are its last |#(u,v) - #(v,u)|
//                     pushes of the majority direction; a self-loop key (P(u) == P(v)) keeps
//                     its last push iff the group has an odd number of pushes; an edge with a
//                     NaN coordinate equals nothing and survives. The key is the pair of
//                     canonical vertex ids (the first pool vertex with an equal position; the
//                     pool holds at most 72 vertices), so groups index a 2,628-entry table.
//                     Survival is decided in parallel from each group's counts and last push
//                     index; only a group that keeps more than one but not all of its majority
//                     pushes needs push order, and those pushes get an ordered reverse pass.
//                     Survivors keep push order (a warp-range compaction).
//   new faces         appended after the kept faces, in horizon order (PushTriangle).
#include <algorithm>

#include "nans_gjk.cuh"

namespace nans
{

constexpr int kGroupSlots = kEpaMaxVerts * (kEpaMaxVerts + 1) / 2;
constexpr int kGroupSlotsPad = (kGroupSlots + 31) & ~31;
constexpr int kLargeThreads = 256;
constexpr int kGiantMaxWarps = 4096;

enum
{
    EPA_ABORT = -2 // a grid barrier timed out; every block leaves the kernel
};

template <int F, int E, int WMAX> struct PolyArena
{
    static constexpr int kFaces = F, kPushes = 3 * F, kEdges = E, kMaxWarps = WMAX;
    float px[kEpaMaxVerts], py[kEpaMaxVerts], pz[kEpaMaxVerts];
    float ax[kEpaMaxVerts], ay[kEpaMaxVerts], az[kEpaMaxVerts];
    float bx[kEpaMaxVerts], by[kEpaMaxVerts], bz[kEpaMaxVerts];
    int vid[kEpaMaxVerts];                   // canonical vertex id, -1 for a NaN coordinate
    float fnx[2][F], fny[2][F], fnz[2][F], fd[2][F];
    unsigned fidx[2][F];                     // a | b << 8 | c << 16
    unsigned short push[3 * F];              // u | v << 8
    unsigned short pgroup[3 * F];            // group slot, 0xffff for a NaN edge
    unsigned char pdir[3 * F];               // 0 / 1 orientation, 2 self-loop
    unsigned char palive[3 * F];             // 0 / 1, 2 = decided by the ordered pass
    unsigned short edge[E];                  // horizon: u | v << 8
    int hcnt[kGroupSlotsPad * WMAX];         // ordered pass: per group and warp, pushes after
};
using BlockArena = PolyArena<kBlockFaces, kBlockEdges, kLargeThreads / 32>;
using GiantArena = PolyArena<kGiantFaces, kGiantEdges, kGiantMaxWarps>;

struct GroupTable
{
    int cnt0[kGroupSlots], cnt1[kGroupSlots];   // pushes per orientation (self-loops in cnt0)
    int last0[kGroupSlots], last1[kGroupSlots]; // last push index per orientation, -1 if none
    int quota[kGroupSlots];                     // survivors left, for the ordered pass
};

struct GridBarrier
{
    unsigned arrive, gen, err, pad;
};

// Team-wide scratch of tier 4 (global memory; tier 3 keeps the same in shared memory).
struct GiantScratch
{
    GroupTable table;
    float af[kGiantMaxWarps];
    int ai[kGiantMaxWarps], c1[kGiantMaxWarps], c2[kGiantMaxWarps];
    int flag;
    GridBarrier bar;
};

// One block.
struct BlockTeam
{
    float *af;
    int *ai, *c1, *c2, *flag;
    __device__ int rank() const { return threadIdx.x; }
    __device__ int size() const { return blockDim.x; }
    __device__ int warp() const { return threadIdx.x >> 5; }
    __device__ int warps() const { return blockDim.x >> 5; }
    __device__ bool sync() const
    {
        __syncthreads();
        return true;
    }
};

// The whole grid of a cooperative launch. The barrier's waits are bounded: past the limit
// the barrier records an error and every later sync fails, so every block leaves.
struct GridTeam
{
    float *af;
    int *ai, *c1, *c2, *flag;
    GridBarrier *bar;
    long long spins;   // polls before a wait gives up
    unsigned extra;    // arrivals beyond the grid's blocks a barrier waits for (0)
    __device__ int rank() const { return blockIdx.x * blockDim.x + threadIdx.x; }
    __device__ int size() const { return gridDim.x * blockDim.x; }
    __device__ int warp() const { return rank() >> 5; }
    __device__ int warps() const { return size() >> 5; }
    __device__ bool sync() const
    {
        __shared__ int s_ok;
        __syncthreads();
        if (threadIdx.x == 0)
        {
            int ok = 1;
            volatile unsigned *vgen = &bar->gen;
            volatile unsigned *verr = &bar->err;
            if (*verr)
                ok = 0;
            else
            {
                const unsigned g = atomicAdd(&bar->gen, 0u);
                __threadfence();
                if (atomicAdd(&bar->arrive, 1u) == gridDim.x - 1 + extra)
                {
                    atomicExch(&bar->arrive, 0u);
                    __threadfence();
                    atomicAdd(&bar->gen, 1u);
                }
                else
                {
                    long long spins = 0;
                    while (*vgen == g)
                    {
                        if (*verr || ++spins > this->spins)
                        {
                            atomicExch(&bar->err, 1u);
                            ok = 0;
                            break;
                        }
                        __nanosleep(64);
                    }
                }
                __threadfence();
            }
            s_ok = ok;
        }
        __syncthreads();
        return s_ok != 0;
    }
};

template <class A> __device__ __forceinline__ v3 lpool(const A &E, int i) { return mk3(E.px[i], E.py[i], E.pz[i]); }

// Vertex i of the pool and its canonical id (first vertex with an equal position).
template <class A> __device__ __forceinline__ void lpool_put(A &E, int i, const GV &g)
{
    E.px[i] = g.p.x;
    E.py[i] = g.p.y;
    E.pz[i] = g.p.z;
    E.ax[i] = g.sa.x;
    E.ay[i] = g.sa.y;
    E.az[i] = g.sa.z;
    E.bx[i] = g.sb.x;
    E.by[i] = g.sb.y;
    E.bz[i] = g.sb.z;
    int id = i;
    if (isnan(g.p.x) || isnan(g.p.y) || isnan(g.p.z))
        id = -1;
    else
        for (int j = 0; j < i; ++j)
            if (eq3(lpool(E, j), g.p))
            {
                id = j;
                break;
            }
    E.vid[i] = id;
}

// PushTriangle (code/nans.cpp:292-322) into bank k, with the face distance cached.
template <class A> __device__ __forceinline__ void lface_put(A &E, int k, int f, int a, int b, int c)
{
    v3 pa = lpool(E, a), pb = lpool(E, b), pc = lpool(E, c);
    v3 n = normalize3(cross3(pb - pa, pc - pa));
    if (dot3(pa, n) < 0.0f)
        n = -1.0f * n;
    E.fidx[k][f] = (unsigned)a | ((unsigned)b << 8) | ((unsigned)c << 16);
    E.fnx[k][f] = n.x;
    E.fny[k][f] = n.y;
    E.fnz[k][f] = n.z;
    E.fd[k][f] = fabsf(dot3(n, pa));
}

template <class A> __device__ __forceinline__ bool lvisible(const A &E, int k, int f, v3 p)
{
    v3 fa = lpool(E, E.fidx[k][f] & 0xffu);
    return dot3(mk3(E.fnx[k][f], E.fny[k][f], E.fnz[k][f]), p - fa) > 0.0f;
}

__device__ __forceinline__ void argmin_step(float &bd, int &bi, float od, int oi)
{
    if (od < bd || (od == bd && oi < bi))
    {
        bd = od;
        bi = oi;
    }
}

__device__ __forceinline__ void warp_argmin(float &bd, int &bi)
{
    for (int o = 16; o > 0; o >>= 1)
        argmin_step(bd, bi, __shfl_xor_sync(0xffffffffu, bd, o), __shfl_xor_sync(0xffffffffu, bi, o));
}

__device__ __forceinline__ int warp_sum(int v)
{
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Exclusive prefix over the team's warps of a per-warp count (lane 0's value is used), and
// the total; scratch holds one int per warp. Every lane receives both.
template <class T> __device__ __forceinline__ bool team_prefix(const T &team, int *scratch, int v, int &before,
                                                              int &total)
{
    const int lane = threadIdx.x & 31, gw = team.warp(), W = team.warps();
    if (lane == 0)
        scratch[gw] = v;
    if (!team.sync())
        return false;
    int b = 0, t = 0;
    for (int q = lane; q < W; q += 32)
    {
        int x = scratch[q];
        t += x;
        if (q < gw)
            b += x;
    }
    before = warp_sum(b);
    total = warp_sum(t);
    return true;
}

// Resumable EPA state at the start of an iteration: (unused, it | bank << 8 | stale << 9,
// face count, vertex count); the faces are those of the bank, the vertices the pool's first.
__device__ __forceinline__ int4 epa_state(int it, int cb, bool stale, int nf, int nv)
{
    return make_int4(0, it | (cb << 8) | ((stale ? 1 : 0) << 9), nf, nv);
}

// ResolveCollision on a team's polytope, from the GJK simplex, or (resume != null) from an
// iteration's starting state already in the arena. On EPA_OVERFLOW, *ovf (rank 0 writes it)
// holds the state at the start of the iteration that overflowed, which the next tier resumes.
template <class T, class A>
__device__ int epa_large(const DevWorld &w, const T &team, A &E, GroupTable &G, int face_limit, const Shape &SA,
                         const Shape &SB, const GV &s0, const GV &s1, const GV &s2, const GV &s3, v3 &out_pa,
                         v3 &out_pb, v3 &out_n, const int4 *resume = nullptr, int4 *ovf = nullptr)
{
    const int r = team.rank(), nt = team.size(), lane = threadIdx.x & 31, gw = team.warp(), W = team.warps();
    const unsigned full = 0xffffffffu;
    if (r == 0 && !resume)
    {
        lpool_put(E, 0, s0);
        lpool_put(E, 1, s1);
        lpool_put(E, 2, s2);
        lpool_put(E, 3, s3);
    }
    for (int i = r; i < kGroupSlots; i += nt)
    {
        G.cnt0[i] = 0;
        G.cnt1[i] = 0;
        G.last0[i] = -1;
        G.last1[i] = -1;
        G.quota[i] = 0;
    }
    if (!team.sync())
        return EPA_ABORT;
    int nf = 4, nv = 4, cb = 0, it0 = 0;
    bool stale = false;
    if (resume)
    {
        it0 = resume->y & 0xff;
        cb = (resume->y >> 8) & 1;
        stale = ((resume->y >> 9) & 1) != 0;
        nf = resume->z;
        nv = resume->w;
    }
    else
    {
        if (r == 0)
            lface_put(E, 0, 0, 0, 1, 2);
        else if (r == 1)
            lface_put(E, 0, 1, 0, 2, 3);
        else if (r == 2)
            lface_put(E, 0, 2, 0, 3, 1);
        else if (r == 3)
            lface_put(E, 0, 3, 1, 3, 2);
        if (!team.sync())
            return EPA_ABORT;
    }
    for (int it = it0; it <= 64; ++it)
    {
        if (nf == 0 && !stale)
            return EPA_NONE;
        // closest face (first minimum; a NaN face 0 stays the closest)
        int ci = 0;
        const float d0 = E.fd[cb][0];
        if (nf > 0 && !isnan(d0))
        {
            float bd = d0;
            int bi = 0;
            for (int f = r; f < nf; f += nt)
                argmin_step(bd, bi, E.fd[cb][f], f);
            warp_argmin(bd, bi);
            if (lane == 0)
            {
                team.af[gw] = bd;
                team.ai[gw] = bi;
            }
            if (!team.sync())
                return EPA_ABORT;
            bd = d0;
            bi = 0;
            for (int q = lane; q < W; q += 32)
                argmin_step(bd, bi, team.af[q], team.ai[q]);
            warp_argmin(bd, bi);
            ci = bi;
        }
        const float cur = E.fd[cb][ci];
        const v3 n = mk3(E.fnx[cb][ci], E.fny[cb][ci], E.fnz[cb][ci]);
        const GV ns = minkowski_support(w.verts, SA, SB, n);
        if (dot3(n, ns.p) - cur < 0.001f)
        {
            unsigned fi = E.fidx[cb][ci];
            int ia = fi & 0xffu, ib = (fi >> 8) & 0xffu, ic = fi >> 16;
            v3 pa = lpool(E, ia), pb = lpool(E, ib), pc = lpool(E, ic);
            v3 p = cur * n;
            v3 v0 = pb - pa, v1 = pc - pa, v2 = p - pa;
            float d00 = dot3(v0, v0), d01 = dot3(v0, v1), d11 = dot3(v1, v1);
            float d20 = dot3(v2, v0), d21 = dot3(v2, v1);
            float den = d00 * d11 - d01 * d01;
            float bv = (d11 * d20 - d01 * d21) / den;
            float bw = (d00 * d21 - d01 * d20) / den;
            float bu = 1.0f - bv - bw;
            if (fabsf(bu) > 1.0f || fabsf(bv) > 1.0f || fabsf(bw) > 1.0f)
                return EPA_NONE;
            if (!isfinite(bu) || !isfinite(bv) || !isfinite(bw))
                return EPA_NONE;
            v3 saa = mk3(E.ax[ia], E.ay[ia], E.az[ia]), sab = mk3(E.ax[ib], E.ay[ib], E.az[ib]),
               sac = mk3(E.ax[ic], E.ay[ic], E.az[ic]);
            v3 sba = mk3(E.bx[ia], E.by[ia], E.bz[ia]), sbb = mk3(E.bx[ib], E.by[ib], E.bz[ib]),
               sbc = mk3(E.bx[ic], E.by[ic], E.bz[ic]);
            out_pa = ((bu * saa) + (bv * sab)) + (bw * sac);
            out_n = -1.0f * n;
            out_pb = ((bu * sba) + (bv * sbb)) + (bw * sbc);
            return EPA_CONTACT;
        }
        if (nf == 0)
            return EPA_NONE; // the stale read repeats identically until the iteration cap
        const int nb = cb ^ 1;
        // visible faces: count per warp range, then ranks
        const int nch = (nf + 31) >> 5, cpw = (nch + W - 1) / W;
        const int c_lo = min(nch, gw * cpw), c_hi = min(nch, c_lo + cpw);
        int wvis = 0;
        for (int ch = c_lo; ch < c_hi; ++ch)
        {
            const int f = ch * 32 + lane;
            wvis += __popc(__ballot_sync(full, f < nf && lvisible(E, cb, f, ns.p)));
        }
        int vis_before = 0, nvis = 0;
        if (!team_prefix(team, team.c1, wvis, vis_before, nvis))
            return EPA_ABORT;
        if (nvis == 0)
            return EPA_NONE; // nothing changes: every later iteration repeats this one
        const int m = 3 * nvis;
        // pushes of the visible faces (edges AB, BC, CA at 3*rank), the other faces to the
        // other bank in order
        {
            int vr = vis_before, kr = c_lo * 32 - vis_before;
            const unsigned below = (1u << lane) - 1u;
            for (int ch = c_lo; ch < c_hi; ++ch)
            {
                const int f = ch * 32 + lane;
                const bool in = f < nf;
                const bool vis = in && lvisible(E, cb, f, ns.p);
                const unsigned bv = __ballot_sync(full, vis), bi = __ballot_sync(full, in);
                const unsigned bk = bi & ~bv;
                if (vis)
                {
                    const int q = vr + __popc(bv & below);
                    const unsigned fi = E.fidx[cb][f];
                    const unsigned a = fi & 0xffu, b = (fi >> 8) & 0xffu, c = fi >> 16;
                    E.push[3 * q] = (unsigned short)(a | (b << 8));
                    E.push[3 * q + 1] = (unsigned short)(b | (c << 8));
                    E.push[3 * q + 2] = (unsigned short)(c | (a << 8));
                }
                else if (in)
                {
                    const int q = kr + __popc(bk & below);
                    E.fidx[nb][q] = E.fidx[cb][f];
                    E.fnx[nb][q] = E.fnx[cb][f];
                    E.fny[nb][q] = E.fny[cb][f];
                    E.fnz[nb][q] = E.fnz[cb][f];
                    E.fd[nb][q] = E.fd[cb][f];
                }
                vr += __popc(bv);
                kr += __popc(bk);
            }
        }
        const int keep = nf - nvis;
        if (r == 0)
            *team.flag = 0;
        if (!team.sync())
            return EPA_ABORT;
        // group counts and last push per orientation
        for (int k = r; k < m; k += nt)
        {
            const unsigned pk = E.push[k];
            const int cu = E.vid[pk & 0xffu], cv = E.vid[pk >> 8];
            if (cu < 0 || cv < 0)
            {
                E.pgroup[k] = 0xffffu;
                continue;
            }
            const int lo = min(cu, cv), hi = max(cu, cv);
            const int g = hi * (hi + 1) / 2 + lo;
            const int dir = (cu < cv) ? 0 : (cu > cv ? 1 : 2);
            E.pgroup[k] = (unsigned short)g;
            E.pdir[k] = (unsigned char)dir;
            if (dir == 1)
            {
                atomicAdd(&G.cnt1[g], 1);
                atomicMax(&G.last1[g], k);
            }
            else
            {
                atomicAdd(&G.cnt0[g], 1);
                atomicMax(&G.last0[g], k);
            }
        }
        if (!team.sync())
            return EPA_ABORT;
        // survivors
        {
            bool hard = false;
            for (int k = r; k < m; k += nt)
            {
                const int g = E.pgroup[k];
                int alive = 1;
                if (g != 0xffff)
                {
                    const int dir = E.pdir[k], c0 = G.cnt0[g], c1 = G.cnt1[g];
                    if (dir == 2)
                        alive = ((c0 & 1) && k == G.last0[g]) ? 1 : 0;
                    else
                    {
                        const int d = c0 - c1, md = d >= 0 ? 0 : 1, q = d >= 0 ? d : -d;
                        if (dir != md || q == 0)
                            alive = 0;
                        else if (q == (md == 0 ? c0 : c1))
                            alive = 1;
                        else if (q == 1)
                            alive = (k == (md == 0 ? G.last0[g] : G.last1[g])) ? 1 : 0;
                        else
                        {
                            alive = 2;
                            G.quota[g] = q;
                            hard = true;
                        }
                    }
                }
                E.palive[k] = (unsigned char)alive;
            }
            if (__any_sync(full, hard) && lane == 0)
                atomicExch(team.flag, 1);
        }
        if (!team.sync())
            return EPA_ABORT;
        if (*(volatile int *)team.flag)
        {
            // Groups that keep some but not all of their majority pushes (quota >= 2): a push
            // survives iff fewer than `quota` pushes of its group come after it. Each warp
            // counts its range's pushes per group, a suffix sum over warps gives every warp the
            // count after its range, and each warp then walks its range backwards.
            const int mch2 = (m + 31) >> 5, mpw2 = (mch2 + W - 1) / W;
            const int h_lo = min(mch2, gw * mpw2), h_hi = min(mch2, h_lo + mpw2);
            for (int i = r; i < kGroupSlots * W; i += nt)
                E.hcnt[i] = 0;
            if (!team.sync())
                return EPA_ABORT;
            for (int ch = h_lo; ch < h_hi; ++ch)
            {
                const int k = ch * 32 + lane;
                const bool cand = k < m && E.palive[k] == 2;
                const int g = cand ? (int)E.pgroup[k] : -1;
                const unsigned peers = __match_any_sync(full, cand ? g : -1 - lane);
                if (cand && lane == 31 - __clz(peers))
                    E.hcnt[g * W + gw] += __popc(peers);
                __syncwarp();
            }
            if (!team.sync())
                return EPA_ABORT;
            for (int g = gw; g < kGroupSlots; g += W)
            {
                if (G.quota[g] < 2)
                    continue;
                int carry = 0; // pushes in warps after the current chunk of warps
                for (int base = ((W - 1) >> 5) << 5; base >= 0; base -= 32)
                {
                    const int q = base + lane;
                    const int v = q < W ? E.hcnt[g * W + q] : 0;
                    int x = v; // inclusive suffix sum within the chunk
                    for (int o = 1; o < 32; o <<= 1)
                    {
                        const int y = __shfl_down_sync(full, x, o);
                        if (lane + o < 32)
                            x += y;
                    }
                    if (q < W)
                        E.hcnt[g * W + q] = carry + x - v;
                    carry += __shfl_sync(full, x, 0);
                }
            }
            if (!team.sync())
                return EPA_ABORT;
            for (int ch = h_hi - 1; ch >= h_lo; --ch)
            {
                const int k = ch * 32 + lane;
                const bool cand = k < m && E.palive[k] == 2;
                const int g = cand ? (int)E.pgroup[k] : -1;
                const unsigned peers = __match_any_sync(full, cand ? g : -1 - lane);
                if (cand)
                {
                    const int later = __popc(peers & ~((2u << lane) - 1u));
                    const int leader = 31 - __clz(peers);
                    int after = 0;
                    if (lane == leader)
                    {
                        after = E.hcnt[g * W + gw];
                        E.hcnt[g * W + gw] = after + __popc(peers);
                    }
                    after = __shfl_sync(peers, after, leader);
                    E.palive[k] = (unsigned char)((after + later) < G.quota[g] ? 1 : 0);
                }
                __syncwarp();
            }
            if (!team.sync())
                return EPA_ABORT;
        }
        // clear the group table for the next iteration
        for (int i = r; i < kGroupSlots; i += nt)
        {
            G.cnt0[i] = 0;
            G.cnt1[i] = 0;
            G.last0[i] = -1;
            G.last1[i] = -1;
            G.quota[i] = 0;
        }
        // horizon = surviving pushes in push order
        const int mch = (m + 31) >> 5, mpw = (mch + W - 1) / W;
        const int m_lo = min(mch, gw * mpw), m_hi = min(mch, m_lo + mpw);
        int wal = 0;
        for (int ch = m_lo; ch < m_hi; ++ch)
        {
            const int k = ch * 32 + lane;
            wal += __popc(__ballot_sync(full, k < m && E.palive[k] == 1));
        }
        int al_before = 0, ne = 0;
        if (!team_prefix(team, team.c2, wal, al_before, ne))
            return EPA_ABORT;
        if (ne > A::kEdges)
        {
            if (ovf && r == 0)
                *ovf = epa_state(it, cb, stale, nf, nv);
            return EPA_OVERFLOW;
        }
        {
            int er = al_before;
            const unsigned below = (1u << lane) - 1u;
            for (int ch = m_lo; ch < m_hi; ++ch)
            {
                const int k = ch * 32 + lane;
                const bool al = k < m && E.palive[k] == 1;
                const unsigned ba = __ballot_sync(full, al);
                if (al)
                    E.edge[er + __popc(ba & below)] = E.push[k];
                er += __popc(ba);
            }
        }
        if (r == 0)
        {
            atomicMax(w.epa_stats + 0, (unsigned)(keep + ne));
            atomicMax(w.epa_stats + 1, (unsigned)ne);
        }
        if (keep + ne > face_limit)
        {
            if (ovf && r == 0)
                *ovf = epa_state(it, cb, stale, nf, nv);
            return EPA_OVERFLOW;
        }
        const int sv = nv++;
        if (r == 0)
        {
            if (keep == 0 && ne == 0)
            {
                // every face removed: slot 0 keeps the last face of the list
                const int l = nf - 1;
                E.fidx[nb][0] = E.fidx[cb][l];
                E.fnx[nb][0] = E.fnx[cb][l];
                E.fny[nb][0] = E.fny[cb][l];
                E.fnz[nb][0] = E.fnz[cb][l];
                E.fd[nb][0] = E.fd[cb][l];
            }
            lpool_put(E, sv, ns);
        }
        if (keep == 0 && ne == 0)
            stale = true;
        if (!team.sync())
            return EPA_ABORT;
        for (int j = r; j < ne; j += nt)
        {
            const unsigned ed = E.edge[j];
            lface_put(E, nb, keep + j, sv, ed & 0xffu, ed >> 8);
        }
        if (!team.sync())
            return EPA_ABORT;
        cb = nb;
        nf = keep + ne;
    }
    return EPA_NONE;
}

// Beyond the giant arena the pair gets no contact, which is what the reference returns for
// every EPA that does not converge within its 65 iterations.
__device__ __forceinline__ void epa_beyond_capacity(const DevWorld &w, int cc)
{
    atomicOr(w.status, (unsigned)ST_EPA_FACES);
    atomicAdd(w.epa_stats + 5, 1u);
    w.epa_stats[3] = (unsigned)cc + 1u;
    w.epa_stats[4] = (unsigned)(w.cand_meta[cc] >> 3) + 1u;
}

// Tier 3: one block per queued candidate. An EPA that outgrows the block arena is queued for
// tier 4 with the state of its last iteration, which stays in this block's arena (the block
// takes no further candidate) for tier 4 to resume. Dynamic shared memory: the group table.
__global__ void __launch_bounds__(kLargeThreads) k_epa_block(DevWorld w)
{
    extern __shared__ unsigned char s_dyn[];
    GroupTable &G = *reinterpret_cast<GroupTable *>(s_dyn);
    __shared__ float s_af[32];
    __shared__ int s_ai[32], s_c1[32], s_c2[32], s_flag, s_q, s_stop;
    __shared__ int4 s_ovf;
    const BlockTeam team{s_af, s_ai, s_c1, s_c2, &s_flag};
    BlockArena &E = *reinterpret_cast<BlockArena *>(w.blk_arena + (size_t)blockIdx.x * sizeof(BlockArena));
    const int n = min(w.work_counter[3], w.ovf_cap);
    for (;;)
    {
        if (threadIdx.x == 0)
            s_q = atomicAdd(w.work_counter + 2, 1);
        __syncthreads();
        const int q = s_q;
        __syncthreads();
        if (q >= n)
            break;
        const int cc = w.ovf_cand[q];
        const Shape A = load_shape(w, w.cand_a[cc]), B = load_shape(w, w.cand_b[cc]);
        GV s0 = {}, s1 = {}, s2 = {}, s3 = {};
        int4 resume = make_int4(0, 0, -1, 0);
        if (q < kHandoverSlots && w.handover[q].hdr[2] >= 0)
        {
            // the warp tier's polytope at the start of the iteration that outgrew it (bank 0)
            const EpaHandover &H = w.handover[q];
            const int nf = H.hdr[2], nv = H.hdr[3];
            for (int i = threadIdx.x; i < nv; i += blockDim.x)
            {
                E.px[i] = H.px[i];
                E.py[i] = H.py[i];
                E.pz[i] = H.pz[i];
                E.ax[i] = H.ax[i];
                E.ay[i] = H.ay[i];
                E.az[i] = H.az[i];
                E.bx[i] = H.bx[i];
                E.by[i] = H.by[i];
                E.bz[i] = H.bz[i];
                E.vid[i] = H.vid[i];
            }
            for (int f = threadIdx.x; f < nf; f += blockDim.x)
            {
                E.fidx[0][f] = H.fidx[f];
                E.fnx[0][f] = H.fnx[f];
                E.fny[0][f] = H.fny[f];
                E.fnz[0][f] = H.fnz[f];
                E.fd[0][f] = H.fd[f];
            }
            resume = epa_state(H.hdr[0], 0, H.hdr[1] != 0, nf, nv);
        }
        else
            gjk(w.verts, A, B, s0, s1, s2, s3); // every thread: same inputs, same simplex
        v3 pa, pb, nn;
        int r = epa_large(w, team, E, G, min(w.blk_face_limit, BlockArena::kFaces), A, B, s0, s1, s2, s3, pa, pb,
                          nn, resume.z >= 0 ? &resume : nullptr, &s_ovf);
        __syncthreads();
        if (threadIdx.x == 0)
        {
            s_stop = 0;
            atomicAdd(w.epa_stats + 2, 1u);
            bool done = true;
            if (r == EPA_OVERFLOW)
            {
                int g = atomicAdd(w.work_counter + 8, 1);
                if (g < w.giant_cap)
                {
                    w.giant_cand[g] = make_int4(cc, s_ovf.y | ((int)blockIdx.x << 10), s_ovf.z, s_ovf.w);
                    atomicAdd(w.epa_stats + 7, 1u);
                    w.hit[cc] = 0;
                    done = false;
                    s_stop = 1;
                }
                else
                {
                    epa_beyond_capacity(w, cc);
                    r = EPA_NONE;
                }
            }
            if (done)
                write_result(w, cc, r, pa, pb, nn);
        }
        __syncthreads();
        if (s_stop)
            break;
    }
}

// Tier 4: the whole grid on one queued candidate at a time (cooperative launch).
__global__ void __launch_bounds__(kLargeThreads) k_epa_giant(DevWorld w)
{
    GiantScratch &S = *reinterpret_cast<GiantScratch *>(w.giant_scratch);
    const GridTeam team{S.af, S.ai, S.c1, S.c2, &S.flag, &S.bar, w.barrier_spins, w.barrier_extra};
    GiantArena &E = *reinterpret_cast<GiantArena *>(w.epa_arena);
    const int n = min(w.work_counter[8], w.giant_cap);
    for (int q = 0; q < n; ++q)
    {
        const int4 gq = w.giant_cand[q];
        const int cc = gq.x;
        const Shape A = load_shape(w, w.cand_a[cc]), B = load_shape(w, w.cand_b[cc]);
        // the block tier's polytope at the start of the iteration that outgrew it
        const BlockArena &src =
            *reinterpret_cast<const BlockArena *>(w.blk_arena + (size_t)(gq.y >> 10) * sizeof(BlockArena));
        const int cb = (gq.y >> 8) & 1, nf = gq.z, nv = gq.w;
        for (int i = team.rank(); i < nv; i += team.size())
        {
            E.px[i] = src.px[i];
            E.py[i] = src.py[i];
            E.pz[i] = src.pz[i];
            E.ax[i] = src.ax[i];
            E.ay[i] = src.ay[i];
            E.az[i] = src.az[i];
            E.bx[i] = src.bx[i];
            E.by[i] = src.by[i];
            E.bz[i] = src.bz[i];
            E.vid[i] = src.vid[i];
        }
        for (int f = team.rank(); f < nf; f += team.size())
        {
            E.fidx[cb][f] = src.fidx[cb][f];
            E.fnx[cb][f] = src.fnx[cb][f];
            E.fny[cb][f] = src.fny[cb][f];
            E.fnz[cb][f] = src.fnz[cb][f];
            E.fd[cb][f] = src.fd[cb][f];
        }
        const int4 resume = make_int4(0, gq.y & 0x3ff, nf, nv);
        GV s0 = {}, s1 = {}, s2 = {}, s3 = {};
        v3 pa, pb, nn;
        int r = epa_large(w, team, E, S.table, GiantArena::kFaces, A, B, s0, s1, s2, s3, pa, pb, nn, &resume);
        if (r == EPA_ABORT)
        {
            if (team.rank() == 0)
            {
                atomicOr(w.status, (unsigned)ST_EPA_TIMEOUT);
                epa_beyond_capacity(w, cc);
                write_result(w, cc, EPA_NONE, pa, pb, nn);
            }
            return;
        }
        if (team.rank() == 0)
        {
            if (r == EPA_OVERFLOW)
            {
                epa_beyond_capacity(w, cc);
                r = EPA_NONE;
            }
            write_result(w, cc, r, pa, pb, nn);
        }
        if (!team.sync()) // the arena is reused by the next candidate
            return;
    }
}

size_t epa_big_bytes() { return sizeof(GiantArena); }
size_t epa_block_bytes() { return sizeof(BlockArena); }
size_t epa_giant_scratch_bytes() { return sizeof(GiantScratch); }

int giant_grid(int sm_count)
{
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_epa_giant, kLargeThreads, 0);
    per = std::max(1, std::min(per, 2));
    return std::min(per * sm_count, kGiantMaxWarps / (kLargeThreads / 32));
}

// The block tier's group table in dynamic shared memory beyond 48 KB. The attribute belongs to
// the current device's context, so every world sets it for its own device when it is created.
int large_kernel_attrs()
{
    return (int)cudaFuncSetAttribute(k_epa_block, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(GroupTable));
}

int launch_narrow_big(cudaStream_t st, const DevWorld &w)
{
    cudaLaunchAttribute prio;
    prio.id = cudaLaunchAttributePriority;
    prio.val.priority = tier_priority();
    cudaLaunchConfig_t bcfg = {};
    bcfg.gridDim = dim3(w.blk_blocks);
    bcfg.blockDim = dim3(kLargeThreads);
    bcfg.dynamicSmemBytes = sizeof(GroupTable);
    bcfg.stream = st;
    bcfg.attrs = &prio;
    bcfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&bcfg, k_epa_block, w);
    if (e != cudaSuccess)
        return (int)e;
    GiantScratch *S = reinterpret_cast<GiantScratch *>(w.giant_scratch);
    e = cudaMemsetAsync(&S->bar, 0, sizeof(GridBarrier), st);
    if (e != cudaSuccess)
        return (int)e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(w.giant_blocks);
    cfg.blockDim = dim3(kLargeThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    attr[1] = prio;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    e = cudaLaunchKernelEx(&cfg, k_epa_giant, w);
    return (int)e;
}

} // namespace nans
