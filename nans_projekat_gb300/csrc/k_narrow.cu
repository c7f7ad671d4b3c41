// Narrowphase tiers 1 and 2: GJK per candidate pair (one lane each), then EPA per hit, one
// per thread on a 12-vertex / 20-face polytope (tier 1) and, for the EPAs that outgrow it,
// one per warp on a 256-face polytope (tier 2; tiers 3 and 4 are in k_epa_large.cu).
//
// GJK follows CheckCollision / EvolveSimplex (code/nans.cpp:571-769, 906-966): the search
// direction is reset to normalize(PB - PA) on every call, Simplex[0] is the oldest point,
// at most 65 calls, the degenerate-direction exit at |d| <= 1e-4 and the support test
// dot(d, P) >= 0. The simplex lives in registers as four named slots. k_gjk gives each pair
// 8 calls; pairs still evolving are queued with their simplex and call index and resumed by
// k_gjk_long, so that long runs share warps with each other. A hit's final simplex is stored
// for the EPA. The tier-1 queue is ordered in two parts: pairs whose EPA ran more than a few
// iterations at the previous step first, then the rest, so that a warp's lanes run EPAs of
// similar length.
//
// EPA follows ResolveCollision (code/nans.cpp:217-328, 771-904) with the polytope in
// fixed-capacity shared-memory buffers instead of std::vector:
//   * vertices are a pool (GJK tetrahedron + one support per iteration);
//   * faces are an ordered list of vertex indices with their normal and distance; removing
//     the visible faces is a stable compaction, new faces are appended in edge order -- the
//     same order vector::erase / push_back produce;
//   * horizon edges are pushed in the order of the visible faces, each push cancelling the
//     FIRST stored edge that is its reverse (vertex equality compares P, code/nans.h:251-254);
//     the warp tier decides every push's fate in parallel from its group of equal edges.
// A face's "recomputed" normal in the closest-face search and the removal test equals its
// stored normal bit for bit (same operands, same operations, the flip is an exact negation),
// so each face's distance |dot(N, A)| is computed once, when the face is created or kept.
// An EPA whose support point no face sees ends at once: nothing changes, so every later
// iteration would repeat it up to the cap. Tier 1 runs one EPA per thread; tier 2 one per
// warp, whose lanes share the per-face loops while the sequential parts run redundantly.
#include <algorithm>

#include "nans_gjk.cuh"
#include "nans_solve.cuh"

namespace nans
{

// Polytope of one warp-cooperative EPA (shared memory). The vertex pool holds the GJK
// tetrahedron plus one support per iteration, with canonical ids; faces are an ordered list
// (vertex indices, normal, cached distance) in one of two banks, the removal pass writing the
// next list into the other; edges are the current horizon, pushes the iteration's horizon
// candidates. FMAX / EMAX bound faces and horizon edges.
template <int FMAX, int EMAX> struct EpaBuf
{
    static constexpr int kFaces = FMAX;
    static constexpr int kEdges = EMAX;
    static constexpr int kPushes = 3 * FMAX;
    float px[kEpaMaxVerts], py[kEpaMaxVerts], pz[kEpaMaxVerts];
    float ax[kEpaMaxVerts], ay[kEpaMaxVerts], az[kEpaMaxVerts];
    float bx[kEpaMaxVerts], by[kEpaMaxVerts], bz[kEpaMaxVerts];
    unsigned char vid[kEpaMaxVerts]; // canonical vertex id (first vertex with an equal P), 0xff: NaN
    float fnx[2][FMAX], fny[2][FMAX], fnz[2][FMAX], fd[2][FMAX]; // two banks: the list and its successor
    unsigned char fa[2][FMAX], fb[2][FMAX], fc[2][FMAX];
    unsigned char ea[EMAX], eb[EMAX];
    unsigned pkey[kPushes];      // horizon push: group lo | hi << 8, orientation << 16, self-loop << 17
    unsigned short puv[kPushes]; // horizon push: u | v << 8
    static constexpr int kShapeCache = 64;
    float sva[3 * kShapeCache], svb[3 * kShapeCache]; // the two shapes' world vertices
};
constexpr unsigned kNanPush = 0xffffffffu; // a push with a NaN vertex: it equals no edge
using EpaFast = EpaBuf<kEpaFastFaces, kEpaFastEdges>; // shared memory, one per warp


template <class B> __device__ __forceinline__ v3 pool_p(const B &E, int i) { return mk3(E.px[i], E.py[i], E.pz[i]); }

template <class B> __device__ __forceinline__ void pool_put(B &E, int i, const GV &g)
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
}

// PushTriangle (code/nans.cpp:292-322) into bank k: N = normalize(cross(B-A, C-A)), flipped to
// face away from the origin; the face's distance to the origin |dot(N, A)| is cached with it
// and returned.
template <class B> __device__ __forceinline__ float face_put(B &E, int k, int f, int a, int b, int c)
{
    v3 pa = pool_p(E, a), pb = pool_p(E, b), pc = pool_p(E, c);
    v3 n = normalize3(cross3(pb - pa, pc - pa));
    if (dot3(pa, n) < 0.0f)
        n = -1.0f * n;
    E.fa[k][f] = (unsigned char)a;
    E.fb[k][f] = (unsigned char)b;
    E.fc[k][f] = (unsigned char)c;
    E.fnx[k][f] = n.x;
    E.fny[k][f] = n.y;
    E.fnz[k][f] = n.z;
    const float d = fabsf(dot3(n, pa));
    E.fd[k][f] = d;
    return d;
}

// The support of one shape from its vertices cached in shared memory (hull_support's order
// and comparisons: the same vertex, bit for bit).
__device__ __forceinline__ v3 cached_hull_support(const float *v, int npts, v3 d)
{
    float best = -FLT_MAX;
    v3 r = mk3(0.0f, 0.0f, 0.0f);
    for (int t = 0; t < npts; ++t)
    {
        const v3 p = mk3(v[3 * t], v[3 * t + 1], v[3 * t + 2]);
        const float dist = dot3(p, d);
        if (dist > best)
        {
            best = dist;
            r = p;
        }
    }
    return r;
}

// minkowski_support with each hull of at most kShapeCache vertices read from the cache.
template <class B>
__device__ __forceinline__ GV cached_support(const DevWorld &w, const B &E, const Shape &A, const Shape &Bs, v3 d)
{
    GV r;
    if (A.npts == 0)
        r.sa = sphere_support(A.p, A.radius, d);
    else if (A.npts <= B::kShapeCache)
        r.sa = cached_hull_support(E.sva, A.npts, d);
    else
        r.sa = hull_support(w.verts, A.off, A.npts, d);
    const v3 nd = -1.0f * d;
    if (Bs.npts == 0)
        r.sb = sphere_support(Bs.p, Bs.radius, nd);
    else if (Bs.npts <= B::kShapeCache)
        r.sb = cached_hull_support(E.svb, Bs.npts, nd);
    else
        r.sb = hull_support(w.verts, Bs.off, Bs.npts, nd);
    r.p = r.sa - r.sb;
    return r;
}

// The same supports with the vertices spread over the warp when both shapes are cached hulls
// of at most 16 vertices: lanes 0-15 evaluate A's vertices against d, lanes 16-31 B's against
// -d, and each half reduces to the first maximum (larger distance, then lower index; NaN and
// distances not above -FLT_MAX never win), which is the sequential scan's vertex.
template <class B>
__device__ __forceinline__ GV warp_support(const DevWorld &w, const B &E, const Shape &A, const Shape &Bs, v3 d,
                                           int lane)
{
    if (A.npts == 0 || Bs.npts == 0 || A.npts > 16 || Bs.npts > 16)
        return cached_support(w, E, A, Bs, d);
    const int half = lane >> 4, t = lane & 15;
    const float *v = half ? E.svb : E.sva;
    const v3 dd = half ? -1.0f * d : d;
    float best = -FLT_MAX;
    int bi = -1;
    if (t < (half ? Bs.npts : A.npts))
    {
        const float dist = dot3(mk3(v[3 * t], v[3 * t + 1], v[3 * t + 2]), dd);
        if (dist > best)
        {
            best = dist;
            bi = t;
        }
    }
    for (int o = 8; o > 0; o >>= 1)
    {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (oi >= 0 && (bi < 0 || ob > best || (ob == best && oi < bi)))
        {
            best = ob;
            bi = oi;
        }
    }
    const int ia = __shfl_sync(0xffffffffu, bi, 0), ib = __shfl_sync(0xffffffffu, bi, 16);
    GV r;
    r.sa = ia >= 0 ? mk3(E.sva[3 * ia], E.sva[3 * ia + 1], E.sva[3 * ia + 2]) : mk3(0.0f, 0.0f, 0.0f);
    r.sb = ib >= 0 ? mk3(E.svb[3 * ib], E.svb[3 * ib + 1], E.svb[3 * ib + 2]) : mk3(0.0f, 0.0f, 0.0f);
    r.p = r.sa - r.sb;
    return r;
}

// Canonical id of pool vertex i (written by lane 0 before the call): the first vertex whose P
// equals it, which is its own canonical id; 0xff when P has a NaN (it equals nothing).
template <class B> __device__ __forceinline__ void pool_canon(B &E, int i, int lane)
{
    const v3 p = pool_p(E, i);
    int id = i;
    if (isnan(p.x) || isnan(p.y) || isnan(p.z))
        id = 0xff;
    else
        for (int base = 0; base < i; base += 32)
        {
            const int j = base + lane;
            const unsigned bal = __ballot_sync(0xffffffffu, j < i && eq3(pool_p(E, j), p));
            if (bal)
            {
                id = base + __ffs(bal) - 1;
                break;
            }
        }
    if (lane == 0)
        E.vid[i] = (unsigned char)id;
    __syncwarp();
}

// Horizon push k = (u, v): its group is the unordered pair of canonical ids.
template <class B> __device__ __forceinline__ void push_put(B &E, int k, int u, int v)
{
    const unsigned cu = E.vid[u], cv = E.vid[v];
    unsigned key = kNanPush;
    if (cu != 0xffu && cv != 0xffu)
        key = min(cu, cv) | (max(cu, cv) << 8) | ((cu > cv ? 1u : 0u) << 16) | ((cu == cv ? 1u : 0u) << 17);
    E.pkey[k] = key;
    E.puv[k] = (unsigned short)(u | (v << 8));
}

// Whether push k of np is on the horizon after PushEdge (code/nans.cpp:232-266) has run over
// all pushes in order. A push cancels the FIRST stored edge that is its reverse, so a group's
// stored edges always run one way and leave in push order: the survivors are the last
// (#majority - #minority) pushes of the majority orientation; in a self-loop group (P(u) ==
// P(v): every push reverses every other) the last push survives iff the count is odd.
template <class B> __device__ __forceinline__ bool push_survives(const B &E, int k, int np)
{
    const unsigned key = E.pkey[k];
    if (key == kNanPush)
        return true;
    const unsigned g = key & 0xffffu, dir = (key >> 16) & 1u;
    int same = 0, opp = 0, after = 0;
    for (int j = 0; j < np; ++j)
    {
        const unsigned kj = E.pkey[j];
        if ((kj & 0xffffu) != g || kj == kNanPush)
            continue;
        if (((kj >> 16) & 1u) == dir)
        {
            ++same;
            after += j > k;
        }
        else
            ++opp;
    }
    if ((key >> 17) & 1u)
        return after == 0 && (same & 1);
    return same > opp && after < same - opp;
}

// Candidate (d, f) for the closest face: the first minimum of the list's distances, NaN
// distances never winning.
__device__ __forceinline__ void closest_step(float &bd, int &bi, float d, int f)
{
    if (d < bd || (d == bd && f < bi))
    {
        bd = d;
        bi = f;
    }
}

// The reference's closest-face scan (CurrentDistance starts at face 0, strict '<'): the first
// minimum over the faces, except that a NaN face 0 stays the closest. (bd, bi) are each lane's
// candidates; returns the face and writes its distance.
template <class B>
__device__ __forceinline__ int closest_face(const B &E, int k, int nf, float bd, int bi, float &cur)
{
    for (int o = 16; o > 0; o >>= 1)
    {
        const float od = __shfl_xor_sync(0xffffffffu, bd, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        closest_step(bd, bi, od, oi);
    }
    int ci = bi;
    if (nf == 0 || isnan(E.fd[k][0]) || ci >= nf)
        ci = 0;
    cur = E.fd[k][ci];
    return ci;
}

// ResolveCollision (code/nans.cpp:787-904) on one warp, the face list in one of two banks.
// One pass over the list tests each face against the new support point, writes the pushes of
// the visible ones and moves the others to the other bank in order (the stable removal); the
// closest face of the next list is reduced from the kept and the new faces as they are
// written. Returns EPA_CONTACT with the contact written, EPA_NONE, or EPA_OVERFLOW when the
// polytope outgrows B; then ovf = (iteration, stale | bank << 1, faces, vertices) describes the
// polytope at the start of that iteration, still in E.
template <class B>
__device__ int epa_run(const DevWorld &w, B &E, const Shape &A, const Shape &Bs, const GV &s0, const GV &s1,
                       const GV &s2, const GV &s3, v3 &out_pa, v3 &out_pb, v3 &out_n, int lane, int4 &ovf)
{
    const unsigned full = 0xffffffffu;
    if (lane == 0)
    {
        pool_put(E, 0, s0);
        pool_put(E, 1, s1);
        pool_put(E, 2, s2);
        pool_put(E, 3, s3);
    }
    if (A.npts > 0 && A.npts <= B::kShapeCache)
        for (int i = lane; i < 3 * A.npts; i += 32)
            E.sva[i] = w.verts[A.off + i];
    if (Bs.npts > 0 && Bs.npts <= B::kShapeCache)
        for (int i = lane; i < 3 * Bs.npts; i += 32)
            E.svb[i] = w.verts[Bs.off + i];
    __syncwarp();
    for (int i = 0; i < 4; ++i)
        pool_canon(E, i, lane);
    // ABC, ACD, ADB, BDC (code/nans.cpp:799-802)
    float bd = INFINITY;
    int bi = 0x7fffffff;
    if (lane < 4)
    {
        const int a = lane == 3 ? 1 : 0, b = lane == 0 ? 1 : (lane == 1 ? 2 : 3), c = lane == 0 ? 2 : (lane == 1 ? 3 : (lane == 2 ? 1 : 2));
        closest_step(bd, bi, face_put(E, 0, lane, a, b, c), lane);
    }
    __syncwarp();
    int cb = 0, nf = 4, nv = 4;
    float cur;
    int ci = closest_face(E, cb, nf, bd, bi, cur);
    // When every face is removed and the horizon cancels out, the reference reads Triangle[0]
    // of the empty vector (code/nans.cpp:807, 824); with libstdc++ that slot still holds the
    // face erased last, the last face of the list before removal. It is kept at index 0.
    bool stale = false;
    for (int it = 0; it <= 64; ++it)
    {
        if (nf == 0 && !stale)
            return EPA_NONE;
        const v3 n = mk3(E.fnx[cb][ci], E.fny[cb][ci], E.fnz[cb][ci]);
        const GV ns = warp_support(w, E, A, Bs, n, lane);
        if (dot3(n, ns.p) - cur < 0.001f)
        {
            // Barycentric (code/nans.cpp:771-785) of N*dist on the closest face
            int ia = E.fa[cb][ci], ib = E.fb[cb][ci], ic = E.fc[cb][ci];
            v3 pa = pool_p(E, ia), pb = pool_p(E, ib), pc = pool_p(E, ic);
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
        // faces that see the new support point (code/nans.cpp:869-891): pushes of the visible
        // ones, the others into the other bank in order
        const int nb = cb ^ 1;
        int nseen = 0, keep = 0;
        bd = INFINITY;
        bi = 0x7fffffff;
        for (int base = 0; base < nf; base += 32)
        {
            const int f = base + lane;
            const bool in = f < nf;
            bool vis = false;
            unsigned char a = 0, b = 0, c = 0;
            v3 fn = mk3(0.0f, 0.0f, 0.0f);
            float d = 0.0f;
            if (in)
            {
                a = E.fa[cb][f];
                b = E.fb[cb][f];
                c = E.fc[cb][f];
                fn = mk3(E.fnx[cb][f], E.fny[cb][f], E.fnz[cb][f]);
                d = E.fd[cb][f];
                vis = dot3(fn, ns.p - pool_p(E, a)) > 0.0f;
            }
            const unsigned bv = __ballot_sync(full, vis), bk = __ballot_sync(full, in && !vis);
            const unsigned below = (1u << lane) - 1u;
            if (vis)
            {
                const int r = nseen + __popc(bv & below);
                push_put(E, 3 * r, a, b);
                push_put(E, 3 * r + 1, b, c);
                push_put(E, 3 * r + 2, c, a);
            }
            else if (in)
            {
                const int dst = keep + __popc(bk & below);
                E.fa[nb][dst] = a;
                E.fb[nb][dst] = b;
                E.fc[nb][dst] = c;
                E.fnx[nb][dst] = fn.x;
                E.fny[nb][dst] = fn.y;
                E.fnz[nb][dst] = fn.z;
                E.fd[nb][dst] = d;
                closest_step(bd, bi, d, dst);
            }
            nseen += __popc(bv);
            keep += __popc(bk);
        }
        __syncwarp();
        if (nseen == 0)
            return EPA_NONE; // nothing changes: every later iteration repeats this one
        // horizon: the pushes decided in parallel; the survivors keep push order
        const int np = 3 * nseen;
        int ne = 0;
        for (int base = 0; base < np; base += 32)
        {
            const int k = base + lane;
            const bool alive = k < np && push_survives(E, k, np);
            const unsigned bal = __ballot_sync(full, alive);
            if (alive)
            {
                const int dst = ne + __popc(bal & ((1u << lane) - 1u));
                if (dst < B::kEdges)
                {
                    const unsigned uv = E.puv[k];
                    E.ea[dst] = (unsigned char)(uv & 0xffu);
                    E.eb[dst] = (unsigned char)(uv >> 8);
                }
            }
            ne += __popc(bal);
        }
        if (ne > B::kEdges || keep + ne > B::kFaces)
        {
            ovf = make_int4(it, (stale ? 1 : 0) | (cb << 1), nf, nv);
            return EPA_OVERFLOW;
        }
        __syncwarp();
        if (keep == 0 && ne == 0)
        {
            // every face removed: slot 0 keeps the last face of the list
            if (lane == 0)
            {
                const int l = nf - 1;
                E.fa[nb][0] = E.fa[cb][l];
                E.fb[nb][0] = E.fb[cb][l];
                E.fc[nb][0] = E.fc[cb][l];
                E.fnx[nb][0] = E.fnx[cb][l];
                E.fny[nb][0] = E.fny[cb][l];
                E.fnz[nb][0] = E.fnz[cb][l];
                E.fd[nb][0] = E.fd[cb][l];
            }
            __syncwarp();
            stale = true;
        }
        // the new support joins the vertex pool; new faces (S, e.A, e.B) in edge order
        const int sv = nv;
        if (lane == 0)
            pool_put(E, sv, ns);
        ++nv;
        __syncwarp();
        pool_canon(E, sv, lane);
        for (int j = lane; j < ne; j += 32)
            closest_step(bd, bi, face_put(E, nb, keep + j, sv, E.ea[j], E.eb[j]), keep + j);
        __syncwarp();
        cb = nb;
        nf = keep + ne;
        ci = closest_face(E, cb, nf, bd, bi, cur);
    }
    return EPA_NONE;
}


// Returns the tier-3 queue index (the caller may leave its state in handover[q]), or -1.
__device__ __forceinline__ int escalate(const DevWorld &w, int c, bool to_big)
{
    w.hit[c] = 0;
    const int sc = w.cand_meta[c] >> 3;
    if (atomicExch(w.scene_late + sc, 1) == 0)
        w.late_list[atomicAdd(w.work_counter + 13, 1)] = sc;
    if (!to_big)
    {
        atomicAdd(w.epa_stats + 6, 1u);
        int q = atomicAdd(w.work_counter + 5, 1);
        if (q < w.med_cap)
        {
            w.med_cand[q] = c;
            return -1;
        }
    }
    int q = atomicAdd(w.work_counter + 3, 1);
    if (q < w.ovf_cap)
    {
        w.ovf_cand[q] = c;
        if (q < kHandoverSlots)
            w.handover[q].hdr[2] = -1; // no state unless the warp tier leaves one
        return q;
    }
    atomicOr(w.status, (unsigned)ST_EPA_FACES);
    return -1;
}

// The warp tier's polytope (state ovf) into handover slot q, for the block tier to resume.
__device__ __forceinline__ void handover_put(const DevWorld &w, const EpaFast &E, int q, int4 ovf, int lane)
{
    EpaHandover &H = w.handover[q];
    const int nf = ovf.z, nv = ovf.w, k = (ovf.y >> 1) & 1;
    for (int i = lane; i < nv; i += 32)
    {
        H.px[i] = E.px[i];
        H.py[i] = E.py[i];
        H.pz[i] = E.pz[i];
        H.ax[i] = E.ax[i];
        H.ay[i] = E.ay[i];
        H.az[i] = E.az[i];
        H.bx[i] = E.bx[i];
        H.by[i] = E.by[i];
        H.bz[i] = E.bz[i];
        H.vid[i] = E.vid[i] == 0xffu ? -1 : (int)E.vid[i];
    }
    for (int f = lane; f < nf; f += 32)
    {
        H.fidx[f] = (unsigned)E.fa[k][f] | ((unsigned)E.fb[k][f] << 8) | ((unsigned)E.fc[k][f] << 16);
        H.fnx[f] = E.fnx[k][f];
        H.fny[f] = E.fny[k][f];
        H.fnz[f] = E.fnz[k][f];
        H.fd[f] = E.fd[k][f];
    }
    __syncwarp();
    if (lane == 0)
    {
        H.hdr[0] = ovf.x;
        H.hdr[1] = ovf.y & 1;
        H.hdr[3] = nv;
        __threadfence();
        H.hdr[2] = nf;
    }
}

// ------------------------------------------------------------------------------------
// Tier 1: one thread per candidate pair, GJK then EPA on a small per-thread polytope.
// Positions of the polytope's vertices, its faces and the horizon live in shared memory in
// field-major layout ([slot][thread], so a warp touches 32 consecutive words); the support
// points SupA/SupB, read only for the final contact point, live in thread-local arrays.
// 12 vertices (8 EPA iterations) and 20 faces hold ~99.7% of the EPAs of the stack workload.
// ------------------------------------------------------------------------------------
constexpr int kTinyThreads = 64;
#ifndef NANS_TINY_V
#define NANS_TINY_V 12
#endif
#ifndef NANS_TINY_F
#define NANS_TINY_F 20
#endif
constexpr int kTinyV = NANS_TINY_V;
constexpr int kTinyF = NANS_TINY_F;
constexpr int kTinyE = 12;
constexpr unsigned kNoCanon = 15u; // a vertex with a NaN coordinate: equal to no vertex
static_assert(kTinyV < 15, "vertex and canonical indices are packed in 4 bits");

struct TinySmem
{
    float px[kTinyV][kTinyThreads], py[kTinyV][kTinyThreads], pz[kTinyV][kTinyThreads];
    float fnx[kTinyF][kTinyThreads], fny[kTinyF][kTinyThreads], fnz[kTinyF][kTinyThreads];
    unsigned fidx[kTinyF][kTinyThreads];       // a | b << 8 | c << 16
    unsigned short edge[kTinyE][kTinyThreads]; // u | v << 4 | canon(u) << 8 | canon(v) << 12
};

struct TinyLocal
{
    float sa[kTinyV][3], sb[kTinyV][3];
};

__device__ __forceinline__ v3 tiny_p(const TinySmem &S, int t, int i) { return mk3(S.px[i][t], S.py[i][t], S.pz[i][t]); }

// Stores vertex i and returns its canonical index: the first vertex whose P equals it (P
// equality is what the reference's edge matching compares), kNoCanon when P has a NaN.
// `canon` holds the canonical indices of vertices 0..i-1, 4 bits each.
__device__ __forceinline__ unsigned tiny_put(TinySmem &S, TinyLocal &L, int t, int i, const GV &g,
                                             unsigned long long canon)
{
    S.px[i][t] = g.p.x;
    S.py[i][t] = g.p.y;
    S.pz[i][t] = g.p.z;
    L.sa[i][0] = g.sa.x;
    L.sa[i][1] = g.sa.y;
    L.sa[i][2] = g.sa.z;
    L.sb[i][0] = g.sb.x;
    L.sb[i][1] = g.sb.y;
    L.sb[i][2] = g.sb.z;
    if (isnan(g.p.x) || isnan(g.p.y) || isnan(g.p.z))
        return kNoCanon;
    for (int j = 0; j < i; ++j)
        if (eq3(tiny_p(S, t, j), g.p))
            return (unsigned)(canon >> (4 * j)) & 15u;
    return (unsigned)i;
}

// PushTriangle (code/nans.cpp:292-322); returns the face's distance |dot(N, A)|, which the
// reference recomputes from the same operands in its closest-face search (bit-equal).
__device__ __forceinline__ float tiny_face(TinySmem &S, int t, int f, int a, int b, int c)
{
    v3 pa = tiny_p(S, t, a), pb = tiny_p(S, t, b), pc = tiny_p(S, t, c);
    v3 n = normalize3(cross3(pb - pa, pc - pa));
    if (dot3(pa, n) < 0.0f)
        n = -1.0f * n;
    S.fidx[f][t] = (unsigned)a | ((unsigned)b << 8) | ((unsigned)c << 16);
    S.fnx[f][t] = n.x;
    S.fny[f][t] = n.y;
    S.fnz[f][t] = n.z;
    return fabsf(dot3(n, pa));
}

// PushEdge (code/nans.cpp:232-266), sequential. The stored edge (x, y) is the reverse of (u, v)
// when P(x) == P(v) and P(y) == P(u): equal canonical indices (a NaN vertex matches nothing).
// Returns false on overflow.
__device__ __forceinline__ bool tiny_edge(TinySmem &S, int t, unsigned long long canon, int &ne, int u, int v)
{
    const unsigned cu = (unsigned)(canon >> (4 * u)) & 15u, cv = (unsigned)(canon >> (4 * v)) & 15u;
    if (cu != kNoCanon && cv != kNoCanon)
    {
        const unsigned want = cv | (cu << 4);
        for (int e = 0; e < ne; ++e)
        {
            if ((unsigned)(S.edge[e][t] >> 8) == want)
            {
                for (int k = e + 1; k < ne; ++k)
                    S.edge[k - 1][t] = S.edge[k][t];
                --ne;
                return true;
            }
        }
    }
    if (ne >= kTinyE)
        return false;
    S.edge[ne][t] = (unsigned short)(u | (v << 4) | (cu << 8) | (cv << 12));
    ++ne;
    return true;
}

// ResolveCollision (code/nans.cpp:787-904) by one thread; same results as epa_run.
// `simp` is the GJK simplex as the GJK pass stored it (4 x (P, SupA, SupB), 36 floats).
// The closest-face search of the next iteration is folded into the removal pass and the face
// creation: a running minimum with strict '<' over the kept faces, then the new ones, in list
// order, is the reference's scan (a NaN first distance keeps face 0, as its scan does).
// The 8 world vertices of an 8-point shape (a box) in registers: the per-thread EPA's support
// maps read them once per EPA instead of at every iteration (the polytopes' shared memory leaves
// the L1 little room). box_support is hull_support's scan: the same order, products and strict
// comparison from -FLT_MAX, so the same vertex bit for bit.
struct Verts8
{
    float x[8], y[8], z[8];
};
__device__ __forceinline__ void load_verts8(const float *verts, int off, Verts8 &r)
{
    const float4 *q = reinterpret_cast<const float4 *>(verts + off);
    float v[24];
#pragma unroll
    for (int i = 0; i < 6; ++i)
    {
        const float4 f = __ldg(q + i);
        v[4 * i] = f.x;
        v[4 * i + 1] = f.y;
        v[4 * i + 2] = f.z;
        v[4 * i + 3] = f.w;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
    {
        r.x[k] = v[3 * k];
        r.y[k] = v[3 * k + 1];
        r.z[k] = v[3 * k + 2];
    }
}
__device__ __forceinline__ v3 box_support(const Verts8 &r, v3 d)
{
    float best = -FLT_MAX;
    v3 out = mk3(0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < 8; ++k)
    {
        const v3 p = mk3(r.x[k], r.y[k], r.z[k]);
        const float dist = dot3(p, d);
        if (dist > best)
        {
            best = dist;
            out = p;
        }
    }
    return out;
}

__device__ int epa_tiny(const DevWorld &w, TinySmem &S, int t, const Shape &A, const Shape &B, const float *simp,
                        v3 &out_pa, v3 &out_pb, v3 &out_n, int &iters)
{
    TinyLocal L;
    const bool ra = A.npts == 8, rb = B.npts == 8;
    Verts8 VA, VB;
    if (ra)
        load_verts8(w.verts, A.off, VA);
    if (rb)
        load_verts8(w.verts, B.off, VB);
    unsigned long long canon = 0ull;
    for (int i = 0; i < 4; ++i)
    {
        const float *q = simp + 9 * i;
        GV g;
        g.p = mk3(q[0], q[1], q[2]);
        g.sa = mk3(q[3], q[4], q[5]);
        g.sb = mk3(q[6], q[7], q[8]);
        canon |= (unsigned long long)tiny_put(S, L, t, i, g, canon) << (4 * i);
    }
    float cur = tiny_face(S, t, 0, 0, 1, 2);
    int ci = 0;
    {
        const float d1 = tiny_face(S, t, 1, 0, 2, 3);
        if (d1 < cur)
        {
            cur = d1;
            ci = 1;
        }
        const float d2 = tiny_face(S, t, 2, 0, 3, 1);
        if (d2 < cur)
        {
            cur = d2;
            ci = 2;
        }
        const float d3 = tiny_face(S, t, 3, 1, 3, 2);
        if (d3 < cur)
        {
            cur = d3;
            ci = 3;
        }
    }
    int nf = 4, nv = 4;
    bool stale = false;
    for (int it = 0; it <= 64; ++it)
    {
        iters = it + 1;
        if (nf == 0 && !stale)
            return EPA_NONE;
        const v3 n = mk3(S.fnx[ci][t], S.fny[ci][t], S.fnz[ci][t]);
        GV ns;
        ns.sa = ra ? box_support(VA, n) : shape_support(w.verts, A, n);
        const v3 nd = -1.0f * n;
        ns.sb = rb ? box_support(VB, nd) : shape_support(w.verts, B, nd);
        ns.p = ns.sa - ns.sb;
        if (dot3(n, ns.p) - cur < 0.001f)
        {
            unsigned fi = S.fidx[ci][t];
            int ia = fi & 0xffu, ib = (fi >> 8) & 0xffu, ic = fi >> 16;
            v3 pa = tiny_p(S, t, ia), pb = tiny_p(S, t, ib), pc = tiny_p(S, t, ic);
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
            v3 saa = mk3(L.sa[ia][0], L.sa[ia][1], L.sa[ia][2]), sab = mk3(L.sa[ib][0], L.sa[ib][1], L.sa[ib][2]),
               sac = mk3(L.sa[ic][0], L.sa[ic][1], L.sa[ic][2]);
            v3 sba = mk3(L.sb[ia][0], L.sb[ia][1], L.sb[ia][2]), sbb = mk3(L.sb[ib][0], L.sb[ib][1], L.sb[ib][2]),
               sbc = mk3(L.sb[ic][0], L.sb[ic][1], L.sb[ic][2]);
            out_pa = ((bu * saa) + (bv * sab)) + (bw * sac);
            out_n = -1.0f * n;
            out_pb = ((bu * sba) + (bv * sbb)) + (bw * sbc);
            return EPA_CONTACT;
        }
        if (nf == 0)
            return EPA_NONE; // the stale read repeats identically until the iteration cap
        // visible faces -> horizon edges, the others compacted in place (code/nans.cpp:869-891),
        // with the running closest-face search over the kept ones
        int ne = 0, keep = 0, nci = 0;
        float ncur = 0.0f;
        for (int f = 0; f < nf; ++f)
        {
            unsigned fi = S.fidx[f][t];
            v3 fa = tiny_p(S, t, fi & 0xffu);
            v3 fn = mk3(S.fnx[f][t], S.fny[f][t], S.fnz[f][t]);
            if (dot3(fn, ns.p - fa) > 0.0f)
            {
                int a = fi & 0xffu, b = (fi >> 8) & 0xffu, c = fi >> 16;
                if (!(tiny_edge(S, t, canon, ne, a, b) && tiny_edge(S, t, canon, ne, b, c) &&
                      tiny_edge(S, t, canon, ne, c, a)))
                    return EPA_OVERFLOW;
            }
            else
            {
                if (keep != f)
                {
                    S.fidx[keep][t] = fi;
                    S.fnx[keep][t] = fn.x;
                    S.fny[keep][t] = fn.y;
                    S.fnz[keep][t] = fn.z;
                }
                const float d = fabsf(dot3(fn, fa));
                if (keep == 0 || d < ncur)
                {
                    ncur = d;
                    nci = keep;
                }
                ++keep;
            }
        }
        if (keep == nf)
            return EPA_NONE; // no face sees the support: every later iteration repeats this one
        if (keep + ne > kTinyF || nv >= kTinyV)
            return EPA_OVERFLOW;
        if (keep == 0 && ne == 0)
        {
            // every face removed: slot 0 keeps the last face of the list (nothing was moved)
            int l = nf - 1;
            const unsigned fi = S.fidx[l][t];
            const v3 fn = mk3(S.fnx[l][t], S.fny[l][t], S.fnz[l][t]);
            S.fidx[0][t] = fi;
            S.fnx[0][t] = fn.x;
            S.fny[0][t] = fn.y;
            S.fnz[0][t] = fn.z;
            ncur = fabsf(dot3(fn, tiny_p(S, t, fi & 0xffu)));
            nci = 0;
            stale = true;
        }
        int sv = nv++;
        canon |= (unsigned long long)tiny_put(S, L, t, sv, ns, canon) << (4 * sv);
        for (int j = 0; j < ne; ++j)
        {
            const unsigned ed = S.edge[j][t];
            const float d = tiny_face(S, t, keep + j, sv, ed & 15u, (ed >> 4) & 15u);
            if (keep + j == 0 || d < ncur)
            {
                ncur = d;
                nci = keep + j;
            }
        }
        nf = keep + ne;
        cur = ncur;
        ci = nci;
    }
    return EPA_NONE;
}

// GJK and the per-thread EPA run as separate kernels. The GJK pass keeps its registers low
// and its code small; a hit's final simplex (4 x (P, SupA, SupB), 36 floats) goes to the
// candidate's solver-constant slot (s_k, 9 float4, written only later by the solver) and the
// candidate to a compact queue (s_order, likewise free until the solver), so the EPA pass runs
// only hits, every lane on an EPA.
__device__ __forceinline__ void store_simplex(const DevWorld &w, int c, const GV &s0, const GV &s1, const GV &s2,
                                              const GV &s3)
{
    float4 *o = w.s_k + 9 * (size_t)c;
    o[0] = make_float4(s0.p.x, s0.p.y, s0.p.z, s0.sa.x);
    o[1] = make_float4(s0.sa.y, s0.sa.z, s0.sb.x, s0.sb.y);
    o[2] = make_float4(s0.sb.z, s1.p.x, s1.p.y, s1.p.z);
    o[3] = make_float4(s1.sa.x, s1.sa.y, s1.sa.z, s1.sb.x);
    o[4] = make_float4(s1.sb.y, s1.sb.z, s2.p.x, s2.p.y);
    o[5] = make_float4(s2.p.z, s2.sa.x, s2.sa.y, s2.sa.z);
    o[6] = make_float4(s2.sb.x, s2.sb.y, s2.sb.z, s3.p.x);
    o[7] = make_float4(s3.p.y, s3.p.z, s3.sa.x, s3.sa.y);
    o[8] = make_float4(s3.sa.z, s3.sb.x, s3.sb.y, s3.sb.z);
}

// Appends c to the EPA queue when `hit` (one atomic per warp and part). Pairs whose EPA took
// more than kEpaLongIters iterations at its last step fill the queue from the back (count in
// work counter 9), the others from the front (work counter 10): the per-thread EPA pass takes
// the long ones first, so that the lanes of a warp run EPAs of similar length.
constexpr int kEpaLongIters = 4;
__device__ __forceinline__ void enqueue_epa(const DevWorld &w, int c, bool hit)
{
    const unsigned act = __activemask();
    const bool lng = hit && w.epa_hist[w.cand_pidx[c]] > kEpaLongIters;
    const unsigned bal = __ballot_sync(act, hit && !lng), ball = __ballot_sync(act, lng);
    if (!hit)
        return;
    const int lane = threadIdx.x & 31;
    const unsigned part = lng ? ball : bal;
    const int leader = __ffs(part) - 1;
    int base = 0;
    if (lane == leader)
        base = atomicAdd(w.work_counter + (lng ? 9 : 10), __popc(part));
    base = __shfl_sync(part, base, leader);
    const int k = base + __popc(part & ((1u << lane) - 1u));
    w.s_order[lng ? w.cand_cap - 1 - k : k] = c;
}

// GJK of candidate c from call `it` with the simplex (s0..s3, n points). With a budget below
// 65, a GJK still evolving is queued for the long pass with its state (the simplex in the
// candidate's s_k slot, n and it in the queue), which resumes it.
// Minkowski support with 8-point shapes' vertices in registers (Verts8), the others read from
// memory: minkowski_support's values.
struct RegSupport
{
    const float *verts;
    const Shape &A, &B;
    bool ra, rb;
    const Verts8 &VA, &VB;
    __device__ __forceinline__ GV operator()(v3 d) const
    {
        GV r;
        r.sa = ra ? box_support(VA, d) : shape_support(verts, A, d);
        const v3 nd = -1.0f * d;
        r.sb = rb ? box_support(VB, nd) : shape_support(verts, B, nd);
        r.p = r.sa - r.sb;
        return r;
    }
};

__device__ __forceinline__ void gjk_one(const DevWorld &w, int c, int ia, int ib, int budget, GV &s0, GV &s1, GV &s2,
                                        GV &s3, int n, int it)
{
    const Shape A = load_shape(w, ia), B = load_shape(w, ib);
    const bool ra = A.npts == 8, rb = B.npts == 8;
    Verts8 VA, VB;
    if (ra)
        load_verts8(w.verts, A.off, VA);
    if (rb)
        load_verts8(w.verts, B.off, VB);
    const int g = gjk_from_with(RegSupport{w.verts, A, B, ra, rb, VA, VB}, A, B, s0, s1, s2, s3, n, it, budget);
    if (g == G_FOUND || g == G_BUDGET)
        store_simplex(w, c, s0, s1, s2, s3);
    if (g == G_BUDGET)
        w.long_cand[atomicAdd(w.work_counter + 7, 1)] = make_int2(c, n | (it << 8));
    else if (g != G_FOUND)
        w.hit[c] = 0;
    enqueue_epa(w, c, g == G_FOUND);
}

// Persistent: warps take 32 candidates at a time from a global queue; each lane runs GJK
// (budget kGjkShort calls); GJKs that need more calls go to the long pass, so that the rare
// long GJK runs share warps with each other instead of stalling 31 finished lanes.
constexpr int kGjkShort = 8;
constexpr int kGjkThreads = 128;
// four blocks per SM (at most 128 registers, room for both shapes' vertices): measured best
// against 5 and 6 (which spill the vertices) on the stack workload
__global__ void __launch_bounds__(kGjkThreads, 4) k_gjk(DevWorld w)
{
    const int lane = threadIdx.x & 31;
    const int n = *w.n_cand;
    // the warp claims its next 32 candidates and reads their bodies while it runs these
    int base = 0;
    if (lane == 0)
        base = atomicAdd(w.work_counter, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    int ia = 0, ib = 0;
    if (base + lane < n)
    {
        ia = w.cand_a[base + lane];
        ib = w.cand_b[base + lane];
    }
    while (base < n)
    {
        int next = 0;
        if (lane == 0)
            next = atomicAdd(w.work_counter, 32);
        next = __shfl_sync(0xffffffffu, next, 0);
        int na = 0, nb = 0;
        if (next + lane < n)
        {
            na = w.cand_a[next + lane];
            nb = w.cand_b[next + lane];
        }
        const int c = base + lane;
        if (c < n)
        {
            const int sc = w.cand_meta[c] >> 3;
            if (c == 0 || (w.cand_meta[c - 1] >> 3) != sc)
                w.cand_begin[sc] = c;
            if (c == n - 1 || (w.cand_meta[c + 1] >> 3) != sc)
                w.cand_end[sc] = c + 1;
            GV s0 = {}, s1 = {}, s2 = {}, s3 = {};
            gjk_one(w, c, ia, ib, kGjkShort, s0, s1, s2, s3, 0, 0);
        }
        base = next;
        ia = na;
        ib = nb;
    }
}

// The long pass: candidates whose GJK needed more than kGjkShort calls, resumed where the
// first pass stopped.
__global__ void __launch_bounds__(kGjkThreads, 4) k_gjk_long(DevWorld w)
{
    const int n = w.work_counter[7];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const int2 q = w.long_cand[i];
        const float4 *o = w.s_k + 9 * (size_t)q.x;
        const float4 k0 = o[0], k1 = o[1], k2 = o[2], k3 = o[3], k4 = o[4], k5 = o[5], k6 = o[6], k7 = o[7], k8 = o[8];
        GV s0, s1, s2, s3;
        s0.p = mk3(k0.x, k0.y, k0.z);
        s0.sa = mk3(k0.w, k1.x, k1.y);
        s0.sb = mk3(k1.z, k1.w, k2.x);
        s1.p = mk3(k2.y, k2.z, k2.w);
        s1.sa = mk3(k3.x, k3.y, k3.z);
        s1.sb = mk3(k3.w, k4.x, k4.y);
        s2.p = mk3(k4.z, k4.w, k5.x);
        s2.sa = mk3(k5.y, k5.z, k5.w);
        s2.sb = mk3(k6.x, k6.y, k6.z);
        s3.p = mk3(k6.w, k7.x, k7.y);
        s3.sa = mk3(k7.z, k7.w, k8.x);
        s3.sb = mk3(k8.y, k8.z, k8.w);
        gjk_one(w, q.x, w.cand_a[q.x], w.cand_b[q.x], 65, s0, s1, s2, s3, q.y & 0xff, q.y >> 8);
    }
}

// ---------------------------------------------------------------------------------------
// GJK with one warp per candidate pair: the support maps evaluated across the warp (lanes
// 0-15 hold shape A's vertices, lanes 16-31 shape B's, each half reduced to the first maximum
// by shuffles), the simplex cases run by every lane on the broadcast values. The same result
// as k_gjk bit for bit; an alternative schedule for the A/B against one thread per pair
// (NANS_WORLD_GJK_WARP), which keeps 32 pairs per warp instruction stream instead of one.
// ---------------------------------------------------------------------------------------
struct WarpSupport
{
    const float *verts;
    const Shape &A, &B;
    v3 v;      // this lane's vertex: A's vertex lane (lanes 0-15) or B's vertex lane - 16
    bool have; // this lane holds a vertex of its half's shape
    int lane;

    // First maximum of dot(vertex, d) over a half's lanes (NaN and values not above -FLT_MAX
    // never win; ties go to the lower index): the sequential scan's vertex.
    __device__ __forceinline__ int half_support(v3 d) const
    {
        float best = -FLT_MAX;
        int bi = -1;
        if (have)
        {
            const float dist = dot3(v, d);
            if (dist > best)
            {
                best = dist;
                bi = lane & 15;
            }
        }
        for (int o = 8; o > 0; o >>= 1)
        {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (oi >= 0 && (bi < 0 || ob > best || (ob == best && oi < bi)))
            {
                best = ob;
                bi = oi;
            }
        }
        return bi; // the vertex's index in the half, -1 for none; the caller fetches the vertex
    }

    __device__ __forceinline__ GV operator()(v3 d) const
    {
        const v3 nd = -1.0f * d;
        // both halves reduce in the same instructions, each against its own direction
        const v3 mine = (lane < 16) ? d : nd;
        const int bi = half_support(mine);
        const int ia = __shfl_sync(0xffffffffu, bi, 0), ib = __shfl_sync(0xffffffffu, bi, 16);
        const float ax = __shfl_sync(0xffffffffu, v.x, ia < 0 ? 0 : ia), ay = __shfl_sync(0xffffffffu, v.y, ia < 0 ? 0 : ia),
                    az = __shfl_sync(0xffffffffu, v.z, ia < 0 ? 0 : ia);
        const float bx = __shfl_sync(0xffffffffu, v.x, 16 + (ib < 0 ? 0 : ib)),
                    by = __shfl_sync(0xffffffffu, v.y, 16 + (ib < 0 ? 0 : ib)),
                    bz = __shfl_sync(0xffffffffu, v.z, 16 + (ib < 0 ? 0 : ib));
        GV r;
        if (A.npts == 0)
            r.sa = sphere_support(A.p, A.radius, d);
        else if (A.npts > 16)
            r.sa = hull_support(verts, A.off, A.npts, d);
        else
            r.sa = ia >= 0 ? mk3(ax, ay, az) : mk3(0.0f, 0.0f, 0.0f);
        if (B.npts == 0)
            r.sb = sphere_support(B.p, B.radius, nd);
        else if (B.npts > 16)
            r.sb = hull_support(verts, B.off, B.npts, nd);
        else
            r.sb = ib >= 0 ? mk3(bx, by, bz) : mk3(0.0f, 0.0f, 0.0f);
        r.p = r.sa - r.sb;
        return r;
    }
};

constexpr int kGjkWarpThreads = 128;
__global__ void __launch_bounds__(kGjkWarpThreads) k_gjk_warp(DevWorld w)
{
    const int lane = threadIdx.x & 31;
    const int n = *w.n_cand;
    for (;;)
    {
        int c = 0;
        if (lane == 0)
            c = atomicAdd(w.work_counter, 1);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= n)
            break;
        if (lane == 0)
        {
            const int sc = w.cand_meta[c] >> 3;
            if (c == 0 || (w.cand_meta[c - 1] >> 3) != sc)
                w.cand_begin[sc] = c;
            if (c == n - 1 || (w.cand_meta[c + 1] >> 3) != sc)
                w.cand_end[sc] = c + 1;
        }
        const Shape A = load_shape(w, w.cand_a[c]), B = load_shape(w, w.cand_b[c]);
        const Shape &S = lane < 16 ? A : B;
        const int t = lane & 15;
        const bool have = S.npts > 0 && S.npts <= 16 && t < S.npts;
        v3 v = mk3(0.0f, 0.0f, 0.0f);
        if (have)
            v = mk3(__ldg(w.verts + S.off + 3 * t), __ldg(w.verts + S.off + 3 * t + 1), __ldg(w.verts + S.off + 3 * t + 2));
        GV s0 = {}, s1 = {}, s2 = {}, s3 = {};
        int np = 0, it = 0;
        const int g = gjk_from_with(WarpSupport{w.verts, A, B, v, have, lane}, A, B, s0, s1, s2, s3, np, it, 65);
        if (lane == 0)
        {
            if (g == G_FOUND)
            {
                store_simplex(w, c, s0, s1, s2, s3);
                const bool lng = w.epa_hist[w.cand_pidx[c]] > kEpaLongIters;
                const int k = atomicAdd(w.work_counter + (lng ? 9 : 10), 1);
                w.s_order[lng ? w.cand_cap - 1 - k : k] = c;
            }
            else
                w.hit[c] = 0;
        }
    }
}

// Tier 1 EPA: one thread per hit from the queue; EPAs that outgrow the per-thread polytope
// are queued for the warp tier.
__global__ void __launch_bounds__(kTinyThreads) k_epa_tiny(DevWorld w)
{
    __shared__ TinySmem S;
    const int lane = threadIdx.x & 31, t = threadIdx.x;
    const int nl = w.work_counter[9], n = nl + w.work_counter[10];
    for (;;)
    {
        int base = 0;
        if (lane == 0)
            base = atomicAdd(w.work_counter + 11, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n)
            break;
        const int i = base + lane;
        if (i >= n)
            continue;
        const int slot = i < nl ? w.cand_cap - 1 - i : i - nl; // the long part first
        if (!dev_check(w, slot >= 0 && slot < w.cand_cap, 12, slot, w.cand_cap))
            continue;
        const int c = w.s_order[slot];
        if (!dev_check(w, c >= 0 && c < w.cand_cap, 13, c, w.cand_cap))
            continue;
        const Shape A = load_shape(w, w.cand_a[c]), B = load_shape(w, w.cand_b[c]);
        v3 pa, pb, nn;
        int iters = 0;
        const int r =
            epa_tiny(w, S, t, A, B, reinterpret_cast<const float *>(w.s_k + 9 * (size_t)c), pa, pb, nn, iters);
        const int pidx = w.cand_pidx[c];
        if (dev_check(w, pidx >= 0 && pidx < w.n_words * 32, 11, pidx, (long long)w.n_words * 32))
            w.epa_hist[pidx] = (unsigned char)(r == EPA_OVERFLOW ? 255 : iters);
        if (r == EPA_OVERFLOW)
            escalate(w, c, false);
        else
            write_result(w, c, r, pa, pb, nn);
    }
}

// Tier 2: one warp per queued candidate, polytope of up to 256 faces in shared memory, from
// the GJK simplex the GJK pass stored with the candidate. Dynamic shared memory: one EpaFast
// per warp.
template <int WARPS> __global__ void __launch_bounds__(WARPS * 32) k_epa_medium(DevWorld w)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    EpaFast *epa = reinterpret_cast<EpaFast *>(smem_raw);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    EpaFast &E = epa[wid];
    const int n = min(w.work_counter[5], w.med_cap);
    for (;;)
    {
        int q = 0;
        if (lane == 0)
            q = atomicAdd(w.work_counter + 6, 1);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= n)
            break;
        const int cc = w.med_cand[q];
        const Shape A = load_shape(w, w.cand_a[cc]), B = load_shape(w, w.cand_b[cc]);
        const float *sq = reinterpret_cast<const float *>(w.s_k + 9 * (size_t)cc);
        GV g[4];
        for (int i = 0; i < 4; ++i)
        {
            g[i].p = mk3(sq[9 * i], sq[9 * i + 1], sq[9 * i + 2]);
            g[i].sa = mk3(sq[9 * i + 3], sq[9 * i + 4], sq[9 * i + 5]);
            g[i].sb = mk3(sq[9 * i + 6], sq[9 * i + 7], sq[9 * i + 8]);
        }
        v3 pa, pb, nn;
        int4 ovf;
        int r = epa_run(w, E, A, B, g[0], g[1], g[2], g[3], pa, pb, nn, lane, ovf);
        __syncwarp();
        int qo = -1;
        if (lane == 0)
        {
            if (r == EPA_OVERFLOW)
                qo = escalate(w, cc, true);
            else
                write_result(w, cc, r, pa, pb, nn);
        }
        qo = __shfl_sync(0xffffffffu, qo, 0);
        if (qo >= 0 && qo < kHandoverSlots)
            handover_put(w, E, qo, ovf, lane);
        __syncwarp();
    }
}



// ---------------------------------------------------------------------------------------
// The fused per-scene step (NANS_WORLD_FUSED_STEP): after the sweep, one launch in which a
// block of kSceneThreads threads takes a scene at a time (largest first) and runs its whole
// detect-and-solve sequence, each phase on the block:
//   (1) the cull: the scene's pairs in the reference's order (code/nans.cpp:1355-1535), kept
//       when their inflated boxes meet (k_cull_mask's test), compacted in order by block scans
//       into the scene's own slots of the pair space (from sc_word0 * 32: the candidate
//       buffers of such a world hold every pair, so no scan across scenes is needed);
//   (2) GJK, one thread per candidate, every EvolveSimplex call in one run;
//   (3) EPA per hit on the per-thread polytope (epa_tiny);
//   (4) the EPAs that outgrew it, one per warp on the warp tier's polytope (epa_run);
//   (5) the solve (solve_scene), unless an EPA outgrew the warp tier: that pair goes to the
//       block- and grid-wide tiers as in the staged step and its scene to the late solve pass.
//       In a CUDA graph those launches sit in a conditional node, which the launch's last block
//       to finish opens only when a scene went late.
// The device functions are the staged kernels' own, so the results are the same bit for bit.
// Every value the phases read from global memory was written by an earlier launch (the sweep)
// or by the same block before a barrier.
// ---------------------------------------------------------------------------------------
constexpr int kSceneThreads = kTinyThreads; // the per-thread polytopes' shared-memory layout
static_assert(kSceneThreads % 32 == 0 && kSceneThreads <= kWaveChunk, "scene step block size");
// the block's dynamic shared memory stays within the 48 KB a launch gets without an opt-in
static_assert(sizeof(TinySmem) <= 48 * 1024 && (kSceneThreads / 32) * sizeof(EpaFast) <= 48 * 1024 &&
                  (size_t)(kSceneStepMaxBodies + 1) * 2 * sizeof(float4) <= 48 * 1024 &&
                  4 * kWaveChunk * sizeof(int) + kSceneStepMaxBodies * sizeof(int) <= 48 * 1024,
              "scene step shared memory");

size_t scene_step_smem(size_t solve_bytes)
{
    return std::max(std::max(sizeof(TinySmem), (size_t)(kSceneThreads / 32) * sizeof(EpaFast)), solve_bytes);
}

__global__ void __launch_bounds__(kSceneThreads) k_scene_step(DevWorld w, float dt, int all_pairs,
                                                               cudaGraphConditionalHandle cond, int signal)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TinySmem &S = *reinterpret_cast<TinySmem *>(smem_raw);
    EpaFast *const epa = reinterpret_cast<EpaFast *>(smem_raw);
    float4 *const s_dyn = reinterpret_cast<float4 *>(smem_raw);
    __shared__ int sh[32];
    __shared__ int s_q, s_nq, s_nw, s_late, s_maxw;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (;;)
    {
        if (tid == 0)
        {
            s_q = atomicAdd(w.work_counter + 14, 1);
            s_nq = 0;
            s_nw = 0;
            s_late = 0;
        }
        __syncthreads();
        const int q = s_q;
        if (q >= w.n_scenes)
            break;
        const int s = w.sc_order[q];
        const int c0 = w.sc_cube0[s], nc = w.sc_nc[s], ns = w.sc_ns[s];
        const long long np = scene_pair_count(nc, ns);
        const int cb = w.sc_word0[s] * 32;
        // (1) the cull, eight consecutive pairs a thread between the block scans
        int nk = 0;
        for (long long base = 0; base < np; base += 8 * kSceneThreads)
        {
            const long long k0 = base + 8ll * tid;
            int t0 = 0, i0 = 0, j0 = 0;
            unsigned m = 0u;
            if (k0 < np)
            {
                decode_pair(k0, nc, ns, t0, i0, j0);
                const int cnt = (int)min(8ll, np - k0);
                for (int o = 0; o < cnt; ++o)
                {
                    int type, i, j, a, b;
                    pair_after(k0, nc, ns, t0, i0, j0, o, type, i, j);
                    pair_ids(w, s, c0, nc, type, i, j, a, b);
                    bool keep = true;
                    if (!all_pairs)
                    {
                        const float4 la = __ldg(w.box_lo + a), ha = __ldg(w.box_hi + a);
                        const float4 lb = __ldg(w.box_lo + b), hb = __ldg(w.box_hi + b);
                        keep = la.x <= hb.x && lb.x <= ha.x && la.y <= hb.y && lb.y <= ha.y && la.z <= hb.z &&
                               lb.z <= ha.z;
                    }
                    if (keep)
                        m |= 1u << o;
                }
            }
            int tot;
            int pos = cb + nk + block_scan_excl(__popc(m), sh, &tot);
            while (m)
            {
                const int o = __ffs(m) - 1;
                m &= m - 1u;
                int type, i, j, a, b;
                pair_after(k0, nc, ns, t0, i0, j0, o, type, i, j);
                pair_ids(w, s, c0, nc, type, i, j, a, b);
                if (dev_check(w, pos < w.cand_cap, 20, pos, w.cand_cap))
                {
                    w.cand_a[pos] = a;
                    w.cand_b[pos] = b;
                    w.cand_meta[pos] = (s << 3) | type;
                    w.cand_pidx[pos] = cb + (int)(k0 + o);
                }
                ++pos;
            }
            nk += tot;
        }
        const int ce = min(cb + nk, w.cand_cap);
        if (tid == 0)
        {
            w.cand_begin[s] = cb;
            w.cand_end[s] = ce;
            w.scene_late[s] = 0;
        }
        __syncthreads(); // the last chunk's candidates, written after its scan
        // (2) GJK; the hits' simplices go to their s_k slots and the hits to s_order[cb ..)
        for (int c = cb + tid; c < ce; c += kSceneThreads)
        {
            const Shape A = load_shape(w, w.cand_a[c]), B = load_shape(w, w.cand_b[c]);
            const bool ra = A.npts == 8, rb = B.npts == 8;
            Verts8 VA, VB;
            if (ra)
                load_verts8(w.verts, A.off, VA);
            if (rb)
                load_verts8(w.verts, B.off, VB);
            GV s0 = {}, s1 = {}, s2 = {}, s3 = {};
            int n = 0, it = 0;
            const int g = gjk_from_with(RegSupport{w.verts, A, B, ra, rb, VA, VB}, A, B, s0, s1, s2, s3, n, it, 65);
            if (g == G_FOUND)
            {
                store_simplex(w, c, s0, s1, s2, s3);
                w.s_order[cb + atomicAdd(&s_nq, 1)] = c;
            }
            else
                w.hit[c] = 0;
        }
        __syncthreads();
        // (3) per-thread EPA; the EPAs that outgrow its polytope go to s_wave[cb ..)
        const int nq = s_nq;
        for (int i = tid; i < nq; i += kSceneThreads)
        {
            const int c = w.s_order[cb + i];
            if (!dev_check(w, c >= cb && c < ce, 21, c, ce))
                continue;
            const Shape A = load_shape(w, w.cand_a[c]), B = load_shape(w, w.cand_b[c]);
            v3 pa, pb, nn;
            int iters = 0;
            const int r =
                epa_tiny(w, S, tid, A, B, reinterpret_cast<const float *>(w.s_k + 9 * (size_t)c), pa, pb, nn, iters);
            w.epa_hist[w.cand_pidx[c]] = (unsigned char)(r == EPA_OVERFLOW ? 255 : iters);
            if (r == EPA_OVERFLOW)
            {
                w.hit[c] = 0;
                atomicAdd(w.epa_stats + 6, 1u);
                w.s_wave[cb + atomicAdd(&s_nw, 1)] = c;
            }
            else
                write_result(w, c, r, pa, pb, nn);
        }
        __syncthreads(); // the per-thread polytopes' memory becomes the warps' polytopes
        // (4) warp tier, from the simplex the GJK phase stored
        const int nw = s_nw;
        for (int i = wid; i < nw; i += kSceneThreads / 32)
        {
            EpaFast &E = epa[wid];
            int cc = w.s_wave[cb + i];
            if (!dev_check(w, cc >= cb && cc < ce, 22, cc, ce))
                cc = -1;
            if (cc < 0)
                continue;
            const Shape A = load_shape(w, w.cand_a[cc]), B = load_shape(w, w.cand_b[cc]);
            const float *sq = reinterpret_cast<const float *>(w.s_k + 9 * (size_t)cc);
            GV g[4];
            for (int v = 0; v < 4; ++v)
            {
                g[v].p = mk3(sq[9 * v], sq[9 * v + 1], sq[9 * v + 2]);
                g[v].sa = mk3(sq[9 * v + 3], sq[9 * v + 4], sq[9 * v + 5]);
                g[v].sb = mk3(sq[9 * v + 6], sq[9 * v + 7], sq[9 * v + 8]);
            }
            v3 pa, pb, nn;
            int4 ovf;
            const int r = epa_run(w, E, A, B, g[0], g[1], g[2], g[3], pa, pb, nn, lane, ovf);
            __syncwarp();
            int qo = -1;
            if (lane == 0)
            {
                if (r == EPA_OVERFLOW)
                {
                    qo = escalate(w, cc, true);
                    s_late = 1;
                }
                else
                    write_result(w, cc, r, pa, pb, nn);
            }
            qo = __shfl_sync(0xffffffffu, qo, 0);
            if (qo >= 0 && qo < kHandoverSlots)
                handover_put(w, E, qo, ovf, lane);
            __syncwarp();
        }
        __syncthreads(); // the warps' polytopes' memory becomes the solver's
        // (5) the solve, unless a pair of the scene went to the large tiers (the late pass)
        if (!s_late)
            solve_scene<false>(w, s, dt, s_dyn, sh, s_maxw);
        __syncthreads();
    }
    // In a graph, the last block to finish opens the conditional node of the large tiers and the
    // late pass when a scene went late (work counter 13, counted by escalate); one call per launch.
    if (signal && tid == 0)
    {
        __threadfence();
        if (atomicAdd(w.work_counter + 15, 1) == (int)gridDim.x - 1 && atomicAdd(w.work_counter + 13, 0) > 0)
            cudaGraphSetConditional(cond, 1u);
    }
}

// The fused step's launch: resident blocks on every SM, no more than the world's scenes.
void launch_scene_step(const DevWorld &w, size_t solve_bytes, float dt, int all_pairs, cudaStream_t st,
                       cudaGraphConditionalHandle cond, int signal)
{
    const size_t smem = scene_step_smem(solve_bytes);
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_scene_step, kSceneThreads, smem);
    const int grid = std::max(1, std::min(w.n_scenes, std::max(1, per) * std::max(1, w.sm_count)));
    k_scene_step<<<grid, kSceneThreads, smem, st>>>(w, dt, all_pairs, cond, signal);
}

static size_t medium_smem(int warps) { return sizeof(EpaFast) * (size_t)warps; }

// The warp tier's dynamic shared memory beyond 48 KB. The attribute belongs to the current
// device's context, so every world sets it for its own device when it is created.
int narrow_kernel_attrs()
{
    return (int)cudaFuncSetAttribute(k_epa_medium<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)medium_smem(4));
}

int narrow_blocks_per_sm(int warps)
{
    (void)warps;
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_gjk, kGjkThreads, 0);
    return per;
}

// Resident blocks of the warp-per-pair GJK on every SM, no more than the pairs need.
static int gjk_warp_grid(const DevWorld &w)
{
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_gjk_warp, kGjkWarpThreads, 0);
    const long long need = (w.pair_total + kGjkWarpThreads / 32 - 1) / (kGjkWarpThreads / 32);
    return (int)std::max(1LL, std::min<long long>((long long)std::max(1, per) * w.sm_count, need));
}

int epa_tiny_grid(int sm_count)
{
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_epa_tiny, kTinyThreads, 0);
    return std::max(1, per) * std::max(1, sm_count);
}

void launch_narrow_tiny(int grid, cudaStream_t st, const DevWorld &w)
{
    if (w.gjk_warp)
        k_gjk_warp<<<gjk_warp_grid(w), kGjkWarpThreads, 0, st>>>(w);
    else
    {
        k_gjk<<<grid, kGjkThreads, 0, st>>>(w);
        k_gjk_long<<<grid, kGjkThreads, 0, st>>>(w);
    }
    k_epa_tiny<<<w.tiny_blocks, kTinyThreads, 0, st>>>(w);
}

int tier_priority()
{
    static int prio = 1;
    if (prio > 0)
    {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        prio = greatest;
    }
    return prio;
}

// The escalation tiers are latency-bound chains on the step's critical path; they are
// launched at the greatest priority so that their blocks are placed before those of the
// solve pass that becomes ready at the same time.
void launch_epa_medium(cudaStream_t st, const DevWorld &w)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(w.medium_blocks);
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = medium_smem(4);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = tier_priority();
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_epa_medium<4>, w);
}





} // namespace nans
