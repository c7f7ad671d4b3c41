// Internal device-side view of a world and the helpers shared by the step kernels.
//
// HBM layout (structure of arrays; one world = S independent scenes):
//   bodies  [0, n_dyn)            dynamic bodies, scene-major; in each scene the cubes
//                                 (boxes and convex hulls) come first, then the spheres
//   bodies  [n_dyn, n_dyn + S)    one static ground box per scene ("floor")
//   pos[b]  float4 (Position, radius)   radius = 0 for cubes and floors
//   ang[b]  float4 (Angles in the reference's degree convention, 0)
//   vel[b], omg[b]  float4 (V, 0), (W, 0)
//   frc[b], trq[b]  float4 external force / torque (read and cleared while force_pending)
//   prm[b]  float4 (Mass, (float)(1.0/(double)Mass), 1.0f/Mass, 1.0f/MOI)
//   scl[b]  float4 (model scale xyz, 0)
//   shape[b] int4 (vert_off in floats, npts, local_off in floats or -1 for the unit-cube
//                  corners, 0); npts = 0 marks a sphere
//   verts   world-space hull vertices, 3 floats each; each shape's block holds whole groups
//           of four vertices (12 floats, 16-byte aligned) because supports read group-wise
//   box_lo/box_hi[b] float4 conservative AABB (xyz)
// Candidate pairs are stored in the reference's enumeration order (scene-major, then
// CC, CF, SF, CS, SS as in code/nans.cpp:1355-1535).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <cfloat>
#include "nans_math.cuh"

namespace nans
{

enum PairType
{
    T_CC = 0,
    T_CS = 1,
    T_CF = 2,
    T_SS = 3,
    T_SF = 4
};

// device status bits (or'ed into DevWorld::status)
enum StatusBits
{
    ST_EPA_FACES = 1u << 0,      // an EPA outgrew the large-polytope buffers (pair: no contact)
    ST_EPA_EDGES = 1u << 1,      // EPA horizon edge buffer full
    ST_CANDIDATES = 1u << 2,     // candidate capacity exceeded
    ST_EPA_EMPTY = 1u << 3,      // EPA face list emptied (reference would read a stale face)
    ST_SOLVER_BODIES = 1u << 4,  // scene too large for the solver's wave table
    ST_EPA_TIMEOUT = 1u << 5,    // a giant-tier grid barrier timed out (pair: no contact)
};

struct EpaHandover; // nans_kernels.cuh

struct DevWorld
{
    int n_scenes;
    int n_dyn;
    int n_all;
    // per scene
    const int *sc_cube0;      // global id of the scene's first cube
    const int *sc_nc;         // cubes (incl. hulls)
    const int *sc_ns;         // spheres
    const int *sc_word0;      // first pair-mask word of the scene (n_scenes + 1 entries)
    const float *sc_cr;
    const float *sc_cf;
    const int *sc_iters;
    const int *sc_order;      // scenes by decreasing body count (solver queue order)
    // per body
    float4 *pos, *ang, *vel, *omg, *frc, *trq;
    const float4 *prm, *scl;
    const int4 *shape;
    const float *local_pts;
    float *verts;
    const float4 *model_in;   // 4 float4 (columns) per body, used when MODEL_FROM_INPUT
    float4 *box_lo, *box_hi;
    const int *body_scene;
    // candidate pairs
    long long pair_total;
    int cand_cap;
    int *cand_a, *cand_b, *cand_meta; // meta = scene << 3 | type
    int *n_cand;                        // device counter
    unsigned *pair_mask;                // one bit per pair, words aligned per scene
    const int *word_scene;              // scene of each mask word
    int n_words;
    int *block_hits;                    // per cull block: culled pairs, then candidate offset
    int *cull_total;                    // candidates before the capacity clamp
    int *cand_begin, *cand_end;         // per scene candidate range
    int *scene_late;                    // per scene: 1 if a candidate went beyond the per-thread
                                        // EPA tier (solved after those tiers)
    int *late_list;                     // the late scenes, in no particular order
    // narrowphase output, per candidate
    int *hit;
    float4 *c_pa, *c_pb, *c_n;
    int *work_counter;                  // [0] narrowphase head, [1] solver head, [2] block-EPA
                                        // head, [3] block-EPA queue length, [5] warp-EPA queue
                                        // length, [6] warp-EPA head, [7] long-GJK queue length,
                                        // [8] giant-EPA queue length, [9] giant-EPA head,
                                        // [10] per-thread EPA queue length (queue: s_order),
                                        // [11] per-thread EPA head, [12] late-solve head,
                                        // [13] late-scene count
    int med_cap;                        // warp-EPA queue capacity
    int *med_cand;                      // candidates queued for the warp tier
    int2 *long_cand;                    // candidates whose GJK needs the long pass: (c, n | it << 8)
    int medium_blocks;                  // warp-tier grid
    int ovf_cap;                        // block-EPA queue capacity
    int *ovf_cand;                      // candidates queued for the block tier
    unsigned char *blk_arena;           // block-tier polytope buffers, one per block
    int blk_blocks;                     // block-tier grid
    int blk_face_limit;                 // block-tier face capacity (lowered only by a test flag)
    int giant_cap;                      // giant-EPA queue capacity
    EpaHandover *handover;              // warp-tier states for the block tier (kHandoverSlots)
    int4 *giant_cand;                   // queued for the giant tier: candidate, state (it | bank << 8 |
                                        // stale << 9 | block << 10), faces, vertices
    unsigned char *epa_arena;           // giant-tier polytope buffers (one, grid-wide)
    unsigned char *giant_scratch;       // giant-tier group table, team scratch and barrier
    int giant_blocks;                   // giant-tier grid (cooperative launch)
    unsigned *epa_stats;                // [0] max faces, [1] max horizon edges, [2] block- and
                                        // giant-tier EPAs, [3] overflowing candidate + 1, [4] its
                                        // scene + 1, [5] EPAs that outgrew the giant tier, [6]
                                        // EPAs escalated to the warp tier, [7] EPAs escalated to
                                        // the giant tier
    // solver scratch, per candidate slot
    int *s_order, *s_wave, *s_perm, *s_wcnt; // s_order doubles as the narrowphase's EPA queue
    float4 *s_k;                        // 9 float4 of per-contact constants; during the
                                        // narrowphase the GJK simplex of a hit
    int *s_last;                        // per body: last wave touching it
    float4 *s_fwd;                      // adjoint tape of the solve (2 float4 per slot) or null
    // warm starting (null when off): per pair of the pair space (index 32 * word + bit) the
    // accumulators (sn, st1, st2) of its last solve and that solve's step number
    float4 *warm;
    int *warm_step;                     // step counter, advanced by the sweep
    int *cand_pidx;                     // per candidate: its pair-space index
    unsigned char *epa_hist;            // per pair-space index: iterations of its last per-thread EPA
    int *s_maxw;                        // per scene: highest wave of the last solve, or null
    unsigned *status;
};

// ------------------------------------------------------------------------------------
// support maps (code/nans.cpp:409-461): argmax of dot(vertex, d) starting at -FLT_MAX with
// a strict '>' so the first maximum wins and (0,0,0) is returned when nothing beats it.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ v3 hull_support(const float *__restrict__ verts, int off, int npts, v3 d)
{
    float best = -FLT_MAX;
    v3 r = mk3(0.0f, 0.0f, 0.0f);
    const float4 *q = reinterpret_cast<const float4 *>(verts + off);
    int groups = (npts + 3) >> 2;
    for (int g = 0; g < groups; ++g)
    {
        float4 q0 = __ldg(q + 3 * g), q1 = __ldg(q + 3 * g + 1), q2 = __ldg(q + 3 * g + 2);
        v3 v[4] = {mk3(q0.x, q0.y, q0.z), mk3(q0.w, q1.x, q1.y), mk3(q1.z, q1.w, q2.x),
                   mk3(q2.y, q2.z, q2.w)};
#pragma unroll
        for (int t = 0; t < 4; ++t)
        {
            if (4 * g + t < npts)
            {
                float dist = dot3(v[t], d);
                if (dist > best)
                {
                    best = dist;
                    r = v[t];
                }
            }
        }
    }
    return r;
}

// GetSphereSupport (code/nans.cpp:432-438): P + r * normalize(d)
__device__ __forceinline__ v3 sphere_support(v3 p, float radius, v3 d)
{
    return p + radius * normalize3(d);
}

struct Shape
{
    v3 p;        // position (for the GJK initial direction and sphere support)
    float radius;
    int off, npts; // hull vertices; npts == 0 -> sphere
};

__device__ __forceinline__ Shape load_shape(const DevWorld &w, int b)
{
    Shape s;
    float4 p = __ldg(w.pos + b);
    int4 sh = __ldg(w.shape + b);
    s.p = mk3(p.x, p.y, p.z);
    s.radius = p.w;
    s.off = sh.x;
    s.npts = sh.y;
    return s;
}

__device__ __forceinline__ v3 shape_support(const float *verts, const Shape &s, v3 d)
{
    if (s.npts == 0)
        return sphere_support(s.p, s.radius, d);
    return hull_support(verts, s.off, s.npts, d);
}

struct GV
{
    v3 p, sa, sb;
};

// CalculateSupport (code/nans.cpp:463-519): Minkowski vertex SupA(d) - SupB(-d)
__device__ __forceinline__ GV minkowski_support(const float *verts, const Shape &A, const Shape &B, v3 d)
{
    GV r;
    r.sa = shape_support(verts, A, d);
    r.sb = shape_support(verts, B, -1.0f * d);
    r.p = r.sa - r.sb;
    return r;
}

// ------------------------------------------------------------------------------------
// pair-space enumeration of one scene in the reference order (code/nans.cpp:1355-1535)
// ------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ long long scene_pair_count(long long nc, long long ns)
{
    return nc * (nc - 1) / 2 + nc + ns + nc * ns + ns * (ns - 1) / 2;
}

// Largest i with row_start(i) = i*n - i*(i+1)/2 <= k, for pairs i < j < n.
__device__ __forceinline__ void tri_decode(long long k, long long n, int &i, int &j)
{
    double a = 2.0 * (double)n - 1.0;
    double disc = a * a - 8.0 * (double)k;
    long long ii = (long long)floor((a - sqrt(disc > 0.0 ? disc : 0.0)) * 0.5);
    if (ii < 0)
        ii = 0;
    if (ii > n - 2)
        ii = n - 2;
    while (ii > 0 && ii * n - ii * (ii + 1) / 2 > k)
        --ii;
    while (ii + 1 <= n - 2 && (ii + 1) * n - (ii + 1) * (ii + 2) / 2 <= k)
        ++ii;
    long long rs = ii * n - ii * (ii + 1) / 2;
    i = (int)ii;
    j = (int)(ii + 1 + (k - rs));
}

// Decodes scene-local pair index k into (type, i, j).
__device__ __forceinline__ void decode_local(long long k, int nc, int ns, int &type, int &i, int &j)
{
    long long ncc = (long long)nc * (nc - 1) / 2;
    if (k < ncc)
    {
        type = T_CC;
        tri_decode(k, nc, i, j);
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
    long long ncs = (long long)nc * ns;
    if (k < ncs)
    {
        type = T_CS;
        i = (int)(k / ns);
        j = (int)(k % ns);
        return;
    }
    k -= ncs;
    type = T_SS;
    tri_decode(k, ns, i, j);
}

// Moves to the first pair of the first non-empty region at or after `type`
// (region order CC, CF, SF, CS, SS); returns false when the scene has no such pair.
__device__ __forceinline__ bool start_region(int nc, int ns, int from, int &type, int &i, int &j)
{
    // region index of each type in enumeration order CC, CF, SF, CS, SS
    int r0 = (from == T_CC) ? 0 : (from == T_CF) ? 1 : (from == T_SF) ? 2 : (from == T_CS) ? 3 : 4;
    for (int r = r0; r < 5; ++r)
    {
        if (r == 0 && nc > 1) { type = T_CC; i = 0; j = 1; return true; }
        if (r == 1 && nc > 0) { type = T_CF; i = j = 0; return true; }
        if (r == 2 && ns > 0) { type = T_SF; i = j = 0; return true; }
        if (r == 3 && nc > 0 && ns > 0) { type = T_CS; i = 0; j = 0; return true; }
        if (r == 4 && ns > 1) { type = T_SS; i = 0; j = 1; return true; }
    }
    return false;
}

// Advances (type, i, j) to the next pair of the same scene; returns false past the end.
__device__ __forceinline__ bool advance_local(int nc, int ns, int &type, int &i, int &j)
{
    switch (type)
    {
    case T_CC:
        if (++j < nc)
            return true;
        ++i;
        j = i + 1;
        if (j < nc)
            return true;
        return start_region(nc, ns, T_CF, type, i, j);
    case T_CF:
        if (++i < nc)
        {
            j = i;
            return true;
        }
        return start_region(nc, ns, T_SF, type, i, j);
    case T_SF:
        if (++i < ns)
        {
            j = i;
            return true;
        }
        return start_region(nc, ns, T_CS, type, i, j);
    case T_CS:
        if (++j < ns)
            return true;
        j = 0;
        if (++i < nc)
            return true;
        return start_region(nc, ns, T_SS, type, i, j);
    default:
        if (++j < ns)
            return true;
        ++i;
        j = i + 1;
        return j < ns;
    }
}

__host__ __device__ __forceinline__ bool type_b_is_floor(int t) { return t == T_CF || t == T_SF; }
__host__ __device__ __forceinline__ bool type_a_is_sphere(int t) { return t == T_SS || t == T_SF; }
__host__ __device__ __forceinline__ bool type_b_is_sphere(int t) { return t == T_CS || t == T_SS; }

// Global body ids of a scene-local pair.
__device__ __forceinline__ void pair_bodies(const DevWorld &w, int scene, int type, int i, int j, int &a,
                                            int &b)
{
    int c0 = __ldg(w.sc_cube0 + scene);
    int nc = __ldg(w.sc_nc + scene);
    int s0 = c0 + nc;
    a = type_a_is_sphere(type) ? s0 + i : c0 + i;
    if (type_b_is_floor(type))
        b = w.n_dyn + scene;
    else
        b = type_b_is_sphere(type) ? s0 + j : c0 + j;
}

} // namespace nans
