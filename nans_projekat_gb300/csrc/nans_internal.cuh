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
#include "nans_pairs.cuh"

namespace nans
{

// device status bits (or'ed into DevWorld::status)
enum StatusBits
{
    ST_EPA_FACES = 1u << 0,      // an EPA outgrew the large-polytope buffers (pair: no contact)
    ST_EPA_EDGES = 1u << 1,      // EPA horizon edge buffer full
    ST_CANDIDATES = 1u << 2,     // candidate capacity exceeded
    ST_EPA_EMPTY = 1u << 3,      // EPA face list emptied (reference would read a stale face)
    ST_SOLVER_BODIES = 1u << 4,  // scene too large for the solver's wave table
    ST_EPA_TIMEOUT = 1u << 5,    // a giant-tier grid barrier timed out (pair: no contact)
    ST_CHECK = 1u << 6,          // a device bounds check failed and the access was skipped
                                 // (the first failure is recorded in DevWorld::check)
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
    const int *sc_rank;       // per scene: its position in sc_order
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
    const int4 *tiles;                  // cube-cube cull tiles: (scene, row block, column block)
    int n_tiles;
    const int4 *rest_tasks;             // cull of the other pairs: (scene, first chunk, chunks)
    int n_rest_tasks;
    const int *word_scene;              // scene of each mask word
    int n_words;
    int *block_hits;                    // per cull block: culled pairs, then candidate offset
    int *cull_total;                    // candidates before the capacity clamp
    int *cull_max;                      // largest cull_total since the host last cleared it
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
                                        // [8] giant-EPA queue length, per-thread EPA queue
                                        // (s_order): [9] its long part (from the back), [10]
                                        // the others, [11] its head; [12] late-solve head,
                                        // [13] late-scene count; fused step: [14] its scene
                                        // head, [15] its blocks done
    int med_cap;                        // warp-EPA queue capacity
    int *med_cand;                      // candidates queued for the warp tier
    int2 *long_cand;                    // candidates whose GJK needs the long pass: (c, n | it << 8)
    int medium_blocks;                  // warp-tier grid
    int tiny_blocks;                    // per-thread EPA grid (resident blocks on every SM)
    int gjk_warp;                       // 1: GJK with one warp per pair (NANS_WORLD_GJK_WARP)
    int sm_count;
    int ovf_cap;                        // block-EPA queue capacity
    int *ovf_cand;                      // candidates queued for the block tier
    unsigned char *blk_arena;           // block-tier polytope buffers, one per block
    int blk_blocks;                     // block-tier grid
    int blk_face_limit;                 // block-tier face capacity (lowered only by a test flag)
    long long barrier_spins;            // grid-wide tier: polls before a barrier wait gives up
    unsigned barrier_extra;             // grid-wide tier: arrivals beyond the grid a barrier waits
                                        // for (0; 1 only under a test flag, an arrival that never
                                        // comes)
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
    int *s_order, *s_wave, *s_wcnt;     // s_order doubles as the narrowphase's EPA queue
    int4 *s_ids;                        // per solve slot (wave order): candidate, body A,
                                        // body B (-1 - B when B is the floor), pair-space index
    float4 *s_k;                        // per solve slot: 9 float4 of contact constants; during
                                        // the narrowphase, per candidate: the GJK simplex of a hit
    int *s_last;                        // per body: last wave touching it
    int solve_cache;                    // scenes of up to this many bodies solve their waves on
                                        // a shared-memory copy of their velocities
    float4 *s_fwd;                      // adjoint tape of the solve (2 float4 per slot) or null
    // warm starting (null when off): per pair of the pair space (index 32 * word + bit) the
    // accumulators (sn, st1, st2) of its last solve and that solve's step number
    float4 *warm;
    int *warm_step;                     // step counter, advanced by the sweep
    int *cand_pidx;                     // per candidate: its pair-space index
    unsigned char *epa_hist;            // per pair-space index: iterations of its last per-thread EPA
    int *s_maxw;                        // per scene: highest wave of the last solve, or null
    unsigned *status;
    int *check;                         // first failed bounds check: site, index, bound
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

// A bounds check that records the first failure (site, index, bound) and lets the caller skip
// the access instead of faulting.
__device__ __forceinline__ bool dev_check(const DevWorld &w, bool ok, int site, long long idx, long long bound)
{
    if (ok)
        return true;
    if (!(atomicOr(w.status, (unsigned)ST_CHECK) & (unsigned)ST_CHECK))
    {
        w.check[0] = site;
        w.check[1] = (int)idx;
        w.check[2] = (int)bound;
    }
    return false;
}

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

} // namespace nans
