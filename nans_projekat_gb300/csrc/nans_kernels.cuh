// Kernel declarations and launch constants shared by the step kernels and the host runtime.
#pragma once
#include "nans_internal.cuh"

namespace nans
{

void set_last_error(const char *msg);

// k_sweep flags
enum SweepFlags
{
    SW_APPLY_VEL = 1,   // apply the previous step's P += dt*V, A += dt*W first
    SW_INTEGRATE = 2,   // RK4 + vertices + AABB
    SW_MODEL_INPUT = 4, // take Model from the uploaded records instead of rebuilding it
    SW_FORCES = 8,      // read (then clear) external forces and torques
    SW_CLEAR_COUNTERS = 16, // zero the work counters first (the fused step, which has no memset)
};

// Global body ids of pair (type, i, j) of scene s whose cubes start at c0 (nc cubes).
__device__ __forceinline__ void pair_ids(const DevWorld &w, int s, int c0, int nc, int type, int i, int j, int &a,
                                         int &b)
{
    const int s0 = c0 + nc;
    a = type_a_is_sphere(type) ? s0 + i : c0 + i;
    if (type_b_is_floor(type))
        b = w.n_dyn + s;
    else
        b = type_b_is_sphere(type) ? s0 + j : c0 + j;
}

constexpr int kCullThreads = 256;
constexpr int kCullTileThreads = 256;
constexpr int kRestChunksPerTask = 64; // 32-pair chunks of non-cube-cube pairs per cull task
constexpr int kSolveLateThreads = 128; // solver blocks of the second pass (late scenes)
constexpr int kSolveLateBlocksPerSm = 6; // second-pass solver blocks per SM (registers allow six)
constexpr int kWaveChunk = 256;     // solver: candidates compacted and labelled per chunk
constexpr size_t kSolveSmemMax = 200 * 1024; // solver: dynamic shared memory per block, at most
constexpr int kMediumBlocksPerSm = 2;    // warp-tier EPA blocks per SM (shared memory allows three)
constexpr int kSceneStepMaxBodies = 1024; // fused per-scene step: bodies per scene, at most

// EPA capacities. Vertices: the GJK tetrahedron plus one support per EPA iteration (at most
// 65, code/nans.cpp:804). Faces grow by two per iteration on a convex polytope, but the
// reference's polytope is not always convex: with bodies flung to large coordinates the
// supports repeat existing vertices, faces degenerate (NaN normals, never removed) and the
// list keeps growing, at times geometrically, for all 65 iterations. On the 16,384-scene
// stack workload ~1.3 EPAs in a thousand outgrow 12 vertices / 20 faces, ~14 in a million
// exceed 128 faces (nearly all of them stay within 256), and the largest met so far (scene
// 10198, step 135) reaches 485,688 faces and a 139,111-edge horizon (the reference's own
// algorithm needs 334 s of one CPU core for it). Tier 1 runs EPA per thread (12 vertices, 20
// faces, 12 edges); tier 2 per warp in shared memory (256 faces, a 64-edge horizon); tier 3
// per block in a global-memory arena of 32,768 faces, two blocks per SM; tier 4 on the whole
// grid (cooperative launch) in an arena of 8,388,608 faces and 4,194,304 horizon edges.
// Beyond that the pair gets no contact and the event is counted (NANS_ERR_EPA_CAPACITY in
// strict worlds).
constexpr int kEpaMaxVerts = 72;
constexpr int kEpaFastFaces = 256;
constexpr int kEpaFastEdges = 64;
constexpr int kBlockFaces = 1 << 15;   // tier 3 arena (two blocks per SM)
constexpr int kBlockEdges = 1 << 15;
constexpr int kBlockPerSm = 2;
constexpr int kGiantFaces = 1 << 23;   // tier 4 arena (one, the whole grid per EPA)
constexpr int kGiantEdges = 1 << 22;
constexpr int kEpaOverflowCap = 65536; // tier-3 EPAs queued per step
constexpr int kHandoverSlots = 1024;   // tier-3 queue entries that can carry the warp tier's state

// The warp tier's polytope at the start of the iteration that outgrew it, for the block tier to
// resume (queue entry q < kHandoverSlots of the tier-3 queue): hdr = (iteration, stale, face
// count or -1 when there is no state, vertex count).
struct EpaHandover
{
    int hdr[4];
    float px[kEpaMaxVerts], py[kEpaMaxVerts], pz[kEpaMaxVerts];
    float ax[kEpaMaxVerts], ay[kEpaMaxVerts], az[kEpaMaxVerts];
    float bx[kEpaMaxVerts], by[kEpaMaxVerts], bz[kEpaMaxVerts];
    int vid[kEpaMaxVerts];
    unsigned fidx[kEpaFastFaces];
    float fnx[kEpaFastFaces], fny[kEpaFastFaces], fnz[kEpaFastFaces], fd[kEpaFastFaces];
};
constexpr int kGiantQueueCap = 4096;   // tier-4 EPAs queued per step
constexpr long long kBarrierSpins = 1ll << 24; // grid barrier polls (64 ns sleeps) before it gives up
constexpr long long kBarrierSpinsTest = 1ll << 12;
constexpr int kWorkCounters = 16;
constexpr int kEpaMediumCap = 1 << 20; // tier-2 EPAs queued per step

__global__ void k_sweep(DevWorld w, float pending_dt, float dt, int flags);
__global__ void k_unpack(DevWorld w, const float *rec_cube, const float *rec_sphere, const float *rec_floor,
                         const int *body_rec, int mode, float4 *prm_out, float4 *model_out);
__global__ void k_pack(DevWorld w, float *rec_cube, float *rec_sphere, float *rec_floor, const int *body_rec,
                       const float2 *size_moi, int vertices_valid);

__global__ void k_sincos(const float *x, float *s, float *c, int n);
__global__ void k_state_in(DevWorld w, const float *stage, const int *body_rec, int n_cubes, int mask);
__global__ void k_state_out(DevWorld w, float *stage, const int *body_rec, int n_cubes, int mask);

__global__ void k_cull_mask(DevWorld w, int all_pairs);
__global__ void k_cull_scan(DevWorld w, int nblocks);
__global__ void k_cull_write(DevWorld w);
__global__ void k_cull_tiles(DevWorld w);
__global__ void k_cull_rest(DevWorld w);
__global__ void k_cull_count(DevWorld w);

int narrow_blocks_per_sm(int warps);
size_t epa_big_bytes();
size_t epa_block_bytes();
size_t epa_giant_scratch_bytes();
int giant_grid(int sm_count);
int launch_narrow_big(cudaStream_t st, const DevWorld &w); // returns a cudaError_t
void launch_narrow_tiny(int grid, cudaStream_t st, const DevWorld &w);
int epa_tiny_grid(int sm_count);   // resident blocks of the per-thread EPA on sm_count SMs
int narrow_kernel_attrs();         // per-device kernel attributes (cudaError_t), set at world creation
int large_kernel_attrs();
void launch_epa_medium(cudaStream_t st, const DevWorld &w);
// the fused per-scene step (cull, GJK, per-thread and warp-tier EPA, solve) over every scene;
// solve_bytes is the solver's dynamic shared memory (solve_smem)
// cond: the handle of the graph's conditional node that runs the large EPA tiers and the late
// solve pass, set to 1 by the launch when a scene went late (signal = 0 outside a graph)
void launch_scene_step(const DevWorld &w, size_t solve_bytes, float dt, int all_pairs, cudaStream_t st,
                       cudaGraphConditionalHandle cond, int signal);
int tier_priority(); // the device's greatest stream priority
int solve_threads(int max_scene_bodies);
// scenes of up to this many bodies solve on a shared-memory copy of their velocities
int solve_cache_bodies(int max_scene_bodies);
// the solver's dynamic shared memory (chunk arrays and per-body waves, or the velocity copy)
size_t solve_smem(int max_scene_bodies, int cache);
int render_scene(const DevWorld &w, int scene, const float eye[3], const float target[3], float fov_deg, int width,
                 int height, unsigned long long *fb, unsigned char *rgb, cudaStream_t st);
// the solver kernels' dynamic shared memory limit (cudaFuncAttributeMaxDynamicSharedMemorySize)
int solve_kernel_attrs(const DevWorld &w, int smem);
void launch_solve(const DevWorld &w, int grid, int threads, size_t smem, cudaStream_t st, float dt, int pass);
__global__ void k_pairs_out(DevWorld w, int scene, float *out_rec, int cap, int *count);

// One step of the differentiable rollout's tape. Contact data is stored by solve slot: slot
// cand_begin[s] + i holds the i-th contact of scene s in wave order, so wave v is the
// contiguous slot range cb + [v == 1 ? 0 : wend[cb + v - 2], wend[cb + v - 1]).
struct TapeStep
{
    int *a, *b, *type;        // per slot: bodies and pair type
    float4 *k;                // per slot: 9 float4 of contact constants (k_solve layout)
    float4 *fwd;              // per slot: (JdVn, JdVt1, JdVt2, flags), (dn, dt1, dt2, Ln)
    int *wend;                // per scene, from its first slot: end of each wave (k_solve's s_wcnt)
    int *cand_begin, *maxw;   // per scene
    float4 *v_pre, *w_pre;    // per dynamic body: V, W before this step's RK4
    float4 *f_ext, *t_ext;    // per dynamic body: external force / torque of this step, or null
    int n;                    // slots (candidate pairs of the step)
};

// Adjoint accumulators, per dynamic body (float4 xyz) / per scene.
struct AdjointBufs
{
    const float4 *gP, *gA;    // dL/d(final position / angles); constant through the rollout
    float4 *gV, *gW;          // in: dL/d(final V, W); out: dL/d(initial V, W)
    float *g_invm, *g_invi;   // accumulated dL/d(1/m), dL/d(1/I)
    float *g_z, *g_zw;        // accumulated dL/dz, dL/dzw of the RK4 closed form
    float *g_mass;            // out: dL/dm (moment of inertia proportional to mass)
    float *g_cr, *g_cf;       // out, per scene: dL/d restitution, dL/d friction
    int *err;                 // [0] first inconsistency found (0 none), [1..3] its indices
};

int adjoint_threads();
__global__ void k_tape_copy(DevWorld w, TapeStep t);
__global__ void k_adjoint(DevWorld w, const TapeStep *steps, int nsteps, float h, AdjointBufs g);
__global__ void k_rec_to_body(const float *in_rec, const int *body_rec, int n_cubes, int n_dyn, float4 *out);
__global__ void k_body_to_rec(const float4 *in, const float *in_scalar, const int *body_rec, int n_cubes, int n_dyn,
                              float *out_rec, int comps);

} // namespace nans
