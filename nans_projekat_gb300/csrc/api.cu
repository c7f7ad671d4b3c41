// Host runtime behind the C ABI (include/nans_gb300.h).
//
// A world owns one CUDA stream and every device buffer of its scenes. The step is the
// stage sequence of the reference's frame function (code/nans.cpp:1758-1762) plus the
// render code's Model rebuild, as six kernels:
//   k_sweep        IntegrateVelocities(prev) + rebuild + IntegrateForces + vertices + AABB
//   k_cull_mask / k_cull_scan / k_cull_write     ordered candidate pairs
//   k_narrow / k_narrow_big   GJK + EPA           (DetectCollisions)
//   k_solve        sequential impulses by waves   (SolveConstraints)
// The last step's IntegrateVelocities is folded into the next step's sweep, or applied by
// nans_world_download.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/nans_gb300.h"
#include "nans_kernels.cuh"

using namespace nans;

static_assert(sizeof(nans_cube) == 244, "cube record layout");
static_assert(sizeof(nans_sphere) == 148, "sphere record layout");
static_assert(sizeof(nans_contact_pair) == 96, "contact_pair record layout");

namespace
{
thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

#define CK(call)                                                                                                    \
    do                                                                                                              \
    {                                                                                                               \
        cudaError_t e_ = (call);                                                                                    \
        if (e_ != cudaSuccess)                                                                                      \
            return fail(NANS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));                         \
    } while (0)

} // namespace

// Lets other translation units of the library report through nans_last_error().
void nans::set_last_error(const char *msg) { g_err = msg; }

namespace
{
constexpr int kSweepThreads = 256;
constexpr int kTuneSteps = 20;       // timed steps per autotuner candidate
} // namespace

struct nans_world
{
    int device = 0;
    uint32_t flags = 0;
    uint32_t max_cand_req = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;   // the later EPA tiers, alongside the first solve pass
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int sm_count = 0;

    int n_scenes = 0, n_dyn = 0, n_all = 0, n_cubes = 0, n_spheres = 0;
    long long pair_total = 0;
    int cand_cap = 0;
    int cull_blocks = 0;    // one thread per pair-mask word
    int max_scene_bodies = 0;

    std::vector<void *> allocs;     // per-upload device buffers
    std::vector<void *> cand_allocs; // candidate-sized buffers
    DevWorld dw{};
    float4 *d_prm = nullptr, *d_scl = nullptr, *d_model_in = nullptr;
    int *d_body_rec = nullptr;
    float2 *d_size_moi = nullptr;
    float *d_rec_cube = nullptr, *d_rec_sphere = nullptr, *d_rec_floor = nullptr;
    float *d_pairs_out = nullptr;
    int pairs_out_cap = 0;
    int *d_small = nullptr; // [0] pair count for k_pairs_out, [1] contact count
    float4 *d_snap = nullptr;

    bool uploaded = false;
    bool pending = false;
    float pending_dt = 0.0f;
    bool model_input = false;
    bool forces_pending = false;
    long long steps_run = 0;

    int narrow_bpsm = 0;     // GJK blocks per SM (0 = occupancy limit)
    int cull_tiles = 1;      // cull by tiles (1) or one lane per pair (0)
    int gjk_cap_blocks = 1;  // GJK blocks the world's pairs can keep busy
    int solve_threads0 = 0;  // solver threads per scene, first pass (0 = by the largest scene)
    int solve_threads1 = kSolveLateThreads; // solver threads per late scene
    int solve_late_bpsm = kSolveLateBlocksPerSm; // late-scene solver blocks per SM
    int medium_bpsm = kMediumBlocksPerSm;        // warp-tier EPA blocks per SM
    int medium_cap_blocks = 1;                   // warp-tier blocks the world's pairs can keep busy
    int tune_trials = 0;
    float tune_ms = 0.0f;
    unsigned char *d_snap_hist = nullptr;
    size_t snap_n = 0, snap_hist_n = 0;  // bodies / bytes the snapshot buffers hold

    cudaGraphExec_t gexec = nullptr;    // batched path: graph of g_steps steady steps
    int g_steps = 0;
    float g_dt = 0.0f;
    int g_cfg = -1;
    cudaGraphExec_t gexec_b = nullptr;  // batched path: the same whose first step has flags gb_flags
    int gb_steps = 0, gb_flags = -1, gb_cfg = -1;
    float gb_dt = 0.0f;
    cudaGraphExec_t gexec1 = nullptr;   // plain path: graph of one step
    float g1_dt = 0.0f, g1_pdt = 0.0f;
    int g1_flags = -1, g1_cfg = -1;
    unsigned long long graph_steps_run = 0, eager_steps_run = 0; // nans_step / nans_batch_step

    // differentiable rollout: the tape lives in a chunked device arena reused across forwards
    bool tape_on = false;           // the solve records its adjoint data (s_fwd, s_maxw)
    bool fused = false;             // NANS_WORLD_FUSED_STEP: one detect-and-solve launch per step
    bool fused_conditional = true;  // its graphs put the large tiers in a conditional node
    bool tape_valid = false;        // the tape describes the rollout that led to the state
    float tape_dt = 0.0f;
    float4 *fwd_buf = nullptr;      // 2 float4 per candidate slot (in cand_allocs)
    int *d_maxw = nullptr;          // per scene (in allocs)
    std::vector<void *> tape_chunks;
    std::vector<size_t> tape_sizes;
    size_t tape_chunk = 0, tape_off = 0, tape_bytes = 0;
    std::vector<TapeStep> tape;
    TapeStep *d_tape = nullptr;     // device copy of the step table
    size_t d_tape_cap = 0;
    float4 *d_adj4 = nullptr;       // gP, gA, gV, gW (in allocs)
    float *d_adj1 = nullptr;        // g_invm, g_invi, g_z, g_zw, g_mass, then g_cr, g_cf per scene
    float *d_stage = nullptr;       // 3 floats per dynamic body, record order
    float *d_state_stage = nullptr; // 4 x 3 floats per dynamic body (state arrays, record order)
};

namespace
{

template <class T> int dalloc(nans_world *w, std::vector<void *> &list, T **p, size_t n)
{
    size_t bytes = std::max<size_t>(1, n) * sizeof(T);
    void *q = nullptr;
    CK(cudaMalloc(&q, bytes));
    list.push_back(q);
    *p = (T *)q;
    return NANS_OK;
}

void free_list(std::vector<void *> &list)
{
    for (void *p : list)
        cudaFree(p);
    list.clear();
}

void drop_graph(nans_world *w)
{
    if (w->gexec)
    {
        cudaGraphExecDestroy(w->gexec);
        w->gexec = nullptr;
    }
    w->g_steps = 0;
    w->g_cfg = -1;
    if (w->gexec_b)
    {
        cudaGraphExecDestroy(w->gexec_b);
        w->gexec_b = nullptr;
    }
    w->gb_cfg = -1;
    if (w->gexec1)
    {
        cudaGraphExecDestroy(w->gexec1);
        w->gexec1 = nullptr;
    }
    w->g1_cfg = -1;
}

int cfg_id(const nans_world *w)
{
    return ((((w->medium_bpsm * 33 + w->solve_late_bpsm) * 2 + w->cull_tiles) * 33 + w->narrow_bpsm) * 9 +
            w->solve_threads0 / 32) * 9 + w->solve_threads1 / 32;
}

int narrow_grid(nans_world *w)
{
    int per = narrow_blocks_per_sm(4);
    if (per < 1)
        per = 1;
    if (w->narrow_bpsm > 0)
        per = std::min(per, w->narrow_bpsm);
    return std::min(per * w->sm_count, w->gjk_cap_blocks);
}

size_t solve_smem(const nans_world *w) { return nans::solve_smem(w->max_scene_bodies, w->dw.solve_cache); }


int alloc_candidates(nans_world *w, int cap)
{
    free_list(w->cand_allocs);
    drop_graph(w);
    w->cand_cap = cap;
    DevWorld &d = w->dw;
    d.cand_cap = cap;
    int rc = NANS_OK;
    auto &L = w->cand_allocs;
    w->fwd_buf = nullptr;
    d.s_fwd = nullptr;
    if ((rc = dalloc(w, L, &d.cand_a, cap)) || (rc = dalloc(w, L, &d.cand_b, cap)) ||
        (rc = dalloc(w, L, &d.cand_meta, cap)) || (rc = dalloc(w, L, &d.hit, cap)) ||
        (rc = dalloc(w, L, &d.c_pa, cap)) || (rc = dalloc(w, L, &d.c_pb, cap)) || (rc = dalloc(w, L, &d.c_n, cap)) ||
        (rc = dalloc(w, L, &d.s_order, cap)) || (rc = dalloc(w, L, &d.s_wave, cap)) ||
        (rc = dalloc(w, L, &d.s_ids, cap)) || (rc = dalloc(w, L, &d.s_wcnt, (size_t)cap + 1)) ||
        (rc = dalloc(w, L, &d.s_k, (size_t)9 * cap)) || (rc = dalloc(w, L, &d.long_cand, cap)))
        return rc;
    if (w->tape_on)
    {
        if ((rc = dalloc(w, L, &w->fwd_buf, (size_t)2 * cap)))
            return rc;
        d.s_fwd = w->fwd_buf;
    }
    if ((rc = dalloc(w, L, &d.cand_pidx, cap)))
        return rc;
    return NANS_OK;
}

bool finite_pos(float x) { return std::isfinite(x) && x > 0.0f; }

bool flags_world_warm(const nans_world *w) { return (w->flags & NANS_WORLD_WARM_START) != 0; }

// Warm-start entries are valid for one step; a state overwrite moves the counter on by two.
__global__ void k_warm_bump(int *step) { *step += 2; }

int warm_invalidate(nans_world *w)
{
    if (w->dw.warm_step)
    {
        k_warm_bump<<<1, 1, 0, w->stream>>>(w->dw.warm_step);
        CK(cudaGetLastError());
    }
    return NANS_OK;
}

struct SceneIn
{
    uint32_t nc, ns;
};

// Builds every static table on the host and uploads records; shared by the single-scene
// and the batched upload.
int upload_impl(nans_world *w, uint32_t nscenes, const uint32_t *snc, const uint32_t *sns, const nans_cube *cubes,
                const nans_sphere *spheres, const nans_cube *floors, const float *cube_scale, const int32_t *hull_npts,
                const float *hull_pts, const nans_step_params *sp, uint32_t flags)
{
    if (!w || nscenes == 0 || !snc || !sns || !floors)
        return fail(NANS_ERR_INVALID_ARGUMENT, "upload: null world/counts/floors or zero scenes");
    long long tc = 0, ts = 0;
    for (uint32_t s = 0; s < nscenes; ++s)
    {
        tc += snc[s];
        ts += sns[s];
    }
    if ((tc > 0 && !cubes) || (ts > 0 && !spheres))
        return fail(NANS_ERR_INVALID_ARGUMENT, "upload: null body records");
    if (tc + ts + nscenes > (long long)INT32_MAX / 4)
        return fail(NANS_ERR_INVALID_ARGUMENT, "upload: too many bodies");
    // validate inputs the step divides by
    for (long long i = 0; i < tc; ++i)
        if (!finite_pos(cubes[i].Mass) || !finite_pos(cubes[i].MOI))
            return fail(NANS_ERR_NAN_INPUT, "upload: cube " + std::to_string(i) + " has a non-finite or non-positive Mass/MOI");
    for (long long i = 0; i < ts; ++i)
        if (!finite_pos(spheres[i].Mass) || !finite_pos(spheres[i].MOI) || !finite_pos(spheres[i].Radius))
            return fail(NANS_ERR_NAN_INPUT, "upload: sphere " + std::to_string(i) + " has a non-finite or non-positive Mass/MOI/Radius");
    for (uint32_t s = 0; s < nscenes; ++s)
        if (!finite_pos(floors[s].Mass) || !finite_pos(floors[s].MOI) || !std::isfinite(floors[s].Size))
            return fail(NANS_ERR_NAN_INPUT, "upload: floor " + std::to_string(s) + " has a non-finite Mass/MOI/Size");
    if (cube_scale)
        for (long long i = 0; i < 3 * tc; ++i)
            if (!std::isfinite(cube_scale[i]))
                return fail(NANS_ERR_NAN_INPUT, "upload: non-finite cube scale");
    if (hull_npts)
        for (long long i = 0; i < tc; ++i)
            if (hull_npts[i] < 0 || hull_npts[i] > 255)
                return fail(NANS_ERR_INVALID_ARGUMENT, "upload: hull point count outside [0, 255]");

    CK(cudaSetDevice(w->device));
    CK(cudaStreamSynchronize(w->stream));
    free_list(w->allocs);
    free_list(w->cand_allocs);
    drop_graph(w);
    w->uploaded = false;
    w->tape_valid = false;
    w->fwd_buf = nullptr;
    w->d_maxw = nullptr;
    w->d_adj4 = nullptr;
    w->d_adj1 = nullptr;
    w->d_stage = nullptr;
    w->d_state_stage = nullptr;

    const int S = (int)nscenes;
    const int ndyn = (int)(tc + ts);
    const int nall = ndyn + S;
    w->n_scenes = S;
    w->n_dyn = ndyn;
    w->n_all = nall;
    w->n_cubes = (int)tc;
    w->n_spheres = (int)ts;

    std::vector<int> sc_cube0(S), sc_nc(S), sc_ns(S), sc_iters(S), sc_order(S), body_scene(nall), body_rec(nall);
    std::vector<int> sc_word0(S + 1);
    long long word_acc = 0;
    std::vector<float> sc_cr(S), sc_cf(S);
    std::vector<int4> shape(nall);
    std::vector<float4> scl(nall);
    std::vector<float2> size_moi(nall);
    std::vector<float> local;
    long long vert_floats = 0;
    int cube_rank = 0, sphere_rank = 0, b = 0, max_bodies = 0;
    long long pair_acc = 0;
    long long hull_off = 0;
    for (int s = 0; s < S; ++s)
    {
        sc_cube0[s] = b;
        sc_nc[s] = (int)snc[s];
        sc_ns[s] = (int)sns[s];
        sc_word0[s] = (int)word_acc;
        const long long np = scene_pair_count(snc[s], sns[s]);
        pair_acc += np;
        word_acc += (np + 31) / 32;
        max_bodies = std::max(max_bodies, (int)(snc[s] + sns[s]));
        if (sp)
        {
            sc_cr[s] = sp[s].cr;
            sc_cf[s] = sp[s].cf;
            sc_iters[s] = sp[s].iterations;
        }
        else
        {
            sc_cr[s] = (float)0.1;
            sc_cf[s] = 0.1f;
            sc_iters[s] = 70;
        }
        for (uint32_t i = 0; i < snc[s]; ++i, ++b)
        {
            const nans_cube &r = cubes[cube_rank];
            int np = hull_npts ? hull_npts[cube_rank] : 0;
            int4 sh;
            sh.x = (int)vert_floats;
            if (np > 0)
            {
                sh.y = np;
                sh.z = (int)local.size();
                for (int k = 0; k < 3 * np; ++k)
                    local.push_back(hull_pts[3 * hull_off + k]);
                hull_off += np;
            }
            else
            {
                sh.y = 8;
                sh.z = -1;
            }
            sh.w = 0;
            // whole groups of four vertices (12 floats): hull_support reads group-wise
            vert_floats += ((sh.y + 3LL) / 4) * 12;
            shape[b] = sh;
            if (cube_scale)
                scl[b] = make_float4(cube_scale[3 * cube_rank], cube_scale[3 * cube_rank + 1],
                                     cube_scale[3 * cube_rank + 2], 0.0f);
            else
                scl[b] = make_float4(r.Size, r.Size, r.Size, 0.0f);
            size_moi[b] = make_float2(r.Size, r.MOI);
            body_scene[b] = s;
            body_rec[b] = cube_rank++;
        }
        for (uint32_t i = 0; i < sns[s]; ++i, ++b)
        {
            const nans_sphere &r = spheres[sphere_rank];
            shape[b] = make_int4(0, 0, -1, 0);
            scl[b] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
            size_moi[b] = make_float2(0.0f, r.MOI);
            body_scene[b] = s;
            body_rec[b] = -(sphere_rank++) - 1;
        }
    }
    sc_word0[S] = (int)word_acc;
    if (word_acc > INT32_MAX)
        return fail(NANS_ERR_SCENE_TOO_LARGE, "upload: more than 2^31 words of pair mask");
    for (int s = 0; s < S; ++s)
    {
        int fb = ndyn + s;
        shape[fb] = make_int4((int)vert_floats, 8, -1, 0);
        vert_floats += 24;
        scl[fb] = make_float4(floors[s].Size, 1.0f, floors[s].Size, 0.0f);
        size_moi[fb] = make_float2(floors[s].Size, floors[s].MOI);
        body_scene[fb] = s;
        body_rec[fb] = s;
    }
    for (int s = 0; s < S; ++s)
        sc_order[s] = s;
    std::stable_sort(sc_order.begin(), sc_order.end(),
                     [&](int x, int y) { return sc_nc[x] + sc_ns[x] > sc_nc[y] + sc_ns[y]; });
    if (4 * kWaveChunk * sizeof(int) + (size_t)max_bodies * sizeof(int) > kSolveSmemMax)
        return fail(NANS_ERR_SCENE_TOO_LARGE, "upload: a scene has more bodies than the solver's wave table holds");
    w->fused = (w->flags & NANS_WORLD_FUSED_STEP) != 0;
    if (w->fused && max_bodies > kSceneStepMaxBodies)
        return fail(NANS_ERR_SCENE_TOO_LARGE, "upload: the fused step takes scenes of at most " +
                                                  std::to_string(kSceneStepMaxBodies) + " bodies");
    if (w->fused && word_acc * 32 > INT32_MAX / 16)
        return fail(NANS_ERR_SCENE_TOO_LARGE, "upload: the fused step needs fewer than 2^27 pairs");

    // cube-cube cull tiles: 32 x 32 blocks of the upper triangle of each scene's cube pairs
    std::vector<int4> tiles;
    // cull tasks for the other pairs: each scene's chunks of 32, at most kRestChunksPerTask a task
    std::vector<int4> rest_tasks;
    for (int s = 0; s < S; ++s)
    {
        const long long ncc = (long long)sc_nc[s] * (sc_nc[s] - 1) / 2;
        const long long chunks = (scene_pair_count(sc_nc[s], sc_ns[s]) - ncc + 31) / 32;
        for (long long c = 0; c < chunks; c += kRestChunksPerTask)
            rest_tasks.push_back(make_int4(s, (int)c, (int)std::min<long long>(kRestChunksPerTask, chunks - c), 0));
    }
    if (rest_tasks.size() > (size_t)INT32_MAX)
        return fail(NANS_ERR_SCENE_TOO_LARGE, "upload: more than 2^31 cull tasks of non-cube-cube pairs");
    for (int s = 0; s < S; ++s)
    {
        const int k = (sc_nc[s] + 31) / 32;
        if (sc_nc[s] < 2)
            continue;
        for (int ti = 0; ti < k; ++ti)
            for (int tj = ti; tj < k; ++tj)
                tiles.push_back(make_int4(s, ti, tj, 0));
    }
    w->pair_total = pair_acc;
    w->max_scene_bodies = max_bodies;
    w->cull_blocks = (int)((word_acc + kCullThreads - 1) / kCullThreads);

    DevWorld &d = w->dw;
    d = DevWorld{};
    d.n_scenes = S;
    d.n_dyn = ndyn;
    d.solve_cache = solve_cache_bodies(max_bodies);
    d.n_all = nall;
    d.pair_total = pair_acc;
    d.n_words = (int)word_acc;
    d.n_tiles = (int)tiles.size();
    auto &L = w->allocs;
    int rc;
    int *p_cube0, *p_nc, *p_ns, *p_iters, *p_order, *p_rank, *p_bscene;
    int *p_word0, *p_wscene;
    int4 *p_tiles;
    int4 *p_rest;
    float *p_cr, *p_cf, *p_local;
    int4 *p_shape;
    if ((rc = dalloc(w, L, &p_cube0, S)) || (rc = dalloc(w, L, &p_nc, S)) || (rc = dalloc(w, L, &p_ns, S)) ||
        (rc = dalloc(w, L, &p_iters, S)) || (rc = dalloc(w, L, &p_order, S)) || (rc = dalloc(w, L, &p_rank, S)) || (rc = dalloc(w, L, &p_word0, S + 1)) ||
        (rc = dalloc(w, L, &p_cr, S)) || (rc = dalloc(w, L, &p_cf, S)) || (rc = dalloc(w, L, &p_bscene, nall)) ||
        (rc = dalloc(w, L, &w->d_body_rec, nall)) || (rc = dalloc(w, L, &p_shape, nall)) ||
        (rc = dalloc(w, L, &w->d_scl, nall)) || (rc = dalloc(w, L, &w->d_size_moi, nall)) ||
        (rc = dalloc(w, L, &p_local, local.size())) || (rc = dalloc(w, L, &d.verts, vert_floats)) ||
        (rc = dalloc(w, L, &d.pos, nall)) || (rc = dalloc(w, L, &d.ang, nall)) || (rc = dalloc(w, L, &d.vel, nall)) ||
        (rc = dalloc(w, L, &d.omg, nall)) || (rc = dalloc(w, L, &d.frc, nall)) || (rc = dalloc(w, L, &d.trq, nall)) ||
        (rc = dalloc(w, L, &w->d_prm, nall)) || (rc = dalloc(w, L, &w->d_model_in, (size_t)4 * nall)) ||
        (rc = dalloc(w, L, &d.box_lo, nall)) || (rc = dalloc(w, L, &d.box_hi, nall)) ||
        (rc = dalloc(w, L, &d.pair_mask, (size_t)word_acc)) || (rc = dalloc(w, L, &p_wscene, (size_t)word_acc)) ||
        (rc = dalloc(w, L, &p_tiles, tiles.size())) || (rc = dalloc(w, L, &p_rest, rest_tasks.size())) ||
        (rc = dalloc(w, L, &d.epa_hist, (size_t)word_acc * 32)) ||
        (rc = dalloc(w, L, &d.block_hits, std::max(1, w->cull_blocks))) || (rc = dalloc(w, L, &d.cull_total, 1)) ||
        (rc = dalloc(w, L, &d.cull_max, 1)) ||
        (rc = dalloc(w, L, &d.n_cand, 1)) ||
        (rc = dalloc(w, L, &d.cand_begin, S)) || (rc = dalloc(w, L, &d.cand_end, S)) ||
        (rc = dalloc(w, L, &d.scene_late, S)) || (rc = dalloc(w, L, &d.late_list, S)) ||
        (rc = dalloc(w, L, &d.work_counter, kWorkCounters)) || (rc = dalloc(w, L, &d.status, 1)) ||
        (rc = dalloc(w, L, &d.ovf_cand, kEpaOverflowCap)) || (rc = dalloc(w, L, &d.med_cand, kEpaMediumCap)) ||
        (rc = dalloc(w, L, &d.epa_arena, epa_big_bytes())) ||
        (rc = dalloc(w, L, &d.giant_scratch, epa_giant_scratch_bytes())) ||
        (rc = dalloc(w, L, &d.blk_arena, epa_block_bytes() * (size_t)(kBlockPerSm * w->sm_count))) ||
        (rc = dalloc(w, L, &d.giant_cand, kGiantQueueCap)) || (rc = dalloc(w, L, &d.handover, kHandoverSlots)) ||
        (rc = dalloc(w, L, &d.epa_stats, 8)) || (rc = dalloc(w, L, &d.check, 4)) ||
        (rc = dalloc(w, L, &w->d_rec_cube, (size_t)61 * tc)) || (rc = dalloc(w, L, &w->d_rec_sphere, (size_t)37 * ts)) ||
        (rc = dalloc(w, L, &w->d_rec_floor, (size_t)61 * S)) || (rc = dalloc(w, L, &w->d_small, 2)) ||
        (rc = dalloc(w, L, &d.s_last, 1)))
        return rc;
    // no EPA seen yet: every pair starts in the short-EPA part of the queue
    CK(cudaMemset(d.epa_hist, 0, std::max(1LL, word_acc * 32)));
    // world vertices are written by the first step; zero until then (the renderer reads them)
    CK(cudaMemset(d.verts, 0, (size_t)std::max(1LL, vert_floats) * sizeof(float)));
    d.sc_cube0 = p_cube0;
    d.sc_nc = p_nc;
    d.sc_ns = p_ns;
    d.sc_iters = p_iters;
    d.sc_order = p_order;
    d.sc_rank = p_rank;
    d.sc_word0 = p_word0;
    d.word_scene = p_wscene;
    d.tiles = p_tiles;
    d.rest_tasks = p_rest;
    d.n_rest_tasks = (int)rest_tasks.size();
    d.sc_cr = p_cr;
    d.sc_cf = p_cf;
    d.body_scene = p_bscene;
    d.shape = p_shape;
    d.local_pts = p_local;
    d.scl = w->d_scl;
    d.prm = w->d_prm;
    d.model_in = w->d_model_in;
    d.ovf_cap = kEpaOverflowCap;
    d.med_cap = kEpaMediumCap;
    // persistent grids: resident blocks on every SM, but no more blocks than the world's pairs
    // (an upper bound of its candidates) can keep busy, so that a small scene's step does not
    // launch hundreds of blocks that exit at once
    const long long maxc = std::max(1LL, pair_acc);
    auto upto = [&](long long per_block, int resident) {
        return (int)std::max(1LL, std::min<long long>(resident, (maxc + per_block - 1) / per_block));
    };
    w->gjk_cap_blocks = upto(128, INT32_MAX);
    w->medium_cap_blocks = upto(4, INT32_MAX);
    d.medium_blocks = std::min(w->medium_bpsm * w->sm_count, w->medium_cap_blocks);
    d.tiny_blocks = upto(64, epa_tiny_grid(w->sm_count));
    d.gjk_warp = (w->flags & NANS_WORLD_GJK_WARP) ? 1 : 0;
    d.sm_count = w->sm_count;
    d.giant_blocks = std::min(giant_grid(w->sm_count), upto(1, INT32_MAX) < 4096 ? 16 : INT32_MAX);
    d.blk_blocks = upto(1, kBlockPerSm * w->sm_count);
    d.blk_face_limit = (w->flags & NANS_WORLD_TEST_GIANT_TIER) ? 0 : kBlockFaces;
    const bool barrier_test = (w->flags & NANS_WORLD_TEST_BARRIER_TIMEOUT) != 0;
    d.barrier_spins = barrier_test ? kBarrierSpinsTest : kBarrierSpins;
    d.barrier_extra = barrier_test ? 1u : 0u;
    d.giant_cap = kGiantQueueCap;
    cudaStream_t st = w->stream;
    CK(cudaMemcpyAsync(p_cube0, sc_cube0.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(p_nc, sc_nc.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(p_ns, sc_ns.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(p_iters, sc_iters.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(p_order, sc_order.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
    std::vector<int> sc_rank(S);
    for (int r = 0; r < S; ++r)
        sc_rank[sc_order[r]] = r;
    CK(cudaMemcpyAsync(p_rank, sc_rank.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(p_word0, sc_word0.data(), (S + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
    if (!tiles.empty())
        CK(cudaMemcpyAsync(p_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
    if (!rest_tasks.empty())
        CK(cudaMemcpyAsync(p_rest, rest_tasks.data(), rest_tasks.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
    {
        std::vector<int> wscene((size_t)word_acc);
        for (int s = 0; s < S; ++s)
            std::fill(wscene.begin() + sc_word0[s], wscene.begin() + sc_word0[s + 1], s);
        if (word_acc)
            CK(cudaMemcpyAsync(p_wscene, wscene.data(), (size_t)word_acc * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st)); // wscene is a local buffer
    }
    CK(cudaMemcpyAsync(p_cr, sc_cr.data(), S * sizeof(float), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(p_cf, sc_cf.data(), S * sizeof(float), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(p_bscene, body_scene.data(), nall * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(w->d_body_rec, body_rec.data(), nall * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(p_shape, shape.data(), nall * sizeof(int4), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(w->d_scl, scl.data(), nall * sizeof(float4), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(w->d_size_moi, size_moi.data(), nall * sizeof(float2), cudaMemcpyHostToDevice, st));
    if (!local.empty())
        CK(cudaMemcpyAsync(p_local, local.data(), local.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    if (tc)
        CK(cudaMemcpyAsync(w->d_rec_cube, cubes, tc * sizeof(nans_cube), cudaMemcpyHostToDevice, st));
    if (ts)
        CK(cudaMemcpyAsync(w->d_rec_sphere, spheres, ts * sizeof(nans_sphere), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(w->d_rec_floor, floors, S * sizeof(nans_cube), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(d.status, 0, sizeof(unsigned), st));
    CK(cudaMemsetAsync(d.giant_scratch, 0, epa_giant_scratch_bytes(), st));
    CK(cudaMemsetAsync(d.epa_stats, 0, 8 * sizeof(unsigned), st));
    CK(cudaMemsetAsync(d.check, 0, 4 * sizeof(int), st));
    CK(cudaMemsetAsync(d.n_cand, 0, sizeof(int), st));
    CK(cudaMemsetAsync(d.cull_max, 0, sizeof(int), st));
    CK(cudaMemsetAsync(d.cand_begin, 0, S * sizeof(int), st));
    CK(cudaMemsetAsync(d.cand_end, 0, S * sizeof(int), st));
    CK(cudaMemsetAsync(d.scene_late, 0, S * sizeof(int), st));
    const int mode = 1 | ((flags & NANS_UPLOAD_KEEP_MODEL) ? 2 : 0);
    k_unpack<<<(nall + kSweepThreads - 1) / kSweepThreads, kSweepThreads, 0, st>>>(
        d, w->d_rec_cube, w->d_rec_sphere, w->d_rec_floor, w->d_body_rec, mode, w->d_prm, w->d_model_in);
    CK(cudaGetLastError());

    if (flags_world_warm(w))
    {
        if (word_acc * 32 > INT32_MAX)
            return fail(NANS_ERR_SCENE_TOO_LARGE, "upload: warm starting needs fewer than 2^31 pairs");
        if ((rc = dalloc(w, L, &d.warm, (size_t)word_acc * 32)) || (rc = dalloc(w, L, &d.warm_step, 1)))
            return rc;
        CK(cudaMemsetAsync(d.warm, 0, (size_t)word_acc * 32 * sizeof(float4), st));
        CK(cudaMemsetAsync(d.warm_step, 0, sizeof(int), st));
    }
    int cap = (int)(w->max_cand_req ? w->max_cand_req : std::min<long long>(16LL * ndyn + 4096, INT32_MAX / 16));
    if (w->fused) // the fused step places each scene's candidates in its own slots of the pair space
        cap = std::max(cap, (int)(word_acc * 32));
    if ((rc = alloc_candidates(w, std::max(1, cap))))
        return rc;
    // the attribute is per device and per kernel, shared by every world on the device: set it to
    // the largest table any world may use, so that one world never lowers another's limit
    if (nans::solve_smem(max_bodies, d.solve_cache) > 48 * 1024)
        CK((cudaError_t)solve_kernel_attrs(d, (int)kSolveSmemMax));
    CK(cudaStreamSynchronize(st));
    w->uploaded = true;
    w->graph_steps_run = 0;
    w->eager_steps_run = 0;
    w->pending = false;
    w->pending_dt = 0.0f;
    w->model_input = (flags & NANS_UPLOAD_KEEP_MODEL) != 0;
    w->forces_pending = true;
    w->steps_run = 0;
    return NANS_OK;
}

// Enqueues the cull (three kernels) on the world's stream.
// The culled pair mask and its per-block counts (the scan's input): by tiles (cube-cube pairs
// 32 x 32 per warp, the other pairs per scene, then the counts), or one lane per pair
// (k_cull_mask: the all-pairs mode, and the tuning's alternative). The same mask either way.
void enqueue_cull_mask(nans_world *w)
{
    cudaStream_t st = w->stream;
    const int all_pairs = (w->flags & NANS_WORLD_ALL_PAIRS) ? 1 : 0;
    if (w->cull_blocks <= 0)
        return;
    if (all_pairs || !w->cull_tiles)
    {
        k_cull_mask<<<w->cull_blocks, kCullThreads, 0, st>>>(w->dw, all_pairs);
        return;
    }
    const int per_block = kCullTileThreads / 32, cap = 8 * w->sm_count;
    cudaMemsetAsync(w->dw.pair_mask, 0, (size_t)w->dw.n_words * sizeof(unsigned), st);
    if (w->dw.n_tiles > 0)
        k_cull_tiles<<<std::min(cap, (w->dw.n_tiles + per_block - 1) / per_block), kCullTileThreads, 0, st>>>(w->dw);
    if (w->dw.n_rest_tasks > 0)
        k_cull_rest<<<std::min(cap, (w->dw.n_rest_tasks + per_block - 1) / per_block), kCullTileThreads, 0, st>>>(
            w->dw);
    k_cull_count<<<w->cull_blocks, kCullThreads, 0, st>>>(w->dw);
}

// Enqueues the cull on the world's stream: mask, scan, ordered write.
void enqueue_cull(nans_world *w)
{
    cudaStream_t st = w->stream;
    enqueue_cull_mask(w);
    k_cull_scan<<<1, 1024, 0, st>>>(w->dw, w->cull_blocks);
    if (w->cull_blocks > 0)
        k_cull_write<<<w->cull_blocks, kCullThreads, 0, st>>>(w->dw);
}

// Narrowphase and solve. The EPA tiers beyond the per-thread one run on the second stream
// while the first solve pass handles every scene they do not touch; the second pass solves
// the rest after them. Both streams are joined before the function returns (also under
// stream capture).
// tl (timeline profiling only, else null): events recorded after the per-thread EPA (stream 1),
// the warp tier and the large tiers (stream 2), solve pass 0 and pass 1 (stream 1).
cudaError_t enqueue_narrow_solve(nans_world *w, float dt, cudaEvent_t *tl)
{
    cudaStream_t st = w->stream, st2 = w->stream2;
    launch_narrow_tiny(narrow_grid(w), st, w->dw);
    if (tl)
        cudaEventRecord(tl[0], st);
    cudaError_t e = cudaEventRecord(w->ev_fork, st);
    if (e == cudaSuccess)
        e = cudaStreamWaitEvent(st2, w->ev_fork, 0);
    if (e != cudaSuccess)
        return e;
    launch_epa_medium(st2, w->dw);
    if (tl)
        cudaEventRecord(tl[1], st2);
    e = (cudaError_t)launch_narrow_big(st2, w->dw);
    if (tl)
        cudaEventRecord(tl[2], st2);
    launch_solve(w->dw, w->n_scenes, w->solve_threads0 ? w->solve_threads0 : solve_threads(w->max_scene_bodies),
                 solve_smem(w), st, dt, 0);
    if (tl)
        cudaEventRecord(tl[3], st);
    cudaError_t e2 = cudaEventRecord(w->ev_join, st2);
    if (e2 == cudaSuccess)
        e2 = cudaStreamWaitEvent(st, w->ev_join, 0);
    // the late scenes (few, and mostly the larger ones) solve with wider blocks: their waves
    // are on the step's critical path
    launch_solve(w->dw, std::min(w->n_scenes, w->solve_late_bpsm * w->sm_count), w->solve_threads1, solve_smem(w), st,
                 dt, 1);
    if (tl)
        cudaEventRecord(tl[4], st);
    return e != cudaSuccess ? e : e2;
}

int sweep_flags(const nans_world *w)
{
    int f = SW_INTEGRATE;
    if (w->pending)
        f |= SW_APPLY_VEL;
    if (w->model_input)
        f |= SW_MODEL_INPUT;
    if (w->forces_pending)
        f |= SW_FORCES;
    return f;
}

void after_step(nans_world *w, float dt)
{
    w->tape_valid = false;
    w->pending = true;
    w->pending_dt = dt;
    w->model_input = false;
    w->forces_pending = false;
    ++w->steps_run;
}

// The fused step (NANS_WORLD_FUSED_STEP, not while a tape is recorded): the sweep (which also
// clears the work counters), one launch that culls, collides and solves every scene, then the
// large EPA tiers and the late solve pass for the scenes with an EPA beyond the warp tier. The
// candidate buffers hold every pair, so nothing is read back.
bool use_fused(const nans_world *w) { return w->fused && !w->tape_on; }

// The large EPA tiers and the late solve pass on stream st.
cudaError_t enqueue_fused_tail(nans_world *w, float dt, cudaStream_t st)
{
    DevWorld &d = w->dw;
    cudaError_t e = (cudaError_t)launch_narrow_big(st, d);
    if (e != cudaSuccess)
        return e;
    launch_solve(d, std::min(w->n_scenes, w->solve_late_bpsm * w->sm_count), w->solve_threads1, solve_smem(w), st,
                 dt, 1);
    return cudaGetLastError();
}

// Eagerly, or captured with the tail launched unconditionally.
cudaError_t enqueue_fused(nans_world *w, float pending_dt, float dt, int flags)
{
    cudaStream_t st = w->stream;
    DevWorld &d = w->dw;
    k_sweep<<<(w->n_all + kSweepThreads - 1) / kSweepThreads, kSweepThreads, 0, st>>>(d, pending_dt, dt,
                                                                                       flags | SW_CLEAR_COUNTERS);
    launch_scene_step(d, solve_smem(w), dt, (w->flags & NANS_WORLD_ALL_PAIRS) ? 1 : 0, st, 0, 0);
    return enqueue_fused_tail(w, dt, st);
}

// Under stream capture: the tail in the body of a conditional (IF) node whose handle the fused
// launch sets only when a scene went late, so that a step with no EPA beyond the warp tier (most
// steps of small scenes) replays three nodes. The body is captured on the second stream.
cudaError_t enqueue_fused_conditional(nans_world *w, float pending_dt, float dt, int flags)
{
    cudaStream_t st = w->stream;
    DevWorld &d = w->dw;
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edges = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &edges, &nd);
    if (e != cudaSuccess)
        return e;
    if (cs != cudaStreamCaptureStatusActive)
        return cudaErrorStreamCaptureInvalidated;
    cudaGraphConditionalHandle h = 0;
    if ((e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault)) != cudaSuccess)
        return e;
    k_sweep<<<(w->n_all + kSweepThreads - 1) / kSweepThreads, kSweepThreads, 0, st>>>(d, pending_dt, dt,
                                                                                       flags | SW_CLEAR_COUNTERS);
    launch_scene_step(d, solve_smem(w), dt, (w->flags & NANS_WORLD_ALL_PAIRS) ? 1 : 0, st, h, 1);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return e;
    if ((e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &edges, &nd)) != cudaSuccess)
        return e;
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    if ((e = cudaGraphAddNode(&node, g, deps, edges, nd, &p)) != cudaSuccess)
        return e;
    if ((e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies)) !=
        cudaSuccess)
        return e;
    cudaGraph_t body = p.conditional.phGraph_out[0];
    if ((e = cudaStreamBeginCaptureToGraph(w->stream2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess)
        return e;
    const cudaError_t et = enqueue_fused_tail(w, dt, w->stream2);
    cudaGraph_t out = nullptr;
    e = cudaStreamEndCapture(w->stream2, &out);
    return et != cudaSuccess ? et : e;
}

// One step, stage by stage. With check_capacity the candidate count is read back after the
// scan and the candidate buffers grow if needed (the plain path).
int step_eager(nans_world *w, float dt, bool check_capacity)
{
    cudaStream_t st = w->stream;
    DevWorld &d = w->dw;
    if (use_fused(w))
    {
        CK(enqueue_fused(w, w->pending_dt, dt, sweep_flags(w)));
        after_step(w, dt);
        return NANS_OK;
    }
    CK(cudaMemsetAsync(d.work_counter, 0, kWorkCounters * sizeof(int), st));
    CK(cudaMemsetAsync(d.cand_begin, 0, w->n_scenes * sizeof(int), st));
    CK(cudaMemsetAsync(d.cand_end, 0, w->n_scenes * sizeof(int), st));
    CK(cudaMemsetAsync(d.scene_late, 0, w->n_scenes * sizeof(int), st));
    k_sweep<<<(w->n_all + kSweepThreads - 1) / kSweepThreads, kSweepThreads, 0, st>>>(d, w->pending_dt, dt,
                                                                                       sweep_flags(w));
    enqueue_cull(w);
    CK(cudaGetLastError());
    if (check_capacity)
    {
        unsigned status = 0;
        CK(cudaMemcpyAsync(&status, d.status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (status & ST_CANDIDATES)
        {
            // the scan recorded the exact total: grow the candidate buffers and write again
            int total = 0;
            CK(cudaMemcpyAsync(&total, d.cull_total, sizeof(int), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            int rc = alloc_candidates(w, (int)std::min<long long>((long long)total + total / 4 + 1024, INT32_MAX / 16));
            if (rc)
                return rc;
            // the block counts were turned into offsets by the scan: count again
            CK(cudaMemsetAsync(d.status, 0, sizeof(unsigned), st));
            enqueue_cull(w);
            CK(cudaGetLastError());
        }
    }
    CK(enqueue_narrow_solve(w, dt, nullptr));
    CK(cudaGetLastError());
    after_step(w, dt);
    return NANS_OK;
}

int status_code(nans_world *w, unsigned status);

int check_status(nans_world *w)
{
    unsigned status = 0;
    CK(cudaMemcpyAsync(&status, w->dw.status, sizeof(unsigned), cudaMemcpyDeviceToHost, w->stream));
    CK(cudaStreamSynchronize(w->stream));
    return status_code(w, status);
}

int set_params_all(nans_world *w, const nans_step_params *p)
{
    std::vector<float> cr(w->n_scenes, p->cr), cf(w->n_scenes, p->cf);
    std::vector<int> it(w->n_scenes, p->iterations);
    CK(cudaMemcpyAsync((void *)w->dw.sc_cr, cr.data(), cr.size() * sizeof(float), cudaMemcpyHostToDevice, w->stream));
    CK(cudaMemcpyAsync((void *)w->dw.sc_cf, cf.data(), cf.size() * sizeof(float), cudaMemcpyHostToDevice, w->stream));
    CK(cudaMemcpyAsync((void *)w->dw.sc_iters, it.data(), it.size() * sizeof(int), cudaMemcpyHostToDevice,
                       w->stream));
    CK(cudaStreamSynchronize(w->stream)); // the host vectors die on return
    return NANS_OK;
}

bool steady(const nans_world *w, float dt)
{
    return w->pending && w->pending_dt == dt && !w->model_input && !w->forces_pending;
}

// Captures gsteps steps into *exec (destroying what it held): the first with the previous
// step's dt pdt0 and sweep flags flags0, the others steady.
int capture_steps(nans_world *w, float dt, int gsteps, cudaGraphExec_t *exec, float pdt0 = 0.0f,
                  int flags0 = SW_INTEGRATE | SW_APPLY_VEL)
{
    if (flags0 & SW_APPLY_VEL)
        pdt0 = dt;
    if (*exec)
    {
        cudaGraphExecDestroy(*exec);
        *exec = nullptr;
    }
    cudaStream_t st = w->stream;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    DevWorld &d = w->dw;
    const bool conditional = use_fused(w) && w->fused_conditional;
    cudaError_t ec = cudaSuccess;
    for (int i = 0; i < gsteps; ++i)
    {
        if (use_fused(w))
        {
            const float pdt = i == 0 ? pdt0 : dt;
            const int fl = i == 0 ? flags0 : (SW_INTEGRATE | SW_APPLY_VEL);
            if (conditional)
            {
                if (ec == cudaSuccess)
                    ec = enqueue_fused_conditional(w, pdt, dt, fl);
            }
            else
                enqueue_fused(w, pdt, dt, fl);
            continue;
        }
        cudaMemsetAsync(d.work_counter, 0, kWorkCounters * sizeof(int), st);
        cudaMemsetAsync(d.cand_begin, 0, w->n_scenes * sizeof(int), st);
        cudaMemsetAsync(d.cand_end, 0, w->n_scenes * sizeof(int), st);
        cudaMemsetAsync(d.scene_late, 0, w->n_scenes * sizeof(int), st);
        k_sweep<<<(w->n_all + kSweepThreads - 1) / kSweepThreads, kSweepThreads, 0, st>>>(
            d, i == 0 ? pdt0 : dt, dt, i == 0 ? flags0 : (SW_INTEGRATE | SW_APPLY_VEL));
        enqueue_cull(w);
        enqueue_narrow_solve(w, dt, nullptr);
    }
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (e == cudaSuccess && ec == cudaSuccess && conditional)
    {
        e = cudaGraphInstantiate(exec, graph, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(graph);
        if (e == cudaSuccess)
            return NANS_OK;
        *exec = nullptr;
    }
    if (conditional)
    {
        // the conditional form did not capture or instantiate here: capture the unconditional
        // tail instead (the same results), and keep to it for this world
        if (graph && e == cudaSuccess && ec != cudaSuccess)
            cudaGraphDestroy(graph);
        cudaGetLastError();
        w->fused_conditional = false;
        return capture_steps(w, dt, gsteps, exec, pdt0, flags0);
    }
    if (e != cudaSuccess)
        return fail(NANS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(exec, graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
    {
        *exec = nullptr;
        return fail(NANS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    return NANS_OK;
}

// The gsteps-step graph for the world's current state: the steady graph, or (after a download
// or a state-array write, whose first step does not apply a pending velocity) the graph whose
// first step runs with the world's current sweep flags. Returns it in *exec.
int ensure_graph(nans_world *w, float dt, int gsteps, cudaGraphExec_t *exec)
{
    int rc;
    if (steady(w, dt))
    {
        if (!(w->gexec && w->g_steps == gsteps && w->g_dt == dt && w->g_cfg == cfg_id(w)))
        {
            w->g_steps = 0;
            w->g_cfg = -1;
            if ((rc = capture_steps(w, dt, gsteps, &w->gexec)))
                return rc;
            w->g_steps = gsteps;
            w->g_dt = dt;
            w->g_cfg = cfg_id(w);
        }
        *exec = w->gexec;
        return NANS_OK;
    }
    const int flags = sweep_flags(w);
    if (!(w->gexec_b && w->gb_steps == gsteps && w->gb_dt == dt && w->gb_flags == flags && w->gb_cfg == cfg_id(w)))
    {
        w->gb_cfg = -1;
        if ((rc = capture_steps(w, dt, gsteps, &w->gexec_b, 0.0f, flags)))
            return rc;
        w->gb_steps = gsteps;
        w->gb_dt = dt;
        w->gb_flags = flags;
        w->gb_cfg = cfg_id(w);
    }
    *exec = w->gexec_b;
    return NANS_OK;
}

// A one-step graph for the world's current step flags (steady or not): the plain path and
// one-step batched calls replay it; it is captured again when the flags, dt or the previous
// step's dt change.
int ensure_graph1(nans_world *w, float dt)
{
    const int flags = sweep_flags(w);
    const float pdt = (flags & SW_APPLY_VEL) ? w->pending_dt : 0.0f;
    if (w->gexec1 && w->g1_dt == dt && w->g1_pdt == pdt && w->g1_flags == flags && w->g1_cfg == cfg_id(w))
        return NANS_OK;
    w->g1_cfg = -1;
    int rc = capture_steps(w, dt, 1, &w->gexec1, pdt, flags);
    if (rc)
        return rc;
    w->g1_dt = dt;
    w->g1_pdt = pdt;
    w->g1_flags = flags;
    w->g1_cfg = cfg_id(w);
    return NANS_OK;
}

// One step from a one-step graph.
int step_graph1(nans_world *w, float dt)
{
    int rc = ensure_graph1(w, dt);
    if (rc)
        return rc;
    CK(cudaGraphLaunch(w->gexec1, w->stream));
    after_step(w, dt);
    ++w->graph_steps_run;
    return NANS_OK;
}

int batch_steps(nans_world *w, float dt, uint32_t nsteps, uint32_t gsteps)
{
    w->tape_valid = false;
    uint32_t done = 0;
    int rc;
    if (gsteps == 1)
    {
        for (uint32_t i = 0; i < nsteps; ++i)
            if ((rc = step_graph1(w, dt)))
                return rc;
        return NANS_OK;
    }
    // the first step after an upload or set_state (external forces, input Model) runs eagerly;
    // whole blocks of gsteps steps replay graphs, the rest replays the one-step graph
    while (done < nsteps && (sweep_flags(w) & (SW_FORCES | SW_MODEL_INPUT)))
    {
        if ((rc = step_eager(w, dt, false)))
            return rc;
        ++done;
        ++w->eager_steps_run;
    }
    uint32_t rem = nsteps - done;
    if (gsteps > 1)
        for (; rem >= gsteps; rem -= gsteps)
        {
            cudaGraphExec_t exec = nullptr;
            if ((rc = ensure_graph(w, dt, (int)gsteps, &exec)))
                return rc;
            CK(cudaGraphLaunch(exec, w->stream));
            after_step(w, dt);
            w->steps_run += gsteps - 1;
            w->graph_steps_run += gsteps;
        }
    for (uint32_t i = 0; i < rem; ++i)
        if ((rc = step_graph1(w, dt)))
            return rc;
    return NANS_OK;
}

// The state snapshot buffer (6 float4 per body: the mutable state) and, with_hist, the copy of
// the per-pair EPA lengths, sized for the current upload.
int ensure_snapshot(nans_world *w, bool with_hist)
{
    const size_t n = (size_t)w->n_all;
    if (w->d_snap && w->snap_n < n)
    {
        cudaFree(w->d_snap);
        w->d_snap = nullptr;
    }
    if (!w->d_snap)
    {
        CK(cudaMalloc(&w->d_snap, 6 * std::max<size_t>(1, n) * sizeof(float4)));
        w->snap_n = n;
    }
    const size_t nhist = (size_t)w->dw.n_words * 32;
    if (with_hist && w->d_snap_hist && w->snap_hist_n < nhist)
    {
        cudaFree(w->d_snap_hist);
        w->d_snap_hist = nullptr;
    }
    if (with_hist && !w->d_snap_hist)
    {
        CK(cudaMalloc(&w->d_snap_hist, std::max<size_t>(1, nhist)));
        w->snap_hist_n = nhist;
    }
    return NANS_OK;
}

// Status bits of the last steps as a return code.
int status_code(nans_world *w, unsigned status)
{
    if (status & ST_CHECK)
    {
        int chk[4] = {0, 0, 0, 0};
        cudaMemcpy(chk, w->dw.check, sizeof(chk), cudaMemcpyDeviceToHost);
        return fail(NANS_ERR_CUDA, "step: a device bounds check failed (site " + std::to_string(chk[0]) + ", index " +
                                       std::to_string(chk[1]) + ", bound " + std::to_string(chk[2]) +
                                       "); the access was skipped");
    }
    if (status & ST_CANDIDATES)
        return fail(NANS_ERR_CAPACITY, "step: more candidate pairs than the world's capacity");
    if (status & ST_EPA_TIMEOUT)
        return fail(NANS_ERR_EPA_CAPACITY, "step: the large-polytope EPA's grid barrier timed out");
    if ((status & (ST_EPA_FACES | ST_EPA_EDGES)) && (w->flags & NANS_WORLD_STRICT_EPA))
        return fail(NANS_ERR_EPA_CAPACITY, "step: an EPA polytope outgrew the large-polytope buffers");
    return NANS_OK;
}

// The plain path with one host synchronisation per call. The world's mutable state is copied
// aside on the device, the steps are enqueued without reading the candidate count back (each
// step replays a one-step CUDA graph, except the first after an upload or a set_state), and the
// status word and the largest candidate count are read once at the end. If a step found more
// candidate pairs than the buffers hold (the cull then caps its writes and flags the step), the
// copy is restored, the buffers grow (to 1.5 times the largest count seen, at least double) and
// the steps run again the same way; after three such rounds they run synchronising after every
// cull. Worlds with warm starting keep that synchronising loop: their contact cache is stamped
// per step and cannot be rolled back. A world whose candidate buffers hold all of its pairs (small
// scenes, such as the reference's own) cannot overflow them and skips the copy.
int plain_steps(nans_world *w, float dt, uint32_t nsteps)
{
    cudaStream_t st = w->stream;
    DevWorld &d = w->dw;
    const size_t n = (size_t)w->n_all;
    int rc;
    if ((long long)w->cand_cap >= d.pair_total)
    {
        // The candidate buffers hold every pair of every scene, and the cull writes at most one
        // candidate per pair, so no step can overflow them: no copy aside, one status read.
        for (uint32_t i = 0; i < nsteps; ++i)
        {
            if (!(sweep_flags(w) & (SW_FORCES | SW_MODEL_INPUT)))
            {
                if ((rc = step_graph1(w, dt)))
                    return rc;
            }
            else
            {
                if ((rc = step_eager(w, dt, false)))
                    return rc;
                ++w->eager_steps_run;
            }
        }
        return check_status(w);
    }
    rc = ensure_snapshot(w, false);
    if (rc)
        return rc;
    float4 *bufs[6] = {d.pos, d.ang, d.vel, d.omg, d.frc, d.trq};
    for (int i = 0; i < 6; ++i)
        CK(cudaMemcpyAsync(w->d_snap + i * n, bufs[i], n * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    const bool s_pending = w->pending, s_model = w->model_input, s_forces = w->forces_pending;
    const float s_pdt = w->pending_dt;
    const long long s_steps = w->steps_run;
    const unsigned long long s_graph = w->graph_steps_run, s_eager = w->eager_steps_run;
    for (int round = 0; round < 3; ++round)
    {
        CK(cudaMemsetAsync(d.cull_max, 0, sizeof(int), st));
        for (uint32_t i = 0; i < nsteps; ++i)
        {
            // graphs for the repeating flags (steady steps, and steps after a download or a state
            // write); the first step after an upload or set_state (forces, input Model) is eager
            if (!(sweep_flags(w) & (SW_FORCES | SW_MODEL_INPUT)))
            {
                if ((rc = step_graph1(w, dt)))
                    return rc;
            }
            else
            {
                if ((rc = step_eager(w, dt, false)))
                    return rc;
                ++w->eager_steps_run;
            }
        }
        unsigned hdr[2] = {0u, 0u};
        CK(cudaMemcpyAsync(&hdr[0], d.status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&hdr[1], d.cull_max, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (!(hdr[0] & ST_CANDIDATES))
            return status_code(w, hdr[0]);
        // roll back and grow
        for (int i = 0; i < 6; ++i)
            CK(cudaMemcpyAsync(bufs[i], w->d_snap + i * n, n * sizeof(float4), cudaMemcpyDeviceToDevice, st));
        w->pending = s_pending;
        w->model_input = s_model;
        w->forces_pending = s_forces;
        w->pending_dt = s_pdt;
        w->steps_run = s_steps;
        w->graph_steps_run = s_graph;
        w->eager_steps_run = s_eager;
        const long long need = (long long)(int)hdr[1];
        const long long grow = std::max(need + need / 2, 2LL * w->cand_cap) + 1024;
        if ((rc = alloc_candidates(w, (int)std::min<long long>(grow, INT32_MAX / 16))))
            return rc;
        CK(cudaMemsetAsync(d.status, 0, sizeof(unsigned), st));
    }
    for (uint32_t i = 0; i < nsteps; ++i)
    {
        if ((rc = step_eager(w, dt, true)))
            return rc;
        ++w->eager_steps_run;
    }
    return check_status(w);
}

int valid_dt(float dt) { return std::isfinite(dt) && dt > 0.0f; }

// Bump allocation from the tape arena (256-byte aligned); new chunks of at least 256 MiB.
template <class T> int tape_alloc(nans_world *w, T **out, size_t n)
{
    const size_t bytes = (std::max<size_t>(1, n) * sizeof(T) + 255) & ~(size_t)255;
    while (w->tape_chunk < w->tape_chunks.size())
    {
        if (w->tape_off + bytes <= w->tape_sizes[w->tape_chunk])
        {
            *out = (T *)((char *)w->tape_chunks[w->tape_chunk] + w->tape_off);
            w->tape_off += bytes;
            w->tape_bytes += bytes;
            return NANS_OK;
        }
        ++w->tape_chunk;
        w->tape_off = 0;
    }
    const size_t size = std::max(bytes, (size_t)256 << 20);
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, size);
    if (e != cudaSuccess)
        return fail(NANS_ERR_CUDA, std::string("diff_forward: tape allocation of ") + std::to_string(size) +
                                       " bytes: " + cudaGetErrorString(e));
    w->tape_chunks.push_back(p);
    w->tape_sizes.push_back(size);
    w->tape_chunk = w->tape_chunks.size() - 1;
    w->tape_off = bytes;
    w->tape_bytes += bytes;
    *out = (T *)p;
    return NANS_OK;
}

// One taped step: velocities before RK4 (and this step's external loads), the plain step with
// the solve recording its adjoint data, then the candidate-indexed data copied by solve slot.
int diff_step(nans_world *w, float dt)
{
    cudaStream_t st = w->stream;
    DevWorld &d = w->dw;
    const size_t nd = (size_t)w->n_dyn;
    const int S = w->n_scenes;
    TapeStep t{};
    int rc;
    if ((rc = tape_alloc(w, &t.v_pre, nd)) || (rc = tape_alloc(w, &t.w_pre, nd)))
        return rc;
    CK(cudaMemcpyAsync(t.v_pre, d.vel, nd * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(t.w_pre, d.omg, nd * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    if (w->forces_pending)
    {
        if ((rc = tape_alloc(w, &t.f_ext, nd)) || (rc = tape_alloc(w, &t.t_ext, nd)))
            return rc;
        CK(cudaMemcpyAsync(t.f_ext, d.frc, nd * sizeof(float4), cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(t.t_ext, d.trq, nd * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    }
    if ((rc = step_eager(w, dt, true)))
        return rc;
    int nc = 0;
    CK(cudaMemcpyAsync(&nc, d.n_cand, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    nc = std::max(0, std::min(nc, w->cand_cap));
    if ((rc = tape_alloc(w, &t.a, nc)) || (rc = tape_alloc(w, &t.b, nc)) || (rc = tape_alloc(w, &t.type, nc)) ||
        (rc = tape_alloc(w, &t.k, (size_t)9 * nc)) || (rc = tape_alloc(w, &t.fwd, (size_t)2 * nc)) ||
        (rc = tape_alloc(w, &t.wend, (size_t)nc)) || (rc = tape_alloc(w, &t.cand_begin, S)) ||
        (rc = tape_alloc(w, &t.maxw, S)))
        return rc;
    t.n = nc;
    const int grid = std::max(1, std::min((std::max(nc, S) + 255) / 256, 8 * w->sm_count));
    k_tape_copy<<<grid, 256, 0, st>>>(d, t);
    CK(cudaGetLastError());
    w->tape.push_back(t);
    return NANS_OK;
}

} // namespace

extern "C" {

const char *nans_last_error(void) { return g_err.c_str(); }

int nans_world_create(const nans_world_desc *desc, nans_world **out)
{
    if (!out)
        return fail(NANS_ERR_INVALID_ARGUMENT, "create: null output pointer");
    *out = nullptr;
    nans_world *w = new nans_world();
    if (desc)
    {
        w->device = desc->device;
        w->flags = desc->flags;
        w->max_cand_req = desc->max_candidates;
    }
    if ((w->flags & NANS_WORLD_FUSED_STEP) && (w->flags & NANS_WORLD_WARM_START))
    {
        delete w;
        return fail(NANS_ERR_INVALID_ARGUMENT, "create: the fused step does not support warm starting");
    }
    cudaError_t e = cudaSetDevice(w->device);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithPriority(&w->stream2, cudaStreamNonBlocking, tier_priority());
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&w->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&w->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&w->sm_count, cudaDevAttrMultiProcessorCount, w->device);
    if (e == cudaSuccess)
        e = (cudaError_t)narrow_kernel_attrs();
    if (e == cudaSuccess)
        e = (cudaError_t)large_kernel_attrs();
    if (e != cudaSuccess)
    {
        if (w->stream)
            cudaStreamDestroy(w->stream);
        if (w->stream2)
            cudaStreamDestroy(w->stream2);
        if (w->ev_fork)
            cudaEventDestroy(w->ev_fork);
        if (w->ev_join)
            cudaEventDestroy(w->ev_join);
        delete w;
        return fail(NANS_ERR_CUDA, std::string("create: ") + cudaGetErrorString(e));
    }
    *out = w;
    return NANS_OK;
}

int nans_world_destroy(nans_world *w)
{
    if (!w)
        return NANS_OK;
    cudaSetDevice(w->device);
    if (w->stream)
        cudaStreamSynchronize(w->stream);
    drop_graph(w);
    free_list(w->allocs);
    free_list(w->cand_allocs);
    if (w->d_pairs_out)
        cudaFree(w->d_pairs_out);
    if (w->d_snap)
        cudaFree(w->d_snap);
    if (w->d_snap_hist)
        cudaFree(w->d_snap_hist);
    for (void *p : w->tape_chunks)
        cudaFree(p);
    if (w->d_tape)
        cudaFree(w->d_tape);
    if (w->stream)
        cudaStreamDestroy(w->stream);
    if (w->stream2)
        cudaStreamDestroy(w->stream2);
    if (w->ev_fork)
        cudaEventDestroy(w->ev_fork);
    if (w->ev_join)
        cudaEventDestroy(w->ev_join);
    delete w;
    return NANS_OK;
}

int nans_world_upload(nans_world *w, const nans_cube *cubes, uint32_t ncubes, const nans_sphere *spheres,
                      uint32_t nspheres, const nans_cube *floor, const float *cube_scale, uint32_t flags)
{
    uint32_t nc = ncubes, ns = nspheres;
    return upload_impl(w, 1, &nc, &ns, cubes, spheres, floor, cube_scale, nullptr, nullptr, nullptr, flags);
}

int nans_batch_upload(nans_world *w, uint32_t nscenes, const uint32_t *scene_ncubes, const uint32_t *scene_nspheres,
                      const nans_cube *cubes, const nans_sphere *spheres, const nans_cube *floors,
                      const float *cube_scale, const int32_t *hull_npts, const float *hull_pts,
                      const nans_step_params *scene_params, uint32_t flags)
{
    return upload_impl(w, nscenes, scene_ncubes, scene_nspheres, cubes, spheres, floors, cube_scale, hull_npts,
                       hull_pts, scene_params, flags);
}

int nans_step(nans_world *w, const nans_step_params *params, float dt, uint32_t nsteps)
{
    if (!w)
        return fail(NANS_ERR_INVALID_ARGUMENT, "step: null world");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "step: no scene uploaded");
    if (!valid_dt(dt))
        return fail(NANS_ERR_INVALID_ARGUMENT, "step: dt must be finite and positive");
    CK(cudaSetDevice(w->device));
    if (params)
    {
        const int rc = set_params_all(w, params);
        if (rc)
            return rc;
    }
    CK(cudaMemsetAsync(w->dw.status, 0, sizeof(unsigned), w->stream));
    if (!flags_world_warm(w))
        return plain_steps(w, dt, nsteps);
    for (uint32_t i = 0; i < nsteps; ++i)
    {
        int rc = step_eager(w, dt, true);
        if (rc)
            return rc;
        ++w->eager_steps_run;
    }
    return check_status(w);
}

int nans_batch_step(nans_world *w, float dt, uint32_t nsteps, uint32_t graph_steps)
{
    if (!w)
        return fail(NANS_ERR_INVALID_ARGUMENT, "batch_step: null world");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "batch_step: no scene uploaded");
    if (!valid_dt(dt))
        return fail(NANS_ERR_INVALID_ARGUMENT, "batch_step: dt must be finite and positive");
    CK(cudaSetDevice(w->device));
    CK(cudaMemsetAsync(w->dw.status, 0, sizeof(unsigned), w->stream));
    int rc = batch_steps(w, dt, nsteps, graph_steps ? graph_steps : 60);
    if (rc)
        return rc;
    return check_status(w);
}

int nans_batch_prepare(nans_world *w, float dt, uint32_t graph_steps)
{
    if (!w)
        return fail(NANS_ERR_INVALID_ARGUMENT, "batch_prepare: null world");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "batch_prepare: no scene uploaded");
    if (!valid_dt(dt))
        return fail(NANS_ERR_INVALID_ARGUMENT, "batch_prepare: dt must be finite and positive");
    CK(cudaSetDevice(w->device));
    const uint32_t g = graph_steps ? graph_steps : 60;
    int rc = NANS_OK;
    if (g == 1)
        rc = ensure_graph1(w, dt);
    else if (!(sweep_flags(w) & (SW_FORCES | SW_MODEL_INPUT)))
    {
        cudaGraphExec_t exec = nullptr;
        rc = ensure_graph(w, dt, (int)g, &exec);
    }
    if (rc)
        return rc;
    CK(cudaStreamSynchronize(w->stream));
    return NANS_OK;
}

int nans_batch_autotune(nans_world *w, float dt)
{
    if (!w || !w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "autotune: no scene uploaded");
    if (!valid_dt(dt))
        return fail(NANS_ERR_INVALID_ARGUMENT, "autotune: dt must be finite and positive");
    CK(cudaSetDevice(w->device));
    cudaStream_t st = w->stream;
    const size_t n = (size_t)w->n_all;
    const size_t nhist = (size_t)w->dw.n_words * 32;
    {
        const int r0 = ensure_snapshot(w, true);
        if (r0)
            return r0;
    }
    // snapshot the mutable state (and the per-pair EPA lengths that order the EPA queue) and the
    // host-side step flags: every candidate runs the same window of the simulation
    float4 *bufs[6] = {w->dw.pos, w->dw.ang, w->dw.vel, w->dw.omg, w->dw.frc, w->dw.trq};
    for (int i = 0; i < 6; ++i)
        CK(cudaMemcpyAsync(w->d_snap + i * n, bufs[i], n * sizeof(float4), cudaMemcpyDeviceToDevice, st));
    if (nhist)
        CK(cudaMemcpyAsync(w->d_snap_hist, w->dw.epa_hist, nhist, cudaMemcpyDeviceToDevice, st));
    const bool s_pending = w->pending, s_model = w->model_input, s_forces = w->forces_pending;
    const float s_pdt = w->pending_dt;
    const long long s_steps = w->steps_run;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int rc = NANS_OK;
    // one candidate: a warm step, then kTuneSteps timed steps from the snapshot, restored after
    auto trial = [&](float &ms) -> int {
        int r = step_eager(w, dt, false);
        cudaEventRecord(e0, st);
        for (int k = 0; k < kTuneSteps && r == NANS_OK; ++k)
            r = step_eager(w, dt, false);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        for (int i = 0; i < 6; ++i)
            cudaMemcpyAsync(bufs[i], w->d_snap + i * n, n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
        if (nhist)
            cudaMemcpyAsync(w->dw.epa_hist, w->d_snap_hist, nhist, cudaMemcpyDeviceToDevice, st);
        w->pending = s_pending;
        w->model_input = s_model;
        w->forces_pending = s_forces;
        w->pending_dt = s_pdt;
        w->steps_run = s_steps;
        return r;
    };
    // coordinate descent over the launch parameters, one at a time from the defaults: the cull
    // method (tiles or one lane per pair), the GJK pass's blocks per SM, the solver's threads per
    // scene in its first pass (1 or 2 warps), its blocks per SM for the late scenes (6 or 2),
    // the warp-tier EPA's blocks per SM (2 or 3) and the late scenes' threads (4 or 2 warps)
    struct Axis
    {
        int *field;
        int cands[4];
        int ncand;
    };
    const int solve0_auto = solve_threads(w->max_scene_bodies);
    Axis axes[] = {
        {&w->cull_tiles, {1, 0, 0, 0}, (w->flags & NANS_WORLD_ALL_PAIRS) ? 1 : 2},
        {&w->narrow_bpsm, {0, 4, 0, 0}, 2},
        {&w->solve_threads0, {solve0_auto, 64, 0, 0}, solve0_auto == 32 ? 2 : 1},
        {&w->solve_late_bpsm, {kSolveLateBlocksPerSm, 2, 0, 0}, 2},
        {&w->medium_bpsm, {kMediumBlocksPerSm, 3, 0, 0}, 2},
        {&w->solve_threads1, {kSolveLateThreads, 64, 0, 0}, 2},
    };
    w->tune_trials = 0;
    for (Axis &ax : axes)
    {
        float best = 1e30f;
        int bestv = *ax.field;
        for (int c = 0; c < ax.ncand && rc == NANS_OK; ++c)
        {
            *ax.field = ax.cands[c];
            w->dw.medium_blocks = std::min(w->medium_bpsm * w->sm_count, w->medium_cap_blocks);
            float ms = 0.0f;
            rc = trial(ms);
            ++w->tune_trials;
            if (ms < best)
            {
                best = ms;
                bestv = ax.cands[c];
            }
        }
        *ax.field = bestv;
        w->dw.medium_blocks = std::min(w->medium_bpsm * w->sm_count, w->medium_cap_blocks);
        w->tune_ms = best / kTuneSteps;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    drop_graph(w);
    CK(cudaStreamSynchronize(st));
    CK(cudaMemsetAsync(w->dw.status, 0, sizeof(unsigned), st));
    return rc;
}

int nans_world_set_tuning(nans_world *w, const int32_t *in)
{
    if (!w || !in)
        return fail(NANS_ERR_INVALID_ARGUMENT, "set_tuning: null world or input");
    const bool threads_ok =
        in[1] >= 32 && in[1] <= 256 && in[1] % 32 == 0 && in[2] >= 32 && in[2] <= 256 && in[2] % 32 == 0;
    if (in[0] < 0 || in[0] > 32 || !threads_ok || (in[3] != 0 && in[3] != 1) || in[4] < 1 || in[4] > 32 ||
        in[5] < 1 || in[5] > 3)
        return fail(NANS_ERR_INVALID_ARGUMENT, "set_tuning: GJK blocks per SM in [0, 32], solver threads multiples of "
                                               "32 in [32, 256], cull method 0 or 1, late solver blocks per SM in "
                                               "[1, 32], warp-tier blocks per SM in [1, 3]");
    if (in[1] < 256 && w->max_scene_bodies > 512)
        return fail(NANS_ERR_INVALID_ARGUMENT, "set_tuning: scenes above 512 bodies need 256 solver threads");
    w->narrow_bpsm = in[0];
    w->solve_threads0 = in[1];
    w->solve_threads1 = in[2];
    w->cull_tiles = in[3];
    w->solve_late_bpsm = in[4];
    w->medium_bpsm = in[5];
    w->dw.medium_blocks = std::min(w->medium_bpsm * w->sm_count, w->medium_cap_blocks);
    return NANS_OK;
}

int nans_world_tuning(nans_world *w, int32_t *out)
{
    if (!w || !out)
        return fail(NANS_ERR_INVALID_ARGUMENT, "tuning: null world or output");
    out[0] = w->narrow_bpsm;
    out[1] = w->solve_threads0 ? w->solve_threads0 : solve_threads(w->max_scene_bodies);
    out[2] = w->solve_threads1;
    out[3] = w->cull_tiles;
    out[4] = w->solve_late_bpsm;
    out[5] = w->medium_bpsm;
    out[6] = w->tune_trials;
    out[7] = (int32_t)(1000.0f * w->tune_ms); // microseconds per step of the chosen candidate
    return NANS_OK;
}

int nans_world_download(nans_world *w, nans_cube *cubes, nans_sphere *spheres, nans_cube *floors)
{
    if (!w)
        return fail(NANS_ERR_INVALID_ARGUMENT, "download: null world");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "download: no scene uploaded");
    CK(cudaSetDevice(w->device));
    cudaStream_t st = w->stream;
    if (w->pending)
    {
        k_sweep<<<(w->n_all + kSweepThreads - 1) / kSweepThreads, kSweepThreads, 0, st>>>(w->dw, w->pending_dt, 0.0f,
                                                                                           SW_APPLY_VEL);
        w->pending = false;
        w->model_input = false;
    }
    k_pack<<<(w->n_all + kSweepThreads - 1) / kSweepThreads, kSweepThreads, 0, st>>>(
        w->dw, w->d_rec_cube, w->d_rec_sphere, w->d_rec_floor, w->d_body_rec, w->d_size_moi, w->steps_run > 0);
    CK(cudaGetLastError());
    if (cubes && w->n_cubes)
        CK(cudaMemcpyAsync(cubes, w->d_rec_cube, w->n_cubes * sizeof(nans_cube), cudaMemcpyDeviceToHost, st));
    if (spheres && w->n_spheres)
        CK(cudaMemcpyAsync(spheres, w->d_rec_sphere, w->n_spheres * sizeof(nans_sphere), cudaMemcpyDeviceToHost, st));
    if (floors)
        CK(cudaMemcpyAsync(floors, w->d_rec_floor, w->n_scenes * sizeof(nans_cube), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return NANS_OK;
}

int nans_world_set_state(nans_world *w, const nans_cube *cubes, const nans_sphere *spheres, uint32_t flags)
{
    if (!w)
        return fail(NANS_ERR_INVALID_ARGUMENT, "set_state: null world");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "set_state: no scene uploaded");
    if ((w->n_cubes && !cubes) || (w->n_spheres && !spheres))
        return fail(NANS_ERR_INVALID_ARGUMENT, "set_state: null body records");
    CK(cudaSetDevice(w->device));
    cudaStream_t st = w->stream;
    if (w->n_cubes)
        CK(cudaMemcpyAsync(w->d_rec_cube, cubes, w->n_cubes * sizeof(nans_cube), cudaMemcpyHostToDevice, st));
    if (w->n_spheres)
        CK(cudaMemcpyAsync(w->d_rec_sphere, spheres, w->n_spheres * sizeof(nans_sphere), cudaMemcpyHostToDevice, st));
    // floors keep their state; with KEEP_MODEL their input model is their rebuilt model
    const int mode = (flags & NANS_UPLOAD_KEEP_MODEL) ? (2 | 4) : 0;
    k_unpack<<<(w->n_all + kSweepThreads - 1) / kSweepThreads, kSweepThreads, 0, st>>>(
        w->dw, w->d_rec_cube, w->d_rec_sphere, w->d_rec_floor, w->d_body_rec, mode, w->d_prm, w->d_model_in);
    CK(cudaGetLastError());
    w->pending = false;
    w->model_input = (flags & NANS_UPLOAD_KEEP_MODEL) != 0;
    w->forces_pending = true;
    w->tape_valid = false;
    return warm_invalidate(w);
}

int nans_diff_forward(nans_world *w, const nans_step_params *params, float dt, uint32_t nsteps)
{
    if (!w)
        return fail(NANS_ERR_INVALID_ARGUMENT, "diff_forward: null world");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "diff_forward: no scene uploaded");
    if (!valid_dt(dt))
        return fail(NANS_ERR_INVALID_ARGUMENT, "diff_forward: dt must be finite and positive");
    if (nsteps == 0)
        return fail(NANS_ERR_INVALID_ARGUMENT, "diff_forward: zero steps");
    if (w->flags & NANS_WORLD_WARM_START)
        return fail(NANS_ERR_INVALID_ARGUMENT, "diff_forward: not available with NANS_WORLD_WARM_START");
    CK(cudaSetDevice(w->device));
    if (params)
    {
        const int rc = set_params_all(w, params);
        if (rc)
            return rc;
    }
    CK(cudaMemsetAsync(w->dw.status, 0, sizeof(unsigned), w->stream));
    w->tape.clear();
    w->tape_chunk = 0;
    w->tape_off = 0;
    w->tape_bytes = 0;
    w->tape_valid = false;
    int rc = NANS_OK;
    if (!w->d_maxw && (rc = dalloc(w, w->allocs, &w->d_maxw, w->n_scenes)))
        return rc;
    if (!w->fwd_buf && (rc = dalloc(w, w->cand_allocs, &w->fwd_buf, (size_t)2 * w->cand_cap)))
        return rc;
    w->tape_on = true;
    w->dw.s_fwd = w->fwd_buf;
    w->dw.s_maxw = w->d_maxw;
    for (uint32_t i = 0; i < nsteps && rc == NANS_OK; ++i)
        rc = diff_step(w, dt);
    w->tape_on = false;
    w->dw.s_fwd = nullptr;
    w->dw.s_maxw = nullptr;
    if (rc)
        return rc;
    if ((rc = check_status(w)))
        return rc;
    w->tape_dt = dt;
    w->tape_valid = true;
    return NANS_OK;
}

int nans_diff_backward(nans_world *w, const nans_diff_grads *g)
{
    if (!w || !g)
        return fail(NANS_ERR_INVALID_ARGUMENT, "diff_backward: null world or gradients");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "diff_backward: no scene uploaded");
    if (!w->tape_valid || w->tape.empty())
        return fail(NANS_ERR_NO_TAPE, "diff_backward: no tape for the current state (nans_diff_forward must be "
                                      "the last call that stepped or set the state)");
    CK(cudaSetDevice(w->device));
    cudaStream_t st = w->stream;
    const size_t nd = (size_t)w->n_dyn;
    const int S = w->n_scenes;
    int rc;
    if (!w->d_adj4 && ((rc = dalloc(w, w->allocs, &w->d_adj4, 4 * nd)) ||
                       (rc = dalloc(w, w->allocs, &w->d_adj1, 5 * nd + 2 * (size_t)S + 4)) ||
                       (rc = dalloc(w, w->allocs, &w->d_stage, 3 * nd))))
        return rc;
    const size_t nst = w->tape.size();
    if (w->d_tape_cap < nst)
    {
        if (w->d_tape)
            cudaFree(w->d_tape);
        w->d_tape = nullptr;
        w->d_tape_cap = 0;
        CK(cudaMalloc(&w->d_tape, nst * sizeof(TapeStep)));
        w->d_tape_cap = nst;
    }
    CK(cudaMemcpyAsync(w->d_tape, w->tape.data(), nst * sizeof(TapeStep), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(w->d_adj1, 0, (5 * nd + 2 * (size_t)S + 4) * sizeof(float), st));
    float4 *gP = w->d_adj4, *gA = gP + nd, *gV = gA + nd, *gW = gV + nd;
    const int nb = (int)((nd + kSweepThreads - 1) / kSweepThreads);
    const float *ins[4] = {g->dl_position, g->dl_angles, g->dl_velocity, g->dl_omega};
    float4 *dst[4] = {gP, gA, gV, gW};
    for (int i = 0; i < 4; ++i)
    {
        if (ins[i] && nd)
            CK(cudaMemcpyAsync(w->d_stage, ins[i], 3 * nd * sizeof(float), cudaMemcpyHostToDevice, st));
        if (nd)
            k_rec_to_body<<<nb, kSweepThreads, 0, st>>>(ins[i] ? w->d_stage : nullptr, w->d_body_rec, w->n_cubes,
                                                         w->n_dyn, dst[i]);
    }
    AdjointBufs b{};
    b.gP = gP;
    b.gA = gA;
    b.gV = gV;
    b.gW = gW;
    b.g_invm = w->d_adj1;
    b.g_invi = b.g_invm + nd;
    b.g_z = b.g_invi + nd;
    b.g_zw = b.g_z + nd;
    b.g_mass = b.g_zw + nd;
    b.g_cr = b.g_mass + nd;
    b.g_cf = b.g_cr + S;
    b.err = reinterpret_cast<int *>(b.g_cf + S);
    const int grid = std::max(1, std::min(S, 16 * w->sm_count));
    k_adjoint<<<grid, adjoint_threads(), 0, st>>>(w->dw, w->d_tape, (int)nst, w->tape_dt, b);
    CK(cudaGetLastError());
    float *outs[4] = {g->position0, g->angles0, g->velocity0, g->omega0};
    const float4 *src[4] = {gP, gA, gV, gW};
    for (int i = 0; i < 4; ++i)
        if (outs[i] && nd)
        {
            k_body_to_rec<<<nb, kSweepThreads, 0, st>>>(src[i], nullptr, w->d_body_rec, w->n_cubes, w->n_dyn,
                                                         w->d_stage, 3);
            CK(cudaMemcpyAsync(outs[i], w->d_stage, 3 * nd * sizeof(float), cudaMemcpyDeviceToHost, st));
        }
    if (g->mass && nd)
    {
        k_body_to_rec<<<nb, kSweepThreads, 0, st>>>(nullptr, b.g_mass, w->d_body_rec, w->n_cubes, w->n_dyn,
                                                     w->d_stage, 1);
        CK(cudaMemcpyAsync(g->mass, w->d_stage, nd * sizeof(float), cudaMemcpyDeviceToHost, st));
    }
    if (g->restitution)
        CK(cudaMemcpyAsync(g->restitution, b.g_cr, S * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (g->friction)
        CK(cudaMemcpyAsync(g->friction, b.g_cf, S * sizeof(float), cudaMemcpyDeviceToHost, st));
    int err[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(err, b.err, sizeof(err), cudaMemcpyDeviceToHost, st));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    if (err[0])
        return fail(NANS_ERR_CUDA, "diff_backward: inconsistent tape (check " + std::to_string(err[0]) + ": " +
                                       std::to_string(err[1]) + ", " + std::to_string(err[2]) + ", " +
                                       std::to_string(err[3]) + ")");
    return NANS_OK;
}

int nans_render_scene(nans_world *w, uint32_t scene, const float eye[3], const float target[3], float fov_deg,
                      uint32_t width, uint32_t height, uint8_t *rgb)
{
    if (!w || !eye || !target || !rgb)
        return fail(NANS_ERR_INVALID_ARGUMENT, "render: null argument");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "render: no scene uploaded");
    if (scene >= (uint32_t)w->n_scenes)
        return fail(NANS_ERR_INVALID_ARGUMENT, "render: scene index out of range");
    if (width < 1 || height < 1 || width > 8192 || height > 8192 || !(fov_deg > 1.0f && fov_deg < 179.0f))
        return fail(NANS_ERR_INVALID_ARGUMENT, "render: image size outside [1, 8192] or field of view outside (1, 179)");
    CK(cudaSetDevice(w->device));
    cudaStream_t st = w->stream;
    const size_t n = (size_t)width * height;
    unsigned long long *fb = nullptr;
    unsigned char *img = nullptr;
    CK(cudaMalloc(&fb, n * sizeof(unsigned long long)));
    cudaError_t e = cudaMalloc(&img, 3 * n);
    if (e == cudaSuccess)
        e = (cudaError_t)render_scene(w->dw, (int)scene, eye, target, fov_deg, (int)width, (int)height, fb, img, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(rgb, img, 3 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    cudaFree(fb);
    if (img)
        cudaFree(img);
    if (e != cudaSuccess)
        return fail(NANS_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
    return NANS_OK;
}

int nans_diff_tape_info(nans_world *w, uint32_t *steps, uint64_t *bytes)
{
    if (!w)
        return fail(NANS_ERR_INVALID_ARGUMENT, "diff_tape_info: null world");
    if (steps)
        *steps = w->tape_valid ? (uint32_t)w->tape.size() : 0;
    if (bytes)
        *bytes = w->tape_valid ? (uint64_t)w->tape_bytes : 0;
    return NANS_OK;
}

int nans_world_set_state_arrays(nans_world *w, const float *position, const float *angles, const float *velocity,
                                const float *omega)
{
    if (!w)
        return fail(NANS_ERR_INVALID_ARGUMENT, "set_state_arrays: null world");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "set_state_arrays: no scene uploaded");
    CK(cudaSetDevice(w->device));
    cudaStream_t st = w->stream;
    const size_t n3 = 3 * (size_t)w->n_dyn;
    int rc;
    if (!w->d_state_stage && (rc = dalloc(w, w->allocs, &w->d_state_stage, 4 * n3)))
        return rc;
    const int nb = (w->n_all + kSweepThreads - 1) / kSweepThreads;
    if (w->pending)
    {
        k_sweep<<<nb, kSweepThreads, 0, st>>>(w->dw, w->pending_dt, 0.0f, SW_APPLY_VEL);
        w->pending = false;
    }
    const float *src[4] = {position, angles, velocity, omega};
    int mask = 0;
    for (int q = 0; q < 4; ++q)
        if (src[q] && n3)
        {
            CK(cudaMemcpyAsync(w->d_state_stage + q * n3, src[q], n3 * sizeof(float), cudaMemcpyHostToDevice, st));
            mask |= 1 << q;
        }
    if (mask)
        k_state_in<<<nb, kSweepThreads, 0, st>>>(w->dw, w->d_state_stage, w->d_body_rec, w->n_cubes, mask);
    CK(cudaGetLastError());
    w->model_input = false;
    w->forces_pending = false;
    w->tape_valid = false;
    return warm_invalidate(w);
}

int nans_world_get_state_arrays(nans_world *w, float *position, float *angles, float *velocity, float *omega)
{
    if (!w)
        return fail(NANS_ERR_INVALID_ARGUMENT, "get_state_arrays: null world");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "get_state_arrays: no scene uploaded");
    CK(cudaSetDevice(w->device));
    cudaStream_t st = w->stream;
    const size_t n3 = 3 * (size_t)w->n_dyn;
    int rc;
    if (!w->d_state_stage && (rc = dalloc(w, w->allocs, &w->d_state_stage, 4 * n3)))
        return rc;
    const int nb = (w->n_all + kSweepThreads - 1) / kSweepThreads;
    if (w->pending)
    {
        k_sweep<<<nb, kSweepThreads, 0, st>>>(w->dw, w->pending_dt, 0.0f, SW_APPLY_VEL);
        w->pending = false;
        w->model_input = false;
    }
    float *dst[4] = {position, angles, velocity, omega};
    int mask = 0;
    for (int q = 0; q < 4; ++q)
        if (dst[q])
            mask |= 1 << q;
    if (mask && n3)
    {
        k_state_out<<<nb, kSweepThreads, 0, st>>>(w->dw, w->d_state_stage, w->d_body_rec, w->n_cubes, mask);
        for (int q = 0; q < 4; ++q)
            if (dst[q])
                CK(cudaMemcpyAsync(dst[q], w->d_state_stage + q * n3, n3 * sizeof(float), cudaMemcpyDeviceToHost,
                                   st));
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    return NANS_OK;
}

int nans_get_pairs(nans_world *w, uint32_t scene, nans_contact_pair *out, uint32_t cap, uint32_t *count)
{
    if (!w || !count)
        return fail(NANS_ERR_INVALID_ARGUMENT, "get_pairs: null world or count");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "get_pairs: no scene uploaded");
    if ((int)scene >= w->n_scenes)
        return fail(NANS_ERR_INVALID_ARGUMENT, "get_pairs: scene index out of range");
    CK(cudaSetDevice(w->device));
    cudaStream_t st = w->stream;
    if ((int)cap > w->pairs_out_cap)
    {
        if (w->d_pairs_out)
            cudaFree(w->d_pairs_out);
        w->d_pairs_out = nullptr;
        CK(cudaMalloc(&w->d_pairs_out, (size_t)std::max<uint32_t>(cap, 1) * sizeof(nans_contact_pair)));
        w->pairs_out_cap = (int)std::max<uint32_t>(cap, 1);
    }
    k_pairs_out<<<1, 256, 0, st>>>(w->dw, (int)scene, w->d_pairs_out, (int)cap, w->d_small);
    CK(cudaGetLastError());
    int n = 0;
    CK(cudaMemcpyAsync(&n, w->d_small, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *count = (uint32_t)n;
    uint32_t m = std::min<uint32_t>((uint32_t)n, cap);
    if (out && m)
    {
        CK(cudaMemcpyAsync(out, w->d_pairs_out, m * sizeof(nans_contact_pair), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return NANS_OK;
}

int nans_world_status(nans_world *w, uint32_t *bits)
{
    if (!w || !bits)
        return fail(NANS_ERR_INVALID_ARGUMENT, "status: null argument");
    if (!w->uploaded)
    {
        *bits = 0;
        return NANS_OK;
    }
    CK(cudaSetDevice(w->device));
    unsigned s = 0;
    CK(cudaMemcpyAsync(&s, w->dw.status, sizeof(unsigned), cudaMemcpyDeviceToHost, w->stream));
    CK(cudaMemsetAsync(w->dw.status, 0, sizeof(unsigned), w->stream));
    CK(cudaStreamSynchronize(w->stream));
    *bits = s;
    return NANS_OK;
}

int nans_world_counts(nans_world *w, uint32_t *candidates, uint32_t *contacts)
{
    if (!w || !w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "counts: no scene uploaded");
    CK(cudaSetDevice(w->device));
    int nc = 0;
    if (w->fused)
    {
        // the fused step's candidates: scene s's in [cand_begin[s], cand_end[s]) of its pair space
        CK(cudaStreamSynchronize(w->stream));
        std::vector<int> cb(w->n_scenes), ce(w->n_scenes), h((size_t)std::max(1, w->cand_cap));
        CK(cudaMemcpy(cb.data(), w->dw.cand_begin, w->n_scenes * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(ce.data(), w->dw.cand_end, w->n_scenes * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(h.data(), w->dw.hit, (size_t)w->cand_cap * sizeof(int), cudaMemcpyDeviceToHost));
        uint32_t t = 0;
        for (int sc = 0; sc < w->n_scenes; ++sc)
        {
            nc += ce[sc] - cb[sc];
            for (int i = cb[sc]; i < ce[sc]; ++i)
                t += h[i] ? 1u : 0u;
        }
        if (candidates)
            *candidates = (uint32_t)nc;
        if (contacts)
            *contacts = t;
        return NANS_OK;
    }
    CK(cudaMemcpyAsync(&nc, w->dw.n_cand, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
    CK(cudaStreamSynchronize(w->stream));
    if (candidates)
        *candidates = (uint32_t)nc;
    if (contacts)
    {
        std::vector<int> h(std::max(1, nc));
        if (nc)
            CK(cudaMemcpy(h.data(), w->dw.hit, nc * sizeof(int), cudaMemcpyDeviceToHost));
        uint32_t t = 0;
        for (int i = 0; i < nc; ++i)
            t += h[i] ? 1u : 0u;
        *contacts = t;
    }
    return NANS_OK;
}

void *nans_world_stream(nans_world *w) { return w ? (void *)w->stream : nullptr; }

int nans_world_epa_stats(nans_world *w, uint32_t *out, int reset)
{
    if (!w || !out)
        return fail(NANS_ERR_INVALID_ARGUMENT, "epa_stats: null argument");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "epa_stats: no scene uploaded");
    CK(cudaSetDevice(w->device));
    CK(cudaMemcpyAsync(out, w->dw.epa_stats, 8 * sizeof(uint32_t), cudaMemcpyDeviceToHost, w->stream));
    if (reset)
        CK(cudaMemsetAsync(w->dw.epa_stats, 0, 8 * sizeof(unsigned), w->stream));
    CK(cudaStreamSynchronize(w->stream));
    return NANS_OK;
}

int nans_device_sincos(const float *x, float *s, float *c, uint32_t n)
{
    if (!x || !s || !c || n == 0)
        return fail(NANS_ERR_INVALID_ARGUMENT, "sincos: null argument or n == 0");
    float *d = nullptr;
    CK(cudaMalloc(&d, 3 * (size_t)n * sizeof(float)));
    cudaError_t e = cudaMemcpy(d, x, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
    {
        k_sincos<<<(n + 255) / 256, 256>>>(d, d + n, d + 2 * (size_t)n, (int)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(s, d + n, n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(c, d + 2 * (size_t)n, n * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess)
        return fail(NANS_ERR_CUDA, std::string("sincos: ") + cudaGetErrorString(e));
    return NANS_OK;
}

int nans_profile_steps(nans_world *w, float dt, uint32_t nsteps, float *stage_ms)
{
    if (!w || !stage_ms)
        return fail(NANS_ERR_INVALID_ARGUMENT, "profile: null argument");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "profile: no scene uploaded");
    if (!valid_dt(dt))
        return fail(NANS_ERR_INVALID_ARGUMENT, "profile: dt must be finite and positive");
    CK(cudaSetDevice(w->device));
    cudaStream_t st = w->stream;
    cudaEvent_t ev[7];
    for (int i = 0; i < 7; ++i)
        CK(cudaEventCreate(&ev[i]));
    for (int i = 0; i < 6; ++i)
        stage_ms[i] = 0.0f;
    DevWorld &d = w->dw;
    for (uint32_t k = 0; k < nsteps; ++k)
    {
        CK(cudaMemsetAsync(d.work_counter, 0, kWorkCounters * sizeof(int), st));
        CK(cudaMemsetAsync(d.cand_begin, 0, w->n_scenes * sizeof(int), st));
        CK(cudaMemsetAsync(d.cand_end, 0, w->n_scenes * sizeof(int), st));
        CK(cudaMemsetAsync(d.scene_late, 0, w->n_scenes * sizeof(int), st));
        CK(cudaEventRecord(ev[0], st));
        k_sweep<<<(w->n_all + kSweepThreads - 1) / kSweepThreads, kSweepThreads, 0, st>>>(d, w->pending_dt, dt,
                                                                                           sweep_flags(w));
        CK(cudaEventRecord(ev[1], st));
        enqueue_cull(w);
        CK(cudaEventRecord(ev[2], st));
        launch_narrow_tiny(narrow_grid(w), st, w->dw);
        CK(cudaEventRecord(ev[3], st));
        launch_epa_medium(st, w->dw);
        CK(cudaEventRecord(ev[4], st));
        CK((cudaError_t)launch_narrow_big(st, w->dw));
        CK(cudaEventRecord(ev[5], st));
        launch_solve(w->dw, w->n_scenes, w->solve_threads0 ? w->solve_threads0 : solve_threads(w->max_scene_bodies),
                 solve_smem(w), st, dt, 0);
        launch_solve(w->dw, std::min(w->n_scenes, w->solve_late_bpsm * w->sm_count), w->solve_threads1, solve_smem(w), st,
                 dt, 1);
        CK(cudaEventRecord(ev[6], st));
        CK(cudaGetLastError());
        after_step(w, dt);
        CK(cudaEventSynchronize(ev[6]));
        for (int i = 0; i < 6; ++i)
        {
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
            stage_ms[i] += ms;
        }
    }
    for (int i = 0; i < 7; ++i)
        cudaEventDestroy(ev[i]);
    return check_status(w);
}

int nans_profile_timeline(nans_world *w, float dt, uint32_t nsteps, float *t_ms)
{
    if (!w || !t_ms)
        return fail(NANS_ERR_INVALID_ARGUMENT, "timeline: null argument");
    if (!w->uploaded)
        return fail(NANS_ERR_NOT_UPLOADED, "timeline: no scene uploaded");
    if (!valid_dt(dt))
        return fail(NANS_ERR_INVALID_ARGUMENT, "timeline: dt must be finite and positive");
    CK(cudaSetDevice(w->device));
    cudaStream_t st = w->stream;
    cudaEvent_t ev[8];
    for (int i = 0; i < 8; ++i)
        CK(cudaEventCreate(&ev[i]));
    for (int i = 0; i < 7; ++i)
        t_ms[i] = 0.0f;
    DevWorld &d = w->dw;
    for (uint32_t k = 0; k < nsteps; ++k)
    {
        CK(cudaEventRecord(ev[0], st));
        CK(cudaMemsetAsync(d.work_counter, 0, kWorkCounters * sizeof(int), st));
        CK(cudaMemsetAsync(d.cand_begin, 0, w->n_scenes * sizeof(int), st));
        CK(cudaMemsetAsync(d.cand_end, 0, w->n_scenes * sizeof(int), st));
        CK(cudaMemsetAsync(d.scene_late, 0, w->n_scenes * sizeof(int), st));
        k_sweep<<<(w->n_all + kSweepThreads - 1) / kSweepThreads, kSweepThreads, 0, st>>>(d, w->pending_dt, dt,
                                                                                           sweep_flags(w));
        CK(cudaEventRecord(ev[1], st));
        enqueue_cull(w);
        CK(cudaEventRecord(ev[2], st));
        CK(enqueue_narrow_solve(w, dt, ev + 3));
        CK(cudaGetLastError());
        after_step(w, dt);
        CK(cudaEventSynchronize(ev[7]));
        for (int i = 0; i < 7; ++i)
        {
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, ev[0], ev[i + 1]));
            t_ms[i] += ms;
        }
    }
    for (int i = 0; i < 8; ++i)
        cudaEventDestroy(ev[i]);
    return check_status(w);
}

int nans_world_path_counts(nans_world *w, uint64_t *graph_steps, uint64_t *eager_steps)
{
    if (!w)
        return fail(NANS_ERR_INVALID_ARGUMENT, "path_counts: null world");
    if (graph_steps)
        *graph_steps = w->graph_steps_run;
    if (eager_steps)
        *eager_steps = w->eager_steps_run;
    return NANS_OK;
}

int nans_launches_per_step(nans_world *w, uint32_t *batched, uint32_t *plain)
{
    if (!w)
        return fail(NANS_ERR_INVALID_ARGUMENT, "launches: null world");
    // sweep, [cull mask, cull write], cull scan, gjk, gjk_long, epa_tiny, epa_medium, block
    // EPA, giant EPA, solve (two passes); fused: sweep, scene step, block EPA, giant EPA, late
    // solve
    uint32_t k = w->fused ? 5u : 10 + (w->cull_blocks > 0 ? 2u : 0u);
    if (batched)
        *batched = k;
    if (plain)
        *plain = k;
    return NANS_OK;
}

} // extern "C"
