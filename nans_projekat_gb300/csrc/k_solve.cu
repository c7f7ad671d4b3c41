// Sequential-impulse solver, one scene per block, scenes taken from a queue.
//
// The reference solves the contact list strictly in order (SolveConstraints,
// code/nans.cpp:1538-1548), each contact reading and then updating the velocities of its
// two bodies (Constraint, code/nans.cpp:1020-1329); the floor is never written
// (:1280, :1311). A contact's result depends only on the current V/W of its two bodies, so
// contacts that touch disjoint dynamic bodies commute exactly. Each contact gets a wave
// number wave = 1 + max(last wave of body A, last wave of body B); contacts of one wave run
// in parallel and waves run in order, which reproduces the sequential result bit for bit.
//
// Per scene: (1) compact the scene's hits in candidate order and (2) label their waves (one
// thread, shared memory; a scene whose candidates fit one chunk keeps its hits in shared memory
// throughout), (3) counting-sort the contacts by wave (wave sizes counted in shared memory),
// (4) place each contact at its slot in wave order with everything that does not depend on
// velocities (normal, tangents, lever arms, effective masses, the Baumgarte term), (5) per
// wave, on a shared-memory copy of the scene's velocities: the 'iterations'-step
// accumulate/clamp loop and the impulse application, in the reference's operation order, with
// each thread's next contact read ahead. The loop's friction bound is the reference's double
// product computed in single precision and certified (nans_fbound.cuh).
#include <algorithm>

#include "nans_solve.cuh"

namespace nans
{

// One scene per block. The waves are latency-bound (a contact's 10-iteration loop per wave),
// so worlds of small scenes use 32-thread blocks (many scenes share an SM) and worlds with a
// scene above 512 bodies 256-thread blocks (its waves hold more contacts).
constexpr int kSolveThreadsMax = 256;

// Dynamic shared memory (solve_smem): during phases 1-4 the chunk's hits (candidate, bodies,
// wave), the wave counts and, per body, the wave of its last contact; during phase 5 the
// scene's velocities V and W (bodies, then the floor) when the scene has at most w.solve_cache
// bodies, else the waves work on the world's arrays.
// pass 0 solves every scene whose contacts are all known after the per-thread EPA tier
// (largest first, a block per scene); pass 1 the scenes with a candidate in the later EPA
// tiers (a persistent grid over the late list), so that pass 0 can run while those tiers do.
template <bool WARM> __global__ void __launch_bounds__(kSolveThreadsMax) k_solve(DevWorld w, float dt, int pass)
{
    extern __shared__ float4 s_dyn[];
    __shared__ int sh[32];
    __shared__ int s_scene, s_maxw;
    const int tid = threadIdx.x;
    for (int round = 0;; ++round)
    {
        if (tid == 0)
        {
            if (pass == 0)
            {
                // one block per scene (the grid covers the scenes; blocks start in index order,
                // so the largest scenes start first), so that blocks retire continuously and
                // the escalation tiers' blocks, launched at a higher priority, find room early
                const int q = blockIdx.x + round * gridDim.x;
                s_scene = (q < w.n_scenes) ? w.sc_order[q] : -1;
                if (s_scene >= 0 && w.scene_late[s_scene])
                    s_scene = -2;
            }
            else if (round == 0)
            {
                // the late scenes among the gridDim.x largest, one per block, first (the largest
                // scenes' waves are the pass's critical path); then the others from the late list
                s_scene = ((int)blockIdx.x < w.n_scenes) ? w.sc_order[blockIdx.x] : -2;
                if (s_scene >= 0 && !w.scene_late[s_scene])
                    s_scene = -2;
            }
            else
            {
                int q = atomicAdd(w.work_counter + 12, 1);
                s_scene = (q < min(w.work_counter[13], w.n_scenes)) ? w.late_list[q] : -1;
                if (s_scene >= 0 && w.sc_rank[s_scene] < (int)gridDim.x)
                    s_scene = -2;
            }
        }
        __syncthreads();
        const int s = s_scene;
        if (s == -1)
            break;
        if (s < 0)
        {
            __syncthreads();
            continue;
        }
        solve_scene<WARM>(w, s, dt, s_dyn, sh, s_maxw);
    }
}

// Writes the contact list of one scene in the reference record layout (code/nans.h:338-372),
// in list order. Single block.
__global__ void k_pairs_out(DevWorld w, int scene, float *out_rec, int cap, int *count)
{
    __shared__ int sh[32];
    const int cb = w.cand_begin[scene], ce = w.cand_end[scene];
    const int c0 = w.sc_cube0[scene], s0 = c0 + w.sc_nc[scene];
    int n = 0;
    for (int base = cb; base < ce; base += blockDim.x)
    {
        int i = base + threadIdx.x;
        int h = (i < ce) ? w.hit[i] : 0;
        int tot;
        int pre = block_scan_excl(h, sh, &tot);
        int slot = n + pre;
        if (h && slot < cap)
        {
            int type = w.cand_meta[i] & 7;
            int a = w.cand_a[i], b = w.cand_b[i];
            int ia = type_a_is_sphere(type) ? a - s0 : a - c0;
            int ib = type_b_is_floor(type) ? ia : (type_b_is_sphere(type) ? b - s0 : b - c0);
            float *r = out_rec + (size_t)slot * 24;
            int *ri = reinterpret_cast<int *>(r);
            for (int q = 0; q < 24; ++q)
                r[q] = 0.0f;
            ri[0] = type;
            float4 pa = w.c_pa[i], pb = w.c_pb[i], nn = w.c_n[i];
            r[7] = pa.x;
            r[8] = pa.y;
            r[9] = pa.z;
            r[10] = pb.x;
            r[11] = pb.y;
            r[12] = pb.z;
            r[13] = nn.x;
            r[14] = nn.y;
            r[15] = nn.z;
            ri[22] = ia;
            ri[23] = ib;
        }
        n += tot;
    }
    if (threadIdx.x == 0)
        *count = n;
}

int solve_threads(int max_scene_bodies) { return max_scene_bodies > 512 ? kSolveThreadsMax : 32; }

int solve_cache_bodies(int max_scene_bodies)
{
    return std::min(max_scene_bodies, (int)(kSolveSmemMax / (2 * sizeof(float4))) - 1);
}

size_t solve_smem(int max_scene_bodies, int cache)
{
    return std::max((size_t)4 * kWaveChunk * sizeof(int) + (size_t)std::max(1, max_scene_bodies) * sizeof(int),
                    (size_t)(cache + 1) * 2 * sizeof(float4));
}

// Warm starting keeps its own instantiation so that the default solve keeps its registers.
int solve_kernel_attrs(const DevWorld &w, int smem)
{
    const void *k = w.warm ? (const void *)k_solve<true> : (const void *)k_solve<false>;
    return (int)cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

void launch_solve(const DevWorld &w, int grid, int threads, size_t smem, cudaStream_t st, float dt, int pass)
{
    if (w.warm)
        k_solve<true><<<grid, threads, smem, st>>>(w, dt, pass);
    else
        k_solve<false><<<grid, threads, smem, st>>>(w, dt, pass);
}

} // namespace nans
