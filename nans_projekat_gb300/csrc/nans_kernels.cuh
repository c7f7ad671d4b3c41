// Kernel declarations and launch constants shared by the step kernels and the host runtime.
#pragma once
#include "nans_internal.cuh"

namespace nans
{

// k_sweep flags
enum SweepFlags
{
    SW_APPLY_VEL = 1,   // apply the previous step's P += dt*V, A += dt*W first
    SW_INTEGRATE = 2,   // RK4 + vertices + AABB
    SW_MODEL_INPUT = 4, // take Model from the uploaded records instead of rebuilding it
    SW_FORCES = 8,      // read (then clear) external forces and torques
};

constexpr int kCullThreads = 256;
constexpr int kPairsPerThread = 32;
constexpr int kPairsPerBlock = kCullThreads * kPairsPerThread;

// EPA shared-memory capacities per warp. Vertices: the GJK tetrahedron plus one support per
// EPA iteration (at most 65, code/nans.cpp:804). Faces grow by two per iteration on a convex
// polytope, but the reference's polytope is not always convex (supports can repeat a vertex,
// visible sets can be non-manifold) and runs of all 65 iterations are common; measured on the
// 16,384-scene workload the face list reached ~200 and the horizon ~10 edges. The buffers hold
// 512 faces and 128 edges and report overflow (NANS_ERR_EPA_CAPACITY) instead of dropping data.
constexpr int kEpaMaxVerts = 72;
constexpr int kEpaMaxFaces = 512;
constexpr int kEpaMaxEdges = 128;

__global__ void k_sweep(DevWorld w, float pending_dt, float dt, int flags);
__global__ void k_unpack(DevWorld w, const float *rec_cube, const float *rec_sphere, const float *rec_floor,
                         const int *body_rec, int mode, float4 *prm_out, float4 *model_out);
__global__ void k_pack(DevWorld w, float *rec_cube, float *rec_sphere, float *rec_floor, const int *body_rec,
                       const float2 *size_moi, int vertices_valid);

__global__ void k_sincos(const float *x, float *s, float *c, int n);

__global__ void k_cull_mask(DevWorld w, int all_pairs);
__global__ void k_scan_blocks(DevWorld w, int nblocks);
__global__ void k_cull_write(DevWorld w);

int narrow_blocks_per_sm(int warps);
void launch_narrow(int warps, int grid, cudaStream_t st, const DevWorld &w);
__global__ void k_solve(DevWorld w, float dt);
__global__ void k_pairs_out(DevWorld w, int scene, float *out_rec, int cap, int *count);

} // namespace nans
