/*
 * nans_gb300.h -- C ABI of the GB300 (sm_103a) physics step.
 *
 * Drop-in for the physics step of L4v/nans_projekat: the stage sequence that the
 * reference's frame entry point runs (code/nans.cpp:1756-1764)
 *     Pairs.clear -> IntegrateForces -> DetectCollisions -> SolveConstraints
 *     -> IntegrateVelocities, then the render code's Model rebuild (:1909-1942)
 * with RK4 integration, GJK detection, EPA contact generation and sequential impulses.
 *
 * Conventions
 *   - Host buffers belong to the caller; device buffers belong to the library.
 *   - Every call returns an int status: NANS_OK (0) or one of the NANS_ERR_* codes; a
 *     one-line description of the last failure on the calling thread is available from
 *     nans_last_error(). No C++ exception crosses this boundary.
 *   - One CUDA stream per world. A world is not thread safe; distinct worlds are.
 *   - Results are bit-identical to the reference step compiled with IEEE single precision
 *     and no FP contraction, for every pair list and every body state.
 *
 * The record types keep the reference's layouts byte for byte (code/nans.h:303-372).
 */
#ifndef NANS_GB300_H
#define NANS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- reference record layouts ---------------------------------------------------- */

/* struct cube (code/nans.h:303-319), 244 bytes; Model is a column-major glm::mat4. */
typedef struct nans_cube
{
    float Model[16];
    float Vertices[8][3];
    float Position[3];
    float V[3];
    float Forces[3];
    float Angles[3];
    float W[3];
    float Torque[3];
    float Size;
    float Mass;
    float MOI;
} nans_cube;

/* struct sphere (code/nans.h:321-336), 148 bytes. */
typedef struct nans_sphere
{
    float Model[16];
    float Position[3];
    float V[3];
    float Forces[3];
    float Angles[3];
    float W[3];
    float Torque[3];
    float Radius;
    float Mass;
    float MOI;
} nans_sphere;

/* enum collision_type (code/nans.h:73-89) */
enum nans_collision_type
{
    NANS_CC = 0,
    NANS_CS = 1,
    NANS_CF = 2,
    NANS_SS = 3,
    NANS_SF = 4
};

/* struct contact_pair (code/nans.h:338-372), 96 bytes. Pairs returned by nans_get_pairs
 * carry Type, PointA, PointB, N, IndexA, IndexB as DetectCollisions leaves them
 * (accumulators and tangents zero); IndexB = IndexA for floor pairs. */
typedef struct nans_contact_pair
{
    int32_t Type;
    float DLNormal;
    float DLNormalSum;
    float DLTangent1;
    float DLTangent1Sum;
    float DLTangent2;
    float DLTangent2Sum;
    float PointA[3];
    float PointB[3];
    float N[3];
    float T1[3];
    float T2[3];
    int32_t IndexA;
    int32_t IndexB;
} nans_contact_pair;

/* ---- status codes ------------------------------------------------------------------ */
#define NANS_OK 0
#define NANS_ERR_INVALID_ARGUMENT 1 /* null pointer, zero count, bad scene index */
#define NANS_ERR_CAPACITY 2         /* more candidate pairs than the world's capacity */
#define NANS_ERR_NAN_INPUT 3        /* non-finite or non-positive mass / MOI / size input */
#define NANS_ERR_CUDA 4             /* a CUDA runtime call failed (see nans_last_error) */
#define NANS_ERR_EPA_CAPACITY 5     /* an EPA polytope outgrew its buffers (strict worlds) */
#define NANS_ERR_NOT_UPLOADED 6     /* the world holds no scene yet */
#define NANS_ERR_SCENE_TOO_LARGE 7  /* a scene has more bodies than the solver supports */
#define NANS_ERR_NO_TAPE 8          /* nans_diff_backward without a current forward tape */

/* ---- world ------------------------------------------------------------------------- */

/* Upload flags */
#define NANS_UPLOAD_KEEP_MODEL 1u  /* first step uses the records' Model matrices as given
                                      (exact continuation of a reference state); default:
                                      rebuild Model from Position/Angles/scale first */

/* World flags */
#define NANS_WORLD_ALL_PAIRS 1u    /* run GJK on every pair (the reference's all-pairs
                                      loop); default: conservative AABB cull first */
#define NANS_WORLD_STRICT_EPA 2u   /* an EPA polytope beyond the large-polytope buffers
                                      (8,388,608 faces) fails the step with
                                      NANS_ERR_EPA_CAPACITY; default: that pair gets no
                                      contact (the reference's result for every EPA that does
                                      not converge) and the event is counted */
#define NANS_WORLD_TEST_GIANT_TIER 4u /* testing: every EPA beyond the warp tier's 256 faces
                                      runs on the grid-wide tier (results are the same) */
#define NANS_WORLD_TEST_BARRIER_TIMEOUT 16u /* testing: the grid-wide tier's barrier waits for
                                      one block more than its grid has (an arrival that never
                                      comes) and gives up after 4,096 polls, so that the bounded
                                      wait's error path runs: the step returns
                                      NANS_ERR_EPA_CAPACITY with the timeout status bit. Use with
                                      NANS_WORLD_TEST_GIANT_TIER. The reference caps its loops
                                      instead (code/nans.cpp:804, 915). */
#define NANS_WORLD_GJK_WARP 32u    /* GJK with one warp per candidate pair, the support maps
                                      evaluated across the lanes; default: one thread per pair,
                                      32 pairs per warp (faster on the benchmark workload).
                                      Results are the same. */
#define NANS_WORLD_FUSED_STEP 64u  /* one launch per step detects and solves each scene (cull,
                                      GJK, EPA on the per-thread and warp tiers, solve; a block
                                      per scene) after the sweep, in place of the staged
                                      kernels; EPAs beyond the warp tier still take the large
                                      tiers and the late solve pass. Same results. For worlds of
                                      small scenes, where the staged step's launch chain is the
                                      cost (the reference's own scene). Scenes of at most 1,024
                                      bodies; the candidate buffers hold every pair (the
                                      max_candidates request is raised to that); not with
                                      NANS_WORLD_WARM_START. nans_profile_steps and
                                      nans_profile_timeline still time the staged kernels; of
                                      the launch parameters nans_batch_autotune and
                                      nans_world_set_tuning set, only the late solve pass's
                                      apply to it. */
#define NANS_WORLD_WARM_START 8u   /* warm starting, the reference's TODO at its pair dedupe
                                      (code/nans.cpp:1386-1389): a pair (type, IndexA,
                                      IndexB) that was in contact at the previous step starts
                                      its accumulated impulses from that step's final values
                                      instead of zero. Changes results (off: the reference's
                                      behaviour). Costs 16 bytes of device memory per pair of
                                      the pair space; set_state and upload start it afresh;
                                      not available with nans_diff_forward. */

typedef struct nans_world_desc
{
    int32_t device;          /* CUDA device ordinal */
    uint32_t flags;          /* NANS_WORLD_* */
    uint32_t max_candidates; /* candidate-pair capacity; 0 = 16 per dynamic body + 4096 */
} nans_world_desc;

/* Solver constants. The reference keeps them as literals: restitution Cr = 0.1
 * (code/nans.cpp:1154), friction Cf = 0.1 (:1159), 70 impulse iterations (:1176). */
typedef struct nans_step_params
{
    float cr;
    float cf;
    int32_t iterations;
} nans_step_params;

typedef struct nans_world nans_world;

/* A world replaces the sdl_state that SimUpdateAndRender casts out of the platform's
 * PermanentStorage and initialises on its first call (code/nans.cpp:1721-1729); the world
 * owns the device memory instead of the platform's mmap block (code/sdl_nans.cpp:541-555). */
int nans_world_create(const nans_world_desc *desc, nans_world **out);
int nans_world_destroy(nans_world *world);

/* One scene: the reference's sdl_state bodies (code/nans.h:374-386). cube_scale holds
 * ncubes x 3 model scales or NULL (Size on every axis, code/nans.cpp:1921-1923); the floor's
 * scale is (Size, 1, Size) (code/nans.cpp:1878-1879). Constants default to the reference's
 * literals until nans_step receives others. */
int nans_world_upload(nans_world *world, const nans_cube *cubes, uint32_t ncubes, const nans_sphere *spheres,
                      uint32_t nspheres, const nans_cube *floor, const float *cube_scale, uint32_t flags);

/* Many independent scenes (the batched form). Records are concatenated scene by scene.
 * hull_npts (per cube, 0 = unit-cube corners) and hull_pts (packed local points) describe
 * convex hulls, a shape the reference does not have; pass NULL for boxes only.
 * scene_params (nscenes entries) or NULL for the reference literals. */
int nans_batch_upload(nans_world *world, uint32_t nscenes, const uint32_t *scene_ncubes,
                      const uint32_t *scene_nspheres, const nans_cube *cubes, const nans_sphere *spheres,
                      const nans_cube *floors, const float *cube_scale, const int32_t *hull_npts,
                      const float *hull_pts, const nans_step_params *scene_params, uint32_t flags);

/* The plain drop-in step: nsteps reference steps on every scene of the world, launched
 * stage by stage, synchronised before returning. params (or NULL to keep the current
 * constants) applies to every scene. Replaces the frame's Pairs.clear(), IntegrateForces,
 * DetectCollisions, SolveConstraints, IntegrateVelocities (code/nans.cpp:1756-1764) and the
 * render code's Model rebuild (code/nans.cpp:1909-1942). */
int nans_step(nans_world *world, const nans_step_params *params, float dt, uint32_t nsteps);

/* The batched step: the same stages as persistent kernels with work queues, nsteps steps
 * replayed from a CUDA graph of graph_steps steps (0 = 60). Synchronised before returning.
 * The step of code/nans.cpp:1756-1764 for many independent sdl_states at once (the reference
 * steps one). */
int nans_batch_step(nans_world *world, float dt, uint32_t nsteps, uint32_t graph_steps);

/* Captures, without running a step, the CUDA graph that the next nans_batch_step(world, dt, n,
 * graph_steps) call would replay first (graph capture and instantiation cost milliseconds for
 * large worlds; a caller that times its steps, or runs them under a deadline, prepares the
 * graph beforehand). No reference counterpart. */
int nans_batch_prepare(nans_world *world, float dt, uint32_t graph_steps);

/* Picks narrowphase / solver launch shapes by timing a few steps on the world's own
 * scenes; the state is restored afterwards. No reference counterpart. */
int nans_batch_autotune(nans_world *world, float dt);

/* Bodies back in the reference layouts, all scenes concatenated in upload order; any of
 * the pointers may be NULL. Applies the last step's pending IntegrateVelocities first. What
 * the reference's render code and next frame read from sdl_state's Cubes, Spheres and Floor
 * (code/nans.h:374-386). */
int nans_world_download(nans_world *world, nans_cube *cubes, nans_sphere *spheres, nans_cube *floors);

/* Overwrites the dynamic fields (Position, V, Forces, Angles, W, Torque and, with
 * NANS_UPLOAD_KEEP_MODEL, Model) of every body from records laid out as at upload: the
 * writes the reference's input handling makes to sdl_state between frames (ShootSphere and
 * the debug moves, code/nans.cpp:112-190). */
int nans_world_set_state(nans_world *world, const nans_cube *cubes, const nans_sphere *spheres, uint32_t flags);

/* The dynamic state as four float[n_bodies][3] arrays in record order (the cubes of every
 * scene in upload order, then the spheres): Position, Angles, V, W. Any pointer may be NULL
 * (that quantity is left as it is / not read back). A compact alternative to the records for
 * hosts that exchange state every step (64 bytes per body instead of 244 / 148). set_state
 * applies the last step's pending IntegrateVelocities first, then overwrites; the next step
 * rebuilds Model from Position / Angles and applies no external forces. get_state applies the
 * pending IntegrateVelocities, like nans_world_download, and synchronises. */
int nans_world_set_state_arrays(nans_world *world, const float *position, const float *angles, const float *velocity,
                                const float *omega);
int nans_world_get_state_arrays(nans_world *world, float *position, float *angles, float *velocity, float *omega);

/* Contact list of one scene after its last DetectCollisions, in the reference's order
 * (CC i<j, CF, SF, CS, SS): sdl_state's Pairs vector (code/nans.h:385, filled at
 * code/nans.cpp:1351-1536). *count receives the full count even when it exceeds cap. */
int nans_get_pairs(nans_world *world, uint32_t scene, nans_contact_pair *out, uint32_t cap, uint32_t *count);

/* Device status bits accumulated since the last call (EPA buffer overflow, ...), cleared.
 * Stands in for the reference's printf diagnostics (code/nans.cpp:752, 1109, 1118, 1324). */
int nans_world_status(nans_world *world, uint32_t *status_bits);

/* Counts of the last step: candidate pairs after the cull and contacts. No reference
 * counterpart (the reference tests every pair). */
int nans_world_counts(nans_world *world, uint32_t *candidates, uint32_t *contacts);

/* Large-polytope EPA statistics since upload (or the last reset): out[0] largest face list
 * and out[1] largest horizon seen by the block and giant tiers, out[2] EPAs that went beyond
 * the warp tier, out[3] candidate index + 1 and out[4] scene + 1 of the last EPA that outgrew
 * the giant tier (0 if none), out[5] EPAs that outgrew it, out[6] EPAs escalated from the
 * per-thread tier to the warp tier, out[7] EPAs escalated from the block tier (32,768 faces)
 * to the giant tier. out holds 8 entries. */
int nans_world_epa_stats(nans_world *world, uint32_t *out, int reset);

/* The world's CUDA stream (a cudaStream_t), for event timing by the caller. No reference
 * counterpart. */
void *nans_world_stream(nans_world *world);

/* Profiling; the reference only shows frame time and FPS in its window title
 * (code/sdl_nans.cpp:994-1005).
 * Runs nsteps steps stage by stage with CUDA events on the world's stream between the
 * stages and adds each stage's device time in milliseconds to stage_ms[0..5]:
 * [0] integrate sweep, [1] pair cull (3 kernels), [2] narrowphase (GJK + per-thread EPA),
 * [3] warp-tier EPA, [4] large-polytope EPA, [5] solver. */
int nans_profile_steps(nans_world *world, float dt, uint32_t nsteps, float *stage_ms);

/* Runs nsteps eager steps with the production stream overlap and adds to t_ms[0..6] the time
 * from the step's start at which each stage ended: [0] sweep, [1] cull, [2] GJK + per-thread
 * EPA, [3] warp-tier EPA (second stream), [4] large-polytope EPA (second stream), [5] solve of
 * the scenes without escalated EPAs, [6] solve of the rest (the step's end). */
int nans_profile_timeline(nans_world *world, float dt, uint32_t nsteps, float *t_ms);

/* Kernel launches per step on the batched path and on the plain path. No reference
 * counterpart. */
int nans_launches_per_step(nans_world *world, uint32_t *batched, uint32_t *plain);

/* The launch parameters nans_batch_autotune chose (or the defaults): out[0] GJK blocks per SM
 * (0 = as many as fit), out[1] solver threads per scene in the first solve pass, out[2] solver
 * threads per late scene, out[3] the cull method (1: cube-cube pairs by 32 x 32 tiles, 0: one
 * lane per pair), out[4] late-scene solver blocks per SM, out[5] warp-tier EPA blocks per SM,
 * out[6] candidates the autotuner timed, out[7] the chosen candidate's microseconds per step.
 * No reference counterpart. */
int nans_world_tuning(nans_world *world, int32_t *out);

/* Sets the launch parameters out[0..5] of nans_world_tuning (for instance a choice of the
 * autotuner kept from an earlier run); results do not depend on them. No reference
 * counterpart. */
int nans_world_set_tuning(nans_world *world, const int32_t *in);

/* Steps run since the last upload by nans_step and nans_batch_step, split into those replayed
 * from a CUDA graph and those launched kernel by kernel (the first step after an upload or a
 * set_state, and steps left over from whole graphs). No reference counterpart. */
int nans_world_path_counts(nans_world *world, uint64_t *graph_steps, uint64_t *eager_steps);

/* The project sine/cosine used by the Model rebuild, evaluated on the device (n values); it
 * replaces the sin/cos inside glm::rotate of the rebuild (code/nans.cpp:1913-1924), so that
 * host and device agree bit for bit. */
int nans_device_sincos(const float *x, float *s, float *c, uint32_t n);

/* ---- differentiable rollout --------------------------------------------------------- */

/* No counterpart in the reference, which computes no gradients. nans_diff_forward runs nsteps
 * plain steps (the same kernels and results as nans_step, bit for bit) and keeps, in device
 * memory, a tape of what the adjoint needs: per step the velocities before RK4 and, per
 * contact, the solver's constants, relative velocities, applied impulses and active set.
 * Tape size per step: 32 bytes per dynamic body plus 192 bytes per candidate pair.
 *
 * nans_diff_backward then returns the gradient of a loss L of the final state (the state
 * nans_world_download returns) with respect to the initial state, the masses and the solver
 * constants. The gradient is that of the rollout with each step's contact set and contact
 * geometry (normals, contact points, depths) held at their forward values; within that, it
 * is exact (up to FP32 rounding): the solver's impulses are differentiated through their
 * closed form (normal impulse max(Ln, 0), friction clamped to +-sqrt(2) Cf Ln) on the active
 * set of the forward pass, and RK4 through its exact polynomial form. Under that model, dL/d
 * initial position and angles equal dL/d final position and angles. Mass gradients take the
 * moment of inertia as proportional to the mass (fixed shape).
 *
 * Per-body arrays are float[n][3] (d_mass: float[n]) in record order: the cubes of all scenes
 * in upload order, then the spheres. Per-scene arrays hold one float per scene. Input
 * pointers may be NULL (zero); output pointers may be NULL (not wanted). The tape stays valid
 * until the next step, upload, set_state or forward; the backward may run several times. */
typedef struct nans_diff_grads
{
    const float *dl_position;  /* in: dL/d final Position */
    const float *dl_angles;    /* in: dL/d final Angles */
    const float *dl_velocity;  /* in: dL/d final V */
    const float *dl_omega;     /* in: dL/d final W */
    float *position0;          /* out: dL/d initial Position */
    float *angles0;            /* out: dL/d initial Angles */
    float *velocity0;          /* out: dL/d initial V */
    float *omega0;             /* out: dL/d initial W */
    float *mass;               /* out: dL/d Mass */
    float *restitution;        /* out, per scene: dL/d Cr */
    float *friction;           /* out, per scene: dL/d Cf */
} nans_diff_grads;

int nans_diff_forward(nans_world *world, const nans_step_params *params, float dt, uint32_t nsteps);
int nans_diff_backward(nans_world *world, const nans_diff_grads *grads);

/* Steps and device bytes held by the current tape. */
int nans_diff_tape_info(nans_world *world, uint32_t *steps, uint64_t *bytes);

/* ---- headless rendering ------------------------------------------------------------ */

/* A picture of one scene for visual debugging, without a graphics API (the reference draws with
 * OpenGL, code/nans.cpp:1853-2025): CUDA kernels rasterise the boxes from the step's world
 * vertices and ray-cast the spheres and the ground's top face; convex hulls appear as their
 * bounding spheres. Camera at `eye` looking at `target`, vertical field of view fov_deg.
 * rgb receives width * height * 3 bytes, rows top to bottom. Shows the state as of the last
 * step (the Model rebuild of the step); not meant for per-frame use (it allocates). */
int nans_render_scene(nans_world *world, uint32_t scene, const float eye[3], const float target[3], float fov_deg,
                      uint32_t width, uint32_t height, uint8_t *rgb);

/* ---- allocation-free solve -------------------------------------------------------- */

/* No counterpart in the reference: an extra entry point for callers that must not allocate
 * GPU memory after start-up -- a host that, like the reference's own platform layer, owns all
 * memory and hands it to the simulation library each frame, an engine whose GPU memory belongs
 * to the application's pool, or a real-time loop that forbids allocation once running. The
 * nans_world_* calls allocate with cudaMalloc; this one allocates nothing.
 *
 * It runs the sequential-impulse solve of one scene's contact list -- the same solve as the
 * world's step, contacts touching disjoint bodies in parallel waves, results bit-identical to
 * solving the list in order -- on device buffers the caller owns:
 *   bodies [0, ncubes) are cubes, [ncubes, nbodies) spheres; d_position, d_velocity and
 *   d_angular_velocity hold nbodies x 3 floats, d_mass and d_moi nbodies floats; velocities
 *   are updated in place. floor (host) holds Position[3], V[3], W[3], Mass, MOI of the static
 *   ground; d_pairs holds npairs contact records as nans_get_pairs returns them.
 * Scratch lives in one fixed device array inside the library (about 2.7 MB on every GPU that
 * loads it, kept until the process exits): at most 16,384 bodies and 16,384 contacts per call,
 * larger requests fail with NANS_ERR_INVALID_ARGUMENT. Every call shares that array, so calls
 * whose kernels overlap on the GPU race; serialise them. The first call on a device (and the
 * first after a cudaDeviceReset of it) looks up the array's device address, with that device
 * current. The call is synchronous on `stream` (a cudaStream_t, NULL for the default stream):
 * it waits for the solve and reads a status word back, so it cannot be recorded into a stream
 * capture. A contact naming a body outside the scene, or the same body on both sides, is
 * skipped and reported as NANS_ERR_INVALID_ARGUMENT. */
int nans_solve_contacts_static(uint32_t nbodies, uint32_t ncubes, const float *d_position, const float *d_mass,
                               const float *d_moi, float *d_velocity, float *d_angular_velocity, const float *floor,
                               const nans_contact_pair *d_pairs, uint32_t npairs, float cr, float cf,
                               int32_t iterations, float dt, void *stream);

/* Description of the last failure on the calling thread ("" if none). The reference reports
 * failures only by printf and Assert (code/nans.h:61-69). */
const char *nans_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* NANS_GB300_H */
