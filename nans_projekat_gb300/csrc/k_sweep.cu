// Body sweep kernels: the fused integrate stage and the record pack/unpack kernels.
//
// k_sweep fuses, per body and in this order:
//   IntegrateVelocities of the previous step   P += dt*V, Angles += dt*W   (code/nans.cpp:1331-1349)
//   the model-matrix rebuild                    Model = T*Rx*Ry*Rz*S       (code/nans.cpp:1913-1923)
//   IntegrateForces of this step                V, W <- RK4; F, T <- 0    (code/nans.cpp:974-1018)
//   UpdateVertices                              vertices = Model * corner  (code/nans.cpp:394-407)
//   a conservative AABB for the pair cull (no reference counterpart)
// It is HBM-bound: one coalesced float4 read and write per state vector.
#include "nans_internal.cuh"
#include "nans_kernels.cuh"

namespace nans
{

// Unit-cube corners in the order of UpdateVertices (code/nans.cpp:399-406).
__constant__ float c_corner[8][3] = {{0.5f, 0.5f, 0.5f},   {0.5f, 0.5f, -0.5f},   {-0.5f, 0.5f, 0.5f},
                                     {-0.5f, 0.5f, -0.5f}, {0.5f, -0.5f, 0.5f},   {0.5f, -0.5f, -0.5f},
                                     {-0.5f, -0.5f, 0.5f}, {-0.5f, -0.5f, -0.5f}};

// MovementFunction (code/nans.cpp:63-70): invm * ((F + (m*9.81)*(0,-1,0)) - 1.5*V)
__device__ __forceinline__ v3 movement(v3 v, v3 f, float m, float invm)
{
    float s = m * 9.81f;
    v3 g = mk3(s * 0.0f, s * -1.0f, s * 0.0f);
    v3 t = (f + g) - (1.5f * v);
    return invm * t;
}

// RotationFunction (code/nans.cpp:72-78): invI * (T - 1.5*W)
__device__ __forceinline__ v3 rotation(v3 w, v3 tq, float invi) { return invi * (tq - (1.5f * w)); }

// RK4 (code/nans.cpp:50-61): Y0 + (1/6) * (((K1 + 2K2) + 2K3) + K4)
__device__ __forceinline__ v3 rk4_move(float dt, v3 y0, v3 f, float m, float invm)
{
    v3 k1 = dt * movement(y0, f, m, invm);
    v3 k2 = dt * movement(y0 + div3(k1, 2.0f), f, m, invm);
    v3 k3 = dt * movement(y0 + div3(k2, 2.0f), f, m, invm);
    v3 k4 = dt * movement(y0 + k3, f, m, invm);
    return y0 + 0x1.555556p-3f * (((k1 + 2.0f * k2) + 2.0f * k3) + k4);
}
__device__ __forceinline__ v3 rk4_rot(float dt, v3 y0, v3 tq, float invi)
{
    v3 k1 = dt * rotation(y0, tq, invi);
    v3 k2 = dt * rotation(y0 + div3(k1, 2.0f), tq, invi);
    v3 k3 = dt * rotation(y0 + div3(k2, 2.0f), tq, invi);
    v3 k4 = dt * rotation(y0 + k3, tq, invi);
    return y0 + 0x1.555556p-3f * (((k1 + 2.0f * k2) + 2.0f * k3) + k4);
}

__device__ __forceinline__ m4 load_model_in(const float4 *mi, int b)
{
    m4 m;
    for (int j = 0; j < 4; ++j)
    {
        float4 c = __ldg(mi + 4 * b + j);
        m.c[j][0] = c.x;
        m.c[j][1] = c.y;
        m.c[j][2] = c.z;
        m.c[j][3] = c.w;
    }
    return m;
}

// Writes hull vertices and returns their AABB (NaN coordinates make it non-finite).
__device__ __forceinline__ void write_vertices(const DevWorld &w, const m4 &model, int4 sh, v3 &lo, v3 &hi)
{
    lo = mk3(FLT_MAX, FLT_MAX, FLT_MAX);
    hi = mk3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    bool finite = true;
    float *out = w.verts + sh.x;
    if (sh.z < 0)
    {
        float v[24];
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            v3 p = xform(model, mk3(c_corner[k][0], c_corner[k][1], c_corner[k][2]));
            v[3 * k] = p.x;
            v[3 * k + 1] = p.y;
            v[3 * k + 2] = p.z;
            finite = finite && isfinite(p.x) && isfinite(p.y) && isfinite(p.z);
            lo = mk3(fminf(lo.x, p.x), fminf(lo.y, p.y), fminf(lo.z, p.z));
            hi = mk3(fmaxf(hi.x, p.x), fmaxf(hi.y, p.y), fmaxf(hi.z, p.z));
        }
        float4 *o4 = reinterpret_cast<float4 *>(out);
#pragma unroll
        for (int q = 0; q < 6; ++q)
            o4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
    else
    {
        const float *lp = w.local_pts + sh.z;
        for (int k = 0; k < sh.y; ++k)
        {
            v3 p = xform(model, mk3(__ldg(lp + 3 * k), __ldg(lp + 3 * k + 1), __ldg(lp + 3 * k + 2)));
            out[3 * k] = p.x;
            out[3 * k + 1] = p.y;
            out[3 * k + 2] = p.z;
            finite = finite && isfinite(p.x) && isfinite(p.y) && isfinite(p.z);
            lo = mk3(fminf(lo.x, p.x), fminf(lo.y, p.y), fminf(lo.z, p.z));
            hi = mk3(fmaxf(hi.x, p.x), fmaxf(hi.y, p.y), fmaxf(hi.z, p.z));
        }
    }
    if (!finite)
        lo.x = __int_as_float(0x7fc00000); // marks the box unbounded in store_box
}

// Stores the AABB the pair cull tests, inflated so that the cull keeps every pair whose
// supports could meet under float rounding: 1e-4 of the larger coordinate magnitude plus
// 1e-5 m. A body with a non-finite coordinate, or one beyond 1e6 m, gets an unbounded box:
// the reference's support map returns (0,0,0) when no vertex beats -FLT_MAX (all dot
// products NaN), so such a body can "touch" any shape that contains the origin, and only
// running GJK on its pairs reproduces that.
__device__ __forceinline__ void store_box(const DevWorld &w, int b, v3 lo, v3 hi)
{
    float mag = fmaxf(fmaxf(fmaxf(fabsf(lo.x), fabsf(hi.x)), fmaxf(fabsf(lo.y), fabsf(hi.y))),
                      fmaxf(fabsf(lo.z), fabsf(hi.z)));
    bool bounded = isfinite(lo.x) && isfinite(lo.y) && isfinite(lo.z) && isfinite(hi.x) && isfinite(hi.y) &&
                   isfinite(hi.z) && mag <= 1e6f;
    if (!bounded)
    {
        w.box_lo[b] = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
        w.box_hi[b] = make_float4(INFINITY, INFINITY, INFINITY, 0.0f);
        return;
    }
    float m = 1e-4f * mag + 1e-5f;
    w.box_lo[b] = make_float4(lo.x - m, lo.y - m, lo.z - m, 0.0f);
    w.box_hi[b] = make_float4(hi.x + m, hi.y + m, hi.z + m, 0.0f);
}

__global__ void k_sweep(DevWorld w, float pending_dt, float dt, int flags)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if ((flags & SW_CLEAR_COUNTERS) && b < kWorkCounters)
        w.work_counter[b] = 0;
    if (b >= w.n_all)
        return;
    const bool is_floor = b >= w.n_dyn;
    int4 sh = __ldg(w.shape + b);
    float4 p4 = w.pos[b];
    float4 a4 = w.ang[b];
    v3 P = xyz(p4), A = xyz(a4);
    if (!is_floor && (flags & SW_APPLY_VEL))
    {
        float4 v4 = w.vel[b], o4 = w.omg[b];
        P = P + pending_dt * xyz(v4);
        A = A + pending_dt * xyz(o4);
        w.pos[b] = f4(P, p4.w);
        w.ang[b] = f4(A, a4.w);
    }
    if (!(flags & SW_INTEGRATE))
        return;
    if (w.warm_step && b == 0)
        atomicAdd(w.warm_step, 1); // a new step: warm-start entries of the last one stay valid
    if (!is_floor)
    {
        float4 pr = __ldg(w.prm + b);
        v3 V = xyz(w.vel[b]), W = xyz(w.omg[b]);
        v3 F = mk3(0.0f, 0.0f, 0.0f), T = mk3(0.0f, 0.0f, 0.0f);
        if (flags & SW_FORCES)
        {
            F = xyz(w.frc[b]);
            T = xyz(w.trq[b]);
            w.frc[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            w.trq[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        V = rk4_move(dt, V, F, pr.x, pr.y);
        W = rk4_rot(dt, W, T, pr.w);
        w.vel[b] = f4(V, 0.0f);
        w.omg[b] = f4(W, 0.0f);
    }
    v3 lo, hi;
    if (sh.y > 0)
    {
        m4 model = (flags & SW_MODEL_INPUT) ? load_model_in(w.model_in, b) : model_of(P, A, xyz(__ldg(w.scl + b)));
        write_vertices(w, model, sh, lo, hi);
    }
    else
    {
        float r = p4.w;
        lo = mk3(P.x - r, P.y - r, P.z - r);
        hi = mk3(P.x + r, P.y + r, P.z + r);
    }
    store_box(w, b, lo, hi);
}

// ------------------------------------------------------------------------------------
// Record pack / unpack: reference records (code/nans.h:303-336) <-> the SoA state.
// ------------------------------------------------------------------------------------
// cube record float offsets
enum
{
    RC_MODEL = 0,
    RC_VERT = 16,
    RC_POS = 40,
    RC_V = 43,
    RC_F = 46,
    RC_ANG = 49,
    RC_W = 52,
    RC_TQ = 55,
    RC_SIZE = 58,
    RC_MASS = 59,
    RC_MOI = 60,
    RC_FLOATS = 61
};
// sphere record float offsets
enum
{
    RS_MODEL = 0,
    RS_POS = 16,
    RS_V = 19,
    RS_F = 22,
    RS_ANG = 25,
    RS_W = 28,
    RS_TQ = 31,
    RS_RADIUS = 34,
    RS_MASS = 35,
    RS_MOI = 36,
    RS_FLOATS = 37
};

__device__ __forceinline__ float4 rd3(const float *r, int o, float w4) { return make_float4(r[o], r[o + 1], r[o + 2], w4); }

// Unpacks records into the state. rec_cube/rec_sphere are indexed by the body's rank
// among cubes / spheres in upload order; floors follow the cubes in rec_floor.
// mode bit 0: also unpack masses/MOI into prm (static data); bit 1: keep Model as input.
// mode bit 2: floors keep their state and get Model = rebuild(Position, Angles, scale) as input
// model (the state update of nans_world_set_state carries no floor records).
__global__ void k_unpack(DevWorld w, const float *rec_cube, const float *rec_sphere, const float *rec_floor,
                         const int *body_rec, int mode, float4 *prm_out, float4 *model_out)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= w.n_all)
        return;
    if (b >= w.n_dyn && (mode & 4))
    {
        m4 m = model_of(xyz(w.pos[b]), xyz(w.ang[b]), xyz(w.scl[b]));
        for (int j = 0; j < 4; ++j)
            model_out[4 * b + j] = make_float4(m.c[j][0], m.c[j][1], m.c[j][2], m.c[j][3]);
        return;
    }
    const float *r;
    bool sphere = false;
    if (b >= w.n_dyn)
        r = rec_floor + (size_t)(b - w.n_dyn) * RC_FLOATS;
    else
    {
        int rk = body_rec[b];
        sphere = rk < 0;
        r = sphere ? rec_sphere + (size_t)(-rk - 1) * RS_FLOATS : rec_cube + (size_t)rk * RC_FLOATS;
    }
    float radius = sphere ? r[RS_RADIUS] : 0.0f;
    int o_pos = sphere ? RS_POS : RC_POS, o_v = sphere ? RS_V : RC_V, o_f = sphere ? RS_F : RC_F;
    int o_a = sphere ? RS_ANG : RC_ANG, o_w = sphere ? RS_W : RC_W, o_t = sphere ? RS_TQ : RC_TQ;
    w.pos[b] = rd3(r, o_pos, radius);
    w.ang[b] = rd3(r, o_a, 0.0f);
    w.vel[b] = rd3(r, o_v, 0.0f);
    w.omg[b] = rd3(r, o_w, 0.0f);
    w.frc[b] = rd3(r, o_f, 0.0f);
    w.trq[b] = rd3(r, o_t, 0.0f);
    if (mode & 1)
    {
        float m = sphere ? r[RS_MASS] : r[RC_MASS];
        float moi = sphere ? r[RS_MOI] : r[RC_MOI];
        // (real32)(1.0 / Mass) in double (code/nans.cpp:68); 1.0f / Mass and 1.0f / MOI in
        // float (code/nans.cpp:76, 1041-1044)
        prm_out[b] = make_float4(m, (float)(1.0 / (double)m), 1.0f / m, 1.0f / moi);
    }
    if ((mode & 2) && !sphere)
    {
        for (int j = 0; j < 4; ++j)
            model_out[4 * b + j] = make_float4(r[RC_MODEL + 4 * j], r[RC_MODEL + 4 * j + 1],
                                               r[RC_MODEL + 4 * j + 2], r[RC_MODEL + 4 * j + 3]);
    }
}

// Packs the state into records. Cube records get Model rebuilt from the current Position /
// Angles (as the reference's render code leaves it after a frame) and the vertices of the
// last integrate stage; sphere records get the render code's sphere Model (scale = Radius,
// code/nans.cpp:1975-1985). Mass, MOI and Size are copied from the static tables.
__global__ void k_pack(DevWorld w, float *rec_cube, float *rec_sphere, float *rec_floor, const int *body_rec,
                       const float2 *size_moi, int vertices_valid)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= w.n_all)
        return;
    float *r;
    bool sphere = false;
    if (b >= w.n_dyn)
        r = rec_floor + (size_t)(b - w.n_dyn) * RC_FLOATS;
    else
    {
        int rk = body_rec[b];
        sphere = rk < 0;
        r = sphere ? rec_sphere + (size_t)(-rk - 1) * RS_FLOATS : rec_cube + (size_t)rk * RC_FLOATS;
    }
    float4 p = w.pos[b], a = w.ang[b], v = w.vel[b], o = w.omg[b], f = w.frc[b], t = w.trq[b];
    float4 pr = w.prm[b];
    v3 P = xyz(p), A = xyz(a);
    v3 S = sphere ? mk3(p.w, p.w, p.w) : xyz(w.scl[b]);
    m4 model = model_of(P, A, S);
    int o_m = sphere ? RS_MODEL : RC_MODEL;
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 4; ++k)
            r[o_m + 4 * j + k] = model.c[j][k];
    int o_pos = sphere ? RS_POS : RC_POS, o_v = sphere ? RS_V : RC_V, o_f = sphere ? RS_F : RC_F;
    int o_a = sphere ? RS_ANG : RC_ANG, o_w = sphere ? RS_W : RC_W, o_t = sphere ? RS_TQ : RC_TQ;
    float vals[6][3] = {{p.x, p.y, p.z}, {v.x, v.y, v.z}, {f.x, f.y, f.z},
                        {a.x, a.y, a.z}, {o.x, o.y, o.z}, {t.x, t.y, t.z}};
    int offs[6] = {o_pos, o_v, o_f, o_a, o_w, o_t};
    for (int q = 0; q < 6; ++q)
        for (int k = 0; k < 3; ++k)
            r[offs[q] + k] = vals[q][k];
    if (sphere)
    {
        r[RS_RADIUS] = p.w;
        r[RS_MASS] = pr.x;
        r[RS_MOI] = size_moi[b].y;
    }
    else
    {
        int4 sh = w.shape[b];
        for (int k = 0; k < 8; ++k)
            for (int c = 0; c < 3; ++c)
                r[RC_VERT + 3 * k + c] = (vertices_valid && k < sh.y) ? w.verts[sh.x + 3 * k + c] : 0.0f;
        r[RC_SIZE] = size_moi[b].x;
        r[RC_MASS] = pr.x;
        r[RC_MOI] = size_moi[b].y;
    }
}

// Dynamic state to and from four float[n][3] arrays in record order (cubes of every scene in
// upload order, then spheres): stage[0] Position, [1] Angles, [2] V, [3] W. mask bit q selects
// array q. The radius kept in pos.w is not touched.
__device__ __forceinline__ size_t state_rec(const int *body_rec, int n_cubes, int b)
{
    const int rk = body_rec[b];
    return (size_t)(rk >= 0 ? rk : n_cubes + (-rk - 1));
}

__global__ void k_state_in(DevWorld w, const float *stage, const int *body_rec, int n_cubes, int mask)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= w.n_dyn)
        return;
    const size_t r = 3 * state_rec(body_rec, n_cubes, b), n3 = 3 * (size_t)w.n_dyn;
    float4 *dst[4] = {w.pos, w.ang, w.vel, w.omg};
    for (int q = 0; q < 4; ++q)
        if (mask & (1 << q))
        {
            const float *x = stage + q * n3 + r;
            const float keep = (q == 0) ? dst[q][b].w : 0.0f;
            dst[q][b] = make_float4(x[0], x[1], x[2], keep);
        }
}

__global__ void k_state_out(DevWorld w, float *stage, const int *body_rec, int n_cubes, int mask)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= w.n_dyn)
        return;
    const size_t r = 3 * state_rec(body_rec, n_cubes, b), n3 = 3 * (size_t)w.n_dyn;
    const float4 *src[4] = {w.pos, w.ang, w.vel, w.omg};
    for (int q = 0; q < 4; ++q)
        if (mask & (1 << q))
        {
            const float4 v = src[q][b];
            float *x = stage + q * n3 + r;
            x[0] = v.x;
            x[1] = v.y;
            x[2] = v.z;
        }
}

// The project sine/cosine on the device, for comparison with the oracle's host copy.
__global__ void k_sincos(const float *x, float *s, float *c, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        nans_sincos(x[i], s + i, c + i);
}

} // namespace nans
