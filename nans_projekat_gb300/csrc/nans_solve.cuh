// The sequential-impulse solver's per-scene parts, shared by the solver kernel (k_solve.cu) and
// the fused per-scene step (k_narrow.cu).
//
// The reference solves the contact list strictly in order (SolveConstraints,
// code/nans.cpp:1538-1548), each contact reading and then updating the velocities of its
// two bodies (Constraint, code/nans.cpp:1020-1329); the floor is never written
// (:1280, :1311). A contact's result depends only on the current V/W of its two bodies, so
// contacts that touch disjoint dynamic bodies commute exactly. Each contact gets a wave
// number wave = 1 + max(last wave of body A, last wave of body B); contacts of one wave run
// in parallel and waves run in order, which reproduces the sequential result bit for bit.
#pragma once
#include "nans_fbound.cuh"
#include "nans_kernels.cuh"

namespace nans
{

__device__ __forceinline__ int block_scan_excl(int v, int *sh, int *total)
{
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1)
    {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        sh[wid] = x;
    __syncthreads();
    if (wid == 0)
    {
        int nw = blockDim.x >> 5;
        int t = (lane < nw) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1)
        {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o)
                t += y;
        }
        if (lane < nw)
            sh[lane] = t;
    }
    __syncthreads();
    int pre = (wid > 0 ? sh[wid - 1] : 0) + x - v;
    *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return pre;
}

// Velocity-independent part of Constraint (code/nans.cpp:1023-1174) for candidate c between
// bodies a and b.
__device__ __forceinline__ void contact_constants(const DevWorld &w, int c, int a, int b, float dt, float4 *k)
{
    v3 n = normalize3(xyz(w.c_n[c]));
    v3 pa = xyz(w.pos[a]), pb = xyz(w.pos[b]);
    float4 pra = w.prm[a], prb = w.prm[b];
    float invi1 = pra.w, invi2 = prb.w, invm1 = pra.z, invm2 = prb.z;
    if (eq3(n, mk3(0.0f, 0.0f, 0.0f)))
        n = normalize3(pb - pa);
    v3 r1 = xyz(w.c_pa[c]) - pa;
    v3 r2 = xyz(w.c_pb[c]) - pb;
    v3 t1 = (n.x >= 0.57735f) ? mk3(n.y, -n.x, 0.0f) : mk3(0.0f, n.z, -n.y);
    v3 t2 = cross3(n, t1);
    float depth = dot3((pa + r1) - (pb + r2), n);
    v3 rn1 = cross3(r1, n), rn2 = cross3(r2, n);
    float jn = invm1 + invm2;
    jn = jn + (invi1 * dot3(rn1, rn1) - invi2 * dot3(-rn2, -rn2));
    jn = 1.0f / jn;
    float bias0 = (-0.3f) / dt * depth;
    v3 r1t1 = cross3(r1, t1), r2t1 = cross3(r2, t1), r1t2 = cross3(r1, t2), r2t2 = cross3(r2, t2);
    float jt1 = invm1 + invm2;
    jt1 = jt1 + (invi1 * dot3(r1t1, r1t1) - invi2 * dot3(-r2t1, -r2t1));
    jt1 = 1.0f / jt1;
    float jt2 = invm1 + invm2;
    jt2 = jt2 + (invi1 * dot3(r1t2, r1t2) - invi2 * dot3(-r2t2, -r2t2));
    jt2 = 1.0f / jt2;
    k[0] = make_float4(n.x, n.y, n.z, jn);
    k[1] = make_float4(t1.x, t1.y, t1.z, jt1);
    k[2] = make_float4(t2.x, t2.y, t2.z, jt2);
    k[3] = make_float4(rn1.x, rn1.y, rn1.z, bias0);
    k[4] = make_float4(rn2.x, rn2.y, rn2.z, invm1);
    k[5] = make_float4(r1t1.x, r1t1.y, r1t1.z, invm2);
    k[6] = make_float4(r2t1.x, r2t1.y, r2t1.z, invi1);
    k[7] = make_float4(r1t2.x, r1t2.y, r1t2.z, invi2);
    k[8] = make_float4(r2t2.x, r2t2.y, r2t2.z, 0.0f);
}

// sqrt(2) * Cf * Sum in double, stored to float (code/nans.cpp:1199, 1214). The product is
// evaluated left to right, so sqrt(2) * Cf (c2) is computed once per scene.
__device__ __forceinline__ double friction_scale(float cf) { return 1.4142135623730951 * (double)cf; }

// The accumulate/clamp loop of Constraint (code/nans.cpp:1176-1230): `iters` rounds of the
// normal impulse (its sum clamped at 0) and the two tangent impulses (their sums clamped to
// the friction bound, which the reference computes once per tangent from the same operands).
// On a GB300 a warp's double-precision instruction holds the FP64 pipe for tens of cycles and
// the bound's multiply and conversions are on the loop's critical path, so the bound comes
// from the certified single-precision product of nans_fbound.cuh (SP_BOUND); when a product
// of the loop is not certified the loop reports false and the caller runs it again with the
// double product. Both give the same values.
template <bool SP_BOUND>
__device__ __forceinline__ bool impulse_loop(float jdvn, float jdvt1, float jdvt2, float bias, float jn, float jt1,
                                             float jt2, double c2, const FBound &fb, int iters, float &sn, float &st1,
                                             float &st2, float &dn, float &dt1, float &dt2)
{
    bool certified = true;
    for (int it = 0; it < iters; ++it)
    {
        float ln = (-jdvn + bias) * jn;
        float old = sn;
        sn = sn + ln;
        if (sn < 0.0f)
            sn = 0.0f;
        dn = sn - old;
        float m;
        if (SP_BOUND)
        {
            bool cert;
            m = fbound_mul(fb, sn, &cert);
            certified = certified && cert;
        }
        else
            m = (float)(c2 * (double)sn);
        float lt1 = (-jdvt1) * jt1;
        old = st1;
        st1 = st1 + lt1;
        if (st1 < -m)
            st1 = -m;
        if (st1 > m)
            st1 = m;
        dt1 = st1 - old;
        float lt2 = (-jdvt2) * jt2;
        old = st2;
        st2 = st2 + lt2;
        if (st2 < -m)
            st2 = -m;
        if (st2 > m)
            st2 = m;
        dt2 = st2 - old;
    }
    return certified;
}

// Velocity-dependent part of Constraint (code/nans.cpp:1149-1156, 1171-1328). With a tape
// attached (w.s_fwd) it also records, per contact, what the adjoint needs: the relative
// normal / tangent velocities, the applied impulses and the active set of the closed form
// (normal impulse max(Ln, 0), tangent impulses clamp(Lt, -mu*Ln, mu*Ln)).
//
// id = the slot's (candidate, body A, body B or -1 - B for the floor, pair-space index), kp its
// constants, hd their first part (read a wave ahead), vel / omg the velocities (the scene's
// shared-memory copy or the world's arrays) at ia / ib.
// The iteration loop's operands (N, T1, T2 with their effective masses, and the Baumgarte
// term), read a wave ahead; the rest of the record is read at the wave's start and needed after
// the loop. (All nine vectors ahead cost the late pass more in resident blocks than it saved.)
// The block wrote these slots itself (placement), so the wave loop reads them with ordinary
// loads, which the SM's L1 may serve: after the block's barrier they see the block's writes.
struct KHead
{
    float4 n, t1, t2; // (N, Jn), (T1, Jt1), (T2, Jt2)
    float bias0;
};
__device__ __forceinline__ KHead load_head(const float4 *kp)
{
    KHead h;
    h.n = kp[0];
    h.t1 = kp[1];
    h.t2 = kp[2];
    h.bias0 = reinterpret_cast<const float *>(kp + 3)[3];
    return h;
}

template <bool WARM>
__device__ __forceinline__ void contact_apply(const DevWorld &w, int4 id, const KHead &hd, const float4 *kp,
                                              float4 *vel, float4 *omg, int ia, int ib, float cr, float cf,
                                              double c2, const FBound &fb, int iters)
{
    const int c = id.x;
    const bool writes_b = id.z >= 0;
    float4 k[9];
#pragma unroll
    for (int q = 3; q < 9; ++q)
        k[q] = kp[q];
    k[0] = hd.n;
    k[1] = hd.t1;
    k[2] = hd.t2;
    v3 n = xyz(k[0]), t1 = xyz(k[1]), t2 = xyz(k[2]);
    float jn = k[0].w, jt1 = k[1].w, jt2 = k[2].w, bias0 = hd.bias0;
    float invm1 = k[4].w, invm2 = k[5].w, invi1 = k[6].w, invi2 = k[7].w;
    v3 V1 = xyz(vel[ia]), W1 = xyz(omg[ia]);
    v3 V2 = xyz(vel[ib]), W2 = xyz(omg[ib]);
    float jdvn = dot3(((V1 + cross3(W1, n)) - V2) - cross3(W2, n), n);
    float jdvt1 = dot3(((V1 + cross3(W1, t1)) - V2) - cross3(W2, t1), t1);
    float jdvt2 = dot3(((V1 + cross3(W1, t2)) - V2) - cross3(W2, t2), t2);
    float bias = bias0 + cr * jdvn;
    float sn = 0.0f, st1 = 0.0f, st2 = 0.0f, dn = 0.0f, dt1 = 0.0f, dt2 = 0.0f;
    int step = 0, pidx = 0;
    if (WARM)
    {
        // warm starting (the reference's TODO at its pair dedupe, code/nans.cpp:1386-1389): a
        // pair in contact at the previous step starts from that step's accumulators
        step = *w.warm_step;
        pidx = id.w;
        const float4 e = w.warm[pidx];
        if (__float_as_int(e.w) == step - 1)
        {
            sn = e.x;
            st1 = e.y;
            st2 = e.z;
        }
    }
    {
        const float sn0 = sn, st10 = st1, st20 = st2;
        if (!(fb.ok && impulse_loop<true>(jdvn, jdvt1, jdvt2, bias, jn, jt1, jt2, c2, fb, iters, sn, st1, st2, dn, dt1,
                                          dt2)))
        {
            sn = sn0;
            st1 = st10;
            st2 = st20;
            dn = dt1 = dt2 = 0.0f;
            impulse_loop<false>(jdvn, jdvt1, jdvt2, bias, jn, jt1, jt2, c2, fb, iters, sn, st1, st2, dn, dt1, dt2);
        }
    }
    if (WARM)
        w.warm[pidx] = make_float4(sn, st1, st2, __int_as_float(step));
    if (w.s_fwd)
    {
        float ln = (-jdvn + bias) * jn;
        float lt1 = (-jdvt1) * jt1, lt2 = (-jdvt2) * jt2;
        float mu = (float)(1.4142135623730951 * (double)cf);
        unsigned flags = 0;
        if (ln > 0.0f && iters > 0)
        {
            flags |= 1u;
            float bound = mu * ln;
            flags |= (lt1 > bound ? 1u : (lt1 < -bound ? 2u : 0u)) << 1;
            flags |= (lt2 > bound ? 1u : (lt2 < -bound ? 2u : 0u)) << 3;
        }
        else
            flags |= (3u << 1) | (3u << 3);
        w.s_fwd[2 * (size_t)c] = make_float4(jdvn, jdvt1, jdvt2, __uint_as_float(flags));
        w.s_fwd[2 * (size_t)c + 1] = make_float4(dn, dt1, dt2, ln);
    }
    v3 li = dn * n, lt1 = dt1 * t1, lt2 = dt2 * t2;
    v3 ai1 = dn * xyz(k[3]), ai2 = dn * xyz(k[4]);
    v3 ai1t1 = dt1 * xyz(k[5]), ai2t1 = dt1 * xyz(k[6]);
    v3 ai1t2 = dt2 * xyz(k[7]), ai2t2 = dt2 * xyz(k[8]);
    V1 = V1 + invm1 * li;
    W1 = W1 + invi1 * ai1;
    V1 = V1 + invm1 * lt1;
    W1 = W1 + invi1 * ai1t1;
    V1 = V1 + invm1 * lt2;
    W1 = W1 + invi1 * ai1t2;
    vel[ia] = f4(V1, 0.0f);
    omg[ia] = f4(W1, 0.0f);
    if (writes_b)
    {
        V2 = V2 - invm2 * li;
        W2 = W2 - invi2 * ai2;
        V2 = V2 - invm2 * lt1;
        W2 = W2 - invi2 * ai2t1;
        V2 = V2 - invm2 * lt2;
        W2 = W2 - invi2 * ai2t2;
        vel[ib] = f4(V2, 0.0f);
        omg[ib] = f4(W2, 0.0f);
    }
}

// Wave labels of a scene's hits b0 .. b0 + n - 1, whose bodies are in s_ab[0 .. n) (A and B + 1,
// 16 bits each; B = -1 for the floor, which orders nothing): thread 0 gives each, in list
// order, wave = 1 + max(last wave of A, last wave of B) (s_last per body, from the scene's
// earlier hits), then the waves go to s_wv and s_wave and their sizes are counted in s_cnt
// (waves <= kWaveChunk). Called by the whole block after a barrier.
__device__ __forceinline__ void label_chunk(const DevWorld &w, int cb, int b0, int n, const int *s_ab, int *s_wv,
                                            int *s_cnt, int *s_last, int *s_maxw)
{
    const int tid = threadIdx.x;
    if (tid == 0)
    {
        int maxw = *s_maxw;
        for (int i = 0; i < n; ++i)
        {
            const int v = s_ab[i];
            const int la = v & 0xffff, lb = (v >> 16) - 1;
            int wv = s_last[la];
            if (lb >= 0)
                wv = max(wv, s_last[lb]);
            wv += 1;
            s_last[la] = wv;
            if (lb >= 0)
                s_last[lb] = wv;
            s_wv[i] = wv;
            maxw = max(maxw, wv);
        }
        *s_maxw = maxw;
    }
    __syncthreads();
    for (int i = tid; i < n; i += blockDim.x)
    {
        const int wv = s_wv[i];
        w.s_wave[cb + b0 + i] = wv;
        if (wv <= kWaveChunk)
            atomicAdd(s_cnt + wv - 1, 1);
    }
    __syncthreads();
}


// Solves scene s with the calling block (every thread calls it; blockDim.x a multiple of 32 and
// at most kWaveChunk): (1) its hits in candidate order, (2) their wave labels, (3) the counting
// sort by wave, (4) the placement with the velocity-independent constants, (5) the waves.
// s_dyn is the dynamic shared memory solve_smem sizes, sh 32 ints and s_maxw one int of shared
// memory. The caller synchronises the block before it reuses that memory.
template <bool WARM>
__device__ __forceinline__ void solve_scene(const DevWorld &w, int s, float dt, float4 *s_dyn, int *sh, int &s_maxw)
{
    int *const s_c = reinterpret_cast<int *>(s_dyn), *const s_ab = s_c + kWaveChunk, *const s_wv = s_ab + kWaveChunk,
               *const s_cnt = s_wv + kWaveChunk, *const s_last = s_cnt + kWaveChunk;
    float4 *const s_vel = s_dyn, *const s_omg = s_dyn + w.solve_cache + 1;
    const int tid = threadIdx.x;
    const int cb = w.cand_begin[s], ce = w.cand_end[s];
    const int c0 = w.sc_cube0[s];
    const int nb = w.sc_nc[s] + w.sc_ns[s];
    // (1) the scene's hits in candidate order and (2) their wave labels. A scene whose
    // candidates fit one chunk (`span` <= kWaveChunk of them, `per` consecutive ones a
    // thread) loads each candidate's hit flag and bodies (scene-local A and B + 1, B = -1
    // for the floor, 16 bits each) at once and keeps its hits in shared memory. A larger
    // scene (whose candidates may be mostly misses) compacts its hits into s_order, eight
    // candidates a thread, then labels them in chunks of kWaveChunk reloaded from there.
    for (int i = tid; i < nb; i += blockDim.x)
        s_last[i] = 0;
    for (int i = tid; i < kWaveChunk; i += blockDim.x)
        s_cnt[i] = 0;
    if (tid == 0)
        s_maxw = 0;
    const int per = kWaveChunk / blockDim.x, span = per * blockDim.x;
    const bool single = ce - cb <= span;
    int nh = 0;
    if (single)
    {
        const int i0 = cb + tid * per;
        unsigned hv = 0u;
        int ab[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            ab[k] = 0;
            if (k < per && i0 + k < ce)
            {
                const int c = i0 + k;
                if (w.hit[c])
                    hv |= 1u << k;
                const int lb = type_b_is_floor(w.cand_meta[c] & 7) ? -1 : w.cand_b[c] - c0;
                ab[k] = (w.cand_a[c] - c0) | ((lb + 1) << 16);
            }
        }
        int p = block_scan_excl(__popc(hv), sh, &nh);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (hv & (1u << k))
            {
                w.s_order[cb + p] = i0 + k;
                s_c[p] = i0 + k;
                s_ab[p] = ab[k];
                ++p;
            }
        __syncthreads();
        label_chunk(w, cb, 0, nh, s_ab, s_wv, s_cnt, s_last, &s_maxw);
    }
    else
    {
        for (int base = cb; base < ce; base += blockDim.x * 8)
        {
            const int i0 = base + tid * 8;
            unsigned hv = 0u;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (i0 + k < ce && w.hit[i0 + k])
                    hv |= 1u << k;
            int tot;
            int pos = cb + nh + block_scan_excl(__popc(hv), sh, &tot);
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (hv & (1u << k))
                    w.s_order[pos++] = i0 + k;
            nh += tot;
        }
        __syncthreads(); // the compaction's last writes to s_order, read back below by other threads
        for (int b0 = 0; b0 < nh; b0 += kWaveChunk)
        {
            const int cnt = min(kWaveChunk, nh - b0);
            for (int i = tid; i < cnt; i += blockDim.x)
            {
                int c = w.s_order[cb + b0 + i];
                if (!dev_check(w, c >= cb && c < ce, 15, c, ce))
                    c = cb;
                const int lb = type_b_is_floor(w.cand_meta[c] & 7) ? -1 : w.cand_b[c] - c0;
                s_ab[i] = (w.cand_a[c] - c0) | ((lb + 1) << 16);
            }
            __syncthreads();
            label_chunk(w, cb, b0, cnt, s_ab, s_wv, s_cnt, s_last, &s_maxw);
        }
    }
    if (nh == 0)
    {
        if (tid == 0 && w.s_maxw)
            w.s_maxw[s] = 0;
        __syncthreads();
        return;
    }
    __syncthreads();
    const int maxw = s_maxw;
    if (tid == 0 && w.s_maxw)
        w.s_maxw[s] = maxw;
    // (3) counting sort by wave. With maxw <= kWaveChunk the wave sizes were counted in
    // s_cnt; their exclusive prefix goes to s_cnt (the placement's cursors) and their ends
    // to s_wcnt[cb + v - 1]. Above that, the counts are made in s_wcnt (maxw entries, and
    // maxw <= nh <= the scene's candidate slots, so scenes never share an entry). Either
    // way, after the placement s_wcnt[cb + v - 1] is the end of wave v (wave 1 starts at 0).
    const bool wide = maxw > kWaveChunk;
    if (wide)
    {
        for (int i = tid; i < maxw; i += blockDim.x)
            w.s_wcnt[cb + i] = 0;
        __syncthreads();
        for (int i = tid; i < nh; i += blockDim.x)
            atomicAdd(w.s_wcnt + cb + w.s_wave[cb + i] - 1, 1);
        __syncthreads();
    }
    {
        int carry = 0;
        for (int base = 0; base < maxw; base += blockDim.x)
        {
            int i = base + tid;
            int v = (i < maxw) ? (wide ? w.s_wcnt[cb + i] : s_cnt[i]) : 0;
            int tot;
            int pre = block_scan_excl(v, sh, &tot);
            if (i < maxw)
            {
                if (wide)
                    w.s_wcnt[cb + i] = carry + pre;
                else
                {
                    s_cnt[i] = carry + pre;
                    w.s_wcnt[cb + i] = carry + pre + v;
                }
            }
            carry += tot;
            __syncthreads();
        }
    }
    // (4) placement in wave order with the velocity-independent constants: slot cb + pos
    // gets the contact's ids and constants. The slots are the scene's own candidate slots
    // (nh <= ce - cb), whose narrowphase use (the simplex of a hit) ended with the per-thread
    // EPA; the order of the contacts inside a wave is immaterial (they commute exactly). A
    // scene of one chunk takes its hits from shared memory, a larger one from s_order.
    for (int i = tid; i < nh; i += blockDim.x)
    {
        int c, a, b, wv;
        if (single)
        {
            const int v = s_ab[i], lb = (v >> 16) - 1;
            c = s_c[i];
            wv = s_wv[i];
            a = c0 + (v & 0xffff);
            b = lb >= 0 ? c0 + lb : w.n_dyn + s;
        }
        else
        {
            c = w.s_order[cb + i];
            wv = w.s_wave[cb + i];
            a = w.cand_a[c];
            b = w.cand_b[c];
        }
        const int pos = cb + (wide ? atomicAdd(w.s_wcnt + cb + wv - 1, 1) : atomicAdd(s_cnt + wv - 1, 1));
        float4 k[9];
        contact_constants(w, c, a, b, dt, k);
#pragma unroll
        for (int q = 0; q < 9; ++q)
            w.s_k[(size_t)9 * pos + q] = k[q];
        w.s_ids[pos] = make_int4(c, a, b >= w.n_dyn ? -1 - b : b, w.cand_pidx ? w.cand_pidx[c] : 0);
    }
    __threadfence_block();
    __syncthreads();
    // (5) waves in order, on the scene's velocities in shared memory when they fit. A wave's
    // bound, a thread's first slot id of the next wave and that slot's first constants are
    // fetched a wave ahead.
    const float cr = w.sc_cr[s], cf = w.sc_cf[s];
    const double c2 = friction_scale(cf);
    const FBound fb = fbound_split(c2);
    const int iters = w.sc_iters[s];
    const bool cached = nb <= w.solve_cache;
    if (cached)
    {
        for (int i = tid; i < nb; i += blockDim.x)
        {
            s_vel[i] = __ldcg(w.vel + c0 + i);
            s_omg[i] = __ldcg(w.omg + c0 + i);
        }
        if (tid == 0)
        {
            s_vel[nb] = __ldcg(w.vel + w.n_dyn + s);
            s_omg[nb] = __ldcg(w.omg + w.n_dyn + s);
        }
        __syncthreads();
    }
    float4 *const vel = cached ? s_vel : w.vel;
    float4 *const omg = cached ? s_omg : w.omg;
    const int off = cached ? c0 : 0;
    // A thread's items are its slots lo + tid, lo + tid + nt, ... of each wave in turn; the
    // record (ids and loop operands) of its next item, in the same wave or the next one, is
    // read while the current one runs.
    const int nt = blockDim.x;
    int lo = 0, hi = w.s_wcnt[cb];
    int hin = maxw > 1 ? w.s_wcnt[cb + 1] : hi;
    int i = tid;       // the thread's current slot
    bool have = false; // id / hd hold slot i's record
    int4 id = make_int4(-1, 0, 0, 0);
    KHead hd = {};
    for (int wv = 1; wv <= maxw; ++wv)
    {
        const int hinn = wv + 1 < maxw ? w.s_wcnt[cb + wv + 1] : hin;
        const bool next_wave = wv < maxw && hi + tid < hin; // the thread has an item in wave wv + 1
        if (i < hi && !have)
        {
            id = w.s_ids[cb + i];
            hd = load_head(w.s_k + (size_t)9 * (cb + i));
        }
        else if (i >= hi)
        {
            // no item in this wave: read the next wave's first one now
            have = next_wave;
            if (next_wave)
            {
                id = w.s_ids[cb + hi + tid];
                hd = load_head(w.s_k + (size_t)9 * (cb + hi + tid));
            }
        }
        while (i < hi)
        {
            const bool in_wave = i + nt < hi;
            const int nx = in_wave ? i + nt : hi + tid;
            const bool nx_ok = in_wave || next_wave;
            int4 idn = make_int4(-1, 0, 0, 0);
            KHead hdn = {};
            if (nx_ok)
            {
                idn = w.s_ids[cb + nx];
                hdn = load_head(w.s_k + (size_t)9 * (cb + nx));
            }
            const int b = id.z >= 0 ? id.z : -1 - id.z;
            const int ib = (cached && id.z < 0) ? nb : b - off;
            contact_apply<WARM>(w, id, hd, w.s_k + (size_t)9 * (cb + i), vel, omg, id.y - off, ib, cr, cf, c2, fb,
                                iters);
            id = idn;
            hd = hdn;
            have = nx_ok;
            i = nx;
        }
        __syncthreads();
        lo = hi;
        hi = hin;
        hin = hinn;
        i = lo + tid;
    }
    if (cached)
    {
        for (int i = tid; i < nb; i += blockDim.x)
        {
            __stcg(w.vel + c0 + i, s_vel[i]);
            __stcg(w.omg + c0 + i, s_omg[i]);
        }
    }
}

} // namespace nans
