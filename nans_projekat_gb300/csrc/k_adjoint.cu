// Adjoint of a rollout of plain steps (the differentiable path).
//
// The step is differentiated with the forward pass's contact set and contact geometry held
// fixed: normal, tangents, lever arms and penetration depth are constants of each step. With
// those fixed, the reference's accumulate/clamp loop (code/nans.cpp:1176-1227), which runs on
// constants, has a closed form: normal impulse dn = max(Ln, 0) with
// Ln = (bias0 + (Cr - 1) JdVn) jn, tangent impulses dt = clamp(Lt, -mu Ln, mu Ln) with
// Lt = -JdVt jt and mu = sqrt(2) Cf; jn, jt are the reciprocals of the effective-mass sums
// (code/nans.cpp:1145-1169). The adjoint differentiates that form through the active set the
// forward solve recorded. The relative velocities reduce to dir . (V1 - V2): the angular terms
// of JdV (code/nans.cpp:1149) are cross products with the direction itself.
//
// RK4 on dv/dt = (1/m)(F + m g) - (1.5/m) v (code/nans.cpp:50-70) is exactly
// V+ = P(z) V + h Q(z) b with z = -1.5 h/m, b = F/m + g, P(z) = 1+z+z^2/2+z^3/6+z^4/24 and
// Q(z) = 1+z/2+z^2/6+z^3/24; the angular rate likewise with zw = -1.5 h/I and b = T/I.
// Positions and angles enter only through P+ = P + h V, A+ = A + h W
// (code/nans.cpp:1331-1349), so their adjoints are constant through the rollout.
//
// Scenes are independent, so one block runs the whole reverse sweep of one scene: steps last
// to first, in each step the solve's waves last to first (contacts of one wave touch disjoint
// dynamic bodies, so their adjoint updates do not race), then the RK4 adjoint of the scene's
// bodies. One launch covers the rollout.
#include "nans_kernels.cuh"

namespace nans
{

constexpr int kAdjointThreads = 128;

// Tape of one step, written after the step's solve. Slot j of scene s (cand_begin[s] <= j <
// cand_begin[s] + contacts) receives the contact the solve ran at that position.
__global__ void k_tape_copy(DevWorld w, TapeStep t)
{
    const int n = min(*w.n_cand, w.cand_cap);
    const int stride = gridDim.x * blockDim.x;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride)
    {
        t.wend[j] = w.s_wcnt[j];
        const int s = w.cand_meta[j] >> 3;
        const int cb = w.cand_begin[s], mw = w.s_maxw[s];
        const int nh = mw > 0 ? w.s_wcnt[cb + mw - 1] : 0;
        if (j - cb >= nh)
            continue;
        const int4 id = w.s_ids[j];
        const int c = id.x;
        t.a[j] = id.y;
        t.b[j] = id.z >= 0 ? id.z : -1 - id.z;
        t.type[j] = w.cand_meta[c] & 7;
#pragma unroll
        for (int q = 0; q < 9; ++q)
            t.k[(size_t)9 * j + q] = w.s_k[(size_t)9 * j + q];
        t.fwd[2 * (size_t)j] = w.s_fwd[2 * (size_t)c];
        t.fwd[2 * (size_t)j + 1] = w.s_fwd[2 * (size_t)c + 1];
    }
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < w.n_scenes; s += stride)
    {
        t.cand_begin[s] = w.cand_begin[s];
        t.maxw[s] = w.s_maxw[s];
    }
}

// Records the first inconsistency met (the tape is checked before it is followed).
__device__ __forceinline__ void adj_error(const AdjointBufs &g, int kind, int x, int y, int z)
{
    if (atomicCAS(g.err, 0, kind) == 0)
    {
        g.err[1] = x;
        g.err[2] = y;
        g.err[3] = z;
    }
}

// Adjoint of one contact's solve (contact_apply in k_solve.cu) on the closed form.
__device__ __forceinline__ void contact_adjoint(const DevWorld &w, const TapeStep &t, int j, float cr, float mu,
                                                AdjointBufs &g, float &gcr, float &gmu)
{
    const int a = t.a[j], b = t.b[j];
    const bool wb = !type_b_is_floor(t.type[j]);
    if (a < 0 || a >= w.n_dyn || (wb && (b < 0 || b >= w.n_dyn)))
    {
        adj_error(g, 3, j, a, b);
        return;
    }
    const float4 *k = t.k + (size_t)9 * j;
    const float4 k0 = k[0], k1 = k[1], k2 = k[2], k3 = k[3], k4 = k[4], k5 = k[5], k6 = k[6], k7 = k[7], k8 = k[8];
    const v3 n = xyz(k0), t1 = xyz(k1), t2 = xyz(k2);
    const float jn = k0.w, jt1 = k1.w, jt2 = k2.w, bias0 = k3.w;
    const float invm1 = k4.w, invm2 = k5.w, invi1 = k6.w, invi2 = k7.w;
    const v3 rn1 = xyz(k3), rn2 = xyz(k4), r1t1 = xyz(k5), r2t1 = xyz(k6), r1t2 = xyz(k7), r2t2 = xyz(k8);
    const float4 f0 = t.fwd[2 * (size_t)j], f1 = t.fwd[2 * (size_t)j + 1];
    const float jdvn = f0.x, jdvt1 = f0.y, jdvt2 = f0.z;
    const unsigned flags = __float_as_uint(f0.w);
    const float dn = f1.x, dt1 = f1.y, dt2 = f1.z, ln = f1.w;

    const v3 gV1 = xyz(g.gV[a]), gW1 = xyz(g.gW[a]);
    v3 gV2 = mk3(0.0f, 0.0f, 0.0f), gW2 = mk3(0.0f, 0.0f, 0.0f);
    if (wb)
    {
        gV2 = xyz(g.gV[b]);
        gW2 = xyz(g.gW[b]);
    }
    // V1 += invm1 (dn n + dt1 t1 + dt2 t2), W1 += invi1 (dn rn1 + dt1 r1t1 + dt2 r1t2); body 2
    // the same with minus signs.
    float gdn = invm1 * dot3(gV1, n) + invi1 * dot3(gW1, rn1);
    float gdt1 = invm1 * dot3(gV1, t1) + invi1 * dot3(gW1, r1t1);
    float gdt2 = invm1 * dot3(gV1, t2) + invi1 * dot3(gW1, r1t2);
    const v3 lin = (dn * n + dt1 * t1) + dt2 * t2;
    float gim1 = dot3(gV1, lin);
    float gii1 = dot3(gW1, (dn * rn1 + dt1 * r1t1) + dt2 * r1t2);
    float gim2 = 0.0f, gii2 = 0.0f;
    if (wb)
    {
        gdn -= invm2 * dot3(gV2, n) + invi2 * dot3(gW2, rn2);
        gdt1 -= invm2 * dot3(gV2, t1) + invi2 * dot3(gW2, r2t1);
        gdt2 -= invm2 * dot3(gV2, t2) + invi2 * dot3(gW2, r2t2);
        gim2 = -dot3(gV2, lin);
        gii2 = -dot3(gW2, (dn * rn2 + dt1 * r2t1) + dt2 * r2t2);
    }
    // tangent clamps by the recorded state: 0 free, 1 at +mu Ln, 2 at -mu Ln, 3 zero
    const unsigned s1 = (flags >> 1) & 3u, s2 = (flags >> 3) & 3u;
    float glt1 = 0.0f, glt2 = 0.0f;
    if (s1 == 0u)
        glt1 = gdt1;
    else if (s1 == 1u)
    {
        gdn += mu * gdt1;
        gmu += gdt1 * ln;
    }
    else if (s1 == 2u)
    {
        gdn -= mu * gdt1;
        gmu -= gdt1 * ln;
    }
    if (s2 == 0u)
        glt2 = gdt2;
    else if (s2 == 1u)
    {
        gdn += mu * gdt2;
        gmu += gdt2 * ln;
    }
    else if (s2 == 2u)
    {
        gdn -= mu * gdt2;
        gmu -= gdt2 * ln;
    }
    const float gln = (flags & 1u) ? gdn : 0.0f;
    // Ln = (bias0 + (Cr - 1) JdVn) jn, Lt = -JdVt jt, j = 1 / D
    const float gjdvn = gln * (cr - 1.0f) * jn;
    gcr += gln * jdvn * jn;
    const float gjn = gln * (bias0 + (cr - 1.0f) * jdvn);
    const float gjdvt1 = -glt1 * jt1, gjt1 = -glt1 * jdvt1;
    const float gjdvt2 = -glt2 * jt2, gjt2 = -glt2 * jdvt2;
    // D = invm1 + invm2 + invi1 |r x d|^2 - invi2 |r2 x d|^2 (the reference's sign)
    const float gDn = -gjn * jn * jn, gDt1 = -gjt1 * jt1 * jt1, gDt2 = -gjt2 * jt2 * jt2;
    gim1 += (gDn + gDt1) + gDt2;
    gii1 += (gDn * dot3(rn1, rn1) + gDt1 * dot3(r1t1, r1t1)) + gDt2 * dot3(r1t2, r1t2);
    const v3 gdir = (gjdvn * n + gjdvt1 * t1) + gjdvt2 * t2;
    g.gV[a] = f4(gV1 + gdir, 0.0f);
    g.g_invm[a] += gim1;
    g.g_invi[a] += gii1;
    if (wb)
    {
        gim2 += (gDn + gDt1) + gDt2;
        gii2 -= (gDn * dot3(rn2, rn2) + gDt1 * dot3(r2t1, r2t1)) + gDt2 * dot3(r2t2, r2t2);
        g.gV[b] = f4(gV2 - gdir, 0.0f);
        g.g_invm[b] += gim2;
        g.g_invi[b] += gii2;
    }
}

// RK4 adjoint of one body: gV <- P(z) gV, gW <- P(zw) gW, plus the z / zw / 1/m / 1/I terms.
__device__ __forceinline__ void rk4_adjoint(const TapeStep &t, int b, float4 pr, float h, AdjointBufs &g)
{
    const float z = -1.5f * h * pr.y, zw = -1.5f * h * pr.w;
    const float P = 1.0f + z * (1.0f + z * (0.5f + z * (1.0f / 6.0f + z * (1.0f / 24.0f))));
    const float Q = 1.0f + z * (0.5f + z * (1.0f / 6.0f + z * (1.0f / 24.0f)));
    const float dP = 1.0f + z * (1.0f + z * (0.5f + z * (1.0f / 6.0f)));
    const float dQ = 0.5f + z * (1.0f / 3.0f + z * 0.125f);
    const float Pw = 1.0f + zw * (1.0f + zw * (0.5f + zw * (1.0f / 6.0f + zw * (1.0f / 24.0f))));
    const float Qw = 1.0f + zw * (0.5f + zw * (1.0f / 6.0f + zw * (1.0f / 24.0f)));
    const float dPw = 1.0f + zw * (1.0f + zw * (0.5f + zw * (1.0f / 6.0f)));
    const float dQw = 0.5f + zw * (1.0f / 3.0f + zw * 0.125f);
    const v3 gv = xyz(g.gV[b]), gw = xyz(g.gW[b]);
    const v3 v = xyz(t.v_pre[b]), om = xyz(t.w_pre[b]);
    v3 F = mk3(0.0f, 0.0f, 0.0f), T = mk3(0.0f, 0.0f, 0.0f);
    if (t.f_ext)
    {
        F = xyz(t.f_ext[b]);
        T = xyz(t.t_ext[b]);
    }
    const v3 bl = pr.y * F + mk3(0.0f, -9.81f, 0.0f);
    const v3 bw = pr.w * T;
    g.g_z[b] += dot3(gv, dP * v + (h * dQ) * bl);
    g.g_zw[b] += dot3(gw, dPw * om + (h * dQw) * bw);
    g.g_invm[b] += (h * Q) * dot3(gv, F);
    g.g_invi[b] += (h * Qw) * dot3(gw, T);
    g.gV[b] = f4(P * gv, 0.0f);
    g.gW[b] = f4(Pw * gw, 0.0f);
}

__global__ void __launch_bounds__(kAdjointThreads) k_adjoint(DevWorld w, const TapeStep *steps, int nsteps, float h,
                                                              AdjointBufs g)
{
    __shared__ float s_red[2][kAdjointThreads];
    const int tid = threadIdx.x;
    for (int s = blockIdx.x; s < w.n_scenes; s += gridDim.x)
    {
        const int b0 = w.sc_cube0[s], nb = w.sc_nc[s] + w.sc_ns[s];
        const float cr = w.sc_cr[s];
        const float mu = (float)(1.4142135623730951 * (double)w.sc_cf[s]);
        float gcr = 0.0f, gmu = 0.0f;
        // the last step's P += h V
        for (int i = tid; i < nb; i += blockDim.x)
        {
            const int b = b0 + i;
            const v3 gp = xyz(g.gP[b]), ga = xyz(g.gA[b]);
            g.gV[b] = f4(xyz(g.gV[b]) + h * gp, 0.0f);
            g.gW[b] = f4(xyz(g.gW[b]) + h * ga, 0.0f);
        }
        __syncthreads();
        for (int k = nsteps - 1; k >= 0; --k)
        {
            const TapeStep t = steps[k];
            const int cb = t.cand_begin[s];
            int maxw = t.maxw[s];
            if (cb < 0 || cb > t.n || maxw < 0 || maxw > t.n - cb)
            {
                if (tid == 0)
                    adj_error(g, 1, k, s, maxw);
                maxw = 0;
            }
            for (int wv = maxw; wv >= 1; --wv)
            {
                const int lo = cb + ((wv == 1) ? 0 : t.wend[cb + wv - 2]), hi = cb + t.wend[cb + wv - 1];
                if (lo < cb || hi > t.n || lo > hi)
                {
                    if (tid == 0)
                        adj_error(g, 2, k, s, wv);
                }
                else
                    for (int j = lo + tid; j < hi; j += blockDim.x)
                        contact_adjoint(w, t, j, cr, mu, g, gcr, gmu);
                __syncthreads();
            }
            for (int i = tid; i < nb; i += blockDim.x)
            {
                const int b = b0 + i;
                rk4_adjoint(t, b, w.prm[b], h, g);
                if (k > 0) // the previous step's P += h V
                {
                    g.gV[b] = f4(xyz(g.gV[b]) + h * xyz(g.gP[b]), 0.0f);
                    g.gW[b] = f4(xyz(g.gW[b]) + h * xyz(g.gA[b]), 0.0f);
                }
            }
            __syncthreads();
        }
        // dL/dm with 1/m, 1/I = c/m, z = -1.5 h/m, zw = -1.5 h c/m
        for (int i = tid; i < nb; i += blockDim.x)
        {
            const int b = b0 + i;
            const float4 pr = w.prm[b];
            const float invm = pr.z, inv_im = pr.w * pr.z;
            g.g_mass[b] = (-g.g_invm[b] * invm * invm - g.g_invi[b] * inv_im) +
                          (g.g_z[b] * (1.5f * h) * invm * invm + g.g_zw[b] * (1.5f * h) * inv_im);
        }
        s_red[0][tid] = gcr;
        s_red[1][tid] = gmu;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1)
        {
            if (tid < o)
            {
                s_red[0][tid] += s_red[0][tid + o];
                s_red[1][tid] += s_red[1][tid + o];
            }
            __syncthreads();
        }
        if (tid == 0)
        {
            g.g_cr[s] = s_red[0][0];
            g.g_cf[s] = 1.4142135623730951f * s_red[1][0];
        }
        __syncthreads();
    }
}

// Record order (cubes of all scenes in upload order, then spheres) <-> body order.
__device__ __forceinline__ int rec_index(const int *body_rec, int n_cubes, int b)
{
    const int rk = body_rec[b];
    return rk >= 0 ? rk : n_cubes + (-rk - 1);
}

__global__ void k_rec_to_body(const float *in_rec, const int *body_rec, int n_cubes, int n_dyn, float4 *out)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_dyn)
        return;
    if (!in_rec)
    {
        out[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const float *r = in_rec + 3 * (size_t)rec_index(body_rec, n_cubes, b);
    out[b] = make_float4(r[0], r[1], r[2], 0.0f);
}

__global__ void k_body_to_rec(const float4 *in, const float *in_scalar, const int *body_rec, int n_cubes, int n_dyn,
                              float *out_rec, int comps)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_dyn)
        return;
    const size_t r = (size_t)rec_index(body_rec, n_cubes, b);
    if (comps == 1)
        out_rec[r] = in_scalar[b];
    else
    {
        const float4 v = in[b];
        out_rec[3 * r] = v.x;
        out_rec[3 * r + 1] = v.y;
        out_rec[3 * r + 2] = v.z;
    }
}

int adjoint_threads() { return kAdjointThreads; }

} // namespace nans
