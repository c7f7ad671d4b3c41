// Allocation-free sequential-impulse solve of one scene's contact list.
//
// Who needs this: callers that must not allocate GPU memory after start-up. The reference's
// own host is the model case -- its platform layer reserves all memory once and hands it to
// the hot-reloaded simulation library every frame, and the library is not supposed to grab
// memory of its own while a frame runs. Engines with a fixed GPU memory budget owned by the
// application's pool, and real-time loops that forbid allocation after initialisation for
// latency reasons, are in the same position. nans_world_* cannot serve them: a world
// allocates its buffers with cudaMalloc.
//
// This entry point runs the same solve as the world's solver (waves of contacts that touch
// disjoint bodies, the reference's operation order, bit-identical results) on device
// buffers that the caller owns, and keeps all of its scratch in one file-scope device
// array of fixed size. It never calls cudaMalloc, cudaFree or an allocating library routine.
//
// Limits: at most kMaxBodies bodies and kMaxContacts contacts per call (larger requests are
// rejected with NANS_ERR_INVALID_ARGUMENT). The array lives on every GPU that loads the
// library until the process exits, and every call shares it: calls whose kernels overlap on
// the GPU (two streams, two threads) race on it, so callers must serialise them. What must
// start at zero is cleared by the kernel itself on every call.
#include <cuda_runtime.h>
#include <mutex>

#include "../../include/nans_gb300.h"
#include "nans_math.cuh"

namespace nans
{
void set_last_error(const char *msg); // api.cu: the message nans_last_error() returns
}

namespace
{

constexpr int kMaxBodies = 16384;
constexpr int kMaxContacts = 16384;
constexpr int kThreads = 256;

// Scratch layout (4-byte words):
//   [0]                          error word (bit 0: a contact names a body outside the scene)
//   [1]                          highest wave number
//   last[kMaxBodies]             wave of the last contact that touched each body
//   wave[kMaxContacts]           wave of each contact
//   wcnt[kMaxContacts + 2]       contacts per wave, then wave starts (counting sort)
//   perm[kMaxContacts]           contacts sorted by wave
//   k[kMaxContacts * 36]         velocity-independent constants, 9 float4 per contact
constexpr size_t kOffLast = 4;
constexpr size_t kOffWave = kOffLast + kMaxBodies;
constexpr size_t kOffWcnt = kOffWave + kMaxContacts;
constexpr size_t kOffPerm = kOffWcnt + kMaxContacts + 4;
constexpr size_t kOffK = kOffPerm + kMaxContacts; // multiple of 4 words: float4-aligned
constexpr size_t kScratchWords = kOffK + (size_t)36 * kMaxContacts;
static_assert(kOffK % 4 == 0, "constants must be 16-byte aligned");

// About 2.7 MB, resident on each device that loads the library.
static __device__ __align__(256) unsigned g_solve_scratch[kScratchWords];

// Device address of g_solve_scratch per device, looked up once with that device current. A
// cudaDeviceReset destroys the device's context, and the library's module, with the array in
// it, is loaded again in the next context, possibly at another address. So each entry also keeps
// the id of the context it was taken in, and the address is looked up again when the device's
// current context has another id.
struct ScratchAddr
{
    void *ptr;
    unsigned long long ctx;
};
std::mutex g_setup_mutex;
ScratchAddr g_scratch_addr[64] = {};

typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);

// Id of the calling thread's current context through the driver's cuCtxGetCurrent and
// cuCtxGetId (CUDA 12.0 and later); 0 when the driver does not provide them. Call with
// g_setup_mutex held.
unsigned long long current_context_id()
{
    static bool looked_up = false;
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!looked_up)
    {
        looked_up = true;
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (CtxGetCurrentFn)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (CtxGetIdFn)f;
    }
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, &id) == 0)
        return id;
    return 0;
}

struct Floor
{
    v3 p, v, w;
    float invm, invi;
};

struct Bodies
{
    const float *pos, *mass, *moi;
    float *vel, *omg;
    int nbodies, ncubes;
};

__device__ __forceinline__ v3 ld3(const float *a, int i) { return mk3(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }
__device__ __forceinline__ void st3(float *a, int i, v3 v)
{
    a[3 * i] = v.x;
    a[3 * i + 1] = v.y;
    a[3 * i + 2] = v.z;
}

// Body index of each side of a contact record (code/nans.h:338-372); -1 = the floor,
// -2 = a contact that is skipped and reported: an index outside the scene, or both sides the
// same body.
__device__ __forceinline__ void sides(const Bodies &B, const nans_contact_pair &c, int &a, int &b)
{
    int t = c.Type;
    bool a_sphere = (t == NANS_SS || t == NANS_SF);
    bool b_floor = (t == NANS_CF || t == NANS_SF);
    bool b_sphere = (t == NANS_CS || t == NANS_SS);
    a = a_sphere ? B.ncubes + c.IndexA : c.IndexA;
    b = b_floor ? -1 : (b_sphere ? B.ncubes + c.IndexB : c.IndexB);
    int nsph = B.nbodies - B.ncubes;
    bool a_ok = c.IndexA >= 0 && (a_sphere ? c.IndexA < nsph : c.IndexA < B.ncubes);
    bool b_ok = b_floor || (c.IndexB >= 0 && (b_sphere ? c.IndexB < nsph : c.IndexB < B.ncubes));
    // a contact whose two sides are one body: the sequential solve would interleave the two
    // sides' updates on that body, which the per-side loads and stores below cannot reproduce
    if (t < 0 || t > 4 || !a_ok || !b_ok || (b >= 0 && a == b))
        a = b = -2;
}

__global__ void __launch_bounds__(kThreads) k_solve_static(unsigned *scratch, Bodies B, Floor F,
                                                            const nans_contact_pair *pairs, int npairs, float cr,
                                                            float cf, int iters, float dt)
{
    unsigned *last = scratch + kOffLast;
    int *wave = reinterpret_cast<int *>(scratch + kOffWave);
    int *wcnt = reinterpret_cast<int *>(scratch + kOffWcnt);
    int *perm = reinterpret_cast<int *>(scratch + kOffPerm);
    float4 *K = reinterpret_cast<float4 *>(scratch + kOffK);
    const int tid = threadIdx.x;
    // clear what must start at zero
    if (tid == 0)
    {
        scratch[0] = 0u;
        scratch[1] = 0u;
    }
    for (int i = tid; i < B.nbodies; i += blockDim.x)
        last[i] = 0u;
    for (int i = tid; i < npairs + 2; i += blockDim.x)
        wcnt[i] = 0;
    __syncthreads();
    // wave labels, in list order (one thread)
    if (tid == 0)
    {
        unsigned maxw = 0;
        for (int k = 0; k < npairs; ++k)
        {
            int a, b;
            sides(B, pairs[k], a, b);
            if (a == -2)
            {
                scratch[0] |= 1u;
                wave[k] = 0; // skipped
                continue;
            }
            unsigned w = last[a];
            if (b >= 0)
                w = max(w, last[b]);
            w += 1u;
            last[a] = w;
            if (b >= 0)
                last[b] = w;
            wave[k] = (int)w;
            maxw = max(maxw, w);
        }
        scratch[1] = maxw;
    }
    __syncthreads();
    const int maxw = (int)scratch[1];
    // counting sort by wave (wave 0 holds skipped contacts)
    for (int k = tid; k < npairs; k += blockDim.x)
        atomicAdd(wcnt + wave[k] + 1, 1);
    __syncthreads();
    if (tid == 0)
        for (int w = 1; w <= maxw + 1; ++w)
            wcnt[w] += wcnt[w - 1];
    __syncthreads();
    for (int k = tid; k < npairs; k += blockDim.x)
        perm[atomicAdd(wcnt + wave[k], 1)] = k;
    // velocity-independent part of Constraint (code/nans.cpp:1023-1174)
    for (int k = tid; k < npairs; k += blockDim.x)
    {
        int a, b;
        sides(B, pairs[k], a, b);
        if (a == -2)
            continue;
        const nans_contact_pair &c = pairs[k];
        v3 n = normalize3(mk3(c.N[0], c.N[1], c.N[2]));
        v3 pa = ld3(B.pos, a);
        v3 pb = (b >= 0) ? ld3(B.pos, b) : F.p;
        float invi1 = 1.0f / B.moi[a], invm1 = 1.0f / B.mass[a];
        float invi2 = (b >= 0) ? 1.0f / B.moi[b] : F.invi;
        float invm2 = (b >= 0) ? 1.0f / B.mass[b] : F.invm;
        if (eq3(n, mk3(0.0f, 0.0f, 0.0f)))
            n = normalize3(pb - pa);
        v3 r1 = mk3(c.PointA[0], c.PointA[1], c.PointA[2]) - pa;
        v3 r2 = mk3(c.PointB[0], c.PointB[1], c.PointB[2]) - pb;
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
        float4 *q = K + (size_t)9 * k;
        q[0] = make_float4(n.x, n.y, n.z, jn);
        q[1] = make_float4(t1.x, t1.y, t1.z, jt1);
        q[2] = make_float4(t2.x, t2.y, t2.z, jt2);
        q[3] = make_float4(rn1.x, rn1.y, rn1.z, bias0);
        q[4] = make_float4(rn2.x, rn2.y, rn2.z, invm1);
        q[5] = make_float4(r1t1.x, r1t1.y, r1t1.z, invm2);
        q[6] = make_float4(r2t1.x, r2t1.y, r2t1.z, invi1);
        q[7] = make_float4(r1t2.x, r1t2.y, r1t2.z, invi2);
        q[8] = make_float4(r2t2.x, r2t2.y, r2t2.z, 0.0f);
    }
    __syncthreads();
    // waves in order; wave w occupies perm[wcnt[w-1], wcnt[w])
    for (int w = 1; w <= maxw; ++w)
    {
        for (int i = wcnt[w - 1] + tid; i < wcnt[w]; i += blockDim.x)
        {
            int k = perm[i];
            int a, b;
            sides(B, pairs[k], a, b);
            const float4 *q = K + (size_t)9 * k;
            v3 n = xyz(q[0]), t1 = xyz(q[1]), t2 = xyz(q[2]);
            float jn = q[0].w, jt1 = q[1].w, jt2 = q[2].w, bias0 = q[3].w;
            float invm1 = q[4].w, invm2 = q[5].w, invi1 = q[6].w, invi2 = q[7].w;
            v3 V1 = ld3(B.vel, a), W1 = ld3(B.omg, a);
            v3 V2 = (b >= 0) ? ld3(B.vel, b) : F.v;
            v3 W2 = (b >= 0) ? ld3(B.omg, b) : F.w;
            float jdvn = dot3(((V1 + cross3(W1, n)) - V2) - cross3(W2, n), n);
            float jdvt1 = dot3(((V1 + cross3(W1, t1)) - V2) - cross3(W2, t1), t1);
            float jdvt2 = dot3(((V1 + cross3(W1, t2)) - V2) - cross3(W2, t2), t2);
            float bias = bias0 + cr * jdvn;
            float sn = 0.0f, st1 = 0.0f, st2 = 0.0f, dn = 0.0f, dt1 = 0.0f, dt2 = 0.0f;
            for (int it = 0; it < iters; ++it)
            {
                float ln = (-jdvn + bias) * jn;
                float old = sn;
                sn = sn + ln;
                if (sn < 0.0f)
                    sn = 0.0f;
                dn = sn - old;
                float lt1 = (-jdvt1) * jt1;
                old = st1;
                st1 = st1 + lt1;
                float m1 = (float)(1.4142135623730951 * (double)cf * (double)sn);
                if (st1 < -m1)
                    st1 = -m1;
                if (st1 > m1)
                    st1 = m1;
                dt1 = st1 - old;
                float lt2 = (-jdvt2) * jt2;
                old = st2;
                st2 = st2 + lt2;
                float m2 = (float)(1.4142135623730951 * (double)cf * (double)sn);
                if (st2 < -m2)
                    st2 = -m2;
                if (st2 > m2)
                    st2 = m2;
                dt2 = st2 - old;
            }
            v3 li = dn * n, lt1 = dt1 * t1, lt2 = dt2 * t2;
            V1 = V1 + invm1 * li;
            W1 = W1 + invi1 * (dn * xyz(q[3]));
            V1 = V1 + invm1 * lt1;
            W1 = W1 + invi1 * (dt1 * xyz(q[5]));
            V1 = V1 + invm1 * lt2;
            W1 = W1 + invi1 * (dt2 * xyz(q[7]));
            st3(B.vel, a, V1);
            st3(B.omg, a, W1);
            if (b >= 0)
            {
                V2 = V2 - invm2 * li;
                W2 = W2 - invi2 * (dn * xyz(q[4]));
                V2 = V2 - invm2 * lt1;
                W2 = W2 - invi2 * (dt1 * xyz(q[6]));
                V2 = V2 - invm2 * lt2;
                W2 = W2 - invi2 * (dt2 * xyz(q[8]));
                st3(B.vel, b, V2);
                st3(B.omg, b, W2);
            }
        }
        __syncthreads();
    }
}

int static_fail(int code, const char *msg)
{
    nans::set_last_error(msg);
    return code;
}

} // namespace

extern "C" int nans_solve_contacts_static(uint32_t nbodies, uint32_t ncubes, const float *d_position,
                                          const float *d_mass, const float *d_moi, float *d_velocity,
                                          float *d_angular_velocity, const float *floor,
                                          const nans_contact_pair *d_pairs, uint32_t npairs, float cr, float cf,
                                          int32_t iterations, float dt, void *stream)
{
    if (nbodies > (uint32_t)kMaxBodies)
        return static_fail(NANS_ERR_INVALID_ARGUMENT,
                           "nans_solve_contacts_static: more than 16384 bodies (static scratch limit)");
    if (npairs > (uint32_t)kMaxContacts)
        return static_fail(NANS_ERR_INVALID_ARGUMENT,
                           "nans_solve_contacts_static: more than 16384 contacts (static scratch limit)");
    if (ncubes > nbodies || !floor || (npairs > 0 && (!d_pairs || nbodies == 0)) ||
        (nbodies > 0 && (!d_position || !d_mass || !d_moi || !d_velocity || !d_angular_velocity)))
        return static_fail(NANS_ERR_INVALID_ARGUMENT, "nans_solve_contacts_static: null or inconsistent argument");
    if (!(dt > 0.0f) || iterations < 0)
        return static_fail(NANS_ERR_INVALID_ARGUMENT, "nans_solve_contacts_static: dt must be positive");
    if (npairs == 0)
        return NANS_OK;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64)
        return static_fail(NANS_ERR_CUDA, "nans_solve_contacts_static: no current CUDA device");
    void *scratch = nullptr;
    {
        // set-up, once per device (again after a reset of that device), with that device
        // current: the device address of the scratch array. cudaSetDevice makes the device's
        // primary context current on this thread, so that its id can be read.
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        e = cudaSetDevice(dev);
        if (e != cudaSuccess)
            return static_fail(NANS_ERR_CUDA, "nans_solve_contacts_static: cudaSetDevice failed");
        const unsigned long long ctx = current_context_id();
        if (!g_scratch_addr[dev].ptr || ctx == 0 || ctx != g_scratch_addr[dev].ctx)
        {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_solve_scratch);
            if (e != cudaSuccess || !p)
                return static_fail(NANS_ERR_CUDA, "nans_solve_contacts_static: cudaGetSymbolAddress failed");
            g_scratch_addr[dev].ptr = p;
            g_scratch_addr[dev].ctx = ctx;
        }
        scratch = g_scratch_addr[dev].ptr;
    }
    Bodies B{d_position, d_mass, d_moi, d_velocity, d_angular_velocity, (int)nbodies, (int)ncubes};
    // floor: Position[3], V[3], W[3], Mass, MOI
    Floor F{mk3(floor[0], floor[1], floor[2]), mk3(floor[3], floor[4], floor[5]), mk3(floor[6], floor[7], floor[8]),
            1.0f / floor[9], 1.0f / floor[10]};
    cudaStream_t st = (cudaStream_t)stream;
    k_solve_static<<<1, kThreads, 0, st>>>((unsigned *)scratch, B, F, d_pairs, (int)npairs, cr, cf, iterations, dt);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return static_fail(NANS_ERR_CUDA, "nans_solve_contacts_static: kernel launch failed");
    // the status word (scratch word 0), read on the caller's stream
    unsigned err = 0;
    e = cudaMemcpyAsync(&err, scratch, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return static_fail(NANS_ERR_CUDA, "nans_solve_contacts_static: kernel failed");
    if (err & 1u)
        return static_fail(NANS_ERR_INVALID_ARGUMENT,
                           "nans_solve_contacts_static: a contact names a body outside the scene, or the same "
                           "body on both sides (skipped)");
    return NANS_OK;
}
