// Headless rasteriser for visual debugging of one scene (no graphics API): boxes as 12
// triangles each from the world vertices the step computes, the ground's top face and the
// spheres ray-cast per pixel, convex hulls drawn as their bounding spheres. Depth test and colour live in one 64-bit word
// per pixel (depth bits high, colour low), so an atomicMin keeps the nearest surface.
#include "nans_kernels.cuh"

namespace nans
{

struct Camera
{
    v3 eye, fwd, right, up;
    float focal; // pixels per unit of tan(angle)
    int width, height;
};

__device__ __forceinline__ bool project(const Camera &c, v3 p, float &sx, float &sy, float &z)
{
    const v3 d = p - c.eye;
    z = dot3(d, c.fwd);
    if (!(z > 1e-3f))
        return false;
    sx = 0.5f * c.width + c.focal * dot3(d, c.right) / z;
    sy = 0.5f * c.height - c.focal * dot3(d, c.up) / z;
    return true;
}

__device__ __forceinline__ unsigned shade(unsigned rgb, float lambert)
{
    const float k = 0.25f + 0.75f * fminf(fmaxf(lambert, 0.0f), 1.0f);
    unsigned r = (unsigned)(((rgb >> 16) & 255u) * k), g = (unsigned)(((rgb >> 8) & 255u) * k),
             b = (unsigned)((rgb & 255u) * k);
    return (r << 16) | (g << 8) | b;
}

__device__ __forceinline__ unsigned body_colour(int b, bool floor)
{
    if (floor)
        return 0x808890u;
    const unsigned h = (unsigned)b * 2654435761u;
    return 0x404040u | (h & 0xbfbfbfu);
}

__device__ __forceinline__ void plot(unsigned long long *fb, const Camera &c, int x, int y, float z, unsigned rgb)
{
    const unsigned long long v = ((unsigned long long)__float_as_uint(z) << 32) | rgb;
    atomicMin(fb + (size_t)y * c.width + x, v);
}

__global__ void k_render_clear(unsigned long long *fb, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        fb[i] = ~0ull;
}

// Box faces from UpdateVertices' corner order (code/nans.cpp:399-406).
__constant__ int c_tri[12][3] = {{0, 1, 3}, {0, 3, 2}, {4, 6, 7}, {4, 7, 5}, {0, 4, 5}, {0, 5, 1},
                                 {2, 3, 7}, {2, 7, 6}, {0, 2, 6}, {0, 6, 4}, {1, 5, 7}, {1, 7, 3}};

// The ground's top face as a plane, ray-cast per pixel (a checkerboard of 1 m squares).
__global__ void k_render_ground(DevWorld w, int scene, Camera cam, unsigned long long *fb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cam.width * cam.height)
        return;
    const int x = i % cam.width, y = i / cam.width;
    const int b = w.n_dyn + scene;
    const v3 gp = xyz(w.pos[b]), gs = xyz(w.scl[b]);
    const float top = gp.y + 0.5f * gs.y;
    const float u = (x + 0.5f - 0.5f * cam.width) / cam.focal, v = (0.5f * cam.height - (y + 0.5f)) / cam.focal;
    const v3 d = normalize3(cam.fwd + u * cam.right + v * cam.up);
    if (fabsf(d.y) < 1e-6f)
        return;
    const float s = (top - cam.eye.y) / d.y;
    if (s <= 0.0f)
        return;
    const v3 hit = cam.eye + s * d;
    if (fabsf(hit.x - gp.x) > 0.5f * gs.x || fabsf(hit.z - gp.z) > 0.5f * gs.z)
        return;
    const bool odd = ((int)floorf(hit.x) + (int)floorf(hit.z)) & 1;
    plot(fb, cam, x, y, dot3(hit - cam.eye, cam.fwd), odd ? 0x70757au : 0x8a9096u);
}

// One thread per box triangle of the scene's cubes.
__global__ void k_render_tris(DevWorld w, int scene, Camera cam, v3 light, unsigned long long *fb)
{
    const int c0 = w.sc_cube0[scene], nc = w.sc_nc[scene];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 12 * nc)
        return;
    const int k = t / 12, f = t % 12;
    const bool floor = false;
    const int b = c0 + k;
    const int4 sh = w.shape[b];
    if (sh.z >= 0 || sh.y != 8)
        return; // convex hulls are drawn as spheres
    const float *vp = w.verts + sh.x;
    v3 p[3];
    for (int q = 0; q < 3; ++q)
    {
        const int v = c_tri[f][q];
        p[q] = mk3(vp[3 * v], vp[3 * v + 1], vp[3 * v + 2]);
    }
    v3 n = normalize3(cross3(p[1] - p[0], p[2] - p[0]));
    const v3 centre = xyz(w.pos[b]);
    if (dot3(n, p[0] - centre) < 0.0f)
        n = -1.0f * n;
    const unsigned rgb = shade(body_colour(b, floor), dot3(n, light));
    float sx[3], sy[3], sz[3];
    for (int q = 0; q < 3; ++q)
        if (!project(cam, p[q], sx[q], sy[q], sz[q]))
            return; // a triangle crossing the camera plane is skipped
    const float area = (sx[1] - sx[0]) * (sy[2] - sy[0]) - (sx[2] - sx[0]) * (sy[1] - sy[0]);
    if (fabsf(area) < 1e-12f)
        return;
    const int x0 = max(0, (int)floorf(fminf(fminf(sx[0], sx[1]), sx[2])));
    const int x1 = min(cam.width - 1, (int)ceilf(fmaxf(fmaxf(sx[0], sx[1]), sx[2])));
    const int y0 = max(0, (int)floorf(fminf(fminf(sy[0], sy[1]), sy[2])));
    const int y1 = min(cam.height - 1, (int)ceilf(fmaxf(fmaxf(sy[0], sy[1]), sy[2])));
    for (int y = y0; y <= y1; ++y)
        for (int x = x0; x <= x1; ++x)
        {
            const float px = x + 0.5f, py = y + 0.5f;
            const float w0 = ((sx[1] - px) * (sy[2] - py) - (sx[2] - px) * (sy[1] - py)) / area;
            const float w1 = ((sx[2] - px) * (sy[0] - py) - (sx[0] - px) * (sy[2] - py)) / area;
            const float w2 = 1.0f - w0 - w1;
            if (w0 < 0.0f || w1 < 0.0f || w2 < 0.0f)
                continue;
            // perspective-correct depth: 1/z interpolates linearly in screen space
            const float iz = w0 / sz[0] + w1 / sz[1] + w2 / sz[2];
            plot(fb, cam, x, y, 1.0f / iz, rgb);
        }
}

// One thread per sphere (spheres, and convex hulls as their bounding spheres).
__global__ void k_render_spheres(DevWorld w, int scene, Camera cam, v3 light, unsigned long long *fb)
{
    const int c0 = w.sc_cube0[scene], nb = w.sc_nc[scene] + w.sc_ns[scene];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb)
        return;
    const int b = c0 + k;
    const int4 sh = w.shape[b];
    const v3 centre = xyz(w.pos[b]);
    float r;
    if (sh.y == 0)
        r = w.pos[b].w;
    else if (sh.z >= 0)
    {
        r = 0.0f;
        for (int q = 0; q < sh.y; ++q)
        {
            const float *v = w.verts + sh.x + 3 * q;
            r = fmaxf(r, len3(mk3(v[0], v[1], v[2]) - centre));
        }
    }
    else
        return; // boxes are triangles
    float cx, cy, cz;
    if (!project(cam, centre, cx, cy, cz) || cz <= r)
        return;
    const float rs = cam.focal * r / (cz - r) + 1.0f;
    const int x0 = max(0, (int)floorf(cx - rs)), x1 = min(cam.width - 1, (int)ceilf(cx + rs));
    const int y0 = max(0, (int)floorf(cy - rs)), y1 = min(cam.height - 1, (int)ceilf(cy + rs));
    const unsigned base = body_colour(b, false);
    for (int y = y0; y <= y1; ++y)
        for (int x = x0; x <= x1; ++x)
        {
            // ray through the pixel centre
            const float u = (x + 0.5f - 0.5f * cam.width) / cam.focal, v = (0.5f * cam.height - (y + 0.5f)) / cam.focal;
            const v3 d = normalize3(cam.fwd + u * cam.right + v * cam.up);
            const v3 oc = cam.eye - centre;
            const float bq = dot3(oc, d), cq = dot3(oc, oc) - r * r;
            const float disc = bq * bq - cq;
            if (disc < 0.0f)
                continue;
            const float s = -bq - sqrtf(disc);
            if (s <= 0.0f)
                continue;
            const v3 hit = cam.eye + s * d;
            const v3 n = normalize3(hit - centre);
            plot(fb, cam, x, y, dot3(hit - cam.eye, cam.fwd), shade(base, dot3(n, light)));
        }
}

__global__ void k_render_resolve(const unsigned long long *fb, int n, unsigned char *rgb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const unsigned long long v = fb[i];
    const unsigned c = (v == ~0ull) ? 0x1c2028u : (unsigned)(v & 0xffffffu);
    rgb[3 * i] = (unsigned char)(c >> 16);
    rgb[3 * i + 1] = (unsigned char)(c >> 8);
    rgb[3 * i + 2] = (unsigned char)c;
}

// Host side: camera from eye / target / vertical field of view; fb holds width * height words
// and rgb 3 * width * height bytes on the device.
int render_scene(const DevWorld &w, int scene, const float eye[3], const float target[3], float fov_deg, int width,
                 int height, unsigned long long *fb, unsigned char *rgb, cudaStream_t st)
{
    Camera c;
    c.eye = mk3(eye[0], eye[1], eye[2]);
    c.fwd = normalize3(mk3(target[0], target[1], target[2]) - c.eye);
    v3 up = mk3(0.0f, 1.0f, 0.0f);
    if (fabsf(dot3(up, c.fwd)) > 0.999f)
        up = mk3(0.0f, 0.0f, 1.0f);
    c.right = normalize3(cross3(c.fwd, up));
    c.up = cross3(c.right, c.fwd);
    c.focal = 0.5f * height / tanf(0.5f * fov_deg * 3.14159265f / 180.0f);
    c.width = width;
    c.height = height;
    const v3 light = normalize3(mk3(0.4f, 1.0f, 0.3f));
    const int n = width * height;
    k_render_clear<<<(n + 255) / 256, 256, 0, st>>>(fb, n);
    int nc = 0, ns = 0; // the scene's counts, for the launch sizes
    cudaMemcpyAsync(&nc, w.sc_nc + scene, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&ns, w.sc_ns + scene, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return (int)e;
    k_render_ground<<<(n + 255) / 256, 256, 0, st>>>(w, scene, c, fb);
    const int ntri = 12 * nc;
    if (ntri > 0)
        k_render_tris<<<(ntri + 127) / 128, 128, 0, st>>>(w, scene, c, light, fb);
    if (nc + ns > 0)
        k_render_spheres<<<(nc + ns + 63) / 64, 64, 0, st>>>(w, scene, c, light, fb);
    k_render_resolve<<<(n + 255) / 256, 256, 0, st>>>(fb, n, rgb);
    return (int)cudaGetLastError();
}

} // namespace nans
