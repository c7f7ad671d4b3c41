// Headless SimUpdateAndRender over the C ABI (include/nans_sim.h): the reference's frame entry
// point (code/nans.cpp:1719-1773) with the physics step on the GPU and rendering left out.
// Host code only; it links libnans_gb300.so.
#include <cmath>
#include <cstring>

#include "../../include/nans_sim.h"

namespace
{

// UpdateVertices' corner order (code/nans.cpp:399-406), for the records' initial vertices.
const float kCorner[8][3] = {{0.5f, 0.5f, 0.5f},   {0.5f, 0.5f, -0.5f},   {-0.5f, 0.5f, 0.5f},
                             {-0.5f, 0.5f, -0.5f}, {0.5f, -0.5f, 0.5f},   {0.5f, -0.5f, -0.5f},
                             {-0.5f, -0.5f, 0.5f}, {-0.5f, -0.5f, -0.5f}};
const float kShootForce = 4001.0f; // SHOOT_FORCE (code/nans.h:48)

void identity(float m[16])
{
    for (int i = 0; i < 16; ++i)
        m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}

void set3(float d[3], float x, float y, float z)
{
    d[0] = x;
    d[1] = y;
    d[2] = z;
}

void normalize(float v[3])
{
    const float inv = 1.0f / std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
    v[0] *= inv;
    v[1] *= inv;
    v[2] *= inv;
}

void cross(const float a[3], const float b[3], float o[3])
{
    o[0] = a[1] * b[2] - b[1] * a[2];
    o[1] = a[2] * b[0] - b[2] * a[0];
    o[2] = a[0] * b[1] - b[0] * a[1];
}

void cube_at(nans_cube &c, float x, float y, float z)
{
    std::memset(&c, 0, sizeof(c));
    identity(c.Model);
    for (int k = 0; k < 8; ++k)
        set3(c.Vertices[k], kCorner[k][0], kCorner[k][1], kCorner[k][2]);
    set3(c.Position, x, y, z);
    c.Size = 1.0f;
    c.Mass = 1.0f;
    c.MOI = (c.Mass / 12.0f) * (2.0f * c.Size * c.Size);
}

// Init (code/nans.cpp:1550-1717): camera, 4 cubes, 1 sphere, the floor (lights are render-only).
void init_scene(nans_sim_state *S)
{
    nans_sim_camera &C = S->Camera;
    C.FOV = 45.0f;
    C.Pitch = 0.0f;
    C.Yaw = -90.0f;
    C.Speed = 0.05f;
    set3(C.Position, 0.0f, 0.0f, 3.0f);
    set3(C.Target, 0.0f, 0.0f, 0.0f);
    float up[3] = {0.0f, 1.0f, 0.0f};
    set3(C.Direction, C.Position[0] - C.Target[0], C.Position[1] - C.Target[1], C.Position[2] - C.Target[2]);
    normalize(C.Direction);
    set3(C.Front, 0.0f, 0.0f, -1.0f);
    cross(up, C.Direction, C.Right);
    normalize(C.Right);
    cross(C.Direction, C.Right, C.Up);

    S->CubeCount = 4;
    cube_at(S->Cubes[0], 2.0f, 3.5f, 2.0f);
    cube_at(S->Cubes[1], 2.0f, 1.0f, 2.0f);
    cube_at(S->Cubes[2], 2.0f, 4.5f, 2.0f);
    cube_at(S->Cubes[3], 1.0f, 1.0f, 1.0f);

    S->SphereCount = 1;
    nans_sphere &sp = S->Spheres[0];
    std::memset(&sp, 0, sizeof(sp));
    identity(sp.Model);
    set3(sp.Position, 0.1f, 1.1f, 1.1f);
    sp.Radius = 0.25f;
    sp.Mass = 2.0f;
    sp.MOI = (float)((2.0f / 5.0f) * sp.Mass * std::pow((double)sp.Radius, 2.0));

    nans_cube &f = S->Floor;
    std::memset(&f, 0, sizeof(f));
    identity(f.Model);
    for (int k = 0; k < 8; ++k)
        set3(f.Vertices[k], kCorner[k][0], kCorner[k][1], kCorner[k][2]);
    set3(f.Position, 1.2f, -0.5f, 1.0f);
    f.Size = 100.0f;
    f.Mass = 100000.0f;
    f.MOI = (f.Mass / 12.0f) * (2.0f * f.Size * f.Size);
}

int upload(nans_sim_state *S)
{
    // a scene of the reference's size (at most 16 cubes and 16 spheres): the fused step, one
    // detect-and-solve launch per step instead of the staged kernels (the same results)
    nans_world_desc desc = {0, NANS_WORLD_FUSED_STEP, 0};
    int rc = nans_world_create(&desc, &S->World);
    if (rc)
        return rc;
    // every cube collides with Size on each axis except cube 3, drawn and collided at
    // (0.5, 1, 0.5) * Size (code/nans.cpp:1930-1941)
    float scale[NANS_SIM_MAX_BODIES][3];
    for (uint32_t i = 0; i < S->CubeCount; ++i)
        set3(scale[i], S->Cubes[i].Size, S->Cubes[i].Size, S->Cubes[i].Size);
    if (S->CubeCount > 3)
        set3(scale[3], 0.5f * S->Cubes[3].Size, S->Cubes[3].Size, 0.5f * S->Cubes[3].Size);
    return nans_world_upload(S->World, S->Cubes, S->CubeCount, S->Spheres, S->SphereCount, &S->Floor, &scale[0][0],
                             NANS_UPLOAD_KEEP_MODEL);
}

bool down(const nans_sim_button &b) { return b.EndedDown != 0; }

// HandleInput (code/nans.cpp:114-190); returns true when a body was changed.
bool handle_input(nans_sim_state *S, const nans_sim_input *In, float dt)
{
    nans_sim_camera &C = S->Camera;
    const nans_sim_button *B = In->Buttons;
    float side[3];
    cross(C.Front, C.Up, side);
    normalize(side);
    if (down(B[NANS_KEY_MOVE_FORWARD]))
        for (int k = 0; k < 3; ++k)
            C.Position[k] += C.Speed * C.Front[k];
    if (down(B[NANS_KEY_MOVE_LEFT]))
        for (int k = 0; k < 3; ++k)
            C.Position[k] -= side[k] * C.Speed;
    if (down(B[NANS_KEY_MOVE_BACK]))
        for (int k = 0; k < 3; ++k)
            C.Position[k] -= C.Speed * C.Front[k];
    if (down(B[NANS_KEY_MOVE_RIGHT]))
        for (int k = 0; k < 3; ++k)
            C.Position[k] += side[k] * C.Speed;
    bool changed = false;
    if (down(B[NANS_KEY_SHOOT]) && S->SphereCount > 0)
    {
        // ShootSphere (code/nans.cpp:105-112)
        nans_sphere &s = S->Spheres[0];
        set3(s.Forces, 0.0f, 0.0f, 0.0f);
        set3(s.Torque, 0.0f, 0.0f, 0.0f);
        set3(s.V, 0.0f, 0.0f, 0.0f);
        set3(s.W, 0.0f, 0.0f, 0.0f);
        std::memcpy(s.Position, C.Position, sizeof(s.Position));
        for (int k = 0; k < 3; ++k)
            s.Forces[k] += kShootForce * C.Front[k];
        changed = true;
    }
    if (S->CubeCount > 3)
    {
        const float step[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        const int keys[6] = {NANS_KEY_DEBUG_LEFT, NANS_KEY_DEBUG_RIGHT, NANS_KEY_DEBUG_UP,
                             NANS_KEY_DEBUG_DOWN, NANS_KEY_DEBUG_FORWARD, NANS_KEY_DEBUG_BACK};
        for (int q = 0; q < 6; ++q)
            if (down(B[keys[q]]))
            {
                for (int k = 0; k < 3; ++k)
                    S->Cubes[3].Position[k] += dt * step[q][k];
                changed = true;
            }
        if (down(B[NANS_KEY_DEBUG_RESET]))
        {
            const float p[4][3] = {{2.0f, 3.5f, 2.0f}, {2.0f, 1.0f, 2.0f}, {2.0f, 4.5f, 2.0f}, {0.0f, 0.0f, 0.0f}};
            for (int i = 0; i < 4; ++i)
            {
                std::memcpy(S->Cubes[i].Position, p[i], sizeof(p[i]));
                set3(S->Cubes[i].V, 0.0f, 0.0f, 0.0f);
                set3(S->Cubes[i].W, 0.0f, 0.0f, 0.0f);
            }
            changed = true;
        }
    }
    return changed;
}

// UpdateCamera (code/nans.cpp:20-38)
void update_camera(nans_sim_state *S, nans_sim_input *In)
{
    nans_sim_camera &C = S->Camera;
    C.Yaw += In->MouseController.XRel * In->MouseController.Sensitivity;
    C.Pitch += -In->MouseController.YRel * In->MouseController.Sensitivity;
    In->MouseController.XRel = 0;
    In->MouseController.YRel = 0;
    if (C.Pitch > 89.0f)
        C.Pitch = 89.0f;
    if (C.Pitch < -89.0f)
        C.Pitch = -89.0f;
    if (C.Position[1] < 0.5f)
        C.Position[1] = 0.5f;
}

float radians(float deg) { return deg * 0.01745329251994329577f; }

} // namespace

extern "C" {

uint64_t nans_sim_state_bytes(void) { return sizeof(nans_sim_state); }

void SimUpdateAndRender(nans_sim_memory *Memory, nans_sim_input *Input, void *Render, float dt)
{
    (void)Render;
    if (!Memory || !Memory->PermanentStorage || Memory->PermanentStorageSize < sizeof(nans_sim_state))
        return;
    nans_sim_state *S = (nans_sim_state *)Memory->PermanentStorage;
    if (!Memory->IsInitialized)
    {
        std::memset(S, 0, sizeof(*S));
        init_scene(S);
        S->LastStatus = upload(S);
        Memory->IsInitialized = 1;
    }
    if (!S->World)
        return;
    if (Input)
    {
        if (handle_input(S, Input, dt))
        {
            int rc = nans_world_set_state(S->World, S->Cubes, S->Spheres, NANS_UPLOAD_KEEP_MODEL);
            if (rc)
                S->LastStatus = rc;
        }
        update_camera(S, Input);
    }
    if (dt > 0.0f)
    {
        // Pairs.clear; IntegrateForces; DetectCollisions; SolveConstraints; IntegrateVelocities
        // with the reference's literals (code/nans.cpp:1154, 1159, 1176)
        const nans_step_params K = {0.1f, 0.1f, 70};
        int rc = nans_step(S->World, &K, dt, 1);
        if (rc == NANS_OK)
            rc = nans_world_download(S->World, S->Cubes, S->Spheres, nullptr);
        uint32_t count = 0;
        if (rc == NANS_OK)
            rc = nans_get_pairs(S->World, 0, S->Pairs, NANS_SIM_MAX_PAIRS, &count);
        S->PairCount = count < NANS_SIM_MAX_PAIRS ? count : NANS_SIM_MAX_PAIRS;
        S->LastStatus = rc;
        ++S->Frames;
    }
    // camera update after physics (code/nans.cpp:1766-1770)
    nans_sim_camera &C = S->Camera;
    float front[3] = {std::cos(radians(C.Yaw)) * std::cos(radians(C.Pitch)), std::sin(radians(C.Pitch)),
                      std::sin(radians(C.Yaw)) * std::cos(radians(C.Pitch))};
    normalize(front);
    std::memcpy(C.Front, front, sizeof(front));
}

} // extern "C"
