// Test infrastructure: the declarations of the reference header code/nans.h, restated so
// that the reference physics (code/nans.cpp) can be compiled headless with body arrays
// larger than its 16-slot cap (code/nans.h:52-53,377-378). code/nans.h closes its include
// guard with `#define NANS_H` at its end (code/nans.h:1,402), so defining NANS_H first and
// supplying these declarations makes code/nans.cpp compile unchanged against them.
//
// Every struct below keeps the field order and types of code/nans.h so that the physics
// reads and writes the same members; only MAX_CUBE_COUNT / MAX_SPHERE_COUNT differ.
// A test checks that this build and the build against the unmodified code/nans.h produce
// bit-identical steps on scenes that fit in 16 slots.
#ifndef NANS_LAYOUT_BIG_H
#define NANS_LAYOUT_BIG_H
#define NANS_H

#include <stdint.h>
#include <cstddef>
#include <GL/glew.h>
#include <glm/glm.hpp>
#include <cstdio>
#include <vector>
#include <time.h>
#include <math.h>

#ifndef NANS_REF_CAPACITY
#define NANS_REF_CAPACITY 8192
#endif

#define global_variable static
#define local_persist static

typedef int8_t int8;
typedef int16_t int16;
typedef int32_t int32;
typedef int64_t int64;
typedef int32 bool32;
typedef uint8_t uint8;
typedef uint16_t uint16;
typedef uint32_t uint32;
typedef uint64_t uint64;
typedef size_t memory_index;
typedef float real32;
typedef double real64;

#define Kibibytes(Value) ((Value)*1024LL)
#define Mebibytes(Value) (Kibibytes(Value) * 1024LL)
#define Gibibytes(Value) (Mebibytes(Value) * 1024LL)
#define Pi32 3.14159265359f
#define ArrayCount(Array) (sizeof(Array) / sizeof((Array)[0]))

#define GRAVITY_ACCEL 9.81f
#define GLOBAL_FRICTION 1.5f
#define SHOOT_FORCE 4001.0f
#define DEFAULT_WINDOW_WIDTH 1920
#define DEFAULT_WINDOW_HEIGHT 1080
#define MAX_CUBE_COUNT NANS_REF_CAPACITY
#define MAX_SPHERE_COUNT NANS_REF_CAPACITY
#define MAX_GJK_ITERATIONS 64
#define MAX_EPA_ERROR 0.001f
#define MAX_EPA_ITERATIONS 64
#define POINT_LIGHT_COUNT 4

#if SLOW_BUILD
#define Assert(Expression) \
    if (!(Expression))     \
    {                      \
        *(volatile int *)0 = 0; \
    }
#else
#define Assert(Expression)
#endif

#define PrintVector(Vector) printf("%f %f %f\n", Vector.x, Vector.y, Vector.z)

enum collision_type { CC = 0, CS, CF, SS, SF };
enum evolve_result { NoIntersection = 0, FoundIntersection, StillEvolving };

struct light
{
    glm::vec3 Position;
    real32 Size;
    real32 Kc, Kl, Kq;
    glm::vec3 Ambient, Diffuse, Specular;
};

struct character
{
    uint32 TextureId;
    glm::ivec2 Size;
    glm::ivec2 Bearing;
    long int Advance;
};

struct sdl_mouse
{
    real32 Sensitivity;
    int32 XRel, YRel, X, Y;
};

struct sdl_button_state
{
    int32 HalfTransitionCount;
    bool32 EndedDown;
};

struct sdl_keyboard
{
    union
    {
        sdl_button_state Buttons[13];
        struct
        {
            sdl_button_state MoveForward, MoveBack, MoveLeft, MoveRight, ShootAction;
            sdl_button_state DebugUp, DebugDown, DebugLeft, DebugRight, DebugForward, DebugBack,
                DebugReset, DebugContinue;
        };
    };
};

struct sdl_input
{
    sdl_keyboard KeyboardController;
    sdl_mouse MouseController;
};

enum sdl_texture { CONTAINER_DIFFUSE = 0, CONTAINER_SPECULAR, EARTH, CHECKERBOARD, AMONG_US_DIFFUSE,
                   AMONG_US_SPECULAR, METAL_ALBEDO, METAL_SPECULAR, TEXTURE_COUNT };
enum sdl_vao { CUBEVAO = 0, SPHEREVAO, FLOORVAO, TEXTVAO, LIGHTVAO, MODELVAO, VAO_COUNT };
enum sdl_vbo { CUBEVBO = 0, SPHEREVBO, FLOORVBO, TEXTVBO, LIGHTVBO, MODELVBO, VBO_COUNT };
enum sdl_shader { SIMPLE_COLOR_SH, TEXT_SH, LIGHTING_SH, SHADER_COUNT };

struct sdl_render
{
    uint32 Shaders[SHADER_COUNT];
    uint32 Textures[TEXTURE_COUNT];
    uint32 VAOs[VAO_COUNT];
    uint32 VBOs[VBO_COUNT];
    uint32 *Indices;
    uint32 *ModelIndices;
    uint32 Num;
    uint32 ModelNum;
    uint32 LightVAO;
    glm::mat4 View;
    glm::mat4 Projection;
};

struct memory
{
    void *PermanentStorage;
    uint64 PermanentStorageSize;
    void *TransientStorage;
    uint64 TransientStorageSize;
    bool32 IsInitialized;
};

struct memory_arena
{
    memory_index Size;
    uint8 *Base;
    memory_index Used;
};

struct vertex
{
    glm::vec3 P, SupA, SupB;
    inline bool operator==(const vertex &R) { return (this->P == R.P); }
};

struct simplex
{
    uint32 Count;
    vertex *Vertices;
};

struct edge
{
    uint32 Count;
    vertex A, B;
};

struct triangle
{
    uint32 Count;
    vertex A, B, C;
    glm::vec3 N;
};

struct sdl_camera
{
    real32 FOV, Pitch, Yaw, Speed;
    glm::vec3 Position, Target, Direction, Up, Front, Right;
};

struct plane
{
    glm::mat4 Model;
    glm::vec3 Position;
    glm::vec3 Vertices[4];
    real32 Size;
};

struct cube
{
    glm::mat4 Model;
    glm::vec3 Vertices[8];
    glm::vec3 Position, V, Forces;
    glm::vec3 Angles, W, Torque;
    real32 Size, Mass, MOI;
};

struct sphere
{
    glm::mat4 Model;
    glm::vec3 Position, V, Forces;
    glm::vec3 Angles, W, Torque;
    real32 Radius, Mass, MOI;
};

struct contact_pair
{
    collision_type Type;
    real32 DLNormal, DLNormalSum;
    real32 DLTangent1, DLTangent1Sum;
    real32 DLTangent2, DLTangent2Sum;
    glm::vec3 PointA, PointB;
    glm::vec3 N, T1, T2;
    int32 IndexA, IndexB;
};

struct sdl_state
{
    cube Cubes[MAX_CUBE_COUNT];
    sphere Spheres[MAX_SPHERE_COUNT];
    cube Floor;
    sdl_camera Camera;
    light Lights[POINT_LIGHT_COUNT];
    uint32 CubeCount;
    uint32 SphereCount;
    std::vector<contact_pair> Pairs;
};

#define SIM_UPDATE_AND_RENDER(name) void name(memory *Memory, sdl_input *Input, sdl_render *Render, real32 dt)
typedef SIM_UPDATE_AND_RENDER(sim_update_and_render);
SIM_UPDATE_AND_RENDER(SimUpdateAndRenderStub) {}

#endif
