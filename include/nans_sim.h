/*
 * nans_sim.h -- headless drop-in for the reference's frame entry point.
 *
 * libnans_sim.so exports SimUpdateAndRender with the signature the reference's platform
 * layer resolves with dlsym (code/nans.h:396-397, code/sdl_nans.cpp:396-431):
 *     void SimUpdateAndRender(memory *Memory, sdl_input *Input, sdl_render *Render, real32 dt)
 * and runs the frame of code/nans.cpp:1719-1762 on the GPU step (libnans_gb300.so): on the
 * first call the reference's Init scene (code/nans.cpp:1550-1717: 4 unit cubes, cube 3 drawn
 * and collided at scale (0.5, 1, 0.5), one sphere, a 100-wide floor, every Model the identity),
 * then per frame the input handling (HandleInput / UpdateCamera, code/nans.cpp:114-190 and
 * 20-38), the physics step with the reference's literals (Cr 0.1, Cf 0.1, 70 iterations) and
 * the camera update (code/nans.cpp:1766-1773). Rendering is left out (headless): Render is
 * accepted and not touched.
 *
 * The platform types keep the reference's layouts (code/nans.h:120-165, 227-235). The state the
 * frame keeps lives in Memory->PermanentStorage as a nans_sim_state (below), which must be at
 * least nans_sim_state_bytes() long. Frames with dt <= 0 (the platform's first frame has
 * dt = 0, code/sdl_nans.cpp:902) handle input but run no physics step: the reference's step
 * divides by dt in its Baumgarte term.
 */
#ifndef NANS_SIM_H
#define NANS_SIM_H

#include <stdint.h>

#include "nans_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* struct memory (code/nans.h:227-235) */
typedef struct nans_sim_memory
{
    void *PermanentStorage;
    uint64_t PermanentStorageSize;
    void *TransientStorage;
    uint64_t TransientStorageSize;
    int32_t IsInitialized;
} nans_sim_memory;

/* struct sdl_button_state (code/nans.h:129-133) */
typedef struct nans_sim_button
{
    int32_t HalfTransitionCount;
    int32_t EndedDown;
} nans_sim_button;

/* the 13 buttons of struct sdl_keyboard in their order (code/nans.h:135-159) */
enum nans_sim_key
{
    NANS_KEY_MOVE_FORWARD = 0,
    NANS_KEY_MOVE_BACK,
    NANS_KEY_MOVE_LEFT,
    NANS_KEY_MOVE_RIGHT,
    NANS_KEY_SHOOT,
    NANS_KEY_DEBUG_UP,
    NANS_KEY_DEBUG_DOWN,
    NANS_KEY_DEBUG_LEFT,
    NANS_KEY_DEBUG_RIGHT,
    NANS_KEY_DEBUG_FORWARD,
    NANS_KEY_DEBUG_BACK,
    NANS_KEY_DEBUG_RESET,
    NANS_KEY_DEBUG_CONTINUE,
    NANS_KEY_COUNT
};

/* struct sdl_mouse (code/nans.h:120-127) */
typedef struct nans_sim_mouse
{
    float Sensitivity;
    int32_t XRel;
    int32_t YRel;
    int32_t X;
    int32_t Y;
} nans_sim_mouse;

/* struct sdl_input (code/nans.h:161-165) */
typedef struct nans_sim_input
{
    nans_sim_button Buttons[NANS_KEY_COUNT];
    nans_sim_mouse MouseController;
} nans_sim_input;

/* struct sdl_camera (code/nans.h:279-293) */
typedef struct nans_sim_camera
{
    float FOV, Pitch, Yaw, Speed;
    float Position[3], Target[3], Direction[3], Up[3], Front[3], Right[3];
} nans_sim_camera;

#define NANS_SIM_MAX_BODIES 16   /* MAX_CUBE_COUNT / MAX_SPHERE_COUNT (code/nans.h:52-53) */
#define NANS_SIM_MAX_PAIRS 1024

/* What the frame keeps in PermanentStorage: the bodies in the reference's records (updated
 * every frame), the camera, the last frame's contact list and the GPU world. */
typedef struct nans_sim_state
{
    nans_cube Cubes[NANS_SIM_MAX_BODIES];
    nans_sphere Spheres[NANS_SIM_MAX_BODIES];
    nans_cube Floor;
    nans_sim_camera Camera;
    uint32_t CubeCount;
    uint32_t SphereCount;
    uint32_t PairCount;  /* contacts of the last frame (the list is cut at NANS_SIM_MAX_PAIRS) */
    nans_contact_pair Pairs[NANS_SIM_MAX_PAIRS];
    uint64_t Frames;     /* physics steps run */
    int32_t LastStatus;  /* NANS_OK or the last error of the GPU step */
    nans_world *World;
} nans_sim_state;

void SimUpdateAndRender(nans_sim_memory *Memory, nans_sim_input *Input, void *Render, float dt);

/* sizeof(nans_sim_state), for hosts that size PermanentStorage. */
uint64_t nans_sim_state_bytes(void);

#ifdef __cplusplus
}
#endif

#endif /* NANS_SIM_H */
