/* A plain C consumer of the C ABI (include/nans_gb300.h), as a cgo / C host would bind it:
 * builds one stack scene in the reference's record layouts and steps it. Prints
 * "create <status>" and, when a world was created, "step <status> pairs <count>", then
 * "last_error <text>". Exit status 0 when every call behaved as documented. */
#include <stdio.h>
#include <string.h>

#include "nans_gb300.h"

int main(void)
{
    nans_cube cubes[2];
    nans_sphere sphere;
    nans_cube floor_box;
    nans_world_desc desc = {0, 0, 0};
    nans_world *world = NULL;
    nans_step_params params = {0.2f, 0.5f, 10};
    uint32_t count = 0;
    int i, rc;

    memset(cubes, 0, sizeof(cubes));
    memset(&sphere, 0, sizeof(sphere));
    memset(&floor_box, 0, sizeof(floor_box));
    for (i = 0; i < 2; ++i)
    {
        cubes[i].Model[0] = cubes[i].Model[5] = cubes[i].Model[10] = cubes[i].Model[15] = 1.0f;
        cubes[i].Position[1] = 0.5f + 1.002f * (float)i;
        cubes[i].Size = 1.0f;
        cubes[i].Mass = 1.0f;
        cubes[i].MOI = 1.0f / 6.0f;
    }
    sphere.Model[0] = sphere.Model[5] = sphere.Model[10] = sphere.Model[15] = 1.0f;
    sphere.Position[0] = -4.0f;
    sphere.Position[1] = 1.0f;
    sphere.V[0] = 10.0f;
    sphere.Radius = 0.5f;
    sphere.Mass = 2.0f;
    sphere.MOI = 0.2f;
    floor_box.Model[0] = floor_box.Model[5] = floor_box.Model[10] = floor_box.Model[15] = 1.0f;
    floor_box.Position[1] = -0.5f;
    floor_box.Size = 20.0f;
    floor_box.Mass = 100000.0f;
    floor_box.MOI = 100000.0f;

    rc = nans_world_create(&desc, &world);
    printf("create %d\n", rc);
    if (rc == NANS_OK)
    {
        rc = nans_world_upload(world, cubes, 2, &sphere, 1, &floor_box, NULL, 0);
        if (rc == NANS_OK)
            rc = nans_step(world, &params, 1.0f / 60.0f, 30);
        if (rc == NANS_OK)
            rc = nans_get_pairs(world, 0, NULL, 0, &count);
        printf("step %d pairs %u\n", rc, count);
        nans_world_destroy(world);
    }
    else if (world != NULL)
        return 1; /* a failed create must leave the output pointer NULL */
    printf("last_error %s\n", nans_last_error());
    return rc == NANS_OK || rc == NANS_ERR_CUDA ? 0 : 1;
}
