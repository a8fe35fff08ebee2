/*
 * A C caller of libboids_gb300.so written the way the reference's frame loop
 * drives BoidSimulation (src/main.cpp:82-93 setup and init, :187-291 the
 * per-step frame write followed by update()), but through the C ABI of
 * include/boids.h: the frame of the state before each update is assembled on
 * the GPU and copied into one of two page-locked buffers while the update
 * runs, and written once its copy has landed.
 *
 *   capi_caller N F T out.bin [grid|allpairs]
 *
 * settings/marun2019.ini parameters, "random_uniform" init with seed 12345.
 * out.bin holds, as native float32: T frames of x,y,z per boid (the state
 * before update t, in id order), then the final positions, velocities and
 * get_force values (9 floats per boid) of the last update.
 *
 * Exit status: 0 on success, 2 on a usage error, 3 when a library call fails
 * (its status and boids_last_error() go to stderr), 4 on a file error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "boids.h"

static int report(const char *what, int rc)
{
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, boids_last_error());
    return 3;
}

int main(int argc, char **argv)
{
    if (argc < 5) {
        fprintf(stderr, "usage: %s N F T out.bin [grid|allpairs]\n", argv[0]);
        return 2;
    }
    const unsigned n = (unsigned)strtoul(argv[1], NULL, 10);
    const double field = strtod(argv[2], NULL);
    const int steps = atoi(argv[3]);
    const char *out = argv[4];
    const int allpairs = argc > 5 && strcmp(argv[5], "allpairs") == 0;
    if (n == 0 || steps < 1) {
        fprintf(stderr, "N and T must be positive\n");
        return 2;
    }

    boids_params p;
    memset(&p, 0, sizeof p);
    p.number_of_agents = n;
    p.field_size = field;
    p.separation_sight_distance = 0.01;
    p.separation_sight_angle = 0.5;
    p.separation_force_coefficient = 0.002;
    p.alignment_sight_distance = 0.05;
    p.alignment_sight_angle = 1.0 / 3;
    p.alignment_force_coefficient = 0.06;
    p.cohesion_sight_distance = 0.05;
    p.cohesion_sight_angle = 0.5;
    p.cohesion_force_coefficient = 0.008;
    p.velocity_max = 0.005;
    p.velocity_min = 0.001;
    p.engine = allpairs ? BOIDS_ENGINE_ALLPAIRS : BOIDS_ENGINE_GRID;
    p.flags = BOIDS_FLAG_RECORD_FORCES;

    boids_sim *sim = NULL;
    int rc = boids_create(&p, &sim);
    if (rc) return report("boids_create", rc);
    if ((rc = boids_init_ex(sim, "random_uniform", 12345, 1))) {
        boids_destroy(sim);
        return report("boids_init_ex", rc);
    }

    FILE *f = fopen(out, "wb");
    if (!f) {
        boids_destroy(sim);
        fprintf(stderr, "Couldn't open: %s\n", out);
        return 4;
    }
    const size_t frame_bytes = (size_t)12 * n;
    float *frame[2] = {NULL, NULL};
    float *pos = malloc(frame_bytes), *vel = malloc(frame_bytes), *force = malloc(3 * frame_bytes);
    int status = 0;
    if (!pos || !vel || !force) {
        fprintf(stderr, "host allocation failed\n");
        status = 4;
        goto done;
    }
    for (int i = 0; i < 2; ++i)
        if ((rc = boids_host_alloc(frame_bytes, (void **)&frame[i]))) {
            status = report("boids_host_alloc", rc);
            goto done;
        }

    for (int t = 0; t < steps; ++t) {
        const int slot = t & 1;
        /* frame t of the state before update t, then the update behind it */
        if ((rc = boids_frame_async(sim, frame[slot], NULL, 0, slot))) {
            status = report("boids_frame_async", rc);
            goto done;
        }
        if ((rc = boids_step(sim, 1))) {
            status = report("boids_step", rc);
            goto done;
        }
        /* write frame t while update t runs */
        if ((rc = boids_frame_wait(sim, slot))) {
            status = report("boids_frame_wait", rc);
            goto done;
        }
        if (fwrite(frame[slot], 1, frame_bytes, f) != frame_bytes) {
            status = 4;
            goto done;
        }
    }
    if ((rc = boids_get_state(sim, pos, vel))) {
        status = report("boids_get_state", rc);
        goto done;
    }
    if ((rc = boids_get_forces(sim, force))) {
        status = report("boids_get_forces", rc);
        goto done;
    }
    if (fwrite(pos, 1, frame_bytes, f) != frame_bytes || fwrite(vel, 1, frame_bytes, f) != frame_bytes ||
        fwrite(force, 1, 3 * frame_bytes, f) != 3 * frame_bytes)
        status = 4;

done:
    if (fclose(f) && !status) status = 4;
    for (int i = 0; i < 2; ++i) boids_host_free(frame[i]);
    free(pos);
    free(vel);
    free(force);
    boids_destroy(sim);
    return status;
}
