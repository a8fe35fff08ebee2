/* boids_compat/dtype.h -- the parameter records of BoidSimulation's public
 * fields (src/dtype.h:40-50; the field name sight_agnle is the reference's
 * own spelling, which its callers use).  A stand-in for builds without the
 * reference's headers. */
#ifndef BOIDS_COMPAT_DTYPE_H
#define BOIDS_COMPAT_DTYPE_H

typedef struct {
    double sight_distance;
    double sight_agnle;
    double force_coefficient;
} interaction_parameters;

typedef struct {
    double max;
    double min;
} velocity_parameters;

#endif
