/* boids_compat/boid.h -- the fields of the reference's Boid (src/boid.h:15-35)
 * that callers of BoidSimulation read and write: id, position, velocity and
 * the reference grid's cell indices.  A stand-in for builds without the
 * reference's headers. */
#ifndef BOIDS_COMPAT_BOID_H
#define BOIDS_COMPAT_BOID_H

#include "vector3D.h"

class Boid {
public:
    Boid() : id(0) {}
    explicit Boid(Vector3D p) : id(0), position(p) {}
    Boid(Vector3D p, Vector3D v) : id(0), position(p), velocity(v) {}
    unsigned id;
    Vector3D position;
    Vector3D velocity;
    int grid_index[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
};

#endif
