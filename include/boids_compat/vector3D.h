/* boids_compat/vector3D.h -- the part of the reference's Vector3D
 * (src/vector3D.h:12-35) that BoidSimulation's public interface exposes: a
 * float triple.  A stand-in for builds without the reference's headers; a
 * reference build uses its own src/vector3D.h instead. */
#ifndef BOIDS_COMPAT_VECTOR3D_H
#define BOIDS_COMPAT_VECTOR3D_H

class Vector3D {
public:
    Vector3D() : x(0.0f), y(0.0f), z(0.0f) {}
    Vector3D(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
    float x, y, z;
};

#endif
