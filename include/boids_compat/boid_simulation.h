/* boids_compat/boid_simulation.h -- class BoidSimulation with the public
 * shape of the reference's (src/boid_simulation.h:15-71), backed by the
 * GB300 engine through the C ABI of boids.h.
 *
 * The reference chooses its engine at link time: src/boid_simulation.cpp
 * (all pairs, target boidsim) and src/boid_simulation_grid.cpp (cell lists,
 * target boidsim_grid) define the members of this one class.  The member
 * definitions in boid_simulation_gb300.hpp are a third such definition.
 *
 *  - Without the reference's headers (this directory on the include path):
 *    include this header; it declares the class and pulls in the member
 *    definitions as inline functions (header-only), with the stand-in types
 *    of boid.h, vector3D.h and dtype.h here.
 *  - In a reference build: keep the reference's own headers and compile one
 *    source file that includes the reference's boid_simulation.h and then
 *    boid_simulation_gb300.hpp with BOIDS_COMPAT_INLINE defined empty, in
 *    place of boid_simulation{,_grid}.cpp, and link libboids_gb300.
 *
 * The engine is BOIDS_COMPAT_ENGINE (default BOIDS_ENGINE_GRID). */
#ifndef BOIDS_COMPAT_BOID_SIMULATION_H
#define BOIDS_COMPAT_BOID_SIMULATION_H

#include <string>

#include "boid.h"
#include "dtype.h"
#include "vector3D.h"

class BoidSimulation {
public:
    BoidSimulation();
    virtual ~BoidSimulation();
    /* note the order: velocity_max before velocity_min, as in the reference */
    void setup(unsigned int number_of_agents, double field_size,
               double separation_sight_distance, double separation_sight_angle,
               double separation_force_coefficient,
               double alignment_sight_distance, double alignment_sight_angle,
               double alignment_force_coefficient,
               double cohesion_sight_distance, double cohesion_sight_angle,
               double cohesion_force_coefficient,
               double velocity_max, double velocity_min,
               std::string initialization, int rand_seed);
    virtual void init();
    virtual void update();
    virtual int get(unsigned int id, float *x, float *y, float *z);
    virtual int get_v(unsigned int id, float *vx, float *vy, float *vz);
    virtual int get(unsigned int id, float *x, float *y, float *z, float *vx, float *vy, float *vz);
    bool is_openmp_enabled() const;
    int get_max_threads() const;
    int get_force(unsigned int id, float *coh_x, float *coh_y, float *coh_z, float *sep_x, float *sep_y,
                  float *sep_z, float *ali_x, float *ali_y, float *ali_z);

    unsigned int N;
    unsigned int time_step;
    double field_size;
    double field_size_X, field_size_Y, field_size_Z;
    interaction_parameters separation, alignment, cohesion;
    velocity_parameters velocity;
    Boid *boids;

    unsigned int GRID_NUM = 9;

protected:
    std::string initialization_type;
    int rand_seed;

    void clear_list_grid();
    void update_list_grid(Boid &boid);
};

#include "boid_simulation_gb300.hpp"

#endif
