/* boids_compat/boid_simulation_gb300.hpp -- the members of class
 * BoidSimulation (src/boid_simulation.h:15-71) over the GB300 engine's C ABI.
 *
 * Included by boids_compat/boid_simulation.h (inline, header-only), or by one
 * source file of a reference build after the reference's own
 * boid_simulation.h, with BOIDS_COMPAT_INLINE defined empty (see there).
 * Only members that the reference's declaration has are used; the engine
 * handle of each object is kept in a table keyed by the object's address.
 *
 * Behaviour, member by member:
 *  setup   creates the engine (boids_create); the reference's refusals
 *          ("Invalid GRID_NUM" and the like) print the message and exit(-1)
 *          as the reference does; boids[] is allocated with ids 0..N-1.
 *  init    boids_init (src/boid_simulation_grid.cpp:95-161); a bad
 *          placement type or file prints and exits like the reference.
 *  update  one boids_step; boids[] is refreshed from the device afterwards,
 *          so it always holds the current state, as in the reference.
 *  get, get_v, get_force
 *          read boids[] and the last update's per-rule forces (the forces
 *          are fetched once per update, on the first get_force).
 *  clear_list_grid, update_list_grid
 *          the reference's rebinning hooks: a caller that wrote boids[] and
 *          rebinned it makes boids[] the state the next update starts from
 *          (it is uploaded then).  Writes to boids[] without them are not
 *          seen by the engine, as the reference's grid engine would not see
 *          them in its cell lists either.
 *  is_openmp_enabled, get_max_threads
 *          false and 1: there are no host threads in the update.
 * grid_index[] of boids[] is not maintained (the reference's own cell lists
 * are not built); boids_get_cells gives it. */
#ifndef BOIDS_COMPAT_BOID_SIMULATION_GB300_HPP
#define BOIDS_COMPAT_BOID_SIMULATION_GB300_HPP

#include <cstdlib>
#include <iostream>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "boids.h"

#ifndef BOIDS_COMPAT_INLINE
#define BOIDS_COMPAT_INLINE inline
#endif
#ifndef BOIDS_COMPAT_ENGINE
#define BOIDS_COMPAT_ENGINE BOIDS_ENGINE_GRID
#endif

namespace boids_compat {

struct State {
    boids_sim *sim = nullptr;
    std::vector<float> pos, vel, force;
    bool dirty = false;      /* boids[] was rebinned by the caller: upload it */
    bool force_ok = false;   /* force[] holds the last update's values */
};

BOIDS_COMPAT_INLINE std::mutex &table_mutex()
{
    static std::mutex m;
    return m;
}

BOIDS_COMPAT_INLINE std::map<const void *, State> &table()
{
    static std::map<const void *, State> t;
    return t;
}

BOIDS_COMPAT_INLINE State &state_of(const void *obj)
{
    std::lock_guard<std::mutex> lock(table_mutex());
    return table()[obj];
}

BOIDS_COMPAT_INLINE void drop_state(const void *obj)
{
    std::lock_guard<std::mutex> lock(table_mutex());
    auto it = table().find(obj);
    if (it == table().end()) return;
    if (it->second.sim) boids_destroy(it->second.sim);
    table().erase(it);
}

/* The reference reports its errors on stderr and exits with -1. */
[[noreturn]] BOIDS_COMPAT_INLINE void die(const std::string &msg)
{
    std::cerr << msg << std::endl;
    std::exit(-1);
}

BOIDS_COMPAT_INLINE void check(int rc, const char *what)
{
    if (rc != BOIDS_OK) die(std::string(what) + ": " + boids_last_error());
}

/* Copies the device state into boids[] (id order: boids[i] is boid i). */
BOIDS_COMPAT_INLINE void pull(State &s, Boid *boids, unsigned n)
{
    check(boids_get_state(s.sim, s.pos.data(), s.vel.data()), "boids_get_state");
    for (unsigned i = 0; i < n; ++i) {
        boids[i].id = i;
        boids[i].position = Vector3D(s.pos[3 * i], s.pos[3 * i + 1], s.pos[3 * i + 2]);
        boids[i].velocity = Vector3D(s.vel[3 * i], s.vel[3 * i + 1], s.vel[3 * i + 2]);
    }
}

}  // namespace boids_compat

BOIDS_COMPAT_INLINE BoidSimulation::BoidSimulation() : N(0), time_step(0), boids(nullptr) {}

BOIDS_COMPAT_INLINE BoidSimulation::~BoidSimulation()
{
    boids_compat::drop_state(this);
    delete[] boids;
}

BOIDS_COMPAT_INLINE void BoidSimulation::setup(unsigned int number_of_agents, double field_size,
                                               double separation_sight_distance, double separation_sight_angle,
                                               double separation_force_coefficient,
                                               double alignment_sight_distance, double alignment_sight_angle,
                                               double alignment_force_coefficient,
                                               double cohesion_sight_distance, double cohesion_sight_angle,
                                               double cohesion_force_coefficient,
                                               double velocity_max, double velocity_min,
                                               std::string initialization, int rand_seed)
{
    boids_compat::drop_state(this);
    field_size_X = field_size_Y = field_size_Z = field_size;
    this->field_size = field_size;
    separation = {separation_sight_distance, separation_sight_angle, separation_force_coefficient};
    alignment = {alignment_sight_distance, alignment_sight_angle, alignment_force_coefficient};
    cohesion = {cohesion_sight_distance, cohesion_sight_angle, cohesion_force_coefficient};
    velocity = {velocity_max, velocity_min};
    N = number_of_agents;
    delete[] boids;
    boids = new Boid[N];
    for (unsigned i = 0; i < N; ++i) boids[i].id = i;
    initialization_type = initialization;
    this->rand_seed = rand_seed;
    time_step = 0;

    boids_params p{};
    p.number_of_agents = number_of_agents;
    p.field_size = field_size;
    p.separation_sight_distance = separation_sight_distance;
    p.separation_sight_angle = separation_sight_angle;
    p.separation_force_coefficient = separation_force_coefficient;
    p.alignment_sight_distance = alignment_sight_distance;
    p.alignment_sight_angle = alignment_sight_angle;
    p.alignment_force_coefficient = alignment_force_coefficient;
    p.cohesion_sight_distance = cohesion_sight_distance;
    p.cohesion_sight_angle = cohesion_sight_angle;
    p.cohesion_force_coefficient = cohesion_force_coefficient;
    p.velocity_max = velocity_max;
    p.velocity_min = velocity_min;
    p.engine = BOIDS_COMPAT_ENGINE;
    p.device = 0;
    p.flags = BOIDS_FLAG_RECORD_FORCES;
    boids_compat::State &s = boids_compat::state_of(this);
    if (boids_create(&p, &s.sim) != BOIDS_OK) boids_compat::die(boids_last_error());
    s.pos.assign((size_t)3 * N, 0.0f);
    s.vel.assign((size_t)3 * N, 0.0f);
    s.force.assign((size_t)9 * N, 0.0f);
    boids_grid_info gi;
    if (boids_get_grid_info(s.sim, &gi) == BOIDS_OK && gi.ref_grid_num > 0) {
        GRID_NUM = (unsigned)gi.ref_grid_num;
        if (BOIDS_COMPAT_ENGINE == BOIDS_ENGINE_GRID)
            std::cout << "# Grid List Optimization enabled" << std::endl << "  grid num:" << GRID_NUM << std::endl;
    }
}

BOIDS_COMPAT_INLINE void BoidSimulation::init()
{
    boids_compat::State &s = boids_compat::state_of(this);
    if (boids_init(s.sim, initialization_type.c_str(), rand_seed) != BOIDS_OK)
        boids_compat::die(boids_last_error());
    boids_compat::pull(s, boids, N);
    s.dirty = false;
    s.force_ok = false;
}

BOIDS_COMPAT_INLINE void BoidSimulation::update()
{
    boids_compat::State &s = boids_compat::state_of(this);
    if (s.dirty) {
        for (unsigned i = 0; i < N; ++i) {
            const Boid &b = boids[i];
            s.pos[3 * i] = b.position.x;
            s.pos[3 * i + 1] = b.position.y;
            s.pos[3 * i + 2] = b.position.z;
            s.vel[3 * i] = b.velocity.x;
            s.vel[3 * i + 1] = b.velocity.y;
            s.vel[3 * i + 2] = b.velocity.z;
        }
        boids_compat::check(boids_set_state(s.sim, s.pos.data(), s.vel.data()), "boids_set_state");
        s.dirty = false;
    }
    boids_compat::check(boids_step(s.sim, 1), "boids_step");
    boids_compat::pull(s, boids, N);
    s.force_ok = false;
}

BOIDS_COMPAT_INLINE int BoidSimulation::get(unsigned int id, float *x, float *y, float *z)
{
    *x = boids[id].position.x;
    *y = boids[id].position.y;
    *z = boids[id].position.z;
    return 0;
}

BOIDS_COMPAT_INLINE int BoidSimulation::get_v(unsigned int id, float *vx, float *vy, float *vz)
{
    *vx = boids[id].velocity.x;
    *vy = boids[id].velocity.y;
    *vz = boids[id].velocity.z;
    return 0;
}

BOIDS_COMPAT_INLINE int BoidSimulation::get(unsigned int id, float *x, float *y, float *z, float *vx, float *vy,
                                            float *vz)
{
    get(id, x, y, z);
    get_v(id, vx, vy, vz);
    return 0;
}

BOIDS_COMPAT_INLINE bool BoidSimulation::is_openmp_enabled() const { return false; }

BOIDS_COMPAT_INLINE int BoidSimulation::get_max_threads() const { return 1; }

BOIDS_COMPAT_INLINE int BoidSimulation::get_force(unsigned int id, float *coh_x, float *coh_y, float *coh_z,
                                                  float *sep_x, float *sep_y, float *sep_z, float *ali_x,
                                                  float *ali_y, float *ali_z)
{
    boids_compat::State &s = boids_compat::state_of(this);
    if (!s.force_ok) {
        /* before the first update the reference's force arrays hold zeros */
        if (boids_get_forces(s.sim, s.force.data()) != BOIDS_OK) s.force.assign(s.force.size(), 0.0f);
        s.force_ok = true;
    }
    const float *f = s.force.data() + (size_t)9 * id;
    *coh_x = f[0]; *coh_y = f[1]; *coh_z = f[2];
    *sep_x = f[3]; *sep_y = f[4]; *sep_z = f[5];
    *ali_x = f[6]; *ali_y = f[7]; *ali_z = f[8];
    return 0;
}

BOIDS_COMPAT_INLINE void BoidSimulation::clear_list_grid() { boids_compat::state_of(this).dirty = true; }

BOIDS_COMPAT_INLINE void BoidSimulation::update_list_grid(Boid &) { boids_compat::state_of(this).dirty = true; }

#endif
