// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A C-ABI shim around the reference engine, compiled together with the
// reference's own, unmodified sources (oracle/build_ref.sh) so that tests can
// run the real BoidSimulation::setup/init/update/get/get_force
// (src/boid_simulation.h:15-71) on chosen states.  Built twice: with
// -DREF_GRID against src/boid_simulation_grid.cpp, and without it against
// src/boid_simulation.cpp (the two files define the same class).
#include "boid_simulation.h"

#include <iostream>
#include <string>

namespace {

// The subclass only re-exposes the protected rebinning calls so that a state
// written through the public `boids` array can be binned the way init() and
// update() bin it (src/boid_simulation_grid.cpp:255,291).
class RefSim : public BoidSimulation {
public:
#ifdef REF_GRID
    void rebin()
    {
        clear_list_grid();
        for (unsigned i = 0; i < N; ++i) update_list_grid(boids[i]);
    }
#else
    void rebin() {}
#endif
};

struct QuietCout {
    QuietCout() { std::cout.setstate(std::ios::failbit); }
    ~QuietCout() { std::cout.clear(); }
};

}  // namespace

extern "C" {

void *ref_create(unsigned n, double field,
                 double sep_r, double sep_a, double sep_c,
                 double ali_r, double ali_a, double ali_c,
                 double coh_r, double coh_a, double coh_c,
                 double vmax, double vmin, const char *init, int seed)
{
    QuietCout q;
    RefSim *s = new RefSim();
    s->setup(n, field, sep_r, sep_a, sep_c, ali_r, ali_a, ali_c, coh_r, coh_a, coh_c,
             vmax, vmin, std::string(init), seed);
    return s;
}

void ref_init(void *h)
{
    QuietCout q;
    static_cast<RefSim *>(h)->init();
}

// Writes the state into the engine's boids (ids = index) and bins it.
void ref_set_state(void *h, const float *pos, const float *vel)
{
    RefSim *s = static_cast<RefSim *>(h);
    for (unsigned i = 0; i < s->N; ++i) {
        s->boids[i].id = i;
        s->boids[i].position = Vector3D(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        s->boids[i].velocity = Vector3D(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
    }
    s->rebin();
}

void ref_update(void *h, int steps)
{
    RefSim *s = static_cast<RefSim *>(h);
    for (int t = 0; t < steps; ++t) s->update();
}

void ref_get_state(void *h, float *pos, float *vel)
{
    RefSim *s = static_cast<RefSim *>(h);
    for (unsigned i = 0; i < s->N; ++i) {
        s->get(i, pos + 3 * i, pos + 3 * i + 1, pos + 3 * i + 2,
               vel + 3 * i, vel + 3 * i + 1, vel + 3 * i + 2);
    }
}

void ref_get_force(void *h, float *f9)
{
    RefSim *s = static_cast<RefSim *>(h);
    for (unsigned i = 0; i < s->N; ++i) {
        float *o = f9 + 9 * i;
        s->get_force(i, o, o + 1, o + 2, o + 3, o + 4, o + 5, o + 6, o + 7, o + 8);
    }
}

void ref_get_grid_index(void *h, int *gi8)
{
    RefSim *s = static_cast<RefSim *>(h);
    for (unsigned i = 0; i < s->N; ++i)
        for (int k = 0; k < 8; ++k) gi8[8 * i + k] = s->boids[i].grid_index[k];
}

int ref_grid_num(void *h) { return (int)static_cast<RefSim *>(h)->GRID_NUM; }

void ref_destroy(void *h) { delete static_cast<RefSim *>(h); }

}  // extern "C"
