/*
 * boids_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU oracle for the per-timestep boid update of maru-n/BoidsSimulatorMPI.
 * It restates, in plain C, the reference's FP32 arithmetic (src/boid.cpp,
 * src/vector3D.cpp, src/boid_simulation.cpp, src/boid_simulation_grid.cpp)
 * and adds an FP64 restatement of the same step.  Only tests/,
 * __graft_entry__.smoke() and bench.py (its CPU-baseline leg and its
 * reference arm) load it, and only as the checker or the timed CPU baseline;
 * the product library never links it.
 *
 * Parity pin: the FP32 restatement is checked bit-for-bit against the
 * reference engine compiled from its own sources (oracle/build_ref.sh) on
 * the cases of the reference's test scripts (test/compare_grid.sh,
 * test/compare_legacy.sh); tests/golden holds vectors generated that way.
 */
#ifndef BOIDS_ORACLE_H
#define BOIDS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters exactly as BoidSimulation::setup receives them
 * (src/boid_simulation.h:19-33, src/dtype.h:39-49). */
typedef struct {
    uint32_t n;
    double field;
    double sep_r, sep_a, sep_c;
    double ali_r, ali_a, ali_c;
    double coh_r, coh_a, coh_c;
    double vmax, vmin;
} orc_params;

/* POSIX drand48 (48-bit LCG), the generator BoidSimulation::init draws from. */
void   orc_srand48(uint64_t *state, long seed);
double orc_drand48(uint64_t *state);

/* Initial state, src/boid_simulation_grid.cpp:95-136.  kind 0 = "random_uniform",
 * kind 1 = "test".  seeded != 0 calls srand48(seed) first (grid engine,
 * src/boid_simulation_grid.cpp:98); seeded == 0 draws from the never-seeded
 * stream, which is what the all-pairs engine does (src/boid_simulation.cpp:81).
 * pos and vel are 3*n floats, id order. */
int orc_init(const orc_params *p, int kind, int seeded, int seed, float *pos, float *vel);

/* One update() of the all-pairs engine, src/boid_simulation.cpp:143-249.
 * force9 (nullable) receives get_force()'s nine floats per boid for this step
 * (src/boid_simulation.cpp:275-290).  nthreads <= 0 lets OpenMP decide. */
void orc_step_allpairs(const orc_params *p, float *pos, float *vel, float *force9, int nthreads);

/* Overlapping cell-list engine of src/boid_simulation_grid.cpp (setup :80-89,
 * update :165-293, update_list_grid :389-451).  The rule loop runs in
 * parallel and the integration plus rebinning serially, as in the reference. */
typedef struct orc_grid orc_grid;
int  orc_grid_geometry(const orc_params *p, float *range, int *grid_num, float *grid_size);
orc_grid *orc_grid_create(const orc_params *p);        /* NULL if setup would abort */
void orc_grid_bin(orc_grid *g, const float *pos);      /* rebin from scratch (init) */
void orc_grid_step(orc_grid *g, float *pos, float *vel, float *force9, int nthreads);
void orc_grid_destroy(orc_grid *g);

/* Boid::grid_index[8] for each boid, src/boid_simulation_grid.cpp:400-443. */
int orc_ref_cells(const orc_params *p, const float *pos, int32_t *grid_index8);

/* Per boid and rule (0 = cohesion, 1 = separation, 2 = alignment): neighbour
 * count and an order-free 64-bit hash of the neighbour ids, from the
 * reference's Boid::isInsideArea decisions (src/boid.cpp:27-42).  Arrays are
 * 3*n, layout [i*3 + rule]. */
void orc_neighbor_sets(const orc_params *p, const float *pos, const float *vel,
                       int32_t *count3, uint64_t *hash3, int nthreads);

/* As orc_neighbor_sets; bucketed == 0 scans all pairs (the check of the buckets). */
void orc_neighbor_sets_ex(const orc_params *p, const float *pos, const float *vel,
                          int32_t *count3, uint64_t *hash3, int nthreads, int bucketed);

/* FP64 restatement of one rule pass: the neighbour sets come from the FP32
 * decisions above and every arithmetic operation is carried out in double.
 * force9 layout matches get_force (coh xyz, sep xyz, ali xyz). */
void orc_forces_f64(const orc_params *p, const float *pos, const float *vel,
                    double *force9, int nthreads);

/* The hash mixing function used for neighbour-set hashes (splitmix64 finaliser). */
uint64_t orc_id_hash(uint32_t id);

#ifdef __cplusplus
}
#endif
#endif
