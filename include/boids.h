/*
 * boids.h -- C ABI of the GB300 boid engine (libboids_gb300.so).
 *
 * Drop-in for the per-timestep update of maru-n/BoidsSimulatorMPI: the
 * reference's class BoidSimulation (src/boid_simulation.h:15-71), whose two
 * link-time variants are the all-pairs engine (src/boid_simulation.cpp,
 * target `boidsim`) and the overlapping-cell-list engine
 * (src/boid_simulation_grid.cpp, target `boidsim_grid`).  Each entry point
 * below names the reference member it replaces.
 *
 * Conventions: plain pointers and sizes only.  Host arrays are in boid-id
 * order, xyz interleaved (3 floats per boid; 9 for forces), the layout the
 * reference's getters and its .ptcl frames use.  Every call returns
 * BOIDS_OK (0) or a negative status; boids_last_error() gives the message.
 * Nothing calls exit().  A handle is not thread-safe; all of its GPU work is
 * ordered on one CUDA stream.
 */
#ifndef BOIDS_GB300_H
#define BOIDS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BOIDS_OK 0
#define BOIDS_EINVAL (-1)  /* bad argument or configuration           */
#define BOIDS_ENOMEM (-2)  /* device or host allocation failed        */
#define BOIDS_ECUDA (-3)   /* CUDA runtime error                      */
#define BOIDS_EIO (-4)     /* initialisation file missing or short    */
#define BOIDS_ESTATE (-5)  /* call out of order (e.g. no state yet)   */
#define BOIDS_ENOTSUP (-6) /* host libm breaks an assumption          */

#define BOIDS_ENGINE_ALLPAIRS 0 /* src/boid_simulation.cpp      (boidsim)      */
#define BOIDS_ENGINE_GRID 1     /* src/boid_simulation_grid.cpp (boidsim_grid) */

/* Keep get_force()'s per-rule forces of every step (36 bytes per boid). */
#define BOIDS_FLAG_RECORD_FORCES 1u

typedef struct boids_sim boids_sim;

/* The arguments of BoidSimulation::setup (src/boid_simulation.h:19-33), in
 * the same order and units.  Note that velocity_max comes before
 * velocity_min, as in the reference. */
typedef struct {
    uint32_t number_of_agents;
    double field_size;
    double separation_sight_distance;
    double separation_sight_angle; /* fraction of pi; >= 1 sees all around */
    double separation_force_coefficient;
    double alignment_sight_distance;
    double alignment_sight_angle;
    double alignment_force_coefficient;
    double cohesion_sight_distance;
    double cohesion_sight_angle;
    double cohesion_force_coefficient;
    double velocity_max;
    double velocity_min;
    int32_t engine;  /* BOIDS_ENGINE_* */
    int32_t device;  /* CUDA device ordinal */
    uint32_t flags;  /* BOIDS_FLAG_* */
    uint32_t reserved;
} boids_params;

/* Grid geometry, for logs and tests.  ref_* is the reference's overlapping
 * grid (INTERACTION_RANGE, GRID_NUM, GRID_SIZE of
 * src/boid_simulation_grid.cpp:80-83); dev_cells_per_axis is this engine's
 * own binning grid (0 when it scans all pairs). */
typedef struct {
    float ref_interaction_range;
    int32_t ref_grid_num;
    float ref_grid_size;
    int32_t dev_cells_per_axis;
    float dev_cell_size;
    int32_t list_capacity;
} boids_grid_info;

/* Per-phase device time since the last reset, measured with CUDA events on
 * the handle's stream when profiling is on (boids_profile_enable). */
typedef struct {
    double bin_ms;     /* cell keys + cell-count scan + scatter          */
    double force_ms;   /* rules + integration (+ next keys)              */
    double other_ms;   /* packing, unpacking, diagnostics                 */
    uint64_t steps;
    uint64_t force_launches;
    uint64_t bin_launches;
} boids_profile_t;

/* BoidSimulation::setup (src/boid_simulation.h:19-33,
 * src/boid_simulation_grid.cpp:48-93).  Allocates device memory for
 * number_of_agents boids.  For BOIDS_ENGINE_GRID the reference's grid check
 * applies: where the reference prints "Invalid GRID_NUM!!!" and exits
 * (src/boid_simulation_grid.cpp:86-89) this returns BOIDS_EINVAL; it also
 * refuses GRID_NUM == 1, where the reference lists a boid several times in
 * its own cell. */
int boids_create(const boids_params *params, boids_sim **out);

/* BoidSimulation::~BoidSimulation (src/boid_simulation.cpp:37-44). */
void boids_destroy(boids_sim *sim);

/* BoidSimulation::init (src/boid_simulation_grid.cpp:95-161,
 * src/boid_simulation.cpp:79-137).  initialization is "random_uniform",
 * "test", or the path of a raw file of native-endian float32
 * x,y,z,vx,vy,vz per boid.  The random draws reproduce the reference's
 * drand48 sequence: the grid engine calls srand48(rand_seed) first, the
 * all-pairs engine draws from the never-seeded stream as the reference does
 * (it only calls srand). */
int boids_init(boids_sim *sim, const char *initialization, int32_t rand_seed);

/* As boids_init, with seed_mode 1 = srand48(rand_seed) first, 0 = the
 * never-seeded stream, -1 = what the handle's engine does in the reference. */
int boids_init_ex(boids_sim *sim, const char *initialization, int32_t rand_seed, int32_t seed_mode);

/* Boid::set_serialized_data for every boid (src/boid.cpp:68-76): uploads a
 * state in id order.  The grid engine requires 0 <= x,y,z <= field_size. */
int boids_set_state(boids_sim *sim, const float *pos3n, const float *vel3n);

/* BoidSimulation::update (src/boid_simulation_grid.cpp:165-293), `steps`
 * times.  Asynchronous on the handle's stream. */
int boids_step(boids_sim *sim, int32_t steps);

/* BoidSimulation::get(id, &x,&y,&z, &vx,&vy,&vz) for every id
 * (src/boid_simulation.h:37-39).  Either pointer may be NULL.  Synchronous. */
int boids_get_state(boids_sim *sim, float *pos3n, float *vel3n);

/* BoidSimulation::get_force for every id (src/boid_simulation_grid.cpp:319-334):
 * cohesion xyz, separation xyz, alignment xyz of the last step.  Needs
 * BOIDS_FLAG_RECORD_FORCES and at least one step. */
int boids_get_forces(boids_sim *sim, float *force9n);

/* Boid::grid_index[8] of every boid for the current positions, computed the
 * way update_list_grid does (src/boid_simulation_grid.cpp:389-443):
 * primary cell first, then overlapped cells, -1 padded.  Needs a geometry
 * the reference accepts. */
int boids_get_cells(boids_sim *sim, int32_t *grid_index8n);

/* For the current state, per boid and rule (0 cohesion, 1 separation,
 * 2 alignment): how many boids pass Boid::isInsideArea (src/boid.cpp:27-42)
 * and the sum of a 64-bit mix of their ids (order-free set fingerprint).
 * Runs this engine's own neighbour search; does not advance the state. */
int boids_get_neighbor_sets(boids_sim *sim, int32_t *count3n, uint64_t *hash3n);

/* Geometry of the handle (see boids_grid_info). */
int boids_get_grid_info(boids_sim *sim, boids_grid_info *info);

/* Run on a caller-owned CUDA stream (a cudaStream_t) from now on; NULL
 * returns to the handle's own stream. */
int boids_set_stream(boids_sim *sim, void *cuda_stream);

/* Wait for the handle's queued GPU work. */
int boids_synchronize(boids_sim *sim);

/* Turn per-phase event timing on or off, read it, reset it. */
int boids_profile_enable(boids_sim *sim, int32_t on);
int boids_profile_read(boids_sim *sim, boids_profile_t *out, int32_t reset);

/* Number of this library's kernels launched by the handle so far. */
uint64_t boids_kernel_launches(boids_sim *sim);

/* Scratch reserved by boids_step_noalloc on every GPU that loads the library. */
#define BOIDS_NOALLOC_SCRATCH_BYTES (32u << 20)

/* One grid-engine update (BoidSimulation::update semantics, bit-identical to
 * boids_step) that allocates no memory -- this entry point has no
 * counterpart in the reference.  It is for callers that cannot let a library
 * allocate device memory: applications that own the GPU through their own
 * pool or a fixed budget, and latency-critical loops that must not run into
 * cudaMalloc/cudaFree, which can synchronize the device.  Inputs and outputs
 * are caller-owned DEVICE arrays in id order (3 floats per boid, xyz); in and
 * out must not overlap.  params->engine must be BOIDS_ENGINE_GRID; positions
 * must lie in [0, field_size] (not checked here).
 *
 * All scratch lives in one static device array of BOIDS_NOALLOC_SCRATCH_BYTES
 * that every GPU loading the library holds until the process exits; a step
 * needing more (roughly 440 000 boids at the reference's density) returns
 * BOIDS_EINVAL.  The first call on a device looks up the array's device
 * address, so make that first call before any stream capture.  Every call
 * shares the array: calls whose GPU work overlaps (other streams, other
 * threads on the same device) race; order them on one stream.  The work is
 * queued on cuda_stream (a cudaStream_t; NULL is the legacy default stream)
 * and the call returns without waiting for it. */
int boids_step_noalloc(const boids_params *params, const float *pos3n_in, const float *vel3n_in,
                       float *pos3n_out, float *vel3n_out, void *cuda_stream);

/* Message of the last failed call on this thread ("" if none). */
const char *boids_last_error(void);

/* Library version string. */
const char *boids_version(void);

#ifdef __cplusplus
}
#endif
#endif
