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
 * ordered on one CUDA stream (a grid update, boids_set_state and
 * boids_get_state fork part of their work onto a side stream of the handle
 * and join it back before they end, so work queued after them on the stream
 * sees their results).
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
/* BOIDS_ENGINE_ALLPAIRS: test every ordered pair on the GPU (N^2 work).
 * Without it the all-pairs engine runs the grid kernels whenever the field
 * holds at least 3 device cells per axis, the state lies in [0, field_size]
 * and the speed limits are below field_size / 2: every pair within the
 * sight radii is still found, each with the same image, and neighbours are
 * summed in the same ascending id order, so the results are bit-identical
 * (the reference's own test/compare_grid.sh asserts grid == all-pairs).
 * The N^2 kernels take at most 65535 * 1024 boids (one update would test
 * 4.5e15 pairs); beyond that boids_step returns BOIDS_ECUDA. */
#define BOIDS_FLAG_ALLPAIRS_KERNELS 2u

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
 * state of number_of_agents boids in id order.  The grid engine requires
 * 0 <= x,y,z <= field_size. */
int boids_set_state(boids_sim *sim, const float *pos3n, const float *vel3n);

/* The state of a population of n boids, n at most the number_of_agents the
 * handle was created with: boids_set_state for the first n ids.  For a
 * domain-decomposed flock, whose rank-local boids (its block's and the
 * margin's, cf. BoidSimulationMultiNode, src/boid_simulation_mpi.cpp:151-243)
 * change in number every update.  The getters, frames and updates then
 * cover those n; boids_init sets the whole population again. */
int boids_set_population(boids_sim *sim, uint32_t n, const float *pos3n, const float *vel3n);

/* BoidSimulation::update (src/boid_simulation_grid.cpp:165-293), `steps`
 * times.  Asynchronous on the handle's stream.  A call of 32 or more steps
 * captures 16 updates into a CUDA graph once (per stream, buffer parity and
 * tuning) and replays it; the grid engine's other updates replay a captured
 * one-update graph; with profiling on every kernel is launched directly.
 * Results are the same bits either way. */
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

/* Which full-size cells the grid engine's CTA-per-cell kernel takes (the
 * thread-per-boid kernel does the rest; results never depend on it):
 * tune[0] dense_min   cells holding this many boids or more,
 * tune[1] defer_min   ... or this many with over
 * tune[2] cand_defer  candidates in the cell's 27-cell neighbourhood,
 * tune[3] lone_cand   ... or any boid with over this many candidates.
 * Defaults 16, 4, 192, 96.  No counterpart in the reference. */
int boids_set_tuning(boids_sim *sim, const int32_t *tune4);
int boids_get_tuning(boids_sim *sim, int32_t *tune4);

/* Time a few updates with each candidate threshold set on a copy of the
 * current state, keep the fastest, and put the state back (grid engine; a
 * no-op for the all-pairs engine).  Crowded flocks favour other thresholds
 * than uniform ones, so long runs may call it again as the flock gathers.
 * get_force values of the last update are lost.  steps_per_trial <= 0 picks
 * a default.  No counterpart in the reference. */
int boids_autotune(boids_sim *sim, int32_t steps_per_trial);

/* Number of this library's kernels launched by the handle so far. */
uint64_t boids_kernel_launches(boids_sim *sim);

/* .ptcl frame output: replaces the per-boid get()/get_v()/get_force() loop
 * of the reference's frame writer (src/main.cpp:246-277).  Queues on the
 * handle's stream the assembly of one frame of the current state, in the
 * byte layout main.cpp writes, and its copy into host memory:
 *   pos_frame  x,y,z per boid in id order (3 floats), or with
 *              with_forces != 0 (--force-data-output) x,y,z followed by
 *              get_force's nine floats of the last step (12 floats per
 *              boid); the forces are zero before the first step, as the
 *              reference's zero-initialised dv arrays are;
 *   vel_frame  vx,vy,vz per boid (--velocity-output), nullable.
 * On a little-endian host these are the bytes fix_byte_order passes through
 * unchanged (src/main.cpp:26-36).  The call returns without waiting; the
 * frame has landed once boids_frame_wait(sim, slot) returns.  slot
 * (0 .. BOIDS_FRAME_SLOTS-1) names the completion event, so that frames can
 * be double-buffered while the next update runs.  Host buffers from
 * boids_host_alloc (page-locked) let the copy overlap the GPU work. */
#define BOIDS_FRAME_SLOTS 4
int boids_frame_async(boids_sim *sim, float *pos_frame, float *vel_frame, int32_t with_forces,
                      int32_t slot);

/* Wait for frame slot's copies.  It only waits on a CUDA event, so a writer
 * thread may call it while another thread queues the next update. */
int boids_frame_wait(boids_sim *sim, int32_t slot);

/* Page-locked host memory (cudaHostAlloc) for frame buffers; no counterpart
 * in the reference, which writes from its AoS boid array. */
int boids_host_alloc(size_t bytes, void **out);
void boids_host_free(void *p);

/* ------------------------------------------------------------------ ensembles
 *
 * A batched ensemble: many independent grid-engine flocks of uneven size,
 * each with its own parameters, stepped together by one launch per kernel
 * per step (the steps replayed from a captured CUDA graph).  No counterpart
 * in the reference, whose executables run one flock per process; every
 * flock's trajectory is bit-identical to a boids_create(BOIDS_ENGINE_GRID)
 * handle with the same parameters and initial state. */
typedef struct boids_ensemble boids_ensemble;

#define BOIDS_INIT_RANDOM_UNIFORM 0
#define BOIDS_INIT_TEST 1

typedef struct {
    boids_params params;  /* engine must be BOIDS_ENGINE_GRID; device and flags are taken from flock 0 */
    int32_t init_kind;    /* BOIDS_INIT_*: the drawn placements of BoidSimulation::init */
    int32_t rand_seed;    /* srand48 seed, as the grid engine's init uses it */
} boids_flock_desc;

/* Per-flock statistics written by boids_ensemble_stats, in this order. */
#define BOIDS_STAT_POLARIZATION 0  /* |sum of unit velocities| / N                      */
#define BOIDS_STAT_MILLING 1       /* |sum of r_hat x v_hat| / N about the centre of mass */
#define BOIDS_STAT_NN_DISTANCE 2   /* mean nearest-neighbour distance, capped at the search radius */
#define BOIDS_STAT_LARGEST_CLUSTER 3  /* largest linked group / N (link: cohesion sight distance) */
#define BOIDS_STAT_COM_X 4         /* centre of mass, periodic (circular) mean, FP64       */
#define BOIDS_STAT_COM_Y 5
#define BOIDS_STAT_COM_Z 6
#define BOIDS_STAT_MOMENTUM_X 7    /* mean velocity (momentum per boid), FP64              */
#define BOIDS_STAT_MOMENTUM_Y 8
#define BOIDS_STAT_MOMENTUM_Z 9
#define BOIDS_STAT_SEARCH_RADIUS 10 /* the cap of the nearest-neighbour search             */
#define BOIDS_STATS_PER_FLOCK 11

int boids_ensemble_create(const boids_flock_desc *flocks, uint32_t count, boids_ensemble **out);
void boids_ensemble_destroy(boids_ensemble *ens);
/* BoidSimulation::init of every flock (grid engine: srand48(rand_seed)). */
int boids_ensemble_init(boids_ensemble *ens);
/* Replace one flock's state (id order, 3 floats per boid). */
int boids_ensemble_set_state(boids_ensemble *ens, uint32_t flock, const float *pos3n, const float *vel3n);
/* `steps` updates of every flock.  Asynchronous on the ensemble's stream. */
int boids_ensemble_step(boids_ensemble *ens, int32_t steps);
/* One flock's state in id order.  Synchronous. */
int boids_ensemble_get_state(boids_ensemble *ens, uint32_t flock, float *pos3n, float *vel3n);
/* BOIDS_STATS_PER_FLOCK doubles per flock for the current state.  Synchronous. */
int boids_ensemble_stats(boids_ensemble *ens, double *out);
/* Time a few steps with each candidate of the dense-cell thresholds (which
 * cells take the CTA-per-cell kernel) on a copy of the current state and
 * keep the fastest; results do not depend on the choice.  steps_per_trial
 * <= 0 picks a default.  Leaves the state as it was. */
int boids_ensemble_autotune(boids_ensemble *ens, int32_t steps_per_trial);
/* Chosen thresholds: dense_min, defer_min, cand_defer, lone_cand. */
int boids_ensemble_tuning(boids_ensemble *ens, int32_t *out4);
/* Set the thresholds of every flock (the meaning of boids_set_tuning);
 * results do not depend on them.  No counterpart in the reference. */
int boids_ensemble_set_tuning(boids_ensemble *ens, const int32_t *tune4);
int boids_ensemble_synchronize(boids_ensemble *ens);
uint64_t boids_ensemble_kernel_launches(boids_ensemble *ens);

/* ------------------------------------------------------------------ sweep surrogate
 *
 * A small network that maps a flock's rule parameters to its order
 * statistics, trained on ensemble runs, to screen parameter sweeps before the
 * plain simulation re-runs the candidates it selects.  No counterpart in the
 * reference.  Layers in -> hidden -> hidden -> out with ReLU; BF16 weights
 * and activations, FP32 accumulation (tensor-core MMA), FP32 master
 * parameters updated by Adam on the mean squared error.  Parameters are laid
 * out W1 [in x hidden], b1, W2 [hidden x hidden], b2, W3 [hidden x out], b3,
 * weight matrices row-major.  Host arrays are row-major, one row per sample. */
typedef struct boids_mlp boids_mlp;
int boids_mlp_create(int32_t n_in, int32_t n_hidden, int32_t n_out, uint64_t seed, int32_t device, boids_mlp **out);
void boids_mlp_destroy(boids_mlp *mlp);
int64_t boids_mlp_param_count(boids_mlp *mlp);
int boids_mlp_get_params(boids_mlp *mlp, float *params);
/* Also resets the optimiser state. */
int boids_mlp_set_params(boids_mlp *mlp, const float *params);
int boids_mlp_forward(boids_mlp *mlp, const float *x, int32_t rows, float *y);
/* One forward and backward pass, no update: the mean squared error and its
 * gradient with respect to every parameter (same layout as the parameters). */
int boids_mlp_gradient(boids_mlp *mlp, const float *x, const float *target, int32_t rows, float *grad,
                       double *loss);
/* Adam over shuffled mini-batches; *last_epoch_loss = mean batch loss of the last epoch. */
int boids_mlp_train(boids_mlp *mlp, const float *x, const float *target, int32_t rows, int32_t epochs,
                    int32_t batch, float lr, uint64_t shuffle_seed, double *last_epoch_loss);

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
 * must lie in [0, field_size].  This call does not check them: other
 * positions give meaningless results, but the kernels clamp every index they
 * derive from a position, so they stay within their buffers.
 *
 * All scratch lives in one static device array of BOIDS_NOALLOC_SCRATCH_BYTES
 * that every GPU loading the library holds until the process exits; a step
 * needing more (roughly 370 000 boids at the reference's density) returns
 * BOIDS_EINVAL.  Each call looks the array's device address up in the
 * current context (a host-side lookup, so a device reset between calls does
 * no harm); the first call on a device also loads the library's device code
 * there, so make that first call before any stream capture.  Every call
 * shares the array and clears what must start at zero: calls whose GPU work
 * overlaps (other streams, other threads on the same device) race; order
 * them on one stream.  params->device is made current for the call and the
 * caller's current device is restored before it returns.  The work is
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
