// boids_engine.h -- constants and kernel launchers shared by the C-ABI host
// code (boids_capi.cpp, compiled by g++) and the kernels (boids_kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "boids_softfp.h"

namespace boidsgpu {

// Every comparison of the reference that mixes a float with a double is
// replaced by an exactly equivalent float comparison against a constant the
// host derives once:
//   (double)f <  d   <=>  f <  up(d)      (up: smallest float >= d)
//   (double)f >  d   <=>  f >  dn(d)      (dn: largest float  <= d)
// The radius test of Boid::isInsideArea (src/boid.cpp:28),
// (double)sqrtf(d2) < r, becomes d2 < d2_lim with d2_lim the smallest float
// whose correctly rounded square root reaches r; the view-cone test
// acos(c) <= pi*a (src/boid.cpp:34-35) becomes cstar <= c <= 1, with cstar
// found on the host with the same acosf the reference calls.
struct RuleConst {
    float d2_lim;     // radius test: d2 < d2_lim
    float cstar;      // smallest c with (double)acosf(c) <= M_PI*sight_angle
    int32_t all_round;  // sight_angle >= 1.0: the cone test is skipped
    int32_t pad;
};

enum { RULE_COH = 0, RULE_SEP = 1, RULE_ALI = 2 };

struct StepConst {
    uint32_t n;          // boids
    int32_t G;           // device cells per axis along y and z (>= 3), 0 for all-pairs
    int32_t Gx;          // device cells along x: 4 * G (each a quarter of a y/z cell)
    double F;            // field size (host side only)
    SoftDouble Fsd;      // the field size in integer form, for exact float +- double
    float Ff;            // (float)F, for approximate filters
    float F_dn;          // dn(F): wrap test x > F
    float halfF_dn;      // dn(F/2): minimum-image tests
    float inv_side;      // y/z cells per unit length of the device grid
    float inv_subx;      // x cells per unit length (4 * inv_side)
    float side;          // y/z cell side (approximate, for row trimming)
    float trim_r2;       // squared radius, with margin, used to trim a boid's rows
    float filt_r2;       // squared radius of the conservative fast filter
    float box_lim;       // all-pairs box filter: ||dx| - F/2| > box_lim
    float halfFf;        // (float)(F/2) for the box filter
    float cc, cs, ca;    // (float) force coefficients: cohesion, separation, alignment
    float vmax_dn, vmin_up;  // speed clamp tests
    float vmax_f, vmin_f;    // speed clamp scale factors (float)vmax, (float)vmin
    float d2_any;        // largest d2_lim of the three rules
    float cone_band;     // approximate cone tests closer than this to a threshold are redone exactly
    // View-cone pre-test of the candidate filters, on when every rule has a
    // cone that rejects c <= 0 (cstar > 0): a candidate whose approximate
    // v . r is below -|v| * dot_eps has an exact v . r < 0 and fails all
    // three rules.  dot_eps bounds the approximation's error per unit |v|.
    float dot_eps;
    int32_t cone_pre;
    // The dense kernel's half-precision filter (two candidates per
    // instruction) works on coordinates relative to the cell's centre times
    // hsc (a power of two putting them within +-0.5) and velocities times
    // hvsc (a power of two putting |v| <= vmax within 0.5).  hfilt bounds the
    // half-precision squared distance of any pair within the filter radius;
    // a pair is dropped behind the boid when its half-precision v . r is
    // below -(hdot0 + hdot1 |v| hvsc), which bounds that dot product's error.
    float hsc, hvsc, hfilt, hdot0, hdot1;
    int32_t id_bits;     // bits needed for the largest boid id, rounded up to a multiple of 4
    RuleConst rule[3];   // cohesion, separation, alignment
    // the reference's overlapping grid, for Boid::grid_index parity
    int32_t refG;
    float refGS, refR;
    // Place of this flock in a batched ensemble (all zero for one flock):
    // its cells are global cells [cell_base, cell_base + Gx*G*G), its boids
    // occupy state slots [slot_base, slot_base + n), and slot = cell start
    // (a prefix over all flocks' counts) + slot_off, the padding that aligns
    // every flock to kSlotAlign slots.  Boid ids are local to the flock.
    uint32_t cell_base;
    uint32_t slot_base;
    uint32_t slot_off;
    uint32_t flock;
    // Which full-size cells the CTA-per-cell kernel takes (the results do not
    // depend on it): those holding dense_min boids or more, those holding
    // defer_min or more whose 27-cell neighbourhood holds over cand_defer
    // boids, and any non-empty cell whose neighbourhood holds over lone_cand.
    uint32_t dense_min, defer_min, cand_defer, lone_cand;
};

// A batched ensemble's flock table, in device memory.  Every block of
// kSlotAlign state slots belongs to one flock, so a CTA of that many threads
// serves one flock and can hold its StepConst in shared memory.
constexpr int kSlotAlign = 128;
struct FlockTable {
    const StepConst *ks;        // per flock
    const uint16_t *blk_flock;  // per block of kSlotAlign slots
    const uint32_t *cell4;      // per flock: cell_base / 4 (ascending)
    uint32_t count;             // flocks
    uint32_t nslots;            // padded slots of all flocks
};

// Device scratch of one engine handle.  Sizes in elements.
struct DevBuffers {
    float4 *pos[2], *vel[2];   // ping-pong state, float4 (w of pos = id bits)
    uint32_t *key, *rank;      // per slot: device cell and rank inside it
    uint32_t *count;           // per cell (padded): boids binned so far
    uint32_t *lstart;          // per cell (padded): exclusive scan inside a tile
    uint32_t *bsum;            // per scan tile: offset of the tile
    uint32_t *ticket;          // scan completion counter (1 word)
    uint32_t *ap_cnt, *ap_list;  // all-pairs: per boid neighbour count and list
    float *forces;             // 9 per boid (id order), optional
    float *stage;              // 6 per boid, host<->device staging
    int32_t *cells8;           // 8 per boid (id order)
    int32_t *dcnt;             // 3 per boid (id order)
    uint64_t *dhash;           // 3 per boid (id order)
    uint32_t *dense_list;      // dense kernel work items (cell, first boid), this step (dense_list_capacity words)
    uint32_t *dense_n;         // dense items, the dense kernel's work queue, deferred sparse boids (3 words)
    uint32_t *defer;           // sparse boids deferred to further passes: (slot, lo_id), 2 words per slot (null: none);
                               // a flock's entries start at its slot_base
    uint32_t *defer_cnt;       // deferred boids per flock (a single flock: dense_n + 2)
    uint64_t *ovf;             // per slot, kOvfCap entries: the accepted neighbours a deferred boid's
                               // first pass could not keep (null: none)
    uint32_t *ovf_n;           // per slot: how many there were (over kOvfCap: the row is incomplete)
    uint64_t *wscratch;        // dense kernel: wcap entries per CTA, a huge cell's candidates filed by window
    uint32_t wcap;             // (null / 0: every window scans the neighbourhood)
    // Side stream on which the deferred boids run beside the dense kernel,
    // forked from and joined back to the engine's stream (null: in order).
    cudaStream_t aux;
    cudaEvent_t fork, join, cjoin;  // cjoin: the classification's end (it runs beside the scatter)
    uint8_t *dflag;            // per full-size cell: 1 when the dense kernel takes it
    void *carry;               // per slot, kCarryBytes: partial sums between id windows (null: no windows)
    uint32_t *flag;            // set_state range check (1 word)
    uint32_t ncell, ncell_pad, nscan_blocks;
    uint32_t dense_grid;       // CTAs of the dense-cell kernel
    uint32_t ap_cap;
};

constexpr int kScanTile = 2048;       // cells per scan block (256 threads x 8)
constexpr int kListCap = 12;          // grid engine, thread-per-boid kernel: sorted neighbours kept per pass
constexpr int kOvfCap = 24;           // accepted neighbours beyond those a deferred boid's first pass keeps
// Defaults, measured on the bench workload (N = 2^20 from a uniform start,
// steps 5-25), the same flock after 1000 steps, and gathered flocks of 16 384
// and 65 536 boids: dense_min 16 beats 12 on all four (3-6 %); lone_cand 64
// costs 5x on the uniform start, as many small cells become CTA work items,
// and lone_cand above 96 costs the small gathered flocks 5-20 %.  Clustered
// flocks run another 15-40 % faster with lower thresholds still, which the
// autotuners pick.
constexpr int kDenseMin = 16;         // default dense_min
constexpr int kDeferMin = 4;          // default defer_min
constexpr int kCandDefer = 192;       // default cand_defer
constexpr int kLoneCand = 96;         // default lone_cand
constexpr int kCarryBytes = 72;       // partial sums of one boid between id windows
constexpr uint32_t kWinScratch = 32768;  // most candidates a CTA files by window (32 windows of 1024)

// Dense-cell threshold sets the autotuners try, {dense_min, defer_min,
// cand_defer, lone_cand}; the first is the default.  Crowded (clustered)
// states favour low thresholds, uniform states high ones.
constexpr uint32_t kNever = 1u << 30;
constexpr uint32_t kTuneCand[][4] = {
    {16, 4, 192, 96}, {12, 4, 192, 96}, {12, 4, 192, 384}, {12, 4, 192, 64}, {12, 4, 192, 48},
    {8, 2, 96, 128}, {4, 2, 64, 128}, {8, 4, 128, 64}, {kNever, kNever, kNever, 1024},
};
constexpr int kTuneCount = sizeof(kTuneCand) / sizeof(kTuneCand[0]);

// The dense kernel's work items are (full-size cell, first boid) pairs, one
// per kDenseRound boids of a dense cell, so that the boids of one crowded
// cell spread over several CTAs.  Words the work list can need in one step:
// at most one item per non-empty cell plus one per kDenseRound boids, two
// words per item.
constexpr int kDenseRound = 128;
inline size_t dense_list_capacity(size_t ncell, size_t n)
{
    const size_t by_cells = ncell / 4;
    return 2 * ((by_cells < n ? by_cells : n) + n / kDenseRound + 1);
}
constexpr int kDenseCap = 512;        // candidates of a dense cell held in shared memory
constexpr int kDenseCtasPerSm = 7;   // resident CTAs of the dense-cell kernel per SM (its launch bounds)
constexpr int kApCap = 256;           // all-pairs engine: neighbours kept per boid (more: an O(N) scan)
constexpr uint32_t kMaxBoids = 1u << 29;  // slot index packs into 29 bits
constexpr int kMaxGridAxis = 812;          // device cells per axis: 4 G^3 < 2^31

// Launchers.  Each returns the launch's cudaError_t and adds the number of
// kernels it launched to *launches.
// Packs ids [i0, i1) of an id-ordered state (slot = id); bad: the range
// check's flag (nullable); bin (nullable): also the grid keys of those slots,
// as launch_grid_keys (a single flock; count cleared beforehand).
cudaError_t launch_pack(const float *pos3, const float *vel3, float4 *pos4, float4 *vel4, uint32_t i0, uint32_t i1,
                        uint32_t *bad, float hi, const StepConst *bin, uint32_t *key, uint32_t *rank,
                        uint32_t *count, cudaStream_t s, uint64_t *launches);
// Slot order -> id order: the slot of every id into slot_of (n words of
// scratch), then ids [i0, i1) gathered into pos3/vel3 (either nullable).
cudaError_t launch_unpack_index(const float4 *pos4, uint32_t *slot_of, uint32_t n, cudaStream_t s,
                                uint64_t *launches);
cudaError_t launch_unpack_gather(const float4 *pos4, const float4 *vel4, const uint32_t *slot_of, float *pos3,
                                 float *vel3, uint32_t i0, uint32_t i1, uint32_t n, cudaStream_t s,
                                 uint64_t *launches);
cudaError_t launch_unpack(const float4 *pos4, const float4 *vel4, uint32_t *slot_of, float *pos3, float *vel3,
                          uint32_t n, cudaStream_t s, uint64_t *launches);
// One .ptcl frame in id order: pframe gets 3 floats per boid, or 12 with
// forces (xyz + the nine get_force floats; zeros when force9 is null);
// vframe (nullable) gets vx,vy,vz.
cudaError_t launch_frame(const float4 *pos4, const float4 *vel4, const float *force9, float *pframe,
                         float *vframe, int with_forces, uint32_t n, cudaStream_t s, uint64_t *launches);
// ft == nullptr: one flock described by k; else a batched ensemble (k unused).
cudaError_t launch_grid_keys(const StepConst &k, const float4 *pos, uint32_t *key, uint32_t *rank,
                             uint32_t *count, cudaStream_t s, uint64_t *launches,
                             const FlockTable *ft = nullptr);
// Scan of the cell counts, then the dense-cell classification (flags and
// work list) of every full-size cell.
cudaError_t launch_grid_scan(const StepConst &k, const DevBuffers &b, cudaStream_t s, uint64_t *launches,
                             const FlockTable *ft = nullptr);
cudaError_t launch_grid_scatter(const StepConst &k, const DevBuffers &b, int from, bool zero_counts,
                                cudaStream_t s, uint64_t *launches, const FlockTable *ft = nullptr);
// Rules + integration over the sorted state b.pos[from]; writes the new state
// to b.pos[1-from] (diag == false) or neighbour-set fingerprints (diag == true).
cudaError_t launch_grid_force(const StepConst &k, const DevBuffers &b, int from, bool diag,
                              bool record_forces, cudaStream_t s, uint64_t *launches,
                              const FlockTable *ft = nullptr);
cudaError_t launch_allpairs(const StepConst &k, const DevBuffers &b, int from, bool diag,
                            bool record_forces, cudaStream_t s, uint64_t *launches);
cudaError_t launch_ref_cells(const StepConst &k, const float4 *pos, int32_t *cells8, cudaStream_t s,
                             uint64_t *launches);

// Opt the dense-cell kernels in to their shared memory on the current device
// (done before a stream capture, where it could not be).
cudaError_t grid_prepare();

// Ensemble statistics of the binned state b.pos[from] (see boids_kernels.cu):
// acc gets kStatAcc doubles per flock, com 3 per flock, largest the largest
// linked group per flock; link is the per-flock link distance; *err != 0
// after the launch means a union-find walk hit its bound.  Uses b.key and
// b.rank as scratch.
constexpr int kStatAcc = 16;
cudaError_t launch_ensemble_stats(const DevBuffers &b, int from, const FlockTable &ft, const float *link,
                                  double *acc, double *com, uint32_t *largest, uint32_t *err, cudaStream_t s,
                                  uint64_t *launches);

}  // namespace boidsgpu
