// boids_capi.cpp -- the C ABI of include/boids.h: engine set-up, state
// transfer, stepping and diagnostics.  The compute is in boids_kernels.cu;
// this file owns the handle, its device memory and its stream.
//
// Built with -ffp-contract=off: the host-side initial-state draws must round
// like the reference's x86 build on any host (aarch64 contracts to FMA by
// default).
#include "boids.h"
#include "boids_engine.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

using boidsgpu::DevBuffers;
using boidsgpu::RuleConst;
using boidsgpu::StepConst;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *where)
{
    return fail(BOIDS_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

// ------------------------------------------------------------------ exact float thresholds

float f_dn(double d)  // largest float <= d
{
    float f = (float)d;
    if ((double)f > d) f = std::nextafter(f, -INFINITY);
    return f;
}

float f_up(double d)  // smallest float >= d
{
    float f = (float)d;
    if ((double)f < d) f = std::nextafter(f, INFINITY);
    return f;
}

int64_t ordinal(float x)
{
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return (u & 0x80000000u) ? -(int64_t)(u & 0x7fffffffu) : (int64_t)u;
}

float from_ordinal(int64_t o)
{
    uint32_t u = o < 0 ? (uint32_t)(-o) | 0x80000000u : (uint32_t)o;
    float x;
    std::memcpy(&x, &u, 4);
    return x;
}

// Boid::isInsideArea's cone test is (double)acosf(c) <= M_PI*a with c a
// float (src/boid.cpp:34-35).  With acosf non-increasing on [-1, 1] the set
// of passing c is [cstar, 1]; cstar is found by bisection over the floats
// with the host's own acosf -- the function the reference calls -- and the
// monotonicity is re-checked in a window around it.
int cone_threshold(double a, float *cstar)
{
    const double T = M_PI * a;
    auto ok = [T](float c) { return (double)std::acos(c) <= T; };  // float overload: acosf
    if (!ok(1.0f)) { *cstar = INFINITY; return 0; }
    if (ok(-1.0f)) { *cstar = -1.0f; return 0; }
    int64_t lo = ordinal(-1.0f), hi = ordinal(1.0f);  // ok(lo) false, ok(hi) true
    while (hi - lo > 1) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (ok(from_ordinal(mid))) hi = mid; else lo = mid;
    }
    for (int64_t o = hi - 4096; o < hi + 4096; ++o) {
        if (o < ordinal(-1.0f) || o > ordinal(1.0f)) continue;
        if (ok(from_ordinal(o)) != (o >= hi))
            return fail(BOIDS_ENOTSUP, "host acosf is not monotone near the view-cone threshold");
    }
    *cstar = from_ordinal(hi);
    return 0;
}

// The radius test (double)sqrtf(d2) < r (src/boid.cpp:28, with
// Vector3D::norm at src/vector3D.cpp:64-67).  sqrtf is correctly rounded,
// hence monotone, so the passing d2 are [0, lim) for the float lim returned.
float radius_d2_limit(double r)
{
    auto inside = [r](float d2) { return (double)std::sqrt(d2) < r; };  // float overload: sqrtf
    if (!inside(0.0f)) return 0.0f;
    if (inside(INFINITY)) return INFINITY;
    int64_t lo = 0, hi = ordinal(INFINITY);  // inside(lo), !inside(hi)
    while (hi - lo > 1) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (inside(from_ordinal(mid))) lo = mid; else hi = mid;
    }
    return from_ordinal(hi);
}

// ------------------------------------------------------------------ drand48

struct Drand48 {
    uint64_t x = 0;  // glibc's state before any srand48 call
    void seed(long s) { x = (((uint64_t)s & 0xffffffffULL) << 16) | 0x330eULL; }
    double next()
    {
        x = (0x5deece66dULL * x + 0xbULL) & 0xffffffffffffULL;
        return (double)x * (1.0 / 281474976710656.0);
    }
};

}  // namespace

// ------------------------------------------------------------------ handle

struct boids_sim {
    boids_params p{};
    StepConst k{};
    DevBuffers b{};
    int engine = 0;        // effective kernels: 0 all-pairs, 1 device grid
    bool ref_geometry_ok = false;
    int cur = 0;           // buffer holding the state
    bool has_state = false;
    bool forces_valid = false;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    uint64_t launches = 0;
    uint64_t steps_done = 0;
    // profiling: event pairs recorded around each phase, resolved on read
    struct Pending {
        cudaEvent_t a, b;
        int slot;  // 0 bin, 1 force, 2 other
    };
    bool prof = false;
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;
    boids_profile_t acc{};
    // .ptcl frames: device assembly buffer (15 floats per boid) and one
    // completion event per slot, made on first use
    float *frame_dev = nullptr;
    cudaEvent_t frame_ev[BOIDS_FRAME_SLOTS] = {};
    // Updates captured into CUDA graphs on first use: [0] kGraphSteps
    // updates, for long runs; [1] one update of the grid engine, so that a
    // single update's kernels reach the GPU in one launch.  Each is valid for
    // the stream, buffer parity and constants it was captured with.
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        cudaStream_t stream = nullptr;
        int cur = -1;
        StepConst k{};
        uint64_t launches = 0;  // kernel launches per replay
        int engine = -1;        // the kernels it was captured with
    };
    StepGraph graphs[2];
    bool graph_off = false;     // capture failed once on this handle
    // set_state/get_state move the state in kXferChunks pieces of ids; with
    // the side stream, one piece is packed (or copied out) while the next is
    // copied (or unpacked): one event per piece
    static constexpr int kXferChunks = 4;
    cudaEvent_t xfer_ev[kXferChunks] = {};
};

namespace {

void free_buffers(DevBuffers &b)
{
    void *ptrs[] = {b.pos[0], b.pos[1], b.vel[0], b.vel[1], b.key, b.rank, b.count, b.lstart,
                    b.bsum, b.ticket, b.ap_cnt, b.ap_list, b.forces, b.stage, b.cells8, b.dcnt, b.dhash,
                    b.dense_list, b.dense_n, b.flag, b.dflag, b.carry, b.defer, b.ovf, b.ovf_n, b.wscratch};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (b.aux) cudaStreamDestroy(b.aux);
    if (b.fork) cudaEventDestroy(b.fork);
    if (b.join) cudaEventDestroy(b.join);
    if (b.cjoin) cudaEventDestroy(b.cjoin);
    b = DevBuffers{};
}

template <class T>
int dalloc(T **p, size_t count, bool zero = false)
{
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * count);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(BOIDS_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    if (zero) {
        e = cudaMemset(*p, 0, sizeof(T) * count);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemset");
    }
    return 0;
}

int use_device(boids_sim *s)
{
    cudaError_t e = cudaSetDevice(s->p.device);
    return e == cudaSuccess ? 0 : cuda_fail(e, "cudaSetDevice");
}

// Reference grid sizing, src/boid_simulation_grid.cpp:80-89.
bool ref_geometry(const boids_params &p, float *R, int *G, float *GS)
{
    double m = (p.cohesion_sight_distance < p.alignment_sight_distance) ? p.alignment_sight_distance
                                                                         : p.cohesion_sight_distance;
    m = (m < p.separation_sight_distance) ? p.separation_sight_distance : m;
    const float r = (float)m;
    const int gn = (int)(p.field_size / (double)(r * 2));
    if (gn <= 0) return false;
    const unsigned g = (unsigned)gn;
    const float gs = (float)(p.field_size / (double)g);
    if (r * 2 >= gs) return false;
    *R = r;
    *G = gn;
    *GS = gs;
    return true;
}

cudaEvent_t take_event(boids_sim *s)
{
    if (!s->pool.empty()) {
        cudaEvent_t e = s->pool.back();
        s->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Adds the elapsed time of every recorded phase to the totals.
void resolve_events(boids_sim *s)
{
    for (auto &q : s->pending) {
        float ms = 0.f;
        cudaEventSynchronize(q.b);
        if (cudaEventElapsedTime(&ms, q.a, q.b) == cudaSuccess) {
            double *slot = q.slot == 0 ? &s->acc.bin_ms : q.slot == 1 ? &s->acc.force_ms : &s->acc.other_ms;
            *slot += ms;
        }
        s->pool.push_back(q.a);
        s->pool.push_back(q.b);
    }
    s->pending.clear();
}

// Brackets the launches of one phase with events on the handle's stream.
struct PhaseTimer {
    boids_sim *s;
    int slot;
    cudaEvent_t a = nullptr;
    PhaseTimer(boids_sim *s_, int slot_) : s(s_), slot(slot_)
    {
        if (!s->prof) return;
        if (s->pending.size() > 8192) resolve_events(s);
        a = take_event(s);
        cudaEventRecord(a, s->stream);
    }
    ~PhaseTimer()
    {
        if (!a) return;
        cudaEvent_t b = take_event(s);
        cudaEventRecord(b, s->stream);
        s->pending.push_back({a, b, slot});
    }
};

int grid_bin_fresh(boids_sim *s)
{
    CK(cudaMemsetAsync(s->b.count, 0, sizeof(uint32_t) * s->b.ncell_pad, s->stream));
    CK(boidsgpu::launch_grid_keys(s->k, s->b.pos[s->cur], s->b.key, s->b.rank, s->b.count, s->stream,
                                  &s->launches));
    return 0;
}

// The drawn placements of BoidSimulation::init, in the reference's draw
// order (src/boid_simulation_grid.cpp:95-136; the all-pairs engine's
// src/boid_simulation.cpp:79-112 draws the same sequence but never calls
// srand48: seeded == false starts from the never-seeded state).
void draw_state(const boids_params &p, bool test, bool seeded, int32_t seed, float *pos, float *vel)
{
    const double F = p.field_size;
    Drand48 d;
    if (seeded) d.seed((long)seed);
    const double vmax = p.velocity_max, vmin = p.velocity_min;
    for (uint32_t i = 0; i < p.number_of_agents; ++i) {
        float *x = pos + (size_t)3 * i, *v = vel + (size_t)3 * i;
        if (test) {  // src/boid_simulation_grid.cpp:100-108
            x[0] = (float)(F * 3 / 8 + d.next() * F / 4);
            x[1] = (float)(F * 3 / 8 + d.next() * F / 4);
            if (d.next() > 0.5) x[2] = (float)(d.next() * F / 4 + F * 3 / 4);
            else x[2] = (float)(d.next() * F / 4);
        } else {  // src/boid_simulation_grid.cpp:123-126
            x[0] = (float)(F * d.next());
            x[1] = (float)(F * d.next());
            x[2] = (float)(F * d.next());
        }
        // src/boid_simulation_grid.cpp:127-132
        const double sp = d.next() * (vmax - vmin) + vmin;
        const double th1 = d.next() * M_PI;
        const double th2 = d.next() * 2.0 * M_PI;
        v[0] = (float)(sp * std::sin(th1) * std::cos(th2));
        v[1] = (float)(sp * std::sin(th1) * std::sin(th2));
        v[2] = (float)(sp * std::cos(th1));
    }
}

// The parameter-derived constants of one flock: the exact float thresholds,
// the reference's overlapping-grid geometry (src/boid_simulation_grid.cpp:80-89,
// whose checks apply to the grid engine) and this engine's device grid (G = 0:
// too few cells per axis, scan all pairs).  *ref_ok: the reference geometry
// is valid (boids_get_cells).
int make_constants(const boids_params &p, StepConst &k, bool *ref_ok)
{
    if (p.number_of_agents > boidsgpu::kMaxBoids)
        return fail(BOIDS_EINVAL, "number_of_agents exceeds 2^29");
    if (!(p.field_size > 0.0) || !std::isfinite(p.field_size))
        return fail(BOIDS_EINVAL, "field_size must be positive and finite");
    if (p.engine != BOIDS_ENGINE_ALLPAIRS && p.engine != BOIDS_ENGINE_GRID)
        return fail(BOIDS_EINVAL, "unknown engine");
    const double radii[3] = {p.cohesion_sight_distance, p.separation_sight_distance, p.alignment_sight_distance};
    for (double r : radii)
        if (std::isnan(r)) return fail(BOIDS_EINVAL, "sight distance is NaN");

    k = StepConst{};
    k.n = p.number_of_agents;
    k.F = p.field_size;
    k.Ff = (float)p.field_size;
    k.F_dn = f_dn(p.field_size);
    k.halfF_dn = f_dn(p.field_size / 2);
    k.halfFf = (float)(p.field_size / 2);
    k.cc = (float)p.cohesion_force_coefficient;
    k.cs = (float)p.separation_force_coefficient;
    k.ca = (float)p.alignment_force_coefficient;
    k.vmax_dn = f_dn(p.velocity_max);
    k.vmin_up = f_up(p.velocity_min);
    k.vmax_f = (float)p.velocity_max;
    k.vmin_f = (float)p.velocity_min;
    k.Fsd = boidsgpu::soft_double(p.field_size);
    k.cone_band = 4e-6f;
    {
        int bits = 0;
        while (bits < 32 && (1ull << bits) < (uint64_t)(k.n ? k.n : 1)) ++bits;
        k.id_bits = std::max(4, (bits + 3) / 4 * 4);
    }
    const double ang[3] = {p.cohesion_sight_angle, p.separation_sight_angle, p.alignment_sight_angle};
    float rmax = 0.f;
    k.d2_any = 0.f;
    for (int r = 0; r < 3; ++r) {
        RuleConst &q = k.rule[r];
        q.d2_lim = radius_d2_limit(radii[r]);
        q.all_round = ang[r] >= 1.0;
        q.cstar = INFINITY;
        if (!q.all_round) {
            if (int rc = cone_threshold(ang[r], &q.cstar)) return rc;
        }
        k.d2_any = std::fmax(k.d2_any, q.d2_lim);
        const float rup = f_up(radii[r]);
        if (rup > rmax) rmax = rup;
    }
    // Conservative filter radius: the exact distance test can only accept a
    // pair whose approximate distance is below this (rounding of the image
    // shift and of the filter's own arithmetic is far below the margin).
    const double ulpF = std::nextafter(std::fmax(k.Ff, 1.0f), INFINITY) - std::fmax(k.Ff, 1.0f);
    const double rf = (double)rmax * (1.0 + 1e-4) + 8.0 * ulpF;
    k.filt_r2 = (float)(rf * rf);
    k.box_lim = (float)(p.field_size / 2 - rf * (1.0 + 1e-4) - 8.0 * ulpF);
    // The filters' relative vector differs from the exact imaged one by a
    // few ulps of the coordinates (at most 2F in magnitude), each dot
    // product by those times |v|_1 <= sqrt(3)|v| plus three roundings of
    // |v| * |r|: 64 ulps and 1e-5 * rf per unit |v| bound both with room.
    k.dot_eps = (float)(64.0 * ulpF + 1e-5 * rf);
    k.cone_pre = 1;
    for (int r = 0; r < 3; ++r)
        if (k.rule[r].all_round || !(k.rule[r].cstar > 0.f)) k.cone_pre = 0;

    // reference overlapping-grid geometry
    float refR = 0.f, refGS = 0.f;
    int refG = 0;
    *ref_ok = ref_geometry(p, &refR, &refG, &refGS);
    if (p.engine == BOIDS_ENGINE_GRID) {
        if (!*ref_ok)
            return fail(BOIDS_EINVAL, "Invalid GRID_NUM: the reference grid engine needs "
                                      "field_size > 2 * max sight distance (src/boid_simulation_grid.cpp:86-89)");
        if (refG == 1)
            return fail(BOIDS_EINVAL, "GRID_NUM == 1: the reference grid engine lists a boid up to 8 times in "
                                      "its own cell (overlap cell == own cell); use the all-pairs engine");
    }
    k.refG = refG;
    k.refGS = refGS;
    k.refR = refR;

    // device binning grid: cells of side >= 1.01 * filter radius, capped.
    // The all-pairs engine gets one too (same results, see
    // BOIDS_FLAG_ALLPAIRS_KERNELS) unless its boids could leave the field in
    // one step.
    const bool pairs_on_grid = p.engine == BOIDS_ENGINE_ALLPAIRS && !(p.flags & BOIDS_FLAG_ALLPAIRS_KERNELS) &&
                               std::fmax(p.velocity_max, p.velocity_min) < p.field_size / 2;
    int G = 0;
    if ((p.engine == BOIDS_ENGINE_GRID || pairs_on_grid) && rf > 0) {
        double g = std::floor(p.field_size / (rf * 1.01));
        const double cap = std::cbrt(std::fmax(2.0 * k.n, 2097152.0));
        if (g > cap) g = std::floor(cap);
        // The 4 G^3 cell keys are formed in int arithmetic (cell_key), so
        // they must stay below 2^31: G <= 812.  With marun2019's radii only
        // flocks of more than 2^28 boids at under half the reference's density
        // reach it; the grid's size never changes a result.
        if (g > boidsgpu::kMaxGridAxis) g = boidsgpu::kMaxGridAxis;
        G = g >= 3 ? (int)g : 0;  // fewer than 3 cells per axis: scan all pairs
    }
    k.G = G;
    k.Gx = 4 * G;
    k.inv_side = G ? (float)(G / p.field_size) : 0.f;
    k.inv_subx = G ? (float)(4.0 * G / p.field_size) : 0.f;
    k.side = G ? (float)(p.field_size / G) : 0.f;
    k.trim_r2 = k.filt_r2 * 1.002f;
    if (G) {
        // Error budget of the half-precision filter, in scaled units: with
        // |coordinates| <= 0.5 each conversion and each difference rounds by
        // at most 2^-12, so a component of the relative vector is off by
        // e <= 3 * 2^-12 (pairs within the radius have |d| < 0.34); each of
        // the three fused steps of |d|^2 and v . d adds 2^-11 relative and
        // 2^-25 absolute.  hfilt: (rf + sqrt(3) e)^2 (1 + 2^-11)^3 + 1e-7.
        // v . d: 3 * 2^-11 * 0.35 from the velocity's own conversion, plus
        // |v| (sqrt(3) e + 3 sqrt(3) 2^-11 0.35) + 1e-7 <= 5.2e-4 + 2.2e-3 |v|;
        // hdot0 and hdot1 take twice that.
        const double side = p.field_size / G;
        k.hsc = (float)std::ldexp(1.0, (int)std::floor(std::log2(0.5 / (1.5 * side))));
        const double vm = k.vmax_f > 0.f ? (double)k.vmax_f : 1.0;
        k.hvsc = (float)std::ldexp(1.0, (int)std::floor(std::log2(0.5 / vm)));
        const double e = 3.0 * std::ldexp(1.0, -12);
        const double r = rf * k.hsc + std::sqrt(3.0) * e;
        const double hf = r * r * std::pow(1.0 + std::ldexp(1.0, -11), 3) + 1e-7;
        k.hfilt = std::nextafter((float)hf, INFINITY);
        k.hdot0 = 1.1e-3f;
        k.hdot1 = 4.4e-3f;
    }
    k.dense_min = boidsgpu::kDenseMin;
    k.lone_cand = boidsgpu::kLoneCand;
    k.defer_min = boidsgpu::kDeferMin;
    k.cand_defer = boidsgpu::kCandDefer;
    return BOIDS_OK;
}

}  // namespace

extern "C" {

const char *boids_last_error(void) { return g_err.c_str(); }

const char *boids_version(void) { return "boids_gb300 0.1 (sm_103a)"; }

int boids_create(const boids_params *params, boids_sim **out)
{
    if (!params || !out) return fail(BOIDS_EINVAL, "boids_create: null argument");
    *out = nullptr;
    const boids_params &p = *params;
    StepConst kc{};
    bool ref_ok = false;
    if (int rc = make_constants(p, kc, &ref_ok)) return rc;
    boids_sim *s = new boids_sim();
    s->p = p;
    s->k = kc;
    s->ref_geometry_ok = ref_ok;
    s->engine = kc.G ? 1 : 0;
    const StepConst &k = s->k;
    const int G = k.G;

    int rc = 0;
    if ((rc = use_device(s))) { delete s; return rc; }
    DevBuffers &b = s->b;
    const size_t n = k.n;
#define ALLOC(...)                          \
    if ((rc = dalloc(__VA_ARGS__))) {       \
        free_buffers(b);                    \
        delete s;                           \
        return rc;                          \
    }
    ALLOC(&b.pos[0], n);
    ALLOC(&b.pos[1], n);
    ALLOC(&b.vel[0], n);
    ALLOC(&b.vel[1], n);
    ALLOC(&b.stage, 6 * n);
    ALLOC(&b.flag, 1, true);
    if (G) {
        b.ncell = (uint32_t)(4 * G) * G * G;
        b.ncell_pad = (b.ncell + 1 + boidsgpu::kScanTile - 1) / boidsgpu::kScanTile * boidsgpu::kScanTile;
        b.nscan_blocks = b.ncell_pad / boidsgpu::kScanTile;
        ALLOC(&b.key, n);
        ALLOC(&b.rank, n);
        ALLOC(&b.count, b.ncell_pad, true);
        ALLOC(&b.lstart, b.ncell_pad);
        ALLOC(&b.bsum, b.nscan_blocks);
        ALLOC(&b.ticket, 1, true);
        const size_t ndense = boidsgpu::dense_list_capacity(b.ncell, n);
        ALLOC(&b.dense_list, ndense);
        ALLOC(&b.dflag, b.ncell / 4);
        {
            unsigned char *carry = nullptr;
            ALLOC(&carry, (size_t)boidsgpu::kCarryBytes * n);
            b.carry = carry;
        }
        ALLOC(&b.dense_n, 3, true);
        ALLOC(&b.defer, 2 * n);
        // the deferred boids' overflow rows (196 B per boid) speed the
        // further passes up and are optional: without them those passes
        // walk the candidates again
        if (n <= (size_t)1 << 26) {
            uint64_t *rows = nullptr;
            uint32_t *counts = nullptr;
            if (cudaMalloc((void **)&rows, sizeof(uint64_t) * boidsgpu::kOvfCap * n) == cudaSuccess) {
                if (cudaMalloc((void **)&counts, sizeof(uint32_t) * n) == cudaSuccess) {
                    b.ovf = rows;
                    b.ovf_n = counts;
                } else {
                    cudaFree(rows);
                }
            }
            cudaGetLastError();
        }
        b.defer_cnt = b.dense_n + 2;
        if (cudaStreamCreateWithFlags(&b.aux, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&b.join, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&b.cjoin, cudaEventDisableTiming) != cudaSuccess) {
            const cudaError_t ce = cudaGetLastError();
            free_buffers(b);
            delete s;
            return cuda_fail(ce, "cudaStreamCreate (side stream)");
        }
        int nsm = 0;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p.device);
        b.dense_grid = (uint32_t)std::max(1, nsm) * boidsgpu::kDenseCtasPerSm;
        b.wcap = (uint32_t)std::min<size_t>(boidsgpu::kWinScratch, std::max<size_t>(n, 1));
        ALLOC(&b.wscratch, (size_t)b.wcap * b.dense_grid);
    }
    if (p.engine == BOIDS_ENGINE_ALLPAIRS) {  // its own kernels, for states the grid cannot take
        b.ap_cap = boidsgpu::kApCap;
        ALLOC(&b.ap_cnt, n, true);
        ALLOC(&b.ap_list, n * b.ap_cap);
    }
    if (p.flags & BOIDS_FLAG_RECORD_FORCES) ALLOC(&b.forces, 9 * n);
#undef ALLOC
    cudaError_t e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        free_buffers(b);
        delete s;
        return cuda_fail(e, "cudaStreamCreate");
    }
    s->stream = s->own_stream;
    *out = s;
    return BOIDS_OK;
}

void boids_destroy(boids_sim *s)
{
    if (!s) return;
    cudaSetDevice(s->p.device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->b.aux) cudaStreamSynchronize(s->b.aux);
    free_buffers(s->b);
    for (auto &gr : s->graphs)
        if (gr.exec) cudaGraphExecDestroy(gr.exec);
    if (s->frame_dev) cudaFree(s->frame_dev);
    for (cudaEvent_t e : s->frame_ev)
        if (e) cudaEventDestroy(e);
    resolve_events(s);
    for (cudaEvent_t e : s->pool) cudaEventDestroy(e);
    for (cudaEvent_t e : s->xfer_ev)
        if (e) cudaEventDestroy(e);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    delete s;
}

namespace {

// First id of transfer piece c (of kXferChunks), on a 1024-id boundary.
static uint32_t xfer_start(uint32_t n, int c)
{
    const uint64_t b = ((uint64_t)n * (uint32_t)c / boids_sim::kXferChunks + 1023) & ~(uint64_t)1023;
    return (uint32_t)std::min<uint64_t>(b, n);
}

// Whether the transfers run in pieces: with the side stream, once the
// pieces' events exist (made on first use; without them, one piece).
static bool xfer_pipelined(boids_sim *s)
{
    if (!s->b.aux) return false;
    for (cudaEvent_t &ev : s->xfer_ev)
        if (!ev && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
            ev = nullptr;
            cudaGetLastError();
            return false;
        }
    return true;
}

static bool graph_ready(boids_sim *s, bool rec, int which);

}  // namespace

namespace {

// boids_set_state for the current population s->k.n.
static int set_state_n(boids_sim *s, const float *pos3n, const float *vel3n)
{
    if ((!pos3n && s->k.n) || (!vel3n && s->k.n)) return fail(BOIDS_EINVAL, "boids_set_state: null argument");
    int rc = use_device(s);
    if (rc) return rc;
    const uint32_t n = s->k.n;
    // the grid kernels bin positions into cells: they must lie in the field
    // (the grid engine refuses other states; the all-pairs engine takes them
    // with its own kernels)
    const bool check = s->k.G != 0;
    float *dpos = s->b.stage, *dvel = s->b.stage + (size_t)3 * n;
    const bool pipe = xfer_pipelined(s);
    {
        PhaseTimer t(s, 2);
        if (check) {
            CK(cudaMemsetAsync(s->b.flag, 0, sizeof(uint32_t), s->stream));
            CK(cudaMemsetAsync(s->b.count, 0, sizeof(uint32_t) * s->b.ncell_pad, s->stream));
        }
        // each piece is copied in on the engine's stream and packed (and,
        // for the grid, binned: the binning clamps every coordinate into the
        // grid, so a state that fails the range check only wastes it) on
        // the side stream while the next piece is copied
        cudaStream_t ps = pipe ? s->b.aux : s->stream;
        const int pieces = pipe ? boids_sim::kXferChunks : 1;
        for (int c = 0; c < pieces; ++c) {
            const uint32_t i0 = pipe ? xfer_start(n, c) : 0, i1 = pipe ? xfer_start(n, c + 1) : n;
            if (i1 <= i0) continue;
            const size_t off = (size_t)3 * i0, bytes = sizeof(float) * 3 * (size_t)(i1 - i0);
            CK(cudaMemcpyAsync(dpos + off, pos3n + off, bytes, cudaMemcpyHostToDevice, s->stream));
            CK(cudaMemcpyAsync(dvel + off, vel3n + off, bytes, cudaMemcpyHostToDevice, s->stream));
            if (pipe) {
                CK(cudaEventRecord(s->xfer_ev[c], s->stream));
                CK(cudaStreamWaitEvent(ps, s->xfer_ev[c], 0));
            }
            CK(boidsgpu::launch_pack(dpos, dvel, s->b.pos[0], s->b.vel[0], i0, i1, check ? s->b.flag : nullptr,
                                     s->k.F_dn > s->k.Ff ? s->k.F_dn : s->k.Ff, check ? &s->k : nullptr, s->b.key,
                                     s->b.rank, s->b.count, ps, &s->launches));
        }
        if (pipe) {
            CK(cudaEventRecord(s->b.join, ps));
            CK(cudaStreamWaitEvent(s->stream, s->b.join, 0));
        }
    }
    s->has_state = false;
    s->forces_valid = false;
    s->cur = 0;
    if (check) {
        uint32_t bad = 0;
        CK(cudaMemcpyAsync(&bad, s->b.flag, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        if (bad && s->p.engine == BOIDS_ENGINE_GRID)
            return fail(BOIDS_EINVAL, "grid engine: positions must lie in [0, field_size]");
        s->engine = bad ? 0 : 1;
    }
    s->has_state = true;
    // the grid engine's one-update graph, captured now if the constants,
    // stream or kernels changed, so that the next update is not the one to
    // wait for the capture (a failed capture only turns the graphs off)
    if (s->engine == 1 && !s->prof) graph_ready(s, s->b.forces != nullptr, 1);
    return BOIDS_OK;
}

}  // namespace

int boids_set_state(boids_sim *s, const float *pos3n, const float *vel3n)
{
    if (!s) return fail(BOIDS_EINVAL, "boids_set_state: null argument");
    s->k.n = s->p.number_of_agents;  // the whole population
    return set_state_n(s, pos3n, vel3n);
}

int boids_set_population(boids_sim *s, uint32_t n, const float *pos3n, const float *vel3n)
{
    if (!s) return fail(BOIDS_EINVAL, "boids_set_population: null handle");
    if (n > s->p.number_of_agents)
        return fail(BOIDS_EINVAL, "boids_set_population: more boids than the handle was created for");
    s->has_state = false;
    s->forces_valid = false;
    s->k.n = n;
    return set_state_n(s, pos3n, vel3n);
}

int boids_init_ex(boids_sim *s, const char *init, int32_t seed, int32_t seed_mode)
{
    if (!s || !init) return fail(BOIDS_EINVAL, "boids_init: null argument");
    const uint32_t n = s->p.number_of_agents;  // the whole population, whatever boids_set_population left
    std::vector<float> pos((size_t)3 * n), vel((size_t)3 * n);
    const std::string kind(init);
    if (kind == "test" || kind == "random_uniform") {
        const bool seeded = seed_mode < 0 ? s->p.engine == BOIDS_ENGINE_GRID : seed_mode != 0;
        draw_state(s->p, kind == "test", seeded, seed, pos.data(), vel.data());
    } else {
        // raw float32 x,y,z,vx,vy,vz per boid (src/boid_simulation.cpp:113-136)
        std::ifstream f(kind, std::ios::binary);
        if (!f) return fail(BOIDS_EIO, "Invalid initial placement type or file name: " + kind);
        std::vector<float> raw((size_t)6 * n);
        f.read(reinterpret_cast<char *>(raw.data()), (std::streamsize)(sizeof(float) * raw.size()));
        if ((size_t)f.gcount() != sizeof(float) * raw.size())
            return fail(BOIDS_EIO, "initialization file holds fewer than number_of_agents boids: " + kind);
        for (uint32_t i = 0; i < n; ++i) {
            for (int c = 0; c < 3; ++c) {
                pos[(size_t)3 * i + c] = raw[(size_t)6 * i + c];
                vel[(size_t)3 * i + c] = raw[(size_t)6 * i + 3 + c];
            }
        }
    }
    int rc = boids_set_state(s, pos.data(), vel.data());
    if (rc) return rc;
    return boids_synchronize(s);  // the host vectors die here
}

int boids_init(boids_sim *s, const char *init, int32_t seed) { return boids_init_ex(s, init, seed, -1); }

namespace {

constexpr int kGraphSteps = 16;  // updates per captured graph

// One update: BoidSimulation::update of the grid or all-pairs engine.
static int step_once(boids_sim *s, bool rec)
{
    if (s->engine == 1) {
        {
            PhaseTimer pt(s, 0);
            CK(boidsgpu::launch_grid_scan(s->k, s->b, s->stream, &s->launches));
            CK(boidsgpu::launch_grid_scatter(s->k, s->b, s->cur, true, s->stream, &s->launches));
            s->acc.bin_launches += 2;
        }
        PhaseTimer pt(s, 1);
        CK(boidsgpu::launch_grid_force(s->k, s->b, 1 - s->cur, false, rec, s->stream, &s->launches));
        s->acc.force_launches += 1;
    } else {
        PhaseTimer pt(s, 1);
        CK(boidsgpu::launch_allpairs(s->k, s->b, s->cur, false, rec, s->stream, &s->launches));
        s->cur = 1 - s->cur;
        s->acc.force_launches += 2;
    }
    s->acc.steps++;
    s->steps_done++;
    return 0;
}

// Graph `which` (0: kGraphSteps updates, 1: one update) for the handle's
// current stream, buffer parity and constants, captured if needed; false
// when it cannot be had.
static bool graph_ready(boids_sim *s, bool rec, int which)
{
    if (s->graph_off || !s->stream) return false;  // the legacy stream cannot be captured
    boids_sim::StepGraph &gr = s->graphs[which];
    if (gr.exec && gr.stream == s->stream && gr.cur == s->cur && gr.engine == s->engine &&
        std::memcmp(&gr.k, &s->k, sizeof(StepConst)) == 0)
        return true;
    if (gr.exec) {
        cudaGraphExecDestroy(gr.exec);
        gr.exec = nullptr;
    }
    if (boidsgpu::grid_prepare() != cudaSuccess) {  // function attributes are set outside the capture
        cudaGetLastError();
        s->graph_off = true;
        return false;
    }
    const uint64_t launches = s->launches, done = s->steps_done;
    const boids_profile_t acc = s->acc;
    const int cur = s->cur;
    const int steps = which == 0 ? kGraphSteps : 1;
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    for (int t = 0; ok && t < steps; ++t) ok = step_once(s, rec) == 0;
    if (cudaStreamEndCapture(s->stream, &g) != cudaSuccess) ok = false;
    gr.launches = s->launches - launches;
    s->launches = launches;
    s->steps_done = done;
    s->acc = acc;
    s->cur = cur;  // nothing ran: only recorded
    if (ok && cudaGraphInstantiate(&gr.exec, g, 0) != cudaSuccess) {
        gr.exec = nullptr;
        ok = false;
    }
    if (g) cudaGraphDestroy(g);
    if (!ok) {
        cudaGetLastError();
        s->graph_off = true;
        return false;
    }
    gr.stream = s->stream;
    gr.cur = s->cur;
    gr.k = s->k;
    gr.engine = s->engine;
    return true;
}

}  // namespace

int boids_step(boids_sim *s, int32_t steps)
{
    if (!s || steps < 0) return fail(BOIDS_EINVAL, "boids_step: bad argument");
    if (!s->has_state) return fail(BOIDS_ESTATE, "boids_step: no state (call boids_init or boids_set_state)");
    int rc = use_device(s);
    if (rc) return rc;
    const bool rec = s->b.forces != nullptr;
    int32_t t = 0;
    // replays of captured graphs (not while timing phases with events): the
    // long runs' kGraphSteps updates at a time, the grid engine's other
    // updates one at a time (the all-pairs engine swaps its state buffers
    // every update, so its single updates are launched directly)
    if (!s->prof) {
        if (steps >= 2 * kGraphSteps && graph_ready(s, rec, 0)) {
            for (; steps - t >= kGraphSteps; t += kGraphSteps) {
                CK(cudaGraphLaunch(s->graphs[0].exec, s->stream));
                s->launches += s->graphs[0].launches;
                s->steps_done += kGraphSteps;
                s->acc.steps += kGraphSteps;
            }
        }
        if (t < steps && s->engine == 1 && graph_ready(s, rec, 1)) {
            for (; t < steps; ++t) {
                CK(cudaGraphLaunch(s->graphs[1].exec, s->stream));
                s->launches += s->graphs[1].launches;
                s->steps_done += 1;
                s->acc.steps += 1;
            }
        }
    }
    for (; t < steps; ++t)
        if ((rc = step_once(s, rec))) return rc;
    if (steps > 0) s->forces_valid = rec;
    return BOIDS_OK;
}

int boids_get_state(boids_sim *s, float *pos3n, float *vel3n)
{
    if (!s) return fail(BOIDS_EINVAL, "boids_get_state: null handle");
    if (!s->has_state) return fail(BOIDS_ESTATE, "boids_get_state: no state");
    int rc = use_device(s);
    if (rc) return rc;
    const uint32_t n = s->k.n;
    float *dpos = pos3n ? s->b.stage : nullptr, *dvel = vel3n ? s->b.stage + (size_t)3 * n : nullptr;
    const bool pipe = xfer_pipelined(s);
    {
        PhaseTimer t(s, 2);
        const float4 *p4 = s->b.pos[s->cur], *v4 = s->b.vel[s->cur];
        // the other state buffer is dead between updates: it holds the
        // id -> slot table
        uint32_t *slot_of = reinterpret_cast<uint32_t *>(s->b.pos[1 - s->cur]);
        CK(boidsgpu::launch_unpack_index(p4, slot_of, n, s->stream, &s->launches));
        // each piece is unpacked on the engine's stream and copied out on
        // the side stream while the next piece is unpacked
        cudaStream_t cs = pipe ? s->b.aux : s->stream;
        const int pieces = pipe ? boids_sim::kXferChunks : 1;
        for (int c = 0; c < pieces; ++c) {
            const uint32_t i0 = pipe ? xfer_start(n, c) : 0, i1 = pipe ? xfer_start(n, c + 1) : n;
            if (i1 <= i0) continue;
            const size_t off = (size_t)3 * i0, bytes = sizeof(float) * 3 * (size_t)(i1 - i0);
            CK(boidsgpu::launch_unpack_gather(p4, v4, slot_of, dpos, dvel, i0, i1, n, s->stream, &s->launches));
            if (pipe) {
                CK(cudaEventRecord(s->xfer_ev[c], s->stream));
                CK(cudaStreamWaitEvent(cs, s->xfer_ev[c], 0));
            }
            if (pos3n) CK(cudaMemcpyAsync(pos3n + off, dpos + off, bytes, cudaMemcpyDeviceToHost, cs));
            if (vel3n) CK(cudaMemcpyAsync(vel3n + off, dvel + off, bytes, cudaMemcpyDeviceToHost, cs));
        }
        if (pipe) {
            CK(cudaEventRecord(s->b.join, cs));
            CK(cudaStreamWaitEvent(s->stream, s->b.join, 0));
        }
    }
    return boids_synchronize(s);
}

int boids_get_forces(boids_sim *s, float *force9n)
{
    if (!s || !force9n) return fail(BOIDS_EINVAL, "boids_get_forces: null argument");
    if (!s->b.forces) return fail(BOIDS_ESTATE, "boids_get_forces: handle created without BOIDS_FLAG_RECORD_FORCES");
    if (!s->forces_valid) return fail(BOIDS_ESTATE, "boids_get_forces: no step since the state was set");
    int rc = use_device(s);
    if (rc) return rc;
    CK(cudaMemcpyAsync(force9n, s->b.forces, sizeof(float) * 9 * s->k.n, cudaMemcpyDeviceToHost, s->stream));
    return boids_synchronize(s);
}

int boids_set_tuning(boids_sim *s, const int32_t *t)
{
    if (!s || !t) return fail(BOIDS_EINVAL, "boids_set_tuning: null argument");
    for (int i = 0; i < 4; ++i)
        if (t[i] < 0) return fail(BOIDS_EINVAL, "boids_set_tuning: negative threshold");
    s->k.dense_min = (uint32_t)t[0];
    s->k.defer_min = (uint32_t)t[1];
    s->k.cand_defer = (uint32_t)t[2];
    s->k.lone_cand = (uint32_t)t[3];
    return BOIDS_OK;
}

int boids_get_tuning(boids_sim *s, int32_t *t)
{
    if (!s || !t) return fail(BOIDS_EINVAL, "boids_get_tuning: null argument");
    const uint32_t v[4] = {s->k.dense_min, s->k.defer_min, s->k.cand_defer, s->k.lone_cand};
    for (int i = 0; i < 4; ++i) t[i] = (int32_t)std::min<uint32_t>(v[i], 0x7fffffffu);
    return BOIDS_OK;
}

int boids_autotune(boids_sim *s, int32_t steps_per_trial)
{
    if (!s) return fail(BOIDS_EINVAL, "boids_autotune: null handle");
    if (!s->has_state) return fail(BOIDS_ESTATE, "boids_autotune: no state");
    if (s->engine != 1) return BOIDS_OK;
    int rc = use_device(s);
    if (rc) return rc;
    if (steps_per_trial <= 0) steps_per_trial = 4;
    const size_t n = s->k.n;
    float4 *sp = nullptr, *sv = nullptr;
    if ((rc = dalloc(&sp, n)) || (rc = dalloc(&sv, n))) {
        if (sp) cudaFree(sp);
        return rc;
    }
    const uint64_t steps_done = s->steps_done;
    const boids_profile_t acc = s->acc;
    const bool prof = s->prof;
    s->prof = false;
    auto restore = [&]() -> int {
        CK(cudaMemcpyAsync(s->b.pos[0], sp, sizeof(float4) * n, cudaMemcpyDeviceToDevice, s->stream));
        CK(cudaMemcpyAsync(s->b.vel[0], sv, sizeof(float4) * n, cudaMemcpyDeviceToDevice, s->stream));
        s->cur = 0;
        return grid_bin_fresh(s);
    };
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (cudaMemcpyAsync(sp, s->b.pos[s->cur], sizeof(float4) * n, cudaMemcpyDeviceToDevice, s->stream) != cudaSuccess ||
        cudaMemcpyAsync(sv, s->b.vel[s->cur], sizeof(float4) * n, cudaMemcpyDeviceToDevice, s->stream) != cudaSuccess ||
        cudaEventCreate(&t0) != cudaSuccess || cudaEventCreate(&t1) != cudaSuccess)
        rc = cuda_fail(cudaGetLastError(), "boids_autotune");
    const StepConst keep = s->k;
    float best = INFINITY;
    int best_i = -1;
    for (int c = 0; !rc && c < boidsgpu::kTuneCount; ++c) {
        s->k.dense_min = boidsgpu::kTuneCand[c][0];
        s->k.defer_min = boidsgpu::kTuneCand[c][1];
        s->k.cand_defer = boidsgpu::kTuneCand[c][2];
        s->k.lone_cand = boidsgpu::kTuneCand[c][3];
        if ((rc = restore()) || (rc = boids_step(s, 1))) break;  // one warm-up update
        float ms = 0.f;
        if (cudaEventRecord(t0, s->stream) != cudaSuccess || (rc = boids_step(s, steps_per_trial)) ||
            cudaEventRecord(t1, s->stream) != cudaSuccess || cudaEventSynchronize(t1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, t0, t1) != cudaSuccess) {
            if (!rc) rc = cuda_fail(cudaGetLastError(), "boids_autotune timing");
            break;
        }
        if (ms < best) {
            best = ms;
            best_i = c;
        }
    }
    s->k = keep;
    if (!rc && best_i >= 0) {
        s->k.dense_min = boidsgpu::kTuneCand[best_i][0];
        s->k.defer_min = boidsgpu::kTuneCand[best_i][1];
        s->k.cand_defer = boidsgpu::kTuneCand[best_i][2];
        s->k.lone_cand = boidsgpu::kTuneCand[best_i][3];
    }
    int rc2 = restore();
    if (!rc2 && cudaStreamSynchronize(s->stream) != cudaSuccess) rc2 = cuda_fail(cudaGetLastError(), "boids_autotune");
    s->steps_done = steps_done;
    s->acc = acc;
    s->prof = prof;
    s->forces_valid = false;
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    cudaFree(sp);
    cudaFree(sv);
    return rc ? rc : rc2;
}

int boids_frame_async(boids_sim *s, float *pframe, float *vframe, int32_t with_forces, int32_t slot)
{
    if (!s || !pframe || slot < 0 || slot >= BOIDS_FRAME_SLOTS)
        return fail(BOIDS_EINVAL, "boids_frame_async: bad argument");
    if (!s->has_state) return fail(BOIDS_ESTATE, "boids_frame_async: no state");
    if (with_forces && !s->b.forces)
        return fail(BOIDS_ESTATE, "boids_frame_async: forces need a handle made with BOIDS_FLAG_RECORD_FORCES");
    int rc = use_device(s);
    if (rc) return rc;
    const size_t n = s->k.n;
    if (!s->frame_dev && (rc = dalloc(&s->frame_dev, (size_t)15 * s->p.number_of_agents))) return rc;
    if (!s->frame_ev[slot]) CK(cudaEventCreateWithFlags(&s->frame_ev[slot], cudaEventDisableTiming));
    const size_t stride = with_forces ? 12 : 3;
    float *dp = s->frame_dev, *dv = s->frame_dev + 12 * n;
    {
        PhaseTimer t(s, 2);
        CK(boidsgpu::launch_frame(s->b.pos[s->cur], s->b.vel[s->cur], s->forces_valid ? s->b.forces : nullptr,
                                  dp, vframe ? dv : nullptr, with_forces ? 1 : 0, (uint32_t)n, s->stream,
                                  &s->launches));
        CK(cudaMemcpyAsync(pframe, dp, sizeof(float) * stride * n, cudaMemcpyDeviceToHost, s->stream));
        if (vframe) CK(cudaMemcpyAsync(vframe, dv, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, s->stream));
    }
    CK(cudaEventRecord(s->frame_ev[slot], s->stream));
    return BOIDS_OK;
}

int boids_frame_wait(boids_sim *s, int32_t slot)
{
    if (!s || slot < 0 || slot >= BOIDS_FRAME_SLOTS) return fail(BOIDS_EINVAL, "boids_frame_wait: bad argument");
    if (!s->frame_ev[slot]) return BOIDS_OK;  // nothing was queued on this slot
    CK(cudaEventSynchronize(s->frame_ev[slot]));
    return BOIDS_OK;
}

int boids_host_alloc(size_t bytes, void **out)
{
    if (!out) return fail(BOIDS_EINVAL, "boids_host_alloc: null argument");
    *out = nullptr;
    cudaError_t e = cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        *out = nullptr;
        cudaGetLastError();
        return fail(BOIDS_ENOMEM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    }
    return BOIDS_OK;
}

void boids_host_free(void *p)
{
    if (p) cudaFreeHost(p);
}

int boids_get_cells(boids_sim *s, int32_t *gi8)
{
    if (!s || !gi8) return fail(BOIDS_EINVAL, "boids_get_cells: null argument");
    if (!s->ref_geometry_ok) return fail(BOIDS_EINVAL, "boids_get_cells: geometry has no valid reference grid");
    if (!s->has_state) return fail(BOIDS_ESTATE, "boids_get_cells: no state");
    int rc = use_device(s);
    if (rc) return rc;
    if (!s->b.cells8 && (rc = dalloc(&s->b.cells8, (size_t)8 * s->p.number_of_agents))) return rc;
    CK(boidsgpu::launch_ref_cells(s->k, s->b.pos[s->cur], s->b.cells8, s->stream, &s->launches));
    CK(cudaMemcpyAsync(gi8, s->b.cells8, sizeof(int32_t) * 8 * s->k.n, cudaMemcpyDeviceToHost, s->stream));
    return boids_synchronize(s);
}

int boids_get_neighbor_sets(boids_sim *s, int32_t *count3n, uint64_t *hash3n)
{
    if (!s || !count3n || !hash3n) return fail(BOIDS_EINVAL, "boids_get_neighbor_sets: null argument");
    if (!s->has_state) return fail(BOIDS_ESTATE, "boids_get_neighbor_sets: no state");
    int rc = use_device(s);
    if (rc) return rc;
    const size_t n = s->k.n, cap = s->p.number_of_agents;  // sized once for the largest population
    if (!s->b.dcnt && (rc = dalloc(&s->b.dcnt, 3 * cap))) return rc;
    if (!s->b.dhash && (rc = dalloc(&s->b.dhash, 3 * cap))) return rc;
    if (s->engine == 1) {
        CK(boidsgpu::launch_grid_scan(s->k, s->b, s->stream, &s->launches));
        CK(boidsgpu::launch_grid_scatter(s->k, s->b, s->cur, false, s->stream, &s->launches));
        CK(boidsgpu::launch_grid_force(s->k, s->b, 1 - s->cur, true, false, s->stream, &s->launches));
    } else {
        CK(boidsgpu::launch_allpairs(s->k, s->b, s->cur, true, false, s->stream, &s->launches));
    }
    CK(cudaMemcpyAsync(count3n, s->b.dcnt, sizeof(int32_t) * 3 * n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(hash3n, s->b.dhash, sizeof(uint64_t) * 3 * n, cudaMemcpyDeviceToHost, s->stream));
    return boids_synchronize(s);
}

int boids_get_grid_info(boids_sim *s, boids_grid_info *info)
{
    if (!s || !info) return fail(BOIDS_EINVAL, "boids_get_grid_info: null argument");
    info->ref_interaction_range = s->k.refR;
    info->ref_grid_num = s->ref_geometry_ok ? s->k.refG : 0;
    info->ref_grid_size = s->k.refGS;
    info->dev_cells_per_axis = s->k.G;
    info->dev_cell_size = s->k.G ? (float)(s->p.field_size / s->k.G) : 0.f;
    info->list_capacity = s->engine == 1 ? boidsgpu::kListCap : boidsgpu::kApCap;
    return BOIDS_OK;
}

int boids_set_stream(boids_sim *s, void *stream)
{
    if (!s) return fail(BOIDS_EINVAL, "boids_set_stream: null handle");
    int rc = use_device(s);
    if (rc) return rc;
    // order the switch: work queued on the old stream completes first
    CK(cudaStreamSynchronize(s->stream));
    s->stream = stream ? static_cast<cudaStream_t>(stream) : s->own_stream;
    return BOIDS_OK;
}

int boids_synchronize(boids_sim *s)
{
    if (!s) return fail(BOIDS_EINVAL, "boids_synchronize: null handle");
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaGetLastError());
    return BOIDS_OK;
}

int boids_profile_enable(boids_sim *s, int32_t on)
{
    if (!s) return fail(BOIDS_EINVAL, "boids_profile_enable: null handle");
    s->prof = on != 0;
    return BOIDS_OK;
}

int boids_profile_read(boids_sim *s, boids_profile_t *out, int32_t reset)
{
    if (!s || !out) return fail(BOIDS_EINVAL, "boids_profile_read: null argument");
    int rc = use_device(s);
    if (rc) return rc;
    resolve_events(s);
    *out = s->acc;
    if (reset) s->acc = boids_profile_t{};
    return BOIDS_OK;
}

uint64_t boids_kernel_launches(boids_sim *s) { return s ? s->launches : 0; }

}  // extern "C"

// ------------------------------------------------------------------ support for boids_step_noalloc

namespace boidsgpu {

// Records an error message for boids_last_error() on behalf of
// boids_noalloc.cu.
int set_last_error(int code, const char *msg) { return fail(code, msg); }

// The step constants boids_create derives for a grid-engine handle, for the
// allocation-free entry point, which has no handle.  Uses no heap memory on
// success.
int flock_constants(const boids_params *params, StepConst *out, const char *who)
{
    const boids_params &p = *params;
    if (p.engine != BOIDS_ENGINE_GRID) return fail(BOIDS_EINVAL, std::string(who) + ": grid engine only");
    StepConst k{};
    bool ref_ok = false;
    if (int rc = make_constants(p, k, &ref_ok)) return rc;
    if (k.G == 0) return fail(BOIDS_EINVAL, std::string(who) + ": field too small for device cells (fewer than 3 "
                                                          "per axis); use a boids_create handle");
    *out = k;
    return BOIDS_OK;
}

void draw_initial_state(const boids_params *p, int test, int32_t seed, float *pos, float *vel)
{
    draw_state(*p, test != 0, true, seed, pos, vel);
}

int grid_constants_noalloc(const boids_params *params, StepConst *out)
{
    const boids_params &p = *params;
    if (p.engine != BOIDS_ENGINE_GRID) return fail(BOIDS_EINVAL, "boids_step_noalloc runs the grid engine only");
    StepConst k{};
    bool ref_ok = false;
    if (int rc = make_constants(p, k, &ref_ok)) return rc;
    if (k.G == 0) return fail(BOIDS_EINVAL, "field too small for device cells: use the handle API");
    *out = k;
    return BOIDS_OK;
}

}  // namespace boidsgpu
