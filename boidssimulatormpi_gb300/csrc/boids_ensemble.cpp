// boids_ensemble.cpp -- batched ensembles (boids_ensemble_* of include/boids.h).
//
// Many independent grid-engine flocks share one set of device buffers and
// are stepped by the same kernels as a single flock, launched once per step
// for all flocks together:
//   * cells: flock f owns global cells [cell_base_f, cell_base_f + Gx*G*G),
//     one counting sort (keys, one scan, scatter) bins every flock at once;
//   * slots: flock f owns slots [slot_base_f, slot_base_f + n_f), slot_base_f
//     a multiple of kSlotAlign, so a CTA of the rule kernels serves a single
//     flock and keeps that flock's constants in shared memory;
//   * a step is captured once into a CUDA graph and replayed.
// Boid ids are local to a flock, so each flock's arithmetic -- and result --
// is exactly that of a boids_create handle with the same parameters.
#include "boids.h"
#include "boids_engine.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

using boidsgpu::DevBuffers;
using boidsgpu::FlockTable;
using boidsgpu::StepConst;

namespace boidsgpu {
int set_last_error(int code, const char *msg);
int flock_constants(const boids_params *params, StepConst *out, const char *who);
void draw_initial_state(const boids_params *p, int test, int32_t seed, float *pos, float *vel);
}  // namespace boidsgpu

namespace {

int fail(int code, const std::string &msg) { return boidsgpu::set_last_error(code, msg.c_str()); }

int cuda_fail(cudaError_t e, const char *where)
{
    return fail(BOIDS_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

constexpr int kGraphSteps = 16;  // steps per captured graph

}  // namespace

struct boids_ensemble {
    std::vector<boids_flock_desc> desc;
    std::vector<StepConst> ks;       // host copy of the flock table
    std::vector<uint16_t> blk_flock;
    std::vector<uint32_t> cell4;
    int device = 0;
    uint32_t nslots = 0, ncell = 0, total_boids = 0;
    DevBuffers b{};
    StepConst *d_ks = nullptr;
    uint16_t *d_blk = nullptr;
    uint32_t *d_cell4 = nullptr;
    float *d_link = nullptr;
    double *d_acc = nullptr, *d_com = nullptr;
    uint32_t *d_largest = nullptr, *d_err = nullptr;
    FlockTable ft{};
    cudaStream_t stream = nullptr;
    int cur = 0;           // buffer holding the state
    bool binned = false;   // b.pos[cur] is freshly binned (the next step skips the counting sort)
    bool keys_stale = false;  // set_state changed b.pos[cur]: recompute every key before the next scan
    bool has_state = false;
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_launches = 0;  // kernel launches per replay
    uint64_t launches = 0;
    uint32_t tune[4] = {boidsgpu::kDenseMin, boidsgpu::kDeferMin, boidsgpu::kCandDefer, boidsgpu::kLoneCand};
};

namespace {

void release(boids_ensemble *e)
{
    if (e->graph) cudaGraphExecDestroy(e->graph);
    DevBuffers &b = e->b;
    if (e->stream) cudaStreamSynchronize(e->stream);
    void *ptrs[] = {b.pos[0], b.pos[1], b.vel[0], b.vel[1], b.key, b.rank, b.count, b.lstart, b.bsum, b.ticket,
                    b.dense_list, b.dense_n, b.dflag, b.carry, b.defer, b.defer_cnt, b.wscratch, e->d_ks, e->d_blk,
                    e->d_cell4,
                    e->d_link, e->d_acc, e->d_com, e->d_largest, e->d_err};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (b.aux) cudaStreamDestroy(b.aux);
    for (cudaEvent_t ev : {b.fork, b.join, b.cjoin})
        if (ev) cudaEventDestroy(ev);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

template <class T>
int dalloc(T **p, size_t count)
{
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * count);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(BOIDS_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    return 0;
}

int use_device(boids_ensemble *e)
{
    cudaError_t r = cudaSetDevice(e->device);
    return r == cudaSuccess ? 0 : cuda_fail(r, "cudaSetDevice");
}

// Counts to zero, then keys and ranks of every boid from its position.
int bin_fresh(boids_ensemble *e)
{
    CK(cudaMemsetAsync(e->b.count, 0, sizeof(uint32_t) * e->b.ncell_pad, e->stream));
    CK(boidsgpu::launch_grid_keys(e->ks[0], e->b.pos[e->cur], e->b.key, e->b.rank, e->b.count, e->stream,
                                  &e->launches, &e->ft));
    e->binned = false;
    e->keys_stale = false;
    return 0;
}

// Keys for the whole ensemble once after any number of set_state calls.
int ensure_keys(boids_ensemble *e) { return e->keys_stale ? bin_fresh(e) : 0; }

// One update of every flock, the launches of boids_step's grid engine.
int step_once(boids_ensemble *e)
{
    if (!e->binned) {
        CK(boidsgpu::launch_grid_scan(e->ks[0], e->b, e->stream, &e->launches, &e->ft));
        CK(boidsgpu::launch_grid_scatter(e->ks[0], e->b, e->cur, true, e->stream, &e->launches, &e->ft));
        e->cur = 1 - e->cur;
    }
    CK(boidsgpu::launch_grid_force(e->ks[0], e->b, e->cur, false, false, e->stream, &e->launches, &e->ft));
    e->cur = 1 - e->cur;
    e->binned = false;
    return 0;
}

// Binning only (the first half of a step), for the statistics.
int bin_now(boids_ensemble *e)
{
    if (e->binned) return 0;
    CK(boidsgpu::launch_grid_scan(e->ks[0], e->b, e->stream, &e->launches, &e->ft));
    CK(boidsgpu::launch_grid_scatter(e->ks[0], e->b, e->cur, true, e->stream, &e->launches, &e->ft));
    e->cur = 1 - e->cur;
    e->binned = true;
    return 0;
}

// Put the state back into buffer 0, where the captured graph expects it.
int normalize(boids_ensemble *e)
{
    if (e->binned || e->cur == 0) return 0;
    const size_t bytes = sizeof(float4) * e->nslots;
    CK(cudaMemcpyAsync(e->b.pos[0], e->b.pos[1], bytes, cudaMemcpyDeviceToDevice, e->stream));
    CK(cudaMemcpyAsync(e->b.vel[0], e->b.vel[1], bytes, cudaMemcpyDeviceToDevice, e->stream));
    e->cur = 0;
    return bin_fresh(e);
}

int capture_graph(boids_ensemble *e)
{
    if (e->graph) return 0;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    const uint64_t before = e->launches;
    for (int t = 0; t < kGraphSteps && !rc; ++t) rc = step_once(e);
    cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
    e->graph_launches = e->launches - before;
    e->launches = before;  // counted when replayed
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&e->graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
        e->graph = nullptr;
        return cuda_fail(ce, "cudaGraphInstantiate");
    }
    return 0;
}

int upload_table(boids_ensemble *e)
{
    for (auto &k : e->ks) {
        k.dense_min = e->tune[0];
        k.defer_min = e->tune[1];
        k.cand_defer = e->tune[2];
        k.lone_cand = e->tune[3];
    }
    CK(cudaMemcpyAsync(e->d_ks, e->ks.data(), sizeof(StepConst) * e->ks.size(), cudaMemcpyHostToDevice, e->stream));
    if (e->graph) {  // re-captured on the next step
        cudaGraphExecDestroy(e->graph);
        e->graph = nullptr;
    }
    return 0;
}

}  // namespace

extern "C" {

int boids_ensemble_create(const boids_flock_desc *flocks, uint32_t count, boids_ensemble **out)
{
    if (!flocks || !out || count == 0) return fail(BOIDS_EINVAL, "boids_ensemble_create: bad argument");
    if (count > 65535) return fail(BOIDS_EINVAL, "boids_ensemble_create: at most 65535 flocks");
    *out = nullptr;
    boids_ensemble *e = new boids_ensemble();
    e->desc.assign(flocks, flocks + count);
    e->device = flocks[0].params.device;
    uint64_t slot = 0, cell = 0, boids = 0;
    for (uint32_t f = 0; f < count; ++f) {
        StepConst k{};
        const boids_flock_desc &d = flocks[f];
        if (d.init_kind != BOIDS_INIT_RANDOM_UNIFORM && d.init_kind != BOIDS_INIT_TEST) {
            delete e;
            return fail(BOIDS_EINVAL, "boids_ensemble_create: unknown init_kind");
        }
        if (int rc = boidsgpu::flock_constants(&d.params, &k, "boids_ensemble_create")) {
            delete e;
            return rc;
        }
        k.flock = f;
        k.cell_base = (uint32_t)cell;
        k.slot_base = (uint32_t)slot;
        k.slot_off = (uint32_t)(slot - boids);
        e->ks.push_back(k);
        e->cell4.push_back((uint32_t)(cell / 4));
        const uint64_t span = ((uint64_t)k.n + boidsgpu::kSlotAlign - 1) / boidsgpu::kSlotAlign * boidsgpu::kSlotAlign;
        for (uint64_t q = 0; q < span / boidsgpu::kSlotAlign; ++q) e->blk_flock.push_back((uint16_t)f);
        slot += span;
        cell += (uint64_t)k.Gx * k.G * k.G;  // a multiple of 4
        boids += k.n;
        if (slot >= boidsgpu::kMaxBoids || cell >= (1ull << 31)) {
            delete e;
            return fail(BOIDS_EINVAL, "boids_ensemble_create: ensemble too large (slots or cells)");
        }
    }
    e->nslots = (uint32_t)slot;
    e->ncell = (uint32_t)cell;
    e->total_boids = (uint32_t)boids;
    int rc = use_device(e);
    if (rc) {
        delete e;
        return rc;
    }
    DevBuffers &b = e->b;
    b.ncell = e->ncell;
    b.ncell_pad = (b.ncell + 1 + boidsgpu::kScanTile - 1) / boidsgpu::kScanTile * boidsgpu::kScanTile;
    b.nscan_blocks = b.ncell_pad / boidsgpu::kScanTile;
    const size_t ns = std::max<size_t>(e->nslots, 1);
#define ALLOC(...)                    \
    if ((rc = dalloc(__VA_ARGS__))) { \
        release(e);                   \
        return rc;                    \
    }
    ALLOC(&b.pos[0], ns);
    ALLOC(&b.pos[1], ns);
    ALLOC(&b.vel[0], ns);
    ALLOC(&b.vel[1], ns);
    ALLOC(&b.key, ns);
    ALLOC(&b.rank, ns);
    ALLOC(&b.count, b.ncell_pad);
    ALLOC(&b.lstart, b.ncell_pad);
    ALLOC(&b.bsum, b.nscan_blocks);
    ALLOC(&b.ticket, 1);
    ALLOC(&b.dense_list, boidsgpu::dense_list_capacity(b.ncell, e->total_boids));
    ALLOC(&b.dense_n, 3);
    ALLOC(&b.dflag, b.ncell / 4);
    {
        unsigned char *carry = nullptr;
        ALLOC(&carry, (size_t)boidsgpu::kCarryBytes * ns);
        b.carry = carry;
    }
    // No deferral queue and no side stream (b.defer, b.aux stay null): with
    // them the gathered ensemble's step was 3 % faster, but the whole
    // 2000-step sweep 4 % slower (49.1 against 47.3 s), the second kernel's
    // one CTA per slot block and the stream joins costing more over the
    // sweep's lighter steps than they save in its heaviest.
    ALLOC(&e->d_ks, count);
    ALLOC(&e->d_blk, e->blk_flock.size());
    ALLOC(&e->d_cell4, count);
    ALLOC(&e->d_link, count);
    ALLOC(&e->d_acc, (size_t)boidsgpu::kStatAcc * count);
    ALLOC(&e->d_com, 3 * (size_t)count);
    ALLOC(&e->d_largest, count);
    ALLOC(&e->d_err, 1);
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, e->device);
    b.dense_grid = (uint32_t)std::max(1, nsm) * boidsgpu::kDenseCtasPerSm;
    {
        uint32_t nmax = 1;
        for (const auto &k : e->ks) nmax = std::max(nmax, k.n);
        b.wcap = std::min(boidsgpu::kWinScratch, nmax);
        ALLOC(&b.wscratch, (size_t)b.wcap * b.dense_grid);
    }
#undef ALLOC
    cudaError_t ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
        e->stream = nullptr;
        release(e);
        return cuda_fail(ce, "cudaStreamCreate");
    }
    std::vector<float> link(count);
    for (uint32_t f = 0; f < count; ++f) link[f] = (float)flocks[f].params.cohesion_sight_distance;
    auto ck = [&](cudaError_t x, const char *w) { return x == cudaSuccess ? 0 : cuda_fail(x, w); };
    if ((rc = ck(cudaMemsetAsync(b.ticket, 0, 4, e->stream), "cudaMemsetAsync")) ||
        (rc = ck(cudaMemsetAsync(b.dense_n, 0, 12, e->stream), "cudaMemsetAsync")) ||
        (rc = ck(cudaMemcpyAsync(e->d_blk, e->blk_flock.data(), 2 * e->blk_flock.size(), cudaMemcpyHostToDevice,
                                 e->stream), "cudaMemcpyAsync")) ||
        (rc = ck(cudaMemcpyAsync(e->d_cell4, e->cell4.data(), 4 * (size_t)count, cudaMemcpyHostToDevice, e->stream),
                 "cudaMemcpyAsync")) ||
        (rc = ck(cudaMemcpyAsync(e->d_link, link.data(), 4 * (size_t)count, cudaMemcpyHostToDevice, e->stream),
                 "cudaMemcpyAsync")) ||
        (rc = upload_table(e)) || (rc = ck(boidsgpu::grid_prepare(), "grid_prepare")) ||
        (rc = ck(cudaStreamSynchronize(e->stream), "cudaStreamSynchronize"))) {
        release(e);
        return rc;
    }
    e->ft = FlockTable{e->d_ks, e->d_blk, e->d_cell4, count, e->nslots};
    *out = e;
    return BOIDS_OK;
}

void boids_ensemble_destroy(boids_ensemble *e)
{
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    release(e);
}

int boids_ensemble_init(boids_ensemble *e)
{
    if (!e) return fail(BOIDS_EINVAL, "boids_ensemble_init: null handle");
    int rc = use_device(e);
    if (rc) return rc;
    std::vector<float4> hp(e->nslots, make_float4(0.f, 0.f, 0.f, 0.f)), hv(e->nslots, make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<float> pos, vel;
    for (size_t f = 0; f < e->desc.size(); ++f) {
        const boids_flock_desc &d = e->desc[f];
        const uint32_t n = e->ks[f].n;
        pos.assign((size_t)3 * n, 0.f);
        vel.assign((size_t)3 * n, 0.f);
        boidsgpu::draw_initial_state(&d.params, d.init_kind == BOIDS_INIT_TEST, d.rand_seed, pos.data(), vel.data());
        const uint32_t base = e->ks[f].slot_base;
        for (uint32_t i = 0; i < n; ++i) {
            float w;
            std::memcpy(&w, &i, 4);
            hp[base + i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], w);
            hv[base + i] = make_float4(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2], 0.f);
        }
    }
    CK(cudaMemcpyAsync(e->b.pos[0], hp.data(), sizeof(float4) * e->nslots, cudaMemcpyHostToDevice, e->stream));
    CK(cudaMemcpyAsync(e->b.vel[0], hv.data(), sizeof(float4) * e->nslots, cudaMemcpyHostToDevice, e->stream));
    e->cur = 0;
    if ((rc = bin_fresh(e))) return rc;
    e->has_state = true;
    CK(cudaStreamSynchronize(e->stream));  // the host vectors die here
    return BOIDS_OK;
}

int boids_ensemble_set_state(boids_ensemble *e, uint32_t flock, const float *pos3n, const float *vel3n)
{
    if (!e || flock >= e->ks.size() || (!pos3n || !vel3n))
        return fail(BOIDS_EINVAL, "boids_ensemble_set_state: bad argument");
    if (!e->has_state) return fail(BOIDS_ESTATE, "boids_ensemble_set_state: call boids_ensemble_init first");
    const StepConst &k = e->ks[flock];
    const float hi = std::max(k.F_dn, k.Ff);
    std::vector<float4> hp(k.n), hv(k.n);
    for (uint32_t i = 0; i < k.n; ++i) {
        const float x = pos3n[3 * i], y = pos3n[3 * i + 1], z = pos3n[3 * i + 2];
        if (!(x >= 0.f && x <= hi && y >= 0.f && y <= hi && z >= 0.f && z <= hi))
            return fail(BOIDS_EINVAL, "grid engine: positions must lie in [0, field_size]");
        float w;
        std::memcpy(&w, &i, 4);
        hp[i] = make_float4(x, y, z, w);
        hv[i] = make_float4(vel3n[3 * i], vel3n[3 * i + 1], vel3n[3 * i + 2], 0.f);
    }
    int rc = use_device(e);
    if (rc) return rc;
    CK(cudaMemcpyAsync(e->b.pos[e->cur] + k.slot_base, hp.data(), sizeof(float4) * k.n, cudaMemcpyHostToDevice,
                       e->stream));
    CK(cudaMemcpyAsync(e->b.vel[e->cur] + k.slot_base, hv.data(), sizeof(float4) * k.n, cudaMemcpyHostToDevice,
                       e->stream));
    e->binned = false;
    if ((rc = normalize(e))) return rc;
    e->keys_stale = true;  // binned once, at the next step or statistics pass
    CK(cudaStreamSynchronize(e->stream));
    return BOIDS_OK;
}

int boids_ensemble_step(boids_ensemble *e, int32_t steps)
{
    if (!e || steps < 0) return fail(BOIDS_EINVAL, "boids_ensemble_step: bad argument");
    if (!e->has_state) return fail(BOIDS_ESTATE, "boids_ensemble_step: call boids_ensemble_init first");
    int rc = use_device(e);
    if (rc) return rc;
    int t = 0;
    if (steps > 0 && e->binned) {  // finish the step the statistics started
        if ((rc = step_once(e))) return rc;
        ++t;
    }
    if ((rc = normalize(e)) || (rc = ensure_keys(e))) return rc;
    if (steps - t >= kGraphSteps) {
        if ((rc = capture_graph(e))) return rc;
        for (; steps - t >= kGraphSteps; t += kGraphSteps) {
            CK(cudaGraphLaunch(e->graph, e->stream));
            e->launches += e->graph_launches;
        }
    }
    for (; t < steps; ++t)
        if ((rc = step_once(e))) return rc;
    return BOIDS_OK;
}

int boids_ensemble_get_state(boids_ensemble *e, uint32_t flock, float *pos3n, float *vel3n)
{
    if (!e || flock >= e->ks.size()) return fail(BOIDS_EINVAL, "boids_ensemble_get_state: bad argument");
    if (!e->has_state) return fail(BOIDS_ESTATE, "boids_ensemble_get_state: no state");
    int rc = use_device(e);
    if (rc) return rc;
    const StepConst &k = e->ks[flock];
    std::vector<float4> hp(k.n), hv(k.n);
    CK(cudaMemcpyAsync(hp.data(), e->b.pos[e->cur] + k.slot_base, sizeof(float4) * k.n, cudaMemcpyDeviceToHost,
                       e->stream));
    CK(cudaMemcpyAsync(hv.data(), e->b.vel[e->cur] + k.slot_base, sizeof(float4) * k.n, cudaMemcpyDeviceToHost,
                       e->stream));
    CK(cudaStreamSynchronize(e->stream));
    for (uint32_t s = 0; s < k.n; ++s) {
        uint32_t id;
        std::memcpy(&id, &hp[s].w, 4);
        if (id >= k.n) return fail(BOIDS_ECUDA, "boids_ensemble_get_state: corrupt state slot");
        if (pos3n) { pos3n[3 * id] = hp[s].x; pos3n[3 * id + 1] = hp[s].y; pos3n[3 * id + 2] = hp[s].z; }
        if (vel3n) { vel3n[3 * id] = hv[s].x; vel3n[3 * id + 1] = hv[s].y; vel3n[3 * id + 2] = hv[s].z; }
    }
    return BOIDS_OK;
}

int boids_ensemble_stats(boids_ensemble *e, double *out)
{
    if (!e || !out) return fail(BOIDS_EINVAL, "boids_ensemble_stats: bad argument");
    if (!e->has_state) return fail(BOIDS_ESTATE, "boids_ensemble_stats: no state");
    int rc = use_device(e);
    if (rc) return rc;
    if ((rc = ensure_keys(e)) || (rc = bin_now(e))) return rc;
    CK(boidsgpu::launch_ensemble_stats(e->b, e->cur, e->ft, e->d_link, e->d_acc, e->d_com, e->d_largest, e->d_err,
                                       e->stream, &e->launches));
    const size_t nf = e->ks.size();
    std::vector<double> acc((size_t)boidsgpu::kStatAcc * nf), com(3 * nf);
    std::vector<uint32_t> largest(nf);
    uint32_t err = 0;
    CK(cudaMemcpyAsync(acc.data(), e->d_acc, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaMemcpyAsync(com.data(), e->d_com, sizeof(double) * com.size(), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaMemcpyAsync(largest.data(), e->d_largest, 4 * nf, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaMemcpyAsync(&err, e->d_err, 4, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    if (err) return fail(BOIDS_ECUDA, "boids_ensemble_stats: union-find walk exceeded its bound");
    for (size_t f = 0; f < nf; ++f) {
        const double *a = &acc[(size_t)boidsgpu::kStatAcc * f];
        const double n = e->ks[f].n ? (double)e->ks[f].n : 1.0;
        double *o = out + (size_t)BOIDS_STATS_PER_FLOCK * f;
        o[BOIDS_STAT_POLARIZATION] = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]) / n;
        o[BOIDS_STAT_MILLING] = std::sqrt(a[12] * a[12] + a[13] * a[13] + a[14] * a[14]) / n;
        o[BOIDS_STAT_NN_DISTANCE] = a[15] / n;
        o[BOIDS_STAT_LARGEST_CLUSTER] = largest[f] / n;
        for (int d = 0; d < 3; ++d) {
            o[BOIDS_STAT_COM_X + d] = com[3 * f + d];
            o[BOIDS_STAT_MOMENTUM_X + d] = a[3 + d] / n;
        }
        o[BOIDS_STAT_SEARCH_RADIUS] = e->ks[f].side;
    }
    return BOIDS_OK;
}

int boids_ensemble_autotune(boids_ensemble *e, int32_t steps_per_trial)
{
    if (!e) return fail(BOIDS_EINVAL, "boids_ensemble_autotune: null handle");
    if (!e->has_state) return fail(BOIDS_ESTATE, "boids_ensemble_autotune: no state");
    int rc = use_device(e);
    if (rc) return rc;
    if (steps_per_trial <= 0) steps_per_trial = 4;
    if ((rc = normalize(e))) return rc;
    if (e->binned) {  // keep the unbinned state in buffer 0
        if ((rc = step_once(e)) || (rc = normalize(e))) return rc;
    }
    const size_t bytes = sizeof(float4) * e->nslots;
    float4 *sp = nullptr, *sv = nullptr;
    if ((rc = dalloc(&sp, e->nslots)) || (rc = dalloc(&sv, e->nslots))) {
        if (sp) cudaFree(sp);
        return rc;
    }
    auto restore = [&]() -> int {
        CK(cudaMemcpyAsync(e->b.pos[0], sp, bytes, cudaMemcpyDeviceToDevice, e->stream));
        CK(cudaMemcpyAsync(e->b.vel[0], sv, bytes, cudaMemcpyDeviceToDevice, e->stream));
        e->cur = 0;
        return bin_fresh(e);
    };
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    float best = INFINITY;
    int best_i = 0;
    rc = 0;
    if (cudaMemcpyAsync(sp, e->b.pos[0], bytes, cudaMemcpyDeviceToDevice, e->stream) != cudaSuccess ||
        cudaMemcpyAsync(sv, e->b.vel[0], bytes, cudaMemcpyDeviceToDevice, e->stream) != cudaSuccess ||
        cudaEventCreate(&t0) != cudaSuccess || cudaEventCreate(&t1) != cudaSuccess)
        rc = cuda_fail(cudaGetLastError(), "boids_ensemble_autotune");
    uint32_t keep[4];
    std::memcpy(keep, e->tune, sizeof keep);
    for (int c = 0; !rc && c < boidsgpu::kTuneCount; ++c) {
        std::memcpy(e->tune, boidsgpu::kTuneCand[c], sizeof e->tune);
        if ((rc = upload_table(e)) || (rc = restore()) || (rc = step_once(e))) break;  // one warm-up step
        if (cudaEventRecord(t0, e->stream) != cudaSuccess) { rc = cuda_fail(cudaGetLastError(), "cudaEventRecord"); break; }
        for (int t = 0; t < steps_per_trial && !rc; ++t) rc = step_once(e);
        if (rc) break;
        float ms = 0.f;
        if (cudaEventRecord(t1, e->stream) != cudaSuccess || cudaEventSynchronize(t1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, t0, t1) != cudaSuccess) {
            rc = cuda_fail(cudaGetLastError(), "autotune timing");
            break;
        }
        if (ms < best) {
            best = ms;
            best_i = (int)c;
        }
    }
    if (!rc) std::memcpy(e->tune, boidsgpu::kTuneCand[best_i], sizeof e->tune);
    else std::memcpy(e->tune, keep, sizeof e->tune);
    int rc2 = upload_table(e);
    if (!rc2) rc2 = restore();
    if (!rc2 && cudaStreamSynchronize(e->stream) != cudaSuccess) rc2 = cuda_fail(cudaGetLastError(), "autotune");
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    cudaFree(sp);
    cudaFree(sv);
    return rc ? rc : rc2;
}

int boids_ensemble_tuning(boids_ensemble *e, int32_t *out4)
{
    if (!e || !out4) return fail(BOIDS_EINVAL, "boids_ensemble_tuning: bad argument");
    for (int i = 0; i < 4; ++i) out4[i] = (int32_t)std::min<uint32_t>(e->tune[i], 0x7fffffffu);
    return BOIDS_OK;
}

int boids_ensemble_set_tuning(boids_ensemble *e, const int32_t *t)
{
    if (!e || !t) return fail(BOIDS_EINVAL, "boids_ensemble_set_tuning: null argument");
    for (int i = 0; i < 4; ++i)
        if (t[i] < 0) return fail(BOIDS_EINVAL, "boids_ensemble_set_tuning: negative threshold");
    int rc = use_device(e);
    if (rc) return rc;
    for (int i = 0; i < 4; ++i) e->tune[i] = (uint32_t)t[i];
    return upload_table(e);
}

int boids_ensemble_synchronize(boids_ensemble *e)
{
    if (!e) return fail(BOIDS_EINVAL, "boids_ensemble_synchronize: null handle");
    int rc = use_device(e);
    if (rc) return rc;
    CK(cudaStreamSynchronize(e->stream));
    return BOIDS_OK;
}

uint64_t boids_ensemble_kernel_launches(boids_ensemble *e) { return e ? e->launches : 0; }

}  // extern "C"
