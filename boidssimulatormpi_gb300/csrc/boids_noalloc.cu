// boids_noalloc.cu -- boids_step_noalloc: one grid-engine update that
// allocates no memory.
//
// Some callers cannot let a library allocate device memory: code embedded in
// a host application that owns every byte of the GPU through its own pool or
// a fixed memory budget, and latency-critical loops that must not run into
// cudaMalloc/cudaFree, which can synchronize the whole device.  For them this
// entry point keeps all of its scratch (the cell-sorted copy of the state,
// cell keys and ranks, the per-cell counts and prefix sums, the dense-cell
// work list) in one statically sized device array that the CUDA driver
// reserves when the library is loaded.  The caller passes the input state and
// the output buffers, both in device memory.
//
// Costs and limits of that choice:
//  * the array holds BOIDS_NOALLOC_SCRATCH_BYTES (32 MiB) on every GPU that
//    loads the library, used or not, until the process exits;
//  * a step that needs more scratch than that is refused with BOIDS_EINVAL
//    (about 370 000 boids at the reference's density);
//  * all calls share the one array: two calls whose GPU work overlaps in time
//    (different streams, or different host threads on one device) race and
//    corrupt each other's results; order them on one stream;
//  * the first call on a device loads the library's device code there (lazy
//    module loading), so make it before any stream capture.
// Each call looks the array's address up in the current context, keeps the
// step constants of the last few parameter sets in fixed host storage, and
// leaves the caller's current device as it found it.
#include "boids.h"
#include "boids_engine.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

namespace boidsgpu {
int set_last_error(int code, const char *msg);
int grid_constants_noalloc(const boids_params *params, StepConst *out);
}  // namespace boidsgpu

// The scratch.  In host code this name only stands for the symbol; its device
// address comes from cudaGetSymbolAddress with the device current.
static __device__ __align__(256) unsigned char g_noalloc_scratch[BOIDS_NOALLOC_SCRATCH_BYTES];

namespace {

// Device address of the scratch in the current device's context, looked up
// on every call: a host-side lookup of microseconds, and never stale (a
// cached address would outlive a cudaDeviceReset, after which the module is
// loaded again into a new context).
int scratch_address(unsigned char **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "boids_step_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        return boidsgpu::set_last_error(BOIDS_ECUDA, msg);
    }
    *out = static_cast<unsigned char *>(p);
    return BOIDS_OK;
}

// The step constants of the last few parameter sets.  Deriving them runs a
// bisection with the host's acosf and a monotonicity check around it (about
// 0.2 ms); a loop that steps the same flock call after call finds them here.
// Fixed storage, no allocation; the fields are compared one by one, so
// padding bytes never matter.
constexpr int kConstCache = 4;
struct ConstEntry {
    bool used;
    boids_params p;
    boidsgpu::StepConst k;
};
std::mutex g_const_mutex;
ConstEntry g_const_cache[kConstCache];
int g_const_next;

bool same_params(const boids_params &a, const boids_params &b)
{
    return a.number_of_agents == b.number_of_agents && a.field_size == b.field_size &&
           a.separation_sight_distance == b.separation_sight_distance &&
           a.separation_sight_angle == b.separation_sight_angle &&
           a.separation_force_coefficient == b.separation_force_coefficient &&
           a.alignment_sight_distance == b.alignment_sight_distance &&
           a.alignment_sight_angle == b.alignment_sight_angle &&
           a.alignment_force_coefficient == b.alignment_force_coefficient &&
           a.cohesion_sight_distance == b.cohesion_sight_distance &&
           a.cohesion_sight_angle == b.cohesion_sight_angle &&
           a.cohesion_force_coefficient == b.cohesion_force_coefficient && a.velocity_max == b.velocity_max &&
           a.velocity_min == b.velocity_min && a.engine == b.engine && a.flags == b.flags;
}

int step_constants(const boids_params *params, boidsgpu::StepConst *out)
{
    {
        std::lock_guard<std::mutex> lock(g_const_mutex);
        for (const ConstEntry &e : g_const_cache) {
            if (e.used && same_params(e.p, *params)) {
                *out = e.k;
                return BOIDS_OK;
            }
        }
    }
    boidsgpu::StepConst k;
    const int rc = boidsgpu::grid_constants_noalloc(params, &k);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(g_const_mutex);
    ConstEntry &e = g_const_cache[g_const_next];
    g_const_next = (g_const_next + 1) % kConstCache;
    e.used = true;
    e.p = *params;
    e.k = k;
    *out = k;
    return BOIDS_OK;
}

// Makes `dev` current for the life of the object and gives the caller's
// current device back at the end.
struct DeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(int dev)
    {
        if ((err = cudaGetDevice(&prev)) != cudaSuccess) {
            prev = -1;
            return;
        }
        if (prev != dev) err = cudaSetDevice(dev);
    }
    ~DeviceScope()
    {
        int now = -1;
        if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
    }
};

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

// Carves the scratch into the engine's buffers; returns the bytes used.
size_t layout(const boidsgpu::StepConst &k, unsigned char *base, boidsgpu::DevBuffers *b)
{
    const size_t n = k.n ? k.n : 1;
    b->ncell = (uint32_t)k.Gx * k.G * k.G;
    b->ncell_pad = (b->ncell + 1 + boidsgpu::kScanTile - 1) / boidsgpu::kScanTile * boidsgpu::kScanTile;
    b->nscan_blocks = b->ncell_pad / boidsgpu::kScanTile;
    const size_t ndense = boidsgpu::dense_list_capacity(b->ncell, n);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base ? base + off : nullptr;
        off += up256(bytes);
        return p;
    };
    for (int i = 0; i < 2; ++i) {
        b->pos[i] = reinterpret_cast<float4 *>(take(16 * n));
        b->vel[i] = reinterpret_cast<float4 *>(take(16 * n));
    }
    b->key = reinterpret_cast<uint32_t *>(take(4 * n));
    b->rank = reinterpret_cast<uint32_t *>(take(4 * n));
    b->count = reinterpret_cast<uint32_t *>(take(4 * (size_t)b->ncell_pad));
    b->lstart = reinterpret_cast<uint32_t *>(take(4 * (size_t)b->ncell_pad));
    b->bsum = reinterpret_cast<uint32_t *>(take(4 * (size_t)b->nscan_blocks));
    b->ticket = reinterpret_cast<uint32_t *>(take(4));
    b->dense_list = reinterpret_cast<uint32_t *>(take(4 * ndense));
    b->dense_n = reinterpret_cast<uint32_t *>(take(12));
    b->dflag = take(b->ncell / 4);
    b->carry = nullptr;  // no id windows: cells over the dense list's capacity stay per-boid
    b->defer = nullptr;  // and the thread-per-boid kernel takes all of its boids' passes
    return off;
}

}  // namespace

extern "C" int boids_step_noalloc(const boids_params *params, const float *pos3n_in, const float *vel3n_in,
                                  float *pos3n_out, float *vel3n_out, void *cuda_stream)
{
    if (!params) return boidsgpu::set_last_error(BOIDS_EINVAL, "boids_step_noalloc: null params");
    const uint32_t n = params->number_of_agents;
    if (n && (!pos3n_in || !vel3n_in || !pos3n_out || !vel3n_out))
        return boidsgpu::set_last_error(BOIDS_EINVAL, "boids_step_noalloc: null state pointer");
    if (params->device < 0)
        return boidsgpu::set_last_error(BOIDS_EINVAL, "boids_step_noalloc: bad device ordinal");
    boidsgpu::StepConst k;
    int rc = step_constants(params, &k);
    if (rc) return rc;
    boidsgpu::DevBuffers b{};
    const size_t need = layout(k, nullptr, &b);
    if (need > BOIDS_NOALLOC_SCRATCH_BYTES) {
        char msg[200];
        std::snprintf(msg, sizeof msg,
                      "boids_step_noalloc: this step needs %zu bytes of scratch, the fixed limit is %u bytes "
                      "(use the handle API for larger flocks)",
                      need, (unsigned)BOIDS_NOALLOC_SCRATCH_BYTES);
        return boidsgpu::set_last_error(BOIDS_EINVAL, msg);
    }
    DeviceScope scope(params->device);
    cudaError_t e = scope.err;
    if (e != cudaSuccess) return boidsgpu::set_last_error(BOIDS_ECUDA, cudaGetErrorString(e));
    unsigned char *base = nullptr;
    if ((rc = scratch_address(&base))) return rc;
    layout(k, base, &b);
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, params->device);
    b.dense_grid = (uint32_t)(nsm > 0 ? nsm : 1) * boidsgpu::kDenseCtasPerSm;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    uint64_t launches = 0;
    // the array keeps the previous call's contents: clear what must start at zero
    if ((e = cudaMemsetAsync(b.count, 0, 4 * (size_t)b.ncell_pad, st)) == cudaSuccess &&
        (e = cudaMemsetAsync(b.ticket, 0, 4, st)) == cudaSuccess &&
        (e = boidsgpu::launch_pack(pos3n_in, vel3n_in, b.pos[0], b.vel[0], 0, n, nullptr, 0.f, &k, b.key, b.rank,
                                   b.count, st, &launches)) == cudaSuccess &&
        (e = boidsgpu::launch_grid_scan(k, b, st, &launches)) == cudaSuccess &&
        (e = boidsgpu::launch_grid_scatter(k, b, 0, true, st, &launches)) == cudaSuccess &&
        (e = boidsgpu::launch_grid_force(k, b, 1, false, false, st, &launches)) == cudaSuccess &&
        // the sorted copy in b.pos[1] is dead once the rules have run: it
        // holds the id -> slot table of the unpacking
        (e = boidsgpu::launch_unpack(b.pos[0], b.vel[0], reinterpret_cast<uint32_t *>(b.pos[1]), pos3n_out,
                                     vel3n_out, n, st, &launches)) == cudaSuccess) {
        return BOIDS_OK;
    }
    char msg[160];
    std::snprintf(msg, sizeof msg, "boids_step_noalloc: %s", cudaGetErrorString(e));
    return boidsgpu::set_last_error(BOIDS_ECUDA, msg);
}
