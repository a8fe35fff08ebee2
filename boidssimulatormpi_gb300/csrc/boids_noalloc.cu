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
//    corrupt each other's results; order them on one stream.
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
// address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[BOIDS_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char *g_scratch_addr[kMaxDevices];  // device address of the array, per device

// Device address of the scratch on `dev`, which must be the current device.
// The first call on a device looks it up; later calls reuse it.
int scratch_address(int dev, unsigned char **out)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            char msg[160];
            std::snprintf(msg, sizeof msg, "boids_step_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return boidsgpu::set_last_error(BOIDS_ECUDA, msg);
        }
        g_scratch_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_addr[dev];
    return BOIDS_OK;
}

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
    if (params->device < 0 || params->device >= kMaxDevices)
        return boidsgpu::set_last_error(BOIDS_EINVAL, "boids_step_noalloc: bad device ordinal");
    boidsgpu::StepConst k;
    int rc = boidsgpu::grid_constants_noalloc(params, &k);
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
    cudaError_t e = cudaSetDevice(params->device);
    if (e != cudaSuccess) return boidsgpu::set_last_error(BOIDS_ECUDA, cudaGetErrorString(e));
    unsigned char *base = nullptr;
    if ((rc = scratch_address(params->device, &base))) return rc;
    layout(k, base, &b);
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, params->device);
    b.dense_grid = (uint32_t)(nsm > 0 ? nsm : 1) * 4;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    uint64_t launches = 0;
    // the array keeps the previous call's contents: clear what must start at zero
    if ((e = cudaMemsetAsync(b.count, 0, 4 * (size_t)b.ncell_pad, st)) == cudaSuccess &&
        (e = cudaMemsetAsync(b.ticket, 0, 4, st)) == cudaSuccess &&
        (e = boidsgpu::launch_pack(pos3n_in, vel3n_in, b.pos[0], b.vel[0], n, nullptr, 0.f, st, &launches)) ==
            cudaSuccess &&
        (e = boidsgpu::launch_grid_keys(k, b.pos[0], b.key, b.rank, b.count, st, &launches)) == cudaSuccess &&
        (e = boidsgpu::launch_grid_scan(k, b, st, &launches)) == cudaSuccess &&
        (e = boidsgpu::launch_grid_scatter(k, b, 0, true, st, &launches)) == cudaSuccess &&
        (e = boidsgpu::launch_grid_force(k, b, 1, false, false, st, &launches)) == cudaSuccess &&
        (e = boidsgpu::launch_unpack(b.pos[0], b.vel[0], pos3n_out, vel3n_out, n, st, &launches)) ==
            cudaSuccess) {
        return BOIDS_OK;
    }
    char msg[160];
    std::snprintf(msg, sizeof msg, "boids_step_noalloc: %s", cudaGetErrorString(e));
    return boidsgpu::set_last_error(BOIDS_ECUDA, msg);
}
