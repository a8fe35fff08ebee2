// boids_kernels.cu -- sm_103a kernels for the per-timestep boid update.
//
// Arithmetic contract: every value the reference computes in float is
// computed here with the same IEEE operations in the same order (explicit
// __f*_rn intrinsics, and the file is built with --fmad=false).  Every
// float-vs-double comparison of the reference is replaced by the equivalent
// float comparison prepared on the host (boids_engine.h), and its two
// float-plus-double roundings by integer emulation (boids_softfp.h): the
// kernels issue no FP64 instruction.  Neighbours are accumulated in
// ascending boid id, the order of the reference's loops
// (src/boid_simulation.cpp:161, src/boid_simulation_grid.cpp:191), so the
// results are bit-identical to the reference's, not merely close.
//
// Grid step = scan of cell counts -> stable-free scatter into cell order ->
// two rule kernels that split the boids by the occupancy of their cell:
//   k_grid_sparse  one thread per boid; candidates of the 27 cells around it
//                  are filtered, exactly tested, and kept sorted by id;
//   k_grid_dense   one CTA per crowded cell; the 27-cell candidates are
//                  radix-sorted by id once in shared memory and every boid of
//                  the cell walks them in that order.
// Both integrate, write the new state in place of the sorted slot and bin it
// for the next step (cell key + rank from an atomic count).
#include "boids_engine.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace boidsgpu {

// ------------------------------------------------------------------ exact reference arithmetic

// Vector3D::norm (src/vector3D.cpp:64-67): sqrt((x*x + y*y) + z*z).
__device__ __forceinline__ float nrm3(float x, float y, float z)
{
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
}

// Minimum-image coordinate of boid j seen from boid i
// (src/boid_simulation_grid.cpp:200-214): float difference compared with
// F/2 in double; the shift is (float)((double)x -+ F), reproduced exactly by
// add_f32_f64_rn without any FP64 instruction.
__device__ __forceinline__ float image1(float xj, float xi, const StepConst &k)
{
    if (__fsub_rn(xj, xi) > k.halfF_dn) return add_f32_f64_rn(xj, k.Fsd, 1);
    if (__fsub_rn(xi, xj) > k.halfF_dn) return add_f32_f64_rn(xj, k.Fsd, 0);
    return xj;
}

__device__ __forceinline__ float3 image3(float3 pj, float3 pi, const StepConst &k)
{
    return make_float3(image1(pj.x, pi.x, k), image1(pj.y, pi.y, k), image1(pj.z, pi.z, k));
}

__device__ __forceinline__ float3 xyz(float4 a) { return make_float3(a.x, a.y, a.z); }

// Per-boid constants of the sight vector: |v| exactly, and an approximate
// reciprocal for the cheap cone pre-test.
struct Sight {
    float3 v;
    float nv, inv_nv;
};

__device__ __forceinline__ Sight make_sight(float3 v)
{
    Sight s;
    s.v = v;
    s.nv = nrm3(v.x, v.y, v.z);
    s.inv_nv = __fdividef(1.0f, s.nv);
    return s;
}

// The three Boid::isInsideArea tests (src/boid.cpp:27-42) for an imaged
// target t; bit 0 cohesion, bit 1 separation, bit 2 alignment.
//
// The cone test compares c = dot / (|v| * |r|) (float, correctly rounded
// division and square root) with cstar.  An approximate cosine (hardware
// reciprocal square root, error < 1e-6) settles every case farther than
// cone_band from cstar and from 1; only the rest pay for the exact c.
__device__ __forceinline__ int pair_flags(float3 pi, const Sight &s, float3 t, const StepConst &k)
{
    const float dx = __fsub_rn(pi.x, t.x), dy = __fsub_rn(pi.y, t.y), dz = __fsub_rn(pi.z, t.z);
    // squared norm, (x*x + y*y) + z*z; relativePos = -d has the same one
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    if (!(d2 < k.d2_any)) return 0;
    const float rx = __fsub_rn(t.x, pi.x), ry = __fsub_rn(t.y, pi.y), rz = __fsub_rn(t.z, pi.z);
    const float dot =
        __fadd_rn(__fadd_rn(__fmul_rn(s.v.x, rx), __fmul_rn(s.v.y, ry)), __fmul_rn(s.v.z, rz));
    const float ca = dot * rsqrtf(d2) * s.inv_nv;  // approximate cosine
    bool exact = !(d2 > 1e-30f) || !(fabsf(ca) < 2.0f);  // tiny distance, 0/0, overflow
    int f = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const RuleConst &q = k.rule[r];
        if (!(d2 < q.d2_lim)) continue;
        if (q.all_round) { f |= 1 << r; continue; }
        if (fabsf(ca - q.cstar) < k.cone_band || fabsf(ca - 1.0f) < k.cone_band) exact = true;
        else if (ca > q.cstar && ca < 1.0f) f |= 1 << r;
    }
    if (exact) {
        const float c = __fdiv_rn(dot, __fmul_rn(s.nv, __fsqrt_rn(d2)));
        f = 0;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const RuleConst &q = k.rule[r];
            const bool in_cone = q.all_round || (c >= q.cstar && c <= 1.0f);  // NaN: false
            if (d2 < q.d2_lim && in_cone) f |= 1 << r;
        }
    }
    return f;
}

struct Acc {
    float3 coh, sep, ali;
    int ncoh, nsep, nali;
    uint64_t h[3];
};

__device__ __forceinline__ void acc_zero(Acc &a)
{
    a.coh = a.sep = a.ali = make_float3(0.f, 0.f, 0.f);
    a.ncoh = a.nsep = a.nali = 0;
    a.h[0] = a.h[1] = a.h[2] = 0;
}

// splitmix64 finaliser: the id fingerprint of the neighbour-set diagnostics.
__device__ __forceinline__ uint64_t id_hash(uint32_t id)
{
    uint64_t z = (uint64_t)id + 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// One accepted neighbour, in the reference's order of rules
// (src/boid_simulation_grid.cpp:219-238).
template <bool DIAG>
__device__ __forceinline__ void acc_add(Acc &a, float3 pi, float3 t, float3 vj, int f, uint32_t idj)
{
    if (f & 1) {
        a.ncoh++;
        a.coh.x = __fadd_rn(a.coh.x, t.x);
        a.coh.y = __fadd_rn(a.coh.y, t.y);
        a.coh.z = __fadd_rn(a.coh.z, t.z);
    }
    if (f & 2) {
        a.nsep++;
        const float dx = __fsub_rn(pi.x, t.x), dy = __fsub_rn(pi.y, t.y), dz = __fsub_rn(pi.z, t.z);
        const float n = nrm3(dx, dy, dz);  // Vector3D::normalized
        a.sep.x = __fadd_rn(a.sep.x, __fdiv_rn(dx, n));
        a.sep.y = __fadd_rn(a.sep.y, __fdiv_rn(dy, n));
        a.sep.z = __fadd_rn(a.sep.z, __fdiv_rn(dz, n));
    }
    if (f & 4) {
        a.nali++;
        a.ali.x = __fadd_rn(a.ali.x, vj.x);
        a.ali.y = __fadd_rn(a.ali.y, vj.y);
        a.ali.z = __fadd_rn(a.ali.z, vj.z);
    }
    if (DIAG) {
        const uint64_t h = id_hash(idj);
        if (f & 1) a.h[0] += h;
        if (f & 2) a.h[1] += h;
        if (f & 4) a.h[2] += h;
    }
}

// Exact test of candidate j (state slot) and, if accepted, accumulation.
template <bool DIAG>
__device__ __forceinline__ void visit(Acc &a, float3 pi, const Sight &s, const float4 *__restrict__ pos,
                                      const float4 *__restrict__ vel, uint32_t j, const StepConst &k)
{
    const float4 pj = __ldg(pos + j);
    const float3 t = image3(xyz(pj), pi, k);
    const int f = pair_flags(pi, s, t, k);
    if (f) {
        const float3 vj = (f & 4) ? xyz(__ldg(vel + j)) : make_float3(0.f, 0.f, 0.f);
        acc_add<DIAG>(a, pi, t, vj, f, __float_as_uint(pj.w));
    }
}

// Rule finalisation (src/boid_simulation_grid.cpp:243-252): returns the three
// scaled rule forces, which are also get_force's values (:319-334).
__device__ __forceinline__ void acc_finish(const Acc &a, float3 pi, float3 vi, const StepConst &k,
                                           float3 &fc, float3 &fs, float3 &fa)
{
    float3 coh = a.coh, ali = a.ali;
    if (a.ncoh != 0) {
        const float q = __int2float_rn(a.ncoh);
        coh.x = __fsub_rn(__fdiv_rn(coh.x, q), pi.x);
        coh.y = __fsub_rn(__fdiv_rn(coh.y, q), pi.y);
        coh.z = __fsub_rn(__fdiv_rn(coh.z, q), pi.z);
    }
    if (a.nali != 0) {
        const float q = __int2float_rn(a.nali);
        ali.x = __fsub_rn(__fdiv_rn(ali.x, q), vi.x);
        ali.y = __fsub_rn(__fdiv_rn(ali.y, q), vi.y);
        ali.z = __fsub_rn(__fdiv_rn(ali.z, q), vi.z);
    }
    fc = make_float3(__fmul_rn(coh.x, k.cc), __fmul_rn(coh.y, k.cc), __fmul_rn(coh.z, k.cc));
    fs = make_float3(__fmul_rn(a.sep.x, k.cs), __fmul_rn(a.sep.y, k.cs), __fmul_rn(a.sep.z, k.cs));
    fa = make_float3(__fmul_rn(ali.x, k.ca), __fmul_rn(ali.y, k.ca), __fmul_rn(ali.z, k.ca));
}

// Periodic wrap (src/boid_simulation_grid.cpp:274-289): (float)(F + x) or
// (float)(x - F), both computed in double by the reference.
__device__ __forceinline__ float wrap1(float x, const StepConst &k)
{
    if (x < 0.0f) return add_f32_f64_rn(x, k.Fsd, 0);
    if (x > k.F_dn) return add_f32_f64_rn(x, k.Fsd, 1);
    return x;
}

// Integration of one boid (src/boid_simulation_grid.cpp:262-289).
__device__ __forceinline__ void integrate(float3 &x, float3 &v, float3 fc, float3 fs, float3 fa,
                                          const StepConst &k)
{
    // dv = c_coh*coh + c_sep*sep + c_ali*ali, left to right
    v.x = __fadd_rn(v.x, __fadd_rn(__fadd_rn(fc.x, fs.x), fa.x));
    v.y = __fadd_rn(v.y, __fadd_rn(__fadd_rn(fc.y, fs.y), fa.y));
    v.z = __fadd_rn(v.z, __fadd_rn(__fadd_rn(fc.z, fs.z), fa.z));
    const float n = nrm3(v.x, v.y, v.z);
    if (n > 0.0f && n > k.vmax_dn) {
        v.x = __fmul_rn(__fdiv_rn(v.x, n), k.vmax_f);
        v.y = __fmul_rn(__fdiv_rn(v.y, n), k.vmax_f);
        v.z = __fmul_rn(__fdiv_rn(v.z, n), k.vmax_f);
    } else if (n > 0.0f && n < k.vmin_up) {
        v.x = __fmul_rn(__fdiv_rn(v.x, n), k.vmin_f);
        v.y = __fmul_rn(__fdiv_rn(v.y, n), k.vmin_f);
        v.z = __fmul_rn(__fdiv_rn(v.z, n), k.vmin_f);
    }
    x.x = wrap1(__fadd_rn(x.x, v.x), k);
    x.y = wrap1(__fadd_rn(x.y, v.y), k);
    x.z = wrap1(__fadd_rn(x.z, v.z), k);
}

// ------------------------------------------------------------------ device grid

__device__ __forceinline__ int cell1(float x, const StepConst &k)
{
    const int c = __float2int_rz(__fmul_rn(x, k.inv_side));
    return min(max(c, 0), k.G - 1);
}

__device__ __forceinline__ uint32_t cell_key(float3 p, const StepConst &k)
{
    return (uint32_t)((cell1(p.z, k) * k.G + cell1(p.y, k)) * k.G + cell1(p.x, k));
}

__device__ __forceinline__ uint32_t cell_start(const uint32_t *__restrict__ lstart,
                                               const uint32_t *__restrict__ bsum, uint32_t c)
{
    return __ldg(lstart + c) + __ldg(bsum + c / kScanTile);
}

// Where a rule kernel writes one boid's result.
struct GridOut {
    float4 *pos_out, *vel_out;
    uint32_t *key_out, *rank_out, *count;  // null for the all-pairs engine
    float *forces;
    int32_t *dcnt;
    uint64_t *dhash;
};

template <bool DIAG>
__device__ __forceinline__ void finish_boid(const Acc &a, float4 p4, float3 vi, uint32_t s, const GridOut &o,
                                            const StepConst &k)
{
    const uint32_t id = __float_as_uint(p4.w);
    if (DIAG) {
        o.dcnt[3 * id + 0] = a.ncoh; o.dcnt[3 * id + 1] = a.nsep; o.dcnt[3 * id + 2] = a.nali;
        o.dhash[3 * id + 0] = a.h[0]; o.dhash[3 * id + 1] = a.h[1]; o.dhash[3 * id + 2] = a.h[2];
        return;
    }
    const float3 pi = xyz(p4);
    float3 fc, fs, fa;
    acc_finish(a, pi, vi, k, fc, fs, fa);
    float3 x = pi, v = vi;
    integrate(x, v, fc, fs, fa, k);
    o.pos_out[s] = make_float4(x.x, x.y, x.z, p4.w);
    o.vel_out[s] = make_float4(v.x, v.y, v.z, 0.f);
    if (o.key_out) {  // binning for the next step
        const uint32_t c = cell_key(x, k);
        o.key_out[s] = c;
        o.rank_out[s] = atomicAdd(o.count + c, 1u);
    }
    if (o.forces) {
        float *f = o.forces + (size_t)9 * id;
        f[0] = fc.x; f[1] = fc.y; f[2] = fc.z;
        f[3] = fs.x; f[4] = fs.y; f[5] = fs.z;
        f[6] = fa.x; f[7] = fa.y; f[8] = fa.z;
    }
}

// ------------------------------------------------------------------ state packing

// Packs an id-ordered state into float4 records (w of pos = id bits).  With
// bad != null, a coordinate outside [0, hi] (or NaN) sets *bad.
__global__ void k_pack(const float *__restrict__ pos3, const float *__restrict__ vel3,
                       float4 *__restrict__ pos4, float4 *__restrict__ vel4, uint32_t n,
                       uint32_t *__restrict__ bad, float hi)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = pos3[3 * i], y = pos3[3 * i + 1], z = pos3[3 * i + 2];
    pos4[i] = make_float4(x, y, z, __uint_as_float(i));
    vel4[i] = make_float4(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2], 0.f);
    if (bad && !(x >= 0.f && x <= hi && y >= 0.f && y <= hi && z >= 0.f && z <= hi)) *bad = 1u;
}

// Slot order -> id order (the reference's getters index by id).
__global__ void k_unpack(const float4 *__restrict__ pos4, const float4 *__restrict__ vel4,
                         float *__restrict__ pos3, float *__restrict__ vel3, uint32_t n)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const float4 p = pos4[s];
    const uint32_t id = __float_as_uint(p.w);
    if (pos3) { pos3[3 * id] = p.x; pos3[3 * id + 1] = p.y; pos3[3 * id + 2] = p.z; }
    if (vel3) {
        const float4 v = vel4[s];
        vel3[3 * id] = v.x; vel3[3 * id + 1] = v.y; vel3[3 * id + 2] = v.z;
    }
}

// ------------------------------------------------------------------ counting-sort binning

__global__ void k_grid_keys(const float4 *__restrict__ pos, uint32_t *__restrict__ key,
                            uint32_t *__restrict__ rank, uint32_t *__restrict__ count, StepConst k)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= k.n) return;
    const uint32_t c = cell_key(xyz(pos[s]), k);
    key[s] = c;
    rank[s] = atomicAdd(count + c, 1u);
}

// Exclusive scan of the per-cell counts.  Each block scans one tile of
// kScanTile cells into lstart and publishes its total; the last block to
// finish (completion ticket, no waiting) turns the totals into tile offsets
// in bsum.  start(c) = lstart[c] + bsum[c / kScanTile].  Cells holding at
// least kDenseMin boids are appended to the dense-cell work list.
constexpr int kScanThreads = 256;
constexpr int kScanItems = kScanTile / kScanThreads;  // 8

template <int NT>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *warp_tot, uint32_t &total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = lane < NT / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < NT / 32) warp_tot[lane] = t;  // inclusive warp totals
    }
    __syncthreads();
    total = warp_tot[NT / 32 - 1];
    const uint32_t before = (w > 0 ? warp_tot[w - 1] : 0) + x - v;
    __syncthreads();  // warp_tot is reused by the next call
    return before;
}

__global__ void __launch_bounds__(kScanThreads)
k_grid_scan(const uint32_t *__restrict__ count, uint32_t *__restrict__ lstart, uint32_t *bsum,
            uint32_t *ticket, uint32_t nblocks, uint32_t *__restrict__ dense_list, uint32_t *dense_n)
{
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    __shared__ bool is_last;
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    const uint4 a = *reinterpret_cast<const uint4 *>(count + base);
    const uint4 b = *reinterpret_cast<const uint4 *>(count + base + 4);
    const uint32_t v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        sum += v[i];
        if (dense_list && v[i] >= (uint32_t)kDenseMin) dense_list[atomicAdd(dense_n, 1u)] = base + i;
    }
    uint32_t total;
    uint32_t run = block_excl_scan<kScanThreads>(sum, warp_tot, total);
    uint32_t o[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) { o[i] = run; run += v[i]; }
    *reinterpret_cast<uint4 *>(lstart + base) = make_uint4(o[0], o[1], o[2], o[3]);
    *reinterpret_cast<uint4 *>(lstart + base + 4) = make_uint4(o[4], o[5], o[6], o[7]);
    if (threadIdx.x == 0) {
        bsum[blockIdx.x] = total;
        __threadfence();
        is_last = atomicAdd(ticket, 1u) == nblocks - 1;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    uint32_t carry = 0;
    for (uint32_t c0 = 0; c0 < nblocks; c0 += kScanThreads) {
        const uint32_t i = c0 + threadIdx.x;
        const uint32_t t = i < nblocks ? __ldcg(bsum + i) : 0u;
        uint32_t chunk;
        const uint32_t ex = block_excl_scan<kScanThreads>(t, warp_tot, chunk);
        if (i < nblocks) bsum[i] = carry + ex;
        carry += chunk;
    }
    if (threadIdx.x == 0) *ticket = 0;  // ready for the next launch
}

__global__ void k_grid_scatter(const float4 *__restrict__ pin, const float4 *__restrict__ vin,
                               const uint32_t *__restrict__ key, const uint32_t *__restrict__ rank,
                               const uint32_t *__restrict__ lstart, const uint32_t *__restrict__ bsum,
                               float4 *__restrict__ pout, float4 *__restrict__ vout,
                               uint32_t *__restrict__ count_to_zero, uint32_t n)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t c = key[s];
    const uint32_t d = cell_start(lstart, bsum, c) + rank[s];
    pout[d] = pin[s];
    vout[d] = vin[s];
    if (count_to_zero) count_to_zero[c] = 0;  // every binned cell, for the next step's keys
}

// ------------------------------------------------------------------ neighbourhood segments

// The 27 cells around (cx, cy, cz) form 9 rows of 3 cells along x; a row is
// one run of consecutive cell indices, or two where x wraps.  Segment q of
// a boid (0 <= q < 9 * runs) is run q % runs of row q / runs.  (sx, sy, sz)
// moves a boid of the segment next to the centre cell across the periodic
// faces (approximately, for the filters only).
struct Seg {
    uint32_t c0, c1;  // cells [c0, c1)
    float sx, sy, sz;
};

__device__ __forceinline__ int seg_runs(int cx, const StepConst &k) { return (cx == 0 || cx == k.G - 1) ? 2 : 1; }

__device__ __forceinline__ Seg segment(int cx, int cy, int cz, int q, int runs, const StepConst &k)
{
    const int G = k.G;
    const int row = q / runs, run = q - row * runs;
    int z = cz + row / 3 - 1, y = cy + row % 3 - 1;
    float sz = 0.f, sy = 0.f;
    if (z < 0) { z += G; sz = -k.Ff; } else if (z >= G) { z -= G; sz = k.Ff; }
    if (y < 0) { y += G; sy = -k.Ff; } else if (y >= G) { y -= G; sy = k.Ff; }
    const uint32_t r0 = (uint32_t)(z * G + y) * (uint32_t)G;
    if (runs == 1) return Seg{r0 + cx - 1, r0 + cx + 2, 0.f, sy, sz};
    if (cx == 0) return run == 0 ? Seg{r0 + G - 1, r0 + G, -k.Ff, sy, sz} : Seg{r0, r0 + 2, 0.f, sy, sz};
    return run == 0 ? Seg{r0 + G - 2, r0 + G, 0.f, sy, sz} : Seg{r0, r0 + 1, k.Ff, sy, sz};
}

// Which kernel takes the boids of a cell: k_grid_dense when its shared
// candidate list fits and either the cell is crowded or its neighbourhood is
// (then sorting once per cell beats sorting per boid), else k_grid_sparse.
__device__ __forceinline__ bool dense_path(uint32_t b, uint32_t ncand)
{
    return ncand <= (uint32_t)kDenseCap && (b >= (uint32_t)kDenseMin || ncand > (uint32_t)kCandDefer);
}

// ------------------------------------------------------------------ sparse cells: thread per boid

// All lanes of a warp walk their own candidate lists in lock-step (a flat
// loop of max-over-warp length).  Candidates passing the squared-distance
// filter are buffered, and the whole warp runs the exact tests on its
// buffers together whenever one of them is full, so the expensive test runs
// with most lanes busy.  Accepted neighbours are kept sorted by id, at most
// kListCap per pass; a boid with more takes further passes, each keeping the
// next kListCap ids, so accumulation is always in ascending id.
constexpr int kBufA = 16;

struct GridIn {
    const float4 *__restrict__ pos;
    const float4 *__restrict__ vel;
    const uint32_t *__restrict__ lstart;
    const uint32_t *__restrict__ bsum;
};

template <bool DIAG>
__global__ void __launch_bounds__(128)
k_grid_sparse(GridIn g, GridOut o, uint32_t *__restrict__ dense_list, uint32_t *__restrict__ dense_n, StepConst k)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    bool act = s < k.n;
    const float4 p4 = act ? g.pos[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 v4 = act ? g.vel[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float3 pi = xyz(p4), vi = xyz(v4);
    const int cx = cell1(pi.x, k), cy = cell1(pi.y, k), cz = cell1(pi.z, k);
    const int runs = seg_runs(cx, k), nseg = 9 * runs;
    uint32_t ncand = 0;
    if (act) {
        for (int q = 0; q < nseg; ++q) {
            const Seg sg = segment(cx, cy, cz, q, runs, k);
            ncand += cell_start(g.lstart, g.bsum, sg.c1) - cell_start(g.lstart, g.bsum, sg.c0);
        }
        const uint32_t cown = (uint32_t)((cz * k.G + cy) * k.G + cx);
        const uint32_t own0 = cell_start(g.lstart, g.bsum, cown);
        const uint32_t b = cell_start(g.lstart, g.bsum, cown + 1) - own0;
        if (dense_path(b, ncand)) {
            // a crowded cell is listed by the scan; a sparse cell with a
            // crowded neighbourhood is listed here, once, by its first boid
            if (b < (uint32_t)kDenseMin && s == own0) dense_list[atomicAdd(dense_n, 1u)] = cown;
            act = false;
        }
    }
    const uint32_t nc = act ? ncand : 0;
    const uint32_t max_nc = __reduce_max_sync(0xffffffffu, nc);
    if (max_nc == 0) return;  // the whole warp is idle

    const Sight sight = make_sight(vi);
    Acc a;
    acc_zero(a);
    uint64_t lst[kListCap];
    uint32_t buf[kBufA];
    int64_t lo = -1;  // ids <= lo were accumulated by earlier passes
    bool need = act;
    while (__any_sync(0xffffffffu, need)) {
        int m = 0, nb = 0;
        uint32_t more = 0;  // accepted neighbours with id > lo in this pass
        auto flush = [&]() {
            for (int q = 0; q < nb; ++q) {
                const uint32_t j = buf[q];
                const float4 pj = __ldg(g.pos + j);
                const uint32_t idj = __float_as_uint(pj.w);
                if ((int64_t)idj <= lo) continue;
                const int f = pair_flags(pi, sight, image3(xyz(pj), pi, k), k);
                if (!f) continue;
                ++more;
                const uint64_t e = ((uint64_t)idj << 32) | (uint64_t)(j | ((uint32_t)f << 29));
                int w;
                if (m < kListCap) w = m++;
                else if (e < lst[kListCap - 1]) w = kListCap - 1;
                else continue;
                while (w > 0 && lst[w - 1] > e) { lst[w] = lst[w - 1]; --w; }
                lst[w] = e;
            }
            nb = 0;
        };
        int qs = -1;
        uint32_t j = 0, jend = 0;
        float qx = 0.f, qy = 0.f, qz = 0.f;
        const uint32_t mine = need ? nc : 0;
        for (uint32_t it = 0; it < max_nc; ++it) {
            if (it < mine) {
                while (j == jend) {  // next non-empty segment
                    const Seg sg = segment(cx, cy, cz, ++qs, runs, k);
                    j = cell_start(g.lstart, g.bsum, sg.c0);
                    jend = cell_start(g.lstart, g.bsum, sg.c1);
                    qx = pi.x - sg.sx; qy = pi.y - sg.sy; qz = pi.z - sg.sz;
                }
                const float4 pj = __ldg(g.pos + j);
                const float dx = pj.x - qx, dy = pj.y - qy, dz = pj.z - qz;
                const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                if (d2 < k.filt_r2 && j != s) buf[nb++] = j;
                ++j;
            }
            if (__any_sync(0xffffffffu, nb == kBufA)) flush();
        }
        flush();
        if (need) {
            for (int q = 0; q < m; ++q) {
                const uint64_t e = lst[q];
                const uint32_t jj = (uint32_t)e & 0x1fffffffu;
                const int f = (int)(((uint32_t)e) >> 29);
                const float3 t = image3(xyz(__ldg(g.pos + jj)), pi, k);
                const float3 vj = (f & 4) ? xyz(__ldg(g.vel + jj)) : make_float3(0.f, 0.f, 0.f);
                acc_add<DIAG>(a, pi, t, vj, f, (uint32_t)(e >> 32));
            }
            if (more <= (uint32_t)m) need = false;
            else lo = (int64_t)(lst[m - 1] >> 32);
        }
    }
    if (act) finish_boid<DIAG>(a, p4, vi, s, o, k);
}

// ------------------------------------------------------------------ dense cells: CTA per cell

// Stable LSD radix sort of n 64-bit keys held in shared memory, on bits
// [lo, lo + nbits), 4 bits per pass; NT threads each own a contiguous run.
// Returns the buffer that holds the sorted keys.
template <int NT>
__device__ uint64_t *block_radix_sort(uint64_t *a, uint64_t *b, uint32_t *hist, int n, int lo, int nbits)
{
    __shared__ uint32_t wsum[NT / 32];
    const int t = threadIdx.x;
    const int K = (n + NT - 1) / NT;
    const int i0 = min(n, t * K), i1 = min(n, i0 + K);
    for (int bit = lo; bit < lo + nbits; bit += 4) {
#pragma unroll
        for (int d = 0; d < 16; ++d) hist[d * NT + t] = 0;
        for (int i = i0; i < i1; ++i) hist[((uint32_t)(a[i] >> bit) & 15u) * NT + t]++;
        __syncthreads();
        // exclusive scan of hist in (digit, thread) order; thread t owns 16 entries
        uint32_t loc[16], sum = 0;
#pragma unroll
        for (int q = 0; q < 16; ++q) { loc[q] = hist[16 * t + q]; sum += loc[q]; }
        uint32_t total;
        uint32_t pre = block_excl_scan<NT>(sum, wsum, total);
#pragma unroll
        for (int q = 0; q < 16; ++q) { hist[16 * t + q] = pre; pre += loc[q]; }
        __syncthreads();
        for (int i = i0; i < i1; ++i) {
            const uint64_t v = a[i];
            b[hist[((uint32_t)(v >> bit) & 15u) * NT + t]++] = v;
        }
        __syncthreads();
        uint64_t *tmp = a; a = b; b = tmp;
    }
    return a;
}

constexpr int kDenseThreads = 64;
constexpr int kBufB = 16;
constexpr int kDenseK = kDenseCap / kDenseThreads;  // candidates per thread when full

// Shared memory of k_grid_dense.  The sort keys and gather slots are dead
// once the candidates are laid out in id order, so that layout reuses them.
struct DenseSmem {
    union {
        uint64_t keys[2][kDenseCap];  // (id << 16) | (segment << 11) | gather index
        float4 spos[kDenseCap];       // candidates in id order, moved next to the cell
    } u;
    union {
        uint32_t gslot[kDenseCap];    // state slot, by gather index
        uint32_t sslot[kDenseCap];    // state slot, by id order
    } v;
    uint32_t hist[16 * kDenseThreads];
    uint16_t bufs[kBufB * kDenseThreads];
    uint32_t seg_j0[18], seg_k0[19];
    float seg_s[18][3];
    int nseg;
};
static_assert(sizeof(DenseSmem) <= 48 * 1024, "dense-cell shared memory exceeds the static limit");
static_assert(kDenseCap <= 2048, "gather index must fit 11 bits");

template <bool DIAG>
__global__ void __launch_bounds__(kDenseThreads)
k_grid_dense(GridIn g, GridOut o, const uint32_t *__restrict__ dense_list, const uint32_t *__restrict__ dense_n,
             StepConst k)
{
    __shared__ DenseSmem sm;
    const int t = threadIdx.x;
    const uint32_t nd = *dense_n;
    for (uint32_t w = blockIdx.x; w < nd; w += gridDim.x) {
        const uint32_t c = dense_list[w];
        const int G = k.G;
        const int cx = (int)(c % G), cy = (int)((c / G) % G), cz = (int)(c / ((uint32_t)G * G));
        const int runs = seg_runs(cx, k), ns = 9 * runs;
        if (t < ns) {
            const Seg sg = segment(cx, cy, cz, t, runs, k);
            sm.seg_j0[t] = cell_start(g.lstart, g.bsum, sg.c0);
            sm.seg_k0[t + 1] = cell_start(g.lstart, g.bsum, sg.c1) - sm.seg_j0[t];  // length for now
            sm.seg_s[t][0] = sg.sx; sm.seg_s[t][1] = sg.sy; sm.seg_s[t][2] = sg.sz;
        }
        __syncthreads();
        if (t == 0) {
            sm.seg_k0[0] = 0;
            for (int q = 0; q < ns; ++q) sm.seg_k0[q + 1] += sm.seg_k0[q];
        }
        __syncthreads();
        const uint32_t ncand = sm.seg_k0[ns];
        const uint32_t own0 = cell_start(g.lstart, g.bsum, c);
        const uint32_t b = cell_start(g.lstart, g.bsum, c + 1) - own0;
        if (!dense_path(b, ncand)) {  // too many candidates: left to k_grid_sparse
            __syncthreads();
            continue;
        }

        // gather (id, segment, gather index) keys, sort them by id
        for (uint32_t q = t; q < ncand; q += kDenseThreads) {
            uint32_t sgi = 0;
            while (q >= sm.seg_k0[sgi + 1]) ++sgi;
            const uint32_t slot = sm.seg_j0[sgi] + (q - sm.seg_k0[sgi]);
            sm.v.gslot[q] = slot;
            sm.u.keys[0][q] = ((uint64_t)__float_as_uint(__ldg(&g.pos[slot].w)) << 16) | (sgi << 11) | q;
        }
        __syncthreads();
        const uint64_t *sorted = block_radix_sort<kDenseThreads>(sm.u.keys[0], sm.u.keys[1], sm.hist,
                                                                 (int)ncand, 16, k.id_bits);
        // lay the candidates out in id order (over the dead sort buffers)
        const int K = ((int)ncand + kDenseThreads - 1) / kDenseThreads;
        const int q0 = t * K;
        uint32_t slot_r[kDenseK], seg_r[kDenseK];
#pragma unroll
        for (int i = 0; i < kDenseK; ++i) {
            if (i < K && q0 + i < (int)ncand) {
                const uint64_t key = sorted[q0 + i];
                slot_r[i] = sm.v.gslot[(uint32_t)key & 0x7ffu];
                seg_r[i] = ((uint32_t)key >> 11) & 0x1fu;
            }
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < kDenseK; ++i) {
            if (i < K && q0 + i < (int)ncand) {
                const float4 p = __ldg(g.pos + slot_r[i]);
                const float *sh = sm.seg_s[seg_r[i]];
                sm.u.spos[q0 + i] = make_float4(p.x + sh[0], p.y + sh[1], p.z + sh[2], p.w);
                sm.v.sslot[q0 + i] = slot_r[i];
            }
        }
        __syncthreads();

        // every boid of the cell walks the candidates in id order; the warp
        // runs its exact tests together whenever a lane's buffer fills
        for (uint32_t r0 = 0; r0 < b; r0 += kDenseThreads) {
            const uint32_t bi = r0 + t;
            const bool act = bi < b;
            const uint32_t s = own0 + (act ? bi : 0);
            const float4 p4 = g.pos[s], v4 = g.vel[s];
            const float3 pi = xyz(p4), vi = xyz(v4);
            const Sight sight = make_sight(vi);
            Acc a;
            acc_zero(a);
            int nb = 0;
            auto flush = [&]() {
                for (int q = 0; q < nb; ++q) {
                    const uint32_t j = sm.v.sslot[sm.bufs[q * kDenseThreads + t]];
                    if (j != s) visit<DIAG>(a, pi, sight, g.pos, g.vel, j, k);
                }
                nb = 0;
            };
            for (uint32_t q = 0; q < ncand; ++q) {
                const float4 pj = sm.u.spos[q];
                const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
                const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                if (act && d2 < k.filt_r2) sm.bufs[nb++ * kDenseThreads + t] = (uint16_t)q;
                if (__any_sync(0xffffffffu, nb == kBufB)) flush();
            }
            flush();
            if (act) finish_boid<DIAG>(a, p4, vi, s, o, k);
        }
        __syncthreads();  // shared arrays are rebuilt for the next cell
    }
}

// ------------------------------------------------------------------ all-pairs engine

// Phase 1: a 2-D grid of (i-tile, j-tile) blocks tests every ordered pair.
// A box filter on the minimum-image offset (||dx| - F/2| > F/2 - R per axis)
// rejects almost all pairs; survivors get the exact tests and accepted
// neighbours are appended to the boid's list (unordered).
constexpr int kApThreads = 128;
constexpr int kApKI = 4;                        // i per thread
constexpr int kApTileI = kApThreads * kApKI;    // 512
constexpr int kApTileJ = 1024;

__global__ void __launch_bounds__(kApThreads)
k_ap_pairs(const float4 *__restrict__ pos, const float4 *__restrict__ vel, uint32_t *__restrict__ cnt,
           uint32_t *__restrict__ list, uint32_t cap, StepConst k)
{
    __shared__ float4 sp[kApTileJ];
    const uint32_t n = k.n;
    const uint32_t j0 = blockIdx.y * kApTileJ;
    const uint32_t jn = min((uint32_t)kApTileJ, n - j0);
    for (uint32_t t = threadIdx.x; t < jn; t += kApThreads) sp[t] = pos[j0 + t];
    float3 pi[kApKI];
    uint32_t ii[kApKI];
    const float nanf_ = __uint_as_float(0x7fffffffu);  // fails every filter test
#pragma unroll
    for (int r = 0; r < kApKI; ++r) {
        ii[r] = blockIdx.x * kApTileI + r * kApThreads + threadIdx.x;
        pi[r] = ii[r] < n ? xyz(pos[ii[r]]) : make_float3(nanf_, nanf_, nanf_);
    }
    __syncthreads();
    const float h = k.halfFf, lim = k.box_lim;
    for (uint32_t t = 0; t < jn; ++t) {
        const float4 pj = sp[t];
#pragma unroll
        for (int r = 0; r < kApKI; ++r) {
            const bool nx = fabsf(fabsf(pj.x - pi[r].x) - h) > lim;
            const bool ny = fabsf(fabsf(pj.y - pi[r].y) - h) > lim;
            const bool nz = fabsf(fabsf(pj.z - pi[r].z) - h) > lim;
            if (nx && ny && nz) {
                const uint32_t i = ii[r], j = j0 + t;
                if (i == j) continue;
                const Sight s = make_sight(xyz(vel[i]));
                const int f = pair_flags(pi[r], s, image3(xyz(pj), pi[r], k), k);
                if (f) {
                    const uint32_t q = atomicAdd(cnt + i, 1u);
                    if (q < cap) list[(size_t)i * cap + q] = j | ((uint32_t)f << 29);
                }
            }
        }
    }
}

// Phase 2: per boid, sort its neighbours by id and accumulate in that order,
// then finish and integrate.  A boid with more than `cap` neighbours scans
// all boids in order instead.
template <bool DIAG>
__global__ void __launch_bounds__(128)
k_ap_accumulate(const float4 *__restrict__ pos, const float4 *__restrict__ vel, uint32_t *__restrict__ cnt,
                const uint32_t *__restrict__ list, uint32_t cap, GridOut o, StepConst k)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const float4 p4 = pos[i], v4 = vel[i];
    const float3 pi = xyz(p4), vi = xyz(v4);
    const uint32_t m = cnt[i];
    cnt[i] = 0;  // ready for the next step
    Acc a;
    acc_zero(a);
    if (m <= cap) {
        uint32_t lst[kApCap];
        for (uint32_t q = 0; q < m; ++q) {
            const uint32_t e = list[(size_t)i * cap + q];
            uint32_t w = q;
            while (w > 0 && (lst[w - 1] & 0x1fffffffu) > (e & 0x1fffffffu)) { lst[w] = lst[w - 1]; --w; }
            lst[w] = e;
        }
        for (uint32_t q = 0; q < m; ++q) {
            const uint32_t j = lst[q] & 0x1fffffffu;
            const int f = (int)(lst[q] >> 29);
            const float3 t = image3(xyz(pos[j]), pi, k);
            const float3 vj = (f & 4) ? xyz(vel[j]) : make_float3(0.f, 0.f, 0.f);
            acc_add<DIAG>(a, pi, t, vj, f, j);
        }
    } else {
        const Sight s = make_sight(vi);
        for (uint32_t j = 0; j < k.n; ++j) {
            if (j == i) continue;
            const float4 pj = pos[j];
            const bool nx = fabsf(fabsf(pj.x - pi.x) - k.halfFf) > k.box_lim;
            const bool ny = fabsf(fabsf(pj.y - pi.y) - k.halfFf) > k.box_lim;
            const bool nz = fabsf(fabsf(pj.z - pi.z) - k.halfFf) > k.box_lim;
            if (nx && ny && nz) visit<DIAG>(a, pi, s, pos, vel, j, k);
        }
    }
    finish_boid<DIAG>(a, p4, vi, i, o, k);
}

// ------------------------------------------------------------------ reference cell indices

// Boid::grid_index as update_list_grid computes it
// (src/boid_simulation_grid.cpp:400-443), written in id order.
__global__ void k_ref_cells(const float4 *__restrict__ pos, int32_t *__restrict__ cells8, StepConst k)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= k.n) return;
    const float4 p = pos[s];
    const uint32_t id = __float_as_uint(p.w);
    const unsigned G = (unsigned)k.refG;
    const float GS = k.refGS, R = k.refR;
    const float c[3] = {p.x, p.y, p.z};
    int g[3][2];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int g0 = __float2int_rz(__fdiv_rn(c[d], GS));
        if ((unsigned)g0 == G) g0 = (int)G - 1;
        const float pig = __fsub_rn(c[d], __fmul_rn(__int2float_rn(g0), GS));
        g[d][0] = g0;
        if (pig <= R) g[d][1] = (int)(((unsigned)(g0 - 1) + G) % G);
        else if (pig >= __fsub_rn(GS, R)) g[d][1] = (int)(((unsigned)g0 + 1) % G);
        else g[d][1] = -1;
    }
    int32_t out[8];
    int n = 0;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        if (g[0][i] == -1) continue;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (g[1][j] == -1) continue;
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                if (g[2][q] == -1) continue;
                out[n++] = (int32_t)((unsigned)g[0][i] + (unsigned)g[1][j] * G + (unsigned)g[2][q] * G * G);
            }
        }
    }
    for (int q = 0; q < 8; ++q) cells8[(size_t)8 * id + q] = q < n ? out[q] : -1;
}

// ------------------------------------------------------------------ launchers

static inline unsigned blocks_for(uint32_t n, unsigned t) { return (n + t - 1) / t; }

cudaError_t launch_pack(const float *pos3, const float *vel3, float4 *pos4, float4 *vel4, uint32_t n,
                        uint32_t *bad, float hi, cudaStream_t st, uint64_t *launches)
{
    if (n == 0) return cudaSuccess;
    k_pack<<<blocks_for(n, 256), 256, 0, st>>>(pos3, vel3, pos4, vel4, n, bad, hi);
    ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_unpack(const float4 *pos4, const float4 *vel4, float *pos3, float *vel3, uint32_t n,
                          cudaStream_t st, uint64_t *launches)
{
    if (n == 0) return cudaSuccess;
    k_unpack<<<blocks_for(n, 256), 256, 0, st>>>(pos4, vel4, pos3, vel3, n);
    ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_grid_keys(const StepConst &k, const float4 *pos, uint32_t *key, uint32_t *rank,
                             uint32_t *count, cudaStream_t st, uint64_t *launches)
{
    if (k.n == 0) return cudaSuccess;
    k_grid_keys<<<blocks_for(k.n, 256), 256, 0, st>>>(pos, key, rank, count, k);
    ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_grid_scan(const DevBuffers &b, cudaStream_t st, uint64_t *launches)
{
    cudaError_t e = cudaMemsetAsync(b.dense_n, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    k_grid_scan<<<b.nscan_blocks, kScanThreads, 0, st>>>(b.count, b.lstart, b.bsum, b.ticket, b.nscan_blocks,
                                                          b.dense_list, b.dense_n);
    ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_grid_scatter(const StepConst &k, const DevBuffers &b, int from, bool zero_counts,
                                cudaStream_t st, uint64_t *launches)
{
    if (k.n == 0) return cudaSuccess;
    k_grid_scatter<<<blocks_for(k.n, 256), 256, 0, st>>>(b.pos[from], b.vel[from], b.key, b.rank, b.lstart,
                                                         b.bsum, b.pos[1 - from], b.vel[1 - from],
                                                         zero_counts ? b.count : nullptr, k.n);
    ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_grid_force(const StepConst &k, const DevBuffers &b, int from, bool diag, bool record_forces,
                              cudaStream_t st, uint64_t *launches)
{
    if (k.n == 0) return cudaSuccess;
    GridIn g{b.pos[from], b.vel[from], b.lstart, b.bsum};
    GridOut o{};
    if (diag) {
        o.dcnt = b.dcnt;
        o.dhash = b.dhash;
    } else {
        o.pos_out = b.pos[1 - from];
        o.vel_out = b.vel[1 - from];
        o.key_out = b.key;
        o.rank_out = b.rank;
        o.count = b.count;
        o.forces = record_forces ? b.forces : nullptr;
    }
    const unsigned nb = blocks_for(k.n, 128);
    const unsigned nd = b.dense_grid;
    if (diag) {
        k_grid_sparse<true><<<nb, 128, 0, st>>>(g, o, b.dense_list, b.dense_n, k);
        k_grid_dense<true><<<nd, kDenseThreads, 0, st>>>(g, o, b.dense_list, b.dense_n, k);
    } else {
        k_grid_sparse<false><<<nb, 128, 0, st>>>(g, o, b.dense_list, b.dense_n, k);
        k_grid_dense<false><<<nd, kDenseThreads, 0, st>>>(g, o, b.dense_list, b.dense_n, k);
    }
    *launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_allpairs(const StepConst &k, const DevBuffers &b, int from, bool diag, bool record_forces,
                            cudaStream_t st, uint64_t *launches)
{
    if (k.n == 0) return cudaSuccess;
    dim3 grid(blocks_for(k.n, kApTileI), blocks_for(k.n, kApTileJ));
    k_ap_pairs<<<grid, kApThreads, 0, st>>>(b.pos[from], b.vel[from], b.ap_cnt, b.ap_list, b.ap_cap, k);
    cudaError_t e = cudaGetLastError();
    ++*launches;
    if (e != cudaSuccess) return e;
    GridOut o{};
    if (diag) {
        o.dcnt = b.dcnt;
        o.dhash = b.dhash;
    } else {
        o.pos_out = b.pos[1 - from];
        o.vel_out = b.vel[1 - from];
        o.forces = record_forces ? b.forces : nullptr;
    }
    const unsigned nb = blocks_for(k.n, 128);
    if (diag) {
        k_ap_accumulate<true><<<nb, 128, 0, st>>>(b.pos[from], b.vel[from], b.ap_cnt, b.ap_list, b.ap_cap, o, k);
    } else {
        k_ap_accumulate<false><<<nb, 128, 0, st>>>(b.pos[from], b.vel[from], b.ap_cnt, b.ap_list, b.ap_cap, o, k);
    }
    ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_ref_cells(const StepConst &k, const float4 *pos, int32_t *cells8, cudaStream_t st,
                             uint64_t *launches)
{
    if (k.n == 0) return cudaSuccess;
    k_ref_cells<<<blocks_for(k.n, 256), 256, 0, st>>>(pos, cells8, k);
    ++*launches;
    return cudaGetLastError();
}

}  // namespace boidsgpu
