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
// Grid step = scan of cell counts -> the scatter into cell order, beside the
// classification of every full-size cell -> rule kernels that split the
// boids by the occupancy of their cell:
//   k_grid_sparse  one thread per boid; candidates of the 27 cells around it
//                  are filtered, exactly tested (the warp's hits dealt to all
//                  its lanes), and kept sorted by id; boids that need more
//                  than one pass are queued, with the neighbours their list
//                  could not keep, for
//   k_grid_sparse_more, which runs their further passes in full warps beside
//   k_grid_dense   one CTA per crowded cell; the 27-cell candidates are
//                  sorted by id once in shared memory, the exact tests mark
//                  rule masks, and ordered sums walk the masks in id order.
// Both integrate, write the new state in place of the sorted slot and bin it
// for the next step (cell key + rank from an atomic count).
#include "boids_engine.h"

#include <cuda_fp16.h>
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

// The cone tests redone with the exact cosine c = dot / (|v| * |r|)
// (correctly rounded division and square root, as the reference's floats).
// Kept out of line: it is rarely needed, and inlined the compiler would
// predicate it into every candidate test.
__device__ __noinline__ int cone_flags_exact(float dot, float nv, float d2, float lim0, float lim1, float lim2,
                                             float cs0, float cs1, float cs2, int round_mask)
{
    const float c = __fdiv_rn(dot, __fmul_rn(nv, __fsqrt_rn(d2)));
    const float lim[3] = {lim0, lim1, lim2}, cs[3] = {cs0, cs1, cs2};
    int f = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const bool in_cone = ((round_mask >> r) & 1) || (c >= cs[r] && c <= 1.0f);  // NaN: false
        if (d2 < lim[r] && in_cone) f |= 1 << r;
    }
    return f;
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
    // v . relativePos with relativePos = t - pi = -d: round-to-nearest is
    // symmetric under negation, so the reference's ((v.x r.x + v.y r.y) +
    // v.z r.z) is exactly the negated sum over d
    const float dot =
        -__fadd_rn(__fadd_rn(__fmul_rn(s.v.x, dx), __fmul_rn(s.v.y, dy)), __fmul_rn(s.v.z, dz));
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
        f = cone_flags_exact(dot, s.nv, d2, k.rule[0].d2_lim, k.rule[1].d2_lim, k.rule[2].d2_lim,
                             k.rule[0].cstar, k.rule[1].cstar, k.rule[2].cstar,
                             k.rule[0].all_round | (k.rule[1].all_round << 1) | (k.rule[2].all_round << 2));
    }
    return f;
}

struct Acc {
    float3 coh, sep, ali;
    int ncoh, nsep, nali;
    uint64_t h[3];
};
static_assert(sizeof(Acc) == kCarryBytes, "the carry buffer holds one Acc per slot");

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

// Device cells: side R' (>= the largest radius with margin) along y and z,
// R'/4 along x.  A y/z "row" of cells is contiguous in the sorted state, and
// the quarter-width x cells let a boid scan only the x-interval a sphere of
// radius R' reaches in each neighbouring row.
__device__ __forceinline__ int cell1(float x, const StepConst &k)
{
    const int c = __float2int_rz(__fmul_rn(x, k.inv_side));
    return min(max(c, 0), k.G - 1);
}

__device__ __forceinline__ int subcell_x(float x, const StepConst &k)
{
    const int c = __float2int_rz(__fmul_rn(x, k.inv_subx));
    return min(max(c, 0), k.Gx - 1);
}

__device__ __forceinline__ uint32_t cell_key(float3 p, const StepConst &k)
{
    return (uint32_t)((cell1(p.z, k) * k.G + cell1(p.y, k)) * k.Gx + subcell_x(p.x, k));
}

__device__ __forceinline__ uint32_t cell_start(const uint32_t *__restrict__ lstart,
                                               const uint32_t *__restrict__ bsum, uint32_t c)
{
    return __ldg(lstart + c) + __ldg(bsum + c / kScanTile);
}

// First state slot of global cell c of the flock described by k.
__device__ __forceinline__ uint32_t slot_start(const uint32_t *__restrict__ lstart,
                                               const uint32_t *__restrict__ bsum, uint32_t c, const StepConst &k)
{
    return cell_start(lstart, bsum, c) + k.slot_off;
}

// The constants of the flock that owns block blk of kSlotAlign slots, copied
// into shared memory by the whole CTA (ends with a barrier).
__device__ __forceinline__ void load_flock(StepConst &dst, const FlockTable &ft, uint32_t f)
{
    static_assert(sizeof(StepConst) % 4 == 0, "StepConst is copied as words");
    const uint32_t *src = reinterpret_cast<const uint32_t *>(ft.ks + f);
    uint32_t *d = reinterpret_cast<uint32_t *>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(StepConst) / 4); i += blockDim.x) d[i] = __ldg(src + i);
    __syncthreads();
}

// Where a rule kernel writes one boid's result.
struct GridOut {
    float4 *pos_out, *vel_out;
    uint32_t *key_out, *rank_out, *count;  // null for the all-pairs engine
    float *forces;
    int32_t *dcnt;
    uint64_t *dhash;
    Acc *carry;  // per slot: partial sums of huge cells between id windows (null: no windows)
    uint32_t *defer, *defer_cnt;  // k_grid_sparse's deferred boids: (slot, lo_id) pairs from the flock's slot_base,
                                  // and their count per flock (null: none)
    uint64_t *ovf;                // per slot, kOvfCap: a deferred boid's accepted neighbours beyond its list
    uint32_t *ovf_n;              // per slot: their number (null: not recorded)
    uint64_t *wscratch;           // k_grid_dense: wcap entries per CTA for bucketing huge cells' windows (null: none)
    uint32_t wcap;
};

template <bool DIAG>
__device__ __forceinline__ void finish_boid(const Acc &a, float4 p4, float3 vi, uint32_t s, const GridOut &o,
                                            const StepConst &k)
{
    // output row of the boid: its id, after the boids of earlier flocks
    const uint32_t id = __float_as_uint(p4.w) + (k.slot_base - k.slot_off);
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
        const uint32_t c = k.cell_base + cell_key(x, k);
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

// Packs ids [i0, i1) of an id-ordered state into float4 records, slot = id
// (w of pos = id bits).  With bad != null, a coordinate outside [0, hi] (or
// NaN) sets *bad.  With key != null the boid is also binned for the grid
// (k_grid_keys' work, fused): cell_key clamps every coordinate into the
// grid, so a state that fails the range check still bins in bounds.
__global__ void k_pack(const float *__restrict__ pos3, const float *__restrict__ vel3,
                       float4 *__restrict__ pos4, float4 *__restrict__ vel4, uint32_t i0, uint32_t i1,
                       uint32_t *__restrict__ bad, float hi, uint32_t *__restrict__ key,
                       uint32_t *__restrict__ rank, uint32_t *__restrict__ count, StepConst k)
{
    const uint32_t i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i1) return;
    const float x = pos3[3 * (size_t)i], y = pos3[3 * (size_t)i + 1], z = pos3[3 * (size_t)i + 2];
    pos4[i] = make_float4(x, y, z, __uint_as_float(i));
    vel4[i] = make_float4(vel3[3 * (size_t)i], vel3[3 * (size_t)i + 1], vel3[3 * (size_t)i + 2], 0.f);
    if (bad && !(x >= 0.f && x <= hi && y >= 0.f && y <= hi && z >= 0.f && z <= hi)) *bad = 1u;
    if (key) {
        const uint32_t c = k.cell_base + cell_key(make_float3(x, y, z), k);
        key[i] = c;
        rank[i] = atomicAdd(count + c, 1u);
    }
}

// Slot order -> id order (the reference's getters index by id), first pass:
// the slot of every id.  A valid state holds each id in [0, n) once; other
// ids are skipped.
__global__ void k_unpack_index(const float4 *__restrict__ pos4, uint32_t *__restrict__ slot_of, uint32_t n)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t id = __float_as_uint(__ldg(reinterpret_cast<const float *>(pos4) + 4 * (size_t)s + 3));
    if (id < n) slot_of[id] = s;
}

// Second pass, ids [i0, i1): a thread per id gathers its records, so that a
// warp's stores are contiguous (a thread per slot would scatter six 4-byte
// stores to random ids).
__global__ void k_unpack_gather(const float4 *__restrict__ pos4, const float4 *__restrict__ vel4,
                                const uint32_t *__restrict__ slot_of, float *__restrict__ pos3,
                                float *__restrict__ vel3, uint32_t i0, uint32_t i1, uint32_t n)
{
    const uint32_t i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i1) return;
    const uint32_t s = min(__ldg(slot_of + i), n - 1);
    if (pos3) {
        const float4 p = __ldg(pos4 + s);
        pos3[3 * (size_t)i] = p.x; pos3[3 * (size_t)i + 1] = p.y; pos3[3 * (size_t)i + 2] = p.z;
    }
    if (vel3) {
        const float4 v = __ldg(vel4 + s);
        vel3[3 * (size_t)i] = v.x; vel3[3 * (size_t)i + 1] = v.y; vel3[3 * (size_t)i + 2] = v.z;
    }
}

// One output frame in the .ptcl layout of src/main.cpp:246-277: position
// (+ get_force's nine floats) per boid, and optionally the velocity, both in
// id order.  A thread per state slot; the scattered stores land in L2.
__global__ void k_frame(const float4 *__restrict__ pos4, const float4 *__restrict__ vel4,
                        const float *__restrict__ force9, float *__restrict__ pframe,
                        float *__restrict__ vframe, int with_forces, uint32_t n)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const float4 p = pos4[s];
    const uint32_t id = __float_as_uint(p.w);
    const size_t stride = with_forces ? 12 : 3;
    float *o = pframe + stride * id;
    o[0] = p.x; o[1] = p.y; o[2] = p.z;
    if (with_forces) {
        const float *f = force9 ? force9 + (size_t)9 * id : nullptr;
#pragma unroll
        for (int c = 0; c < 9; ++c) o[3 + c] = f ? f[c] : 0.0f;
    }
    if (vframe) {
        const float4 v = vel4[s];
        vframe[(size_t)3 * id] = v.x; vframe[(size_t)3 * id + 1] = v.y; vframe[(size_t)3 * id + 2] = v.z;
    }
}

// ------------------------------------------------------------------ counting-sort binning

template <bool MULTI>
__global__ void k_grid_keys(const float4 *__restrict__ pos, uint32_t *__restrict__ key,
                            uint32_t *__restrict__ rank, uint32_t *__restrict__ count, StepConst kp, FlockTable ft)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (MULTI ? ft.nslots : kp.n)) return;
    const StepConst &k = MULTI ? ft.ks[ft.blk_flock[s / kSlotAlign]] : kp;
    if (s - k.slot_base >= k.n) return;  // padding between flocks
    const uint32_t c = k.cell_base + cell_key(xyz(pos[s]), k);
    key[s] = c;
    rank[s] = atomicAdd(count + c, 1u);
}

// Exclusive scan of the per-cell counts.  Each block scans one tile of
// kScanTile cells into lstart and publishes its total; the last block to
// finish (completion ticket, no waiting) turns the totals into tile offsets
// in bsum.  start(c) = lstart[c] + bsum[c / kScanTile].
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
            uint32_t *ticket, uint32_t nblocks)
{
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    __shared__ bool is_last;
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    const uint4 a = *reinterpret_cast<const uint4 *>(count + base);
    const uint4 b = *reinterpret_cast<const uint4 *>(count + base + 4);
    const uint32_t v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) sum += v[i];
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

template <bool MULTI>
__global__ void k_grid_scatter(const float4 *__restrict__ pin, const float4 *__restrict__ vin,
                               const uint32_t *__restrict__ key, const uint32_t *__restrict__ rank,
                               const uint32_t *__restrict__ lstart, const uint32_t *__restrict__ bsum,
                               float4 *__restrict__ pout, float4 *__restrict__ vout,
                               uint32_t *__restrict__ count_to_zero, uint32_t n, FlockTable ft)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t off = 0;
    if (MULTI) {
        if (s >= ft.nslots) return;
        const StepConst &k = ft.ks[ft.blk_flock[s / kSlotAlign]];
        if (s - k.slot_base >= k.n) return;
        off = k.slot_off;
    } else if (s >= n) {
        return;
    }
    const uint32_t c = key[s];
    const uint32_t d = cell_start(lstart, bsum, c) + rank[s] + off;
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

// Segment q of the 27 full-size cells around full-size cell (cx, cy, cz),
// in x-cell indices (4 per full-size cell).
__device__ __forceinline__ Seg segment(int cx, int cy, int cz, int q, int runs, const StepConst &k)
{
    const int G = k.G, Gx = k.Gx;
    const int row = q / runs, run = q - row * runs;
    int z = cz + row / 3 - 1, y = cy + row % 3 - 1;
    float sz = 0.f, sy = 0.f;
    if (z < 0) { z += G; sz = -k.Ff; } else if (z >= G) { z -= G; sz = k.Ff; }
    if (y < 0) { y += G; sy = -k.Ff; } else if (y >= G) { y -= G; sy = k.Ff; }
    const uint32_t r0 = (uint32_t)(z * G + y) * (uint32_t)Gx;
    const int x0 = 4 * cx;
    if (runs == 1) return Seg{r0 + x0 - 4, r0 + x0 + 8, 0.f, sy, sz};
    if (cx == 0) return run == 0 ? Seg{r0 + Gx - 4, r0 + Gx, -k.Ff, sy, sz} : Seg{r0, r0 + 8, 0.f, sy, sz};
    return run == 0 ? Seg{r0 + Gx - 8, r0 + Gx, 0.f, sy, sz} : Seg{r0, r0 + 4, k.Ff, sy, sz};
}

// Which kernel takes the boids of a full-size cell: k_grid_dense when the
// cell is crowded (dense_min boids or more), or holds defer_min or more with
// over cand_defer candidates in its 27 cells, or holds any boid with over
// lone_cand candidates (sorting a crowded neighbourhood once per cell beats
// sorting it per boid); else k_grid_sparse.  Cells with more than kDenseCap
// candidates need the dense kernel's id windows (windows != 0).
__device__ __forceinline__ bool dense_rule(uint32_t b, uint32_t ncand, const StepConst &k, int windows)
{
    const bool want = b >= k.dense_min || (b >= k.defer_min && ncand > k.cand_defer) || ncand > k.lone_cand;
    return b > 0 && want && (ncand <= (uint32_t)kDenseCap || windows);
}

// Per full-size cell, after the scan (from the cell starts alone, so that it
// can run beside the scatter): the dense flag the thread-per-boid kernel
// reads, and the dense kernel's work list.
template <bool MULTI>
__global__ void k_grid_classify(const uint32_t *__restrict__ lstart,
                                const uint32_t *__restrict__ bsum, uint8_t *__restrict__ dflag,
                                uint32_t *__restrict__ dense_list, uint32_t *__restrict__ dense_n, uint32_t nfull,
                                int windows, StepConst kp, FlockTable ft)
{
    const uint32_t cg = blockIdx.x * blockDim.x + threadIdx.x;
    if (cg >= nfull) return;
    // boids of the cell from the scan (the counts may be zeroed meanwhile by
    // the scatter, which runs beside this kernel)
    const uint32_t b = cell_start(lstart, bsum, 4 * cg + 4) - cell_start(lstart, bsum, 4 * cg);
    uint8_t flag = 0;
    if (b > 0) {
        uint32_t f = 0;
        if (MULTI) {  // the flock: last with cell4 <= cg
            uint32_t hi = ft.count;
            while (hi - f > 1) {
                const uint32_t mid = (f + hi) / 2;
                if (__ldg(ft.cell4 + mid) <= cg) f = mid; else hi = mid;
            }
        }
        const StepConst &k = MULTI ? ft.ks[f] : kp;
        const uint32_t c = cg - k.cell_base / 4;
        const int G = k.G;
        const int cx = (int)(c % G), cy = (int)((c / G) % G), cz = (int)(c / ((uint32_t)G * G));
        const int runs = seg_runs(cx, k);
        uint32_t ncand = 0;
        for (int q = 0; q < 9 * runs; ++q) {
            const Seg sg = segment(cx, cy, cz, q, runs, k);
            ncand += cell_start(lstart, bsum, k.cell_base + sg.c1) - cell_start(lstart, bsum, k.cell_base + sg.c0);
        }
        if (dense_rule(b, ncand, k, windows)) {
            flag = 1;
            const uint32_t items = (b + kDenseRound - 1) / kDenseRound;
            const uint32_t at = atomicAdd(dense_n, items);
            for (uint32_t r = 0; r < items; ++r) {
                dense_list[2 * (at + r)] = cg;
                dense_list[2 * (at + r) + 1] = r * kDenseRound;
            }
        }
    }
    dflag[cg] = flag;
}

// ------------------------------------------------------------------ sparse cells: thread per boid

// One thread per boid (slot).  In each of the 9 neighbouring y/z rows the
// boid scans only the x cells a sphere of radius sqrt(trim_r2) around it
// reaches, and drops rows it cannot reach.
//
// All lanes of a warp walk their own candidates in lock-step (a flat loop of
// max-over-warp length).  Candidates passing the squared-distance filter are
// buffered, and whenever one buffer is nearly full the warp runs the exact
// tests of all its lanes' hits, dealt to its lanes 32 at a time whichever
// lane found them, so the expensive test runs with nearly every lane busy.  The filter drops candidates behind the boid (the view-cone
// pre-test, StepConst::dot_eps).  Accepted neighbours are kept sorted by id,
// at most kListA per pass; a boid with more takes further passes, each
// keeping the next kListA ids, so accumulation is always in ascending id --
// for a single flock in k_grid_sparse_more, so that those passes run in full
// warps.  The per-boid tables (segments, hit buffer, sorted list) live in
// shared memory, one column per thread: as local memory they overflow L1 and
// every access goes to L2.
constexpr int kBufA = 13;
constexpr int kListA = kListCap;
constexpr int kRT = 128;      // threads of k_grid_sparse
constexpr int kSegA = 18;     // at most 9 rows x 2 runs (a run split where x wraps)
// Candidates loaded together in the filter loop: 3 keeps the kernel within
// 80 registers (6 CTAs per SM, as the shared tables allow) and is 1-2 %
// faster than 2; 4 takes 96 registers, 5 CTAs per SM, and is 6 % slower.
constexpr int kCandStep = 3;
static_assert(kBufA > kCandStep, "the hit buffer holds an iteration's hits");

struct GridIn {
    const float4 *__restrict__ pos;
    const float4 *__restrict__ vel;
    const uint32_t *__restrict__ lstart;
    const uint32_t *__restrict__ bsum;
    const uint8_t *__restrict__ dflag;  // per full-size cell: taken by k_grid_dense
};

struct SparseSmem {
    uint32_t seg0[kSegA][kRT];   // first slot | x shift << 29 | (z shift < 0) << 31
    uint32_t seg1[kSegA][kRT];   // end slot   | y shift << 29 | (z shift > 0) << 31
    uint32_t buf[kBufA][kRT];    // filter hits: slot | shifted << 31
    uint64_t lst[kListA][kRT];   // accepted neighbours, sorted: id << 32 | slot | flags << 29
};

// The segments of the boid at pi, whose full-size cell is (cy, cz) along y
// and z, into the thread's columns of sm.seg0/seg1: in each neighbour row,
// the x cells that a sphere of radius sqrt(trim_r2) around it reaches.
// Empty runs are not stored.  Returns the number of candidates.
__device__ __forceinline__ uint32_t sparse_segments(SparseSmem &sm, int t, float3 pi, int cy, int cz,
                                                    const GridIn &g, const StepConst &k)
{
    const int G = k.G, Gx = k.Gx;
    const float eps = k.side * 1e-5f;
    int nseg = 0;
    uint32_t ncand = 0;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        const int dz = r / 3 - 1, dy = r % 3 - 1;
        const float ddy = dy == 0 ? 0.f : fmaxf(0.f, dy < 0 ? pi.y - (float)cy * k.side - eps
                                                          : (float)(cy + 1) * k.side - pi.y - eps);
        const float ddz = dz == 0 ? 0.f : fmaxf(0.f, dz < 0 ? pi.z - (float)cz * k.side - eps
                                                          : (float)(cz + 1) * k.side - pi.z - eps);
        const float rem = k.trim_r2 - ddy * ddy - ddz * ddz;
        if (!(rem > 0.f)) continue;
        const float rx = sqrtf(rem);
        // a boid in the field reaches at most one row length beyond either
        // end; the clamp only keeps a state outside the field (never made
        // by the update, refused by boids_set_state) within the cell tables
        const int lo = max(__float2int_rd((pi.x - rx) * k.inv_subx), 1 - Gx);
        const int hi = min(__float2int_rd((pi.x + rx) * k.inv_subx), 2 * Gx - 2);
        int a0 = lo, a1 = hi + 1, c0 = 0, c1 = 0;  // x-cell runs [a0, a1) and [c0, c1)
        uint32_t ca = 0, cb = 0;  // x shifts of the runs, 2-bit two's complement: 3 = -F, 1 = +F
        if (lo < 0) { a0 = lo + Gx; a1 = Gx; ca = 3; c1 = min(hi + 1, Gx); }
        else if (hi >= Gx) { a1 = Gx; c1 = hi + 1 - Gx; cb = 1; }
        int zz = cz + dz, yy = cy + dy;
        zz = zz < 0 ? zz + G : (zz >= G ? zz - G : zz);
        yy = yy < 0 ? yy + G : (yy >= G ? yy - G : yy);
        const uint32_t rb = k.cell_base + (uint32_t)(zz * G + yy) * (uint32_t)Gx;
        // y and z shifts of the row, as the x shifts
        const uint32_t ysh = cy + dy < 0 ? 3u : (cy + dy >= G ? 1u : 0u);
        const uint32_t w0 = cz + dz < 0 ? 0x80000000u : 0u, w1 = (ysh << 29) | (cz + dz >= G ? 0x80000000u : 0u);
        if (a1 > a0) {
            const uint32_t j0 = slot_start(g.lstart, g.bsum, rb + a0, k), j1 = slot_start(g.lstart, g.bsum, rb + a1, k);
            if (j1 > j0) {
                sm.seg0[nseg][t] = j0 | (ca << 29) | w0;
                sm.seg1[nseg][t] = j1 | w1;
                ncand += j1 - j0;
                ++nseg;
            }
        }
        if (c1 > c0) {
            const uint32_t j0 = slot_start(g.lstart, g.bsum, rb + c0, k), j1 = slot_start(g.lstart, g.bsum, rb + c1, k);
            if (j1 > j0) {
                sm.seg0[nseg][t] = j0 | (cb << 29) | w0;
                sm.seg1[nseg][t] = j1 | w1;
                ncand += j1 - j0;
                ++nseg;
            }
        }
    }
    return ncand;
}

// The m neighbours of the thread's column of sm.lst (sorted by id) added to
// a in that order, each entry's loads issued one entry ahead.
template <bool DIAG>
__device__ __forceinline__ void list_accumulate(const SparseSmem &sm, int t, int m, float3 pi, Acc &a,
                                                const GridIn &g, const StepConst &k)
{
    uint64_t e_next = m > 0 ? sm.lst[0][t] : 0;
    float4 p_next = make_float4(0.f, 0.f, 0.f, 0.f), v_next = p_next;
    if (m > 0) {
        p_next = __ldg(g.pos + ((uint32_t)e_next & 0x1fffffffu));
        v_next = __ldg(g.vel + ((uint32_t)e_next & 0x1fffffffu));
    }
    for (int q = 0; q < m; ++q) {
        const uint64_t e = e_next;
        const float4 pj = p_next, vv = v_next;
        if (q + 1 < m) {
            e_next = sm.lst[q + 1][t];
            p_next = __ldg(g.pos + ((uint32_t)e_next & 0x1fffffffu));
            v_next = __ldg(g.vel + ((uint32_t)e_next & 0x1fffffffu));
        }
        const int f = (int)(((uint32_t)e) >> 29);
        const float3 tt = image3(xyz(pj), pi, k);
        const float3 vj = (f & 4) ? xyz(vv) : make_float3(0.f, 0.f, 0.f);
        acc_add<DIAG>(a, pi, tt, vj, f, (uint32_t)(e >> 32));
    }
}

// One pass of a warp (all lanes call it together) over the candidates of its
// lanes that still need one: the filter, the exact tests of the buffered
// hits, and the accepted neighbours with ids above lo_id kept sorted in the
// thread's column of sm.lst, at most kListA.  Those lanes then accumulate
// their list; a lane that accepted more than the list held keeps need and
// moves lo_id up to the last id it accumulated.  With ovf (this lane's row),
// every accepted neighbour that leaves the list or never enters it is
// appended there, up to kOvfCap of them, and counted in ovf_n.
template <bool DIAG>
__device__ __forceinline__ void sparse_pass(SparseSmem &sm, int t, uint32_t s, float3 pi, const Sight &sight,
                                            float dot_lim, uint32_t nc, bool &need, int64_t &lo_id, Acc &a,
                                            const GridIn &g, const StepConst &k, uint64_t *ovf, uint32_t &ovf_n)
{
    const float3 vi = sight.v;
    const uint32_t mine = need ? nc : 0;
    const uint32_t max_nc = __reduce_max_sync(0xffffffffu, mine);
    int m = 0, nb = 0;
    uint32_t more = 0;  // accepted neighbours with id > lo_id in this pass
    int qs = -1;
    uint32_t j = 0, jend = 0;  // global slots [j, jend) of the current segment
    uint32_t swrap = 0;        // 1 << 31 when the segment crosses a periodic face
    float qx = 0.f, qy = 0.f, qz = 0.f;
    // the next segment (none is empty): its slots and the query point
    auto advance = [&]() {
        ++qs;
        const uint32_t w0 = sm.seg0[qs][t], w1 = sm.seg1[qs][t];
        j = w0 & 0x1fffffffu;
        jend = w1 & 0x1fffffffu;
        // the candidate's image is pj + shift: test pj against pi - shift
        const int vx = (int)(w0 << 1) >> 30, vy = (int)(w1 << 1) >> 30;
        const int vz = (int)(w1 >> 31) - (int)(w0 >> 31);
        qx = __fmaf_rn(-__int2float_rn(vx), k.Ff, pi.x);
        qy = __fmaf_rn(-__int2float_rn(vy), k.Ff, pi.y);
        qz = __fmaf_rn(-__int2float_rn(vz), k.Ff, pi.z);
        swrap = ((w0 | w1) & 0xe0000000u) ? 0x80000000u : 0u;
    };
    auto filter = [&](float4 pj, float3 q, uint32_t jc, uint32_t wrap) {
        const float dx = pj.x - q.x, dy = pj.y - q.y, dz = pj.z - q.z;
        const float d2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
        const float dv = __fmaf_rn(vi.z, dz, __fmaf_rn(vi.y, dy, __fmul_rn(vi.x, dx)));
        if (d2 < k.filt_r2 && dv >= dot_lim && jc != s) sm.buf[nb++][t] = jc | wrap;
    };
    // kCandStep candidates per iteration, so that their loads are in flight
    // together; the buffers are flushed with room for the next kCandStep hits
    for (uint32_t it = 0; it < max_nc; it += kCandStep) {
        bool vc[kCandStep];
        uint32_t cc[kCandStep], sc[kCandStep];  // candidate slots and their wrap flags
        float3 qc[kCandStep];
        float4 pc[kCandStep];
#pragma unroll
        for (int u = 0; u < kCandStep; ++u) {
            vc[u] = it + u < mine;
            cc[u] = 0;
            sc[u] = 0;
            qc[u] = make_float3(0.f, 0.f, 0.f);
            if (vc[u]) {
                if (j == jend) advance();
                cc[u] = j++;
                qc[u] = make_float3(qx, qy, qz);
                sc[u] = swrap;
            }
        }
#pragma unroll
        for (int u = 0; u < kCandStep; ++u) pc[u] = vc[u] ? __ldg(g.pos + cc[u]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < kCandStep; ++u)
            if (vc[u]) filter(pc[u], qc[u], cc[u], sc[u]);
        // exact tests of the buffered hits, the whole warp together
        if (__any_sync(0xffffffffu, nb > kBufA - kCandStep) || it + kCandStep >= max_nc) {
            // The warp's hits are tested 32 at a time whatever lane found
            // them (hit i of the lanes' buffers laid end to end goes to lane
            // i % 32), so that a lane with many hits does not hold the warp
            // for as many rounds; each verdict goes back into the finder's
            // buffer (slot | rules << 29, rules 0: not accepted), and each
            // lane then files its own accepted hits in its sorted list.
            const int lane = t & 31, wbase = t & ~31;
            int incl = nb;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            const int excl = incl - nb;
            const int lo32 = (int)lo_id;  // ids are below 2^29
            __syncwarp();  // the buffers are written
            for (int base = 0; base < total; base += 32) {
                const int i = base + lane;
                int L = 0;  // the last lane whose hits start at or before i
#pragma unroll
                for (int st = 16; st > 0; st >>= 1) {
                    const int e = __shfl_sync(0xffffffffu, excl, L + st);
                    if (e <= i) L += st;
                }
                const int q = i - __shfl_sync(0xffffffffu, excl, L);
                const float3 po = make_float3(__shfl_sync(0xffffffffu, pi.x, L), __shfl_sync(0xffffffffu, pi.y, L),
                                              __shfl_sync(0xffffffffu, pi.z, L));
                Sight so;
                so.v = make_float3(__shfl_sync(0xffffffffu, sight.v.x, L), __shfl_sync(0xffffffffu, sight.v.y, L),
                                   __shfl_sync(0xffffffffu, sight.v.z, L));
                so.nv = __shfl_sync(0xffffffffu, sight.nv, L);
                so.inv_nv = __shfl_sync(0xffffffffu, sight.inv_nv, L);
                const int olo = __shfl_sync(0xffffffffu, lo32, L);
                if (i < total) {
                    const uint32_t wb = sm.buf[q][wbase + L];
                    const uint32_t jb = wb & 0x7fffffffu;
                    const float4 pj = __ldg(g.pos + jb);
                    int f = 0;
                    if ((int)__float_as_uint(pj.w) > olo) {
                        // a filter hit from a segment without periodic shift is
                        // nearer than F/2 on every axis: its own minimum image
                        const float3 tt = (wb >> 31) ? image3(xyz(pj), po, k) : xyz(pj);
                        f = pair_flags(po, so, tt, k);
                    }
                    sm.buf[q][wbase + L] = jb | ((uint32_t)f << 29);
                }
            }
            __syncwarp();  // the verdicts are written
            for (int q = 0; q < nb; ++q) {
                const uint32_t en = sm.buf[q][t];
                if (!(en >> 29)) continue;
                const uint32_t jb = en & 0x1fffffffu;
                const uint32_t idj = __float_as_uint(__ldg(&g.pos[jb].w));
                ++more;
                const uint64_t e = ((uint64_t)idj << 32) | (uint64_t)en;
                int w;
                if (m < kListA) {
                    w = m++;
                } else {
                    // the list is full: e or its last entry leaves it
                    const uint64_t last = sm.lst[kListA - 1][t];
                    w = e < last ? kListA - 1 : -1;
                    if (ovf) {
                        if (ovf_n < (uint32_t)kOvfCap) ovf[ovf_n] = w < 0 ? e : last;
                        ++ovf_n;
                    }
                    if (w < 0) continue;
                }
                while (w > 0 && sm.lst[w - 1][t] > e) { sm.lst[w][t] = sm.lst[w - 1][t]; --w; }
                sm.lst[w][t] = e;
            }
            __syncwarp();  // the buffers are free for the next hits
            nb = 0;
        }
    }
    if (need) {
        list_accumulate<DIAG>(sm, t, m, pi, a, g, k);
        if (more <= (uint32_t)m) need = false;
        else lo_id = (int64_t)(sm.lst[m - 1][t] >> 32);
    }
}

// A deferred boid's further passes from its overflow row (on <= kOvfCap
// entries, every accepted neighbour with an id above lo_id): the next
// kListA ids sorted in the thread's column of sm.lst and accumulated, until
// none is left.  Per lane; no candidate is walked again.
template <bool DIAG>
__device__ __forceinline__ void ovf_passes(SparseSmem &sm, int t, const uint64_t *__restrict__ row, uint32_t on,
                                           int64_t lo_id, float3 pi, Acc &a, const GridIn &g, const StepConst &k)
{
    for (;;) {
        int m = 0;
        uint32_t more = 0;
        for (uint32_t q = 0; q < on; ++q) {
            const uint64_t e = row[q];
            if ((int64_t)(e >> 32) <= lo_id) continue;
            ++more;
            int w;
            if (m < kListA) w = m++;
            else if (e < sm.lst[kListA - 1][t]) w = kListA - 1;
            else continue;
            while (w > 0 && sm.lst[w - 1][t] > e) { sm.lst[w][t] = sm.lst[w - 1][t]; --w; }
            sm.lst[w][t] = e;
        }
        list_accumulate<DIAG>(sm, t, m, pi, a, g, k);
        if (more <= (uint32_t)m) return;
        lo_id = (int64_t)(sm.lst[m - 1][t] >> 32);
    }
}

template <bool DIAG, bool MULTI>
__global__ void __launch_bounds__(kRT)
k_grid_sparse(GridIn g, GridOut o, StepConst kp, FlockTable ft)
{
    static_assert(kRT == kSlotAlign, "a CTA serves one flock");
    __shared__ SparseSmem sm;
    // the flock's constants (an ensemble's CTA serves one flock); one word otherwise
    __shared__ __align__(8) uint32_t kf_words[MULTI ? sizeof(StepConst) / 4 : 1];
    StepConst &kf = *reinterpret_cast<StepConst *>(kf_words);
    if (MULTI) load_flock(kf, ft, ft.blk_flock[blockIdx.x]);
    const StepConst &k = MULTI ? kf : kp;
    const int G = k.G;
    const int t = threadIdx.x;
    const int lane = t & 31, wid = t >> 5;
    const unsigned below = (1u << lane) - 1u;
    // This CTA's boids outside dense cells (the others are k_grid_dense's),
    // compacted onto its first threads so that warps run full and the
    // warps left over exit at once.
    // (cslot[t] is read only by thread t before it first writes its own
    // buffer column, which cslot shares)
    uint32_t *cslot = sm.buf[0];
    __shared__ uint32_t wcount[kRT / 32];
    const uint32_t s0 = blockIdx.x * kRT + t;
    bool mine = s0 - k.slot_base < k.n;
    if (mine) {
        const float4 q = g.pos[s0];
        const uint32_t fc = k.cell_base / 4 +
                            (uint32_t)((cell1(q.z, k) * G + cell1(q.y, k)) * G + cell1(q.x, k));
        mine = !__ldg(g.dflag + fc);
    }
    const unsigned bal = __ballot_sync(0xffffffffu, mine);
    if (lane == 0) wcount[wid] = __popc(bal);
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (int i = 0; i < kRT / 32; ++i) {
        if (i < wid) before += wcount[i];
        total += wcount[i];
    }
    if (mine) cslot[before + __popc(bal & below)] = s0;
    __syncthreads();
    if ((uint32_t)(wid * 32) >= total) return;  // the whole warp is idle
    const bool act = (uint32_t)t < total;
    const uint32_t s = act ? cslot[t] : s0;
    const float4 p4 = act ? g.pos[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 v4 = act ? g.vel[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float3 pi = xyz(p4);
    const uint32_t nc = act ? sparse_segments(sm, t, pi, cell1(pi.y, k), cell1(pi.z, k), g, k) : 0;
    const Sight sight = make_sight(xyz(v4));
    const float dot_lim = k.cone_pre ? -(sight.nv * k.dot_eps) : -INFINITY;  // cone pre-test
    Acc a;
    acc_zero(a);
    int64_t lo_id = -1;  // ids <= lo_id were accumulated by earlier passes
    bool need = act;
    uint32_t ovf_n = 0;
    sparse_pass<DIAG>(sm, t, s, pi, sight, dot_lim, nc, need, lo_id, a, g, k,
                      o.ovf && act ? o.ovf + (size_t)s * kOvfCap : nullptr, ovf_n);
    if (o.defer) {
        // Boids with more accepted neighbours than one list holds go to
        // k_grid_sparse_more with their partial sums: every further pass
        // walks all of a lane's candidates, however few lanes of the warp
        // still need one, and there they run in full warps.
        const unsigned nbal = __ballot_sync(0xffffffffu, need);
        uint32_t q0 = 0;
        if (lane == 0 && nbal) q0 = atomicAdd(o.defer_cnt + k.flock, (uint32_t)__popc(nbal));
        q0 = __shfl_sync(0xffffffffu, q0, 0);
        if (need) {
            const uint32_t q = k.slot_base + q0 + __popc(nbal & below);
            o.defer[2 * q] = s;
            o.defer[2 * q + 1] = (uint32_t)lo_id;
            o.carry[s] = a;
            if (o.ovf) o.ovf_n[s] = ovf_n;
        } else if (act) {
            finish_boid<DIAG>(a, p4, sight.v, s, o, k);
        }
        return;
    }
    while (__any_sync(0xffffffffu, need))
        sparse_pass<DIAG>(sm, t, s, pi, sight, dot_lim, nc, need, lo_id, a, g, k, nullptr, ovf_n);
    if (act) finish_boid<DIAG>(a, p4, sight.v, s, o, k);
}

// The boids k_grid_sparse deferred: thread per queued boid, its segments
// recomputed, further passes from its partial sums.  A single flock's queue
// is walked grid-stride; in an ensemble CTA b takes the b-th block of 128
// entries of its flock's queue (the flock of slot block b), so that a CTA
// serves one flock.
template <bool DIAG, bool MULTI>
__global__ void __launch_bounds__(kRT)
k_grid_sparse_more(GridIn g, GridOut o, StepConst kp, FlockTable ft)
{
    __shared__ SparseSmem sm;
    __shared__ __align__(8) uint32_t kf_words[MULTI ? sizeof(StepConst) / 4 : 1];
    StepConst &kf = *reinterpret_cast<StepConst *>(kf_words);
    const int t = threadIdx.x;
    uint32_t first = 0, count, stride;  // entries [first + base, first + count), base += stride
    uint32_t base = blockIdx.x * kRT;
    if (MULTI) {
        const uint32_t f = ft.blk_flock[blockIdx.x];
        const uint32_t sb = __ldg(&ft.ks[f].slot_base);
        count = o.defer_cnt[f];
        base = blockIdx.x * kRT - sb;  // this CTA's block of the flock's queue
        if (base >= count) return;     // uniform over the CTA
        first = sb;
        stride = count;                // one block per CTA
        load_flock(kf, ft, f);
    } else {
        count = o.defer_cnt[0];
        stride = gridDim.x * kRT;
    }
    const StepConst &k = MULTI ? kf : kp;
    for (; base < count; base += stride) {
        if (base + (uint32_t)(t & ~31) >= count) break;  // the whole warp is idle
        const uint32_t i = base + t;
        const bool act = i < count;
        const uint32_t s = act ? o.defer[2 * (first + i)] : 0u;
        int64_t lo_id = act ? (int64_t)o.defer[2 * (first + i) + 1] : -1;
        Acc a;
        if (act) a = o.carry[s];
        else acc_zero(a);
        const float4 p4 = act ? g.pos[s] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 v4 = act ? g.vel[s] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float3 pi = xyz(p4);
        // a boid whose first pass recorded all the neighbours it could not
        // keep takes them from its overflow row; the others walk their
        // candidates again
        const uint32_t on = act && o.ovf ? o.ovf_n[s] : (uint32_t)kOvfCap + 1;
        const bool from_row = on <= (uint32_t)kOvfCap;
        if (from_row) ovf_passes<DIAG>(sm, t, o.ovf + (size_t)s * kOvfCap, on, lo_id, pi, a, g, k);
        bool need = act && !from_row;
        const uint32_t nc = need ? sparse_segments(sm, t, pi, cell1(pi.y, k), cell1(pi.z, k), g, k) : 0;
        const Sight sight = make_sight(xyz(v4));
        const float dot_lim = k.cone_pre ? -(sight.nv * k.dot_eps) : -INFINITY;
        uint32_t ovf_n = 0;
        while (__any_sync(0xffffffffu, need))
            sparse_pass<DIAG>(sm, t, s, pi, sight, dot_lim, nc, need, lo_id, a, g, k, nullptr, ovf_n);
        if (act) finish_boid<DIAG>(a, p4, sight.v, s, o, k);
    }
}

// ------------------------------------------------------------------ dense cells: CTA per cell

// Stable LSD radix sort of n 64-bit keys held in shared memory, on bits
// [lo, lo + nbits), kRadixBits bits per pass; NT threads each own a
// contiguous run.  hist holds kRadixWords(NT) words: counter i lives at
// i + i / 16, which keeps the (digit, thread) column walks free of bank
// conflicts.  Returns the buffer that holds the sorted keys.  It is the
// CTA-per-cell kernel's fallback sort (block_bucket_sort), so it favours a
// small counter table over few passes.
__device__ __forceinline__ int hpad(int i) { return i + (i >> 4); }
constexpr int kRadixBits = 2, kRadixDigits = 1 << kRadixBits;
__host__ __device__ constexpr int kRadixWords(int nt) { return kRadixDigits * nt + kRadixDigits * nt / 16; }

template <int NT>
__device__ uint64_t *block_radix_sort(uint64_t *a, uint64_t *b, uint32_t *hist, int n, int lo, int nbits)
{
    __shared__ uint32_t wsum[NT / 32];
    constexpr int D = kRadixDigits;
    const int t = threadIdx.x;
    // an odd run length keeps the threads' 64-bit reads a[t * K + i] at most
    // 2-way bank conflicted
    const int K = ((n + NT - 1) / NT) | 1;
    const int i0 = min(n, t * K), i1 = min(n, i0 + K);
    for (int bit = lo; bit < lo + nbits; bit += kRadixBits) {
#pragma unroll
        for (int d = 0; d < D; ++d) hist[hpad(d * NT + t)] = 0;
        for (int i = i0; i < i1; ++i) hist[hpad((int)((uint32_t)(a[i] >> bit) & (D - 1)) * NT + t)]++;
        __syncthreads();
        // exclusive scan of hist in (digit, thread) order; thread t owns D entries
        uint32_t loc[D], sum = 0;
#pragma unroll
        for (int q = 0; q < D; ++q) { loc[q] = hist[hpad(D * t + q)]; sum += loc[q]; }
        uint32_t total;
        uint32_t pre = block_excl_scan<NT>(sum, wsum, total);
#pragma unroll
        for (int q = 0; q < D; ++q) { hist[hpad(D * t + q)] = pre; pre += loc[q]; }
        __syncthreads();
        for (int i = i0; i < i1; ++i) {
            const uint64_t v = a[i];
            b[hist[hpad((int)((uint32_t)(v >> bit) & (D - 1)) * NT + t)]++] = v;
        }
        __syncthreads();
        uint64_t *tmp = a; a = b; b = tmp;
    }
    return a;
}

// Sort of n (<= kDenseCap) 64-bit keys (id << 16 | payload) by id, ids
// distinct: one bucket pass over the ids' actual range, then each key's place
// inside its bucket by counting the smaller ids there.  Keys whose ids bunch
// into a few buckets (more than kBucketMax in one) go to the radix sort
// instead, so the result never depends on the id distribution and the cost
// never grows quadratically.  NT threads; `cnt` holds kRadixWords(NT) >=
// kBuckets + 1 words.
// Returns the buffer that holds the sorted keys.
constexpr int kBuckets = 512;
constexpr int kBucketMax = 24;
static_assert(kRadixWords(128) >= kBuckets + 1, "the bucket counters fit the radix table");

template <int NT>
__device__ uint64_t *block_bucket_sort(uint64_t *a, uint64_t *b, uint32_t *cnt, int n, int id_bits)
{
    static_assert(kBuckets % NT == 0, "buckets per thread");
    constexpr int kPer = kBuckets / NT;
    __shared__ uint32_t red[2][NT / 32];
    __shared__ uint32_t info[2];  // id shift, largest bucket
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    // the ids' range
    uint32_t mn = 0xffffffffu, mx = 0;
    for (int i = t; i < n; i += NT) {
        const uint32_t id = (uint32_t)(a[i] >> 16);
        mn = min(mn, id);
        mx = max(mx, id);
    }
    mn = __reduce_min_sync(0xffffffffu, mn);
    mx = __reduce_max_sync(0xffffffffu, mx);
    if (lane == 0) { red[0][wid] = mn; red[1][wid] = mx; }
    for (int i = t; i <= kBuckets; i += NT) cnt[i] = 0;
    __syncthreads();
    mn = red[0][0];
    mx = red[1][0];
#pragma unroll
    for (int w = 1; w < NT / 32; ++w) { mn = min(mn, red[0][w]); mx = max(mx, red[1][w]); }
    // bucket = (id - mn) >> shift, shift the least with range >> shift < kBuckets
    const uint32_t range = n > 0 ? mx - mn : 0;
    const int shift = range < (uint32_t)kBuckets ? 0 : 32 - __clz(range) - 9;  // kBuckets = 2^9
    // each key's rank among its bucket's arrivals, and the bucket counts
    uint32_t rk[kDenseCap / NT], bk[kDenseCap / NT];
#pragma unroll
    for (int r = 0; r < kDenseCap / NT; ++r) {
        const int i = t + r * NT;
        if (i < n) {
            bk[r] = ((uint32_t)(a[i] >> 16) - mn) >> shift;
            rk[r] = atomicAdd(&cnt[bk[r]], 1u);
        }
    }
    __syncthreads();
    // exclusive scan of the counts; the largest bucket
    uint32_t loc[kPer], sum = 0, big = 0;
#pragma unroll
    for (int q = 0; q < kPer; ++q) { loc[q] = cnt[t * kPer + q]; sum += loc[q]; big = max(big, loc[q]); }
    big = __reduce_max_sync(0xffffffffu, big);
    if (lane == 0) red[1][wid] = big;
    uint32_t total;
    uint32_t pre = block_excl_scan<NT>(sum, red[0], total);
#pragma unroll
    for (int q = 0; q < kPer; ++q) { cnt[t * kPer + q] = pre; pre += loc[q]; }
    if (t == 0) {
        uint32_t m = 0;
#pragma unroll
        for (int w = 0; w < NT / 32; ++w) m = max(m, red[1][w]);
        info[1] = m;
    }
    if (t == NT - 1) cnt[kBuckets] = pre;
    __syncthreads();
    if (info[1] > (uint32_t)kBucketMax) return block_radix_sort<NT>(a, b, cnt, n, 16, id_bits);
    // file the keys by bucket, then place each inside its bucket
#pragma unroll
    for (int r = 0; r < kDenseCap / NT; ++r) {
        const int i = t + r * NT;
        if (i < n) b[cnt[bk[r]] + rk[r]] = a[i];
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kDenseCap / NT; ++r) {
        const int i = t + r * NT;
        if (i < n) {
            const uint32_t b0 = cnt[bk[r]], b1 = cnt[bk[r] + 1];
            const uint64_t key = b[b0 + rk[r]];
            const uint32_t id = (uint32_t)(key >> 16);
            uint32_t below = 0;
            for (uint32_t j = b0; j < b1; ++j) below += (uint32_t)(b[j] >> 16) < id;
            a[b0 + below] = key;
        }
    }
    __syncthreads();
    return a;
}

constexpr int kDT = 128;                       // threads of k_grid_dense
constexpr int kDenseKT = kDenseCap / kDT;      // candidates per thread when the list is full

constexpr int kMaxCuts = 32;                   // id windows of a huge cell planned at once

// Accepted neighbours are marked in three bit masks per boid (cohesion,
// separation, alignment) over the id-ordered candidate list; the ordered sums
// then walk the masks.  kMaskWords words hold the masks of one round of
// boids, so a round takes at most kMaskWords / (3 * words) boids.
constexpr int kMaskWords = kDenseCap + kRadixWords(kDT);
// At most kSumsMax boids per round: the per-boid table of the exact tests and
// the per-boid results of the ordered sums hold that many.
constexpr int kSumsMax = 72;
// Filter hits queued per warp for the exact tests: a filter iteration adds at
// most two per lane, so the queue is flushed once it holds kQueue - 64.
constexpr int kQueue = 192;

// Shared memory of k_grid_dense.  Regions whose lifetimes do not overlap
// share storage: the sort keys become the id-ordered candidate array, the
// gather slots and radix histogram become the rule masks, and the filter-hit
// buffers become the per-boid sums.
struct DenseSmem {
    union {
        uint64_t keys[2][kDenseCap];  // (id << 16) | (segment << 11) | gather index
        float4 spos[kDenseCap];       // candidates in id order, periodic images; w = slot
    } u;
    union {
        struct {
            uint32_t gslot[kDenseCap];      // state slot, by gather index
            uint32_t hist[kRadixWords(kDT)];  // sort counters (block_bucket_sort, block_radix_sort)
        } s;
        uint32_t masks[kMaskWords];         // rule r of round boid i: words (r * nbr + i) * wstride ...
    } v;
    union {
        struct {
            uint32_t queue[kDT / 32][kQueue];  // per warp: filter hits, round boid << 11 | candidate
            float4 obs[2][kSumsMax];           // per round boid: (position, |v|), (velocity, 1/|v|)
        } a;
        Acc sums[kSumsMax];                    // the ordered sums of each boid of the round
    } w;
    uint32_t seg_j0[18], seg_k0[19];
    float seg_s[18][3];
    uint32_t work, flock;
    uint32_t nw, cut;              // huge cells: window size, histogram cut
    uint32_t wcut[kMaxCuts], nwcut, wbin;  // huge cells: planned window ends (in bins of wbin ids)
    uint32_t woff[kMaxCuts + 1];           // and, when bucketed, each planned window's first scratch entry
    uint32_t wbucketed;
    uint32_t wtot[kDT / 32];       // block scan scratch
    float svx[kDenseCap], svy[kDenseCap], svz[kDenseCap];  // candidates' velocities, id order
    // candidates' coordinates relative to the cell centre, scaled by hsc, in
    // half precision, two candidates per word (one pad entry for odd counts)
    __half2 hx[kDenseCap / 2 + 1], hy[kDenseCap / 2 + 1], hz[kDenseCap / 2 + 1];
    StepConst kf;  // the current cell's flock (batched ensembles)
};
static_assert(kDenseCap <= 2048, "gather index must fit 11 bits");

// The candidates of the id-ordered list hold their periodic images as seen
// from the cell, exactly as the reference computes them: a candidate of a
// segment across a periodic face is shifted by the field size on that axis
// ((float)((double)x -+ F)), the others are unshifted.  That is the
// reference's own minimum image for every pair it can accept: such a pair is
// nearer than the largest sight radius R, which is at most F/3 (at least 3
// device cells per axis), so across a face the reference's test
// |xj - xi| > F/2 holds (|xj - xi| > F - R) and inside the field it fails
// (|xj - xi| < R).  Where the reference images a candidate otherwise, it is
// farther than R from the boid in both placements and no rule accepts it.

// The ordered sums of a round's boids run as jobs, each a (job, boid) pair
// taken by one lane, job-major so that the lanes of a warp run the same code:
// jobs 0-5 are the cohesion sum's x, y, z and the alignment sum's x, y, z
// (jobs 0 and 3 also count), job 6 the separation sum (all three components,
// from the normalised offsets), job 7 the neighbour-set id hashes
// (diagnostics only).  Each walks its rule's mask word by word from candidate
// 0 up: ascending id, the reference's order of accumulation, so every float
// sum is the reference's sequence of additions.  A job's running value starts
// from the earlier id windows' partial sums (carry) or zero, and ends in out.
__device__ __forceinline__ void dense_sum_job(const DenseSmem &sm, const uint32_t *m, uint32_t words, uint32_t job,
                                              const Acc *carry, Acc &out)
{
    const bool coh = job < 3;
    const uint32_t c = job % 3;
    // the summands: the candidates' imaged positions, or their velocities
    const float *base = coh ? reinterpret_cast<const float *>(sm.u.spos) + c
                            : (c == 0 ? sm.svx : (c == 1 ? sm.svy : sm.svz));
    const uint32_t sh = coh ? 2u : 0u;  // element q at base[q << sh]
    float *dst = reinterpret_cast<float *>(&out) + (coh ? 0 : 6) + c;
    float acc = carry ? reinterpret_cast<const float *>(carry)[(coh ? 0 : 6) + c] : 0.f;
    int cnt = 0;
    uint32_t next = words > 0 ? m[0] : 0u;  // each mask word is read one word ahead
    for (uint32_t w = 0; w < words; ++w) {
        uint32_t bits = next;
        if (w + 1 < words) next = m[w + 1];
        cnt += __popc(bits);
        const uint32_t q0 = w * 32;
        // four entries per iteration: their loads in flight together, their
        // additions in order
        while (bits) {
            const uint32_t b0 = (uint32_t)__ffs(bits) - 1;
            bits &= bits - 1;
            const bool h1 = bits != 0;
            const uint32_t b1 = h1 ? (uint32_t)__ffs(bits) - 1 : b0;
            bits &= bits - 1;
            const bool h2 = bits != 0;
            const uint32_t b2 = h2 ? (uint32_t)__ffs(bits) - 1 : b0;
            bits &= bits - 1;
            const bool h3 = bits != 0;
            const uint32_t b3 = h3 ? (uint32_t)__ffs(bits) - 1 : b0;
            bits &= bits - 1;
            const float v0 = base[(q0 + b0) << sh], v1 = base[(q0 + b1) << sh];
            const float v2 = base[(q0 + b2) << sh], v3 = base[(q0 + b3) << sh];
            acc = __fadd_rn(acc, v0);
            if (h1) acc = __fadd_rn(acc, v1);
            if (h2) acc = __fadd_rn(acc, v2);
            if (h3) acc = __fadd_rn(acc, v3);
        }
    }
    *dst = acc;
    if (c == 0) {
        int *n = coh ? &out.ncoh : &out.nali;
        *n = cnt + (carry ? (coh ? carry->ncoh : carry->nali) : 0);
    }
}

// Job 6: the separation sum (Vector3D::normalized of pi - t, as acc_add).
__device__ __forceinline__ void dense_sep_job(const DenseSmem &sm, const uint32_t *m, uint32_t words, float3 pi,
                                              const Acc *carry, Acc &out)
{
    float3 sep = carry ? carry->sep : make_float3(0.f, 0.f, 0.f);
    int cnt = carry ? carry->nsep : 0;
    uint32_t next = words > 0 ? m[0] : 0u;
    for (uint32_t w = 0; w < words; ++w) {
        uint32_t bits = next;
        if (w + 1 < words) next = m[w + 1];
        cnt += __popc(bits);
        while (bits) {
            const uint32_t q = w * 32 + (uint32_t)(__ffs(bits) - 1);
            bits &= bits - 1;
            const float4 t = sm.u.spos[q];
            const float dx = __fsub_rn(pi.x, t.x), dy = __fsub_rn(pi.y, t.y), dz = __fsub_rn(pi.z, t.z);
            const float n = nrm3(dx, dy, dz);
            sep.x = __fadd_rn(sep.x, __fdiv_rn(dx, n));
            sep.y = __fadd_rn(sep.y, __fdiv_rn(dy, n));
            sep.z = __fadd_rn(sep.z, __fdiv_rn(dz, n));
        }
    }
    out.sep = sep;
    out.nsep = cnt;
}

// Job 7 (diagnostics): the order-free id fingerprints of the three sets.
__device__ __forceinline__ void dense_hash_job(const DenseSmem &sm, const uint32_t *m0, uint32_t rstride,
                                               uint32_t words, const Acc *carry, Acc &out,
                                               const float4 *__restrict__ pos)
{
    for (uint32_t r = 0; r < 3; ++r) {
        const uint32_t *m = m0 + r * rstride;
        uint64_t h = carry ? carry->h[r] : 0;
        for (uint32_t w = 0; w < words; ++w) {
            uint32_t bits = m[w];
            while (bits) {
                const uint32_t q = w * 32 + (uint32_t)(__ffs(bits) - 1);
                bits &= bits - 1;
                const uint32_t j = __float_as_uint(sm.u.spos[q].w);
                h += id_hash(__float_as_uint(__ldg(&pos[j].w)));
            }
        }
        out.h[r] = h;
    }
}

// Id window of a huge cell (more than kDenseCap candidates): the largest hi
// such that the candidates with ids in [lo, hi) fit the shared list.  A
// histogram of the candidates' ids over kWinBins bins is cut where the
// running count passes kDenseCap; if the first bin alone is over, the span
// narrows to that bin.  A boid is a candidate at most once (G >= 3), so a
// bin one id wide always fits and the search ends.
constexpr int kWinBins = 1024;

__device__ uint32_t dense_window(DenseSmem &sm, const GridIn &g, int ns, uint32_t lo, uint32_t nid)
{
    static_assert(kWinBins * 4 <= sizeof(sm.u.keys[0]), "window histogram lives in the first sort buffer");
    static_assert(kWinBins % kDT == 0, "bins per thread");
    constexpr int kPer = kWinBins / kDT;
    uint32_t *hist = reinterpret_cast<uint32_t *>(sm.u.keys[0]);
    const int t = threadIdx.x;
    uint32_t span_hi = nid;
    for (;;) {
        const uint32_t w = (span_hi - lo + kWinBins - 1) / kWinBins;
        for (int i = t; i < kWinBins; i += kDT) hist[i] = 0;
        if (t == 0) sm.cut = kWinBins;
        __syncthreads();
        for (int sgi = 0; sgi < ns; ++sgi) {
            const uint32_t j0 = sm.seg_j0[sgi], len = sm.seg_k0[sgi + 1] - sm.seg_k0[sgi];
            for (uint32_t q = t; q < len; q += kDT) {
                const uint32_t id = __float_as_uint(__ldg(&g.pos[j0 + q].w));
                if (id >= lo && id < span_hi) atomicAdd(&hist[(id - lo) / w], 1u);
            }
        }
        __syncthreads();
        uint32_t loc = 0;
#pragma unroll 8
        for (int i = 0; i < kPer; ++i) loc += hist[t * kPer + i];
        uint32_t total;
        uint32_t run = block_excl_scan<kDT>(loc, sm.wtot, total);
        if (run + loc > (uint32_t)kDenseCap) {
            for (int i = 0; i < kPer; ++i) {
                run += hist[t * kPer + i];
                if (run > (uint32_t)kDenseCap) {
                    atomicMin(&sm.cut, (uint32_t)(t * kPer + i));
                    break;
                }
            }
        }
        __syncthreads();
        const uint32_t cut = sm.cut;
        __syncthreads();  // hist and cut are rewritten next
        if (cut >= (uint32_t)kWinBins) return span_hi;
        if (cut > 0) return lo + cut * w;
        span_hi = lo + w;  // w > 1 here: a one-id bin holds at most one candidate
    }
}

// The id windows of a huge cell planned from one histogram of its
// candidates' ids over [0, nid) (kWinBins bins of wbin ids): window ends are
// cut greedily where the running count would pass kDenseCap, at most
// kMaxCuts of them.  Windows beyond the plan, or past a single bin that alone
// overflows the list, are cut by dense_window instead.  One histogram pass
// for all windows, where dense_window needs one per window.  With a scratch
// of cap entries (this CTA's) that holds the planned windows, a second pass
// files the candidates by bin, and each planned window is then read from
// the scratch instead of scanning the whole neighbourhood again; an entry is
// id << 34 | segment << 29 | slot.

__device__ void dense_window_plan(DenseSmem &sm, const GridIn &g, int ns, uint32_t nid, uint64_t *scratch,
                                  uint32_t cap)
{
    static_assert((kWinBins + 1) * 4 <= sizeof(sm.u), "the prefix counts live in the sort buffers");
    static_assert(kWinBins % kDT == 0, "bins per thread");
    constexpr int kPer = kWinBins / kDT;
    uint32_t *hist = reinterpret_cast<uint32_t *>(&sm.u);
    const int t = threadIdx.x;
    const uint32_t w = (nid + kWinBins - 1) / kWinBins;
    for (int i = t; i <= kWinBins; i += kDT) hist[i] = 0;
    __syncthreads();
    for (int sgi = 0; sgi < ns; ++sgi) {
        const uint32_t j0 = sm.seg_j0[sgi], len = sm.seg_k0[sgi + 1] - sm.seg_k0[sgi];
        for (uint32_t q = t; q < len; q += kDT) atomicAdd(&hist[__float_as_uint(__ldg(&g.pos[j0 + q].w)) / w], 1u);
    }
    __syncthreads();
    // exclusive prefix: hist[b] = candidates in bins below b, hist[kWinBins] = all
    uint32_t loc[kPer], sum = 0;
#pragma unroll
    for (int i = 0; i < kPer; ++i) { loc[i] = hist[t * kPer + i]; sum += loc[i]; }
    uint32_t total;
    uint32_t pre = block_excl_scan<kDT>(sum, sm.wtot, total);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kPer; ++i) { hist[t * kPer + i] = pre; pre += loc[i]; }
    if (t == kDT - 1) hist[kWinBins] = pre;
    __syncthreads();
    if (t == 0) {
        uint32_t start = 0, nc = 0;
        while (start < (uint32_t)kWinBins && nc < (uint32_t)kMaxCuts) {
            const uint32_t target = hist[start] + (uint32_t)kDenseCap;
            uint32_t lo_b = start, hi_b = kWinBins + 1;  // hist[lo_b] <= target < hist[hi_b]
            while (hi_b - lo_b > 1) {
                const uint32_t mid = (lo_b + hi_b) / 2;
                if (hist[mid] <= target) lo_b = mid; else hi_b = mid;
            }
            if (lo_b == start) break;  // bin `start` alone holds more than the list
            sm.wcut[nc++] = lo_b;
            start = lo_b;
        }
        sm.nwcut = nc;
        sm.wbin = w;
        sm.woff[0] = 0;
        for (uint32_t c = 0; c < nc; ++c) sm.woff[c + 1] = hist[sm.wcut[c]];
        // bucket the planned windows' candidates when the scratch holds them
        sm.wbucketed = nc > 0 && scratch != nullptr && sm.woff[nc] <= cap;
    }
    __syncthreads();
    if (!sm.wbucketed) return;
    // File every candidate of the planned windows at its bin's next entry
    // (the prefix counts become running ends): a window is then the
    // contiguous run woff[c] .. woff[c + 1] of the scratch, in bin order.
    const uint32_t last_bin = sm.wcut[sm.nwcut - 1];
    for (int sgi = 0; sgi < ns; ++sgi) {
        const uint32_t j0 = sm.seg_j0[sgi], len = sm.seg_k0[sgi + 1] - sm.seg_k0[sgi];
        for (uint32_t q = t; q < len; q += kDT) {
            const uint32_t slot = j0 + q;
            const uint32_t id = __float_as_uint(__ldg(&g.pos[slot].w));
            const uint32_t bin = id / w;
            if (bin < last_bin)
                scratch[atomicAdd(&hist[bin], 1u)] = ((uint64_t)id << 34) | ((uint64_t)sgi << 29) | slot;
        }
    }
    __syncthreads();
}

// One CTA takes one work item at a time (dynamic queue): a crowded cell and
// up to 128 of its boids (a cell with more boids is several items, taken by
// several CTAs).  The cell's 27-cell candidates are radix-sorted by id once
// per item.  The item's boids go in rounds; the round's nbr boids x the
// candidate list is split over all threads: each boid gets L = 128/nbr
// lanes, lane l walks chunk l of the id-ordered list with the
// half-precision filter and exact tests, and marks the accepted neighbours
// in the boid's three rule masks (bit q = candidate q).  The ordered sums
// then run as jobs, one float sum (or the separation sum) per lane of the
// boid, each walking its mask from candidate 0 up: ascending id, as the
// reference accumulates.  A cell with more than kDenseCap candidates is done
// in ascending id windows that each fit the list; the sums are carried from
// window to window through o.carry.
template <bool DIAG, bool MULTI>
__global__ void __launch_bounds__(kDT, kDenseCtasPerSm)
k_grid_dense(GridIn g, GridOut o, const uint32_t *__restrict__ dense_list, uint32_t *__restrict__ dense_n,
             StepConst kp, FlockTable ft)
{
    extern __shared__ __align__(16) unsigned char dense_smem_raw[];
    DenseSmem &sm = *reinterpret_cast<DenseSmem *>(dense_smem_raw);
    const int t = threadIdx.x;
    for (;;) {
        if (t == 0) sm.work = atomicAdd(dense_n + 1, 1u);
        __syncthreads();
        const uint32_t w = sm.work;
        if (w >= dense_n[0]) break;
        const uint32_t cg = dense_list[2 * w];        // global full-size cell
        const uint32_t rbeg = dense_list[2 * w + 1];  // the item's first boid of the cell
        if (MULTI) {
            if (t == 0) {  // the flock: last with cell4 <= cg
                uint32_t lo = 0, hi = ft.count;
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) / 2;
                    if (__ldg(ft.cell4 + mid) <= cg) lo = mid; else hi = mid;
                }
                sm.flock = lo;
            }
            __syncthreads();
            load_flock(sm.kf, ft, sm.flock);
        }
        const StepConst &k = MULTI ? sm.kf : kp;
        const uint32_t c = cg - k.cell_base / 4;  // full-size cell inside the flock
        const int G = k.G;
        const int cx = (int)(c % G), cy = (int)((c / G) % G), cz = (int)(c / ((uint32_t)G * G));
        const int runs = seg_runs(cx, k), ns = 9 * runs;
        if (t < 32) {  // the segments, and their starts in the gather order (a warp scan of their lengths)
            uint32_t len = 0;
            if (t < ns) {
                const Seg sg = segment(cx, cy, cz, t, runs, k);
                const uint32_t j0 = slot_start(g.lstart, g.bsum, k.cell_base + sg.c0, k);
                len = slot_start(g.lstart, g.bsum, k.cell_base + sg.c1, k) - j0;
                sm.seg_j0[t] = j0;
                sm.seg_s[t][0] = sg.sx; sm.seg_s[t][1] = sg.sy; sm.seg_s[t][2] = sg.sz;
            }
            uint32_t incl = len;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (t >= o) incl += y;
            }
            if (t < ns) sm.seg_k0[t + 1] = incl;
            if (t == 0) sm.seg_k0[0] = 0;
        }
        __syncthreads();
        const uint32_t ncand = sm.seg_k0[ns];
        const uint32_t own0 = slot_start(g.lstart, g.bsum, 4 * cg, k);
        const uint32_t b = slot_start(g.lstart, g.bsum, 4 * cg + 4, k) - own0;
        const bool huge = ncand > (uint32_t)kDenseCap;
        if (huge && !o.carry) {  // not listed so by k_grid_classify; kept for safety
            __syncthreads();
            continue;
        }

        if (huge)
            dense_window_plan(sm, g, ns, k.n, o.wscratch ? o.wscratch + (size_t)blockIdx.x * o.wcap : nullptr,
                              o.wcap);
        uint32_t lo = 0;  // this window's ids: [lo, hi)
        uint32_t wi = 0;  // windows done
        for (;;) {
            uint32_t hi = k.n, nw = ncand;
            if (huge) {
                const bool planned = wi < sm.nwcut;
                hi = planned ? min(k.n, sm.wcut[wi] * sm.wbin) : dense_window(sm, g, ns, lo, k.n);
                // gather the window's (id, segment, gather index) keys
                if (planned && sm.wbucketed) {  // its run of the scratch
                    const uint64_t *run = o.wscratch + (size_t)blockIdx.x * o.wcap + sm.woff[wi];
                    const uint32_t len = sm.woff[wi + 1] - sm.woff[wi];
                    for (uint32_t q = t; q < len; q += kDT) {
                        const uint64_t e = __ldcg(run + q);
                        sm.v.s.gslot[q] = (uint32_t)e & 0x1fffffffu;
                        sm.u.keys[0][q] = ((e >> 34) << 16) | (((uint32_t)(e >> 29) & 0x1fu) << 11) | q;
                    }
                    if (t == 0) sm.nw = len;
                } else {  // a scan of the whole neighbourhood for the window's ids
                    if (t == 0) sm.nw = 0;
                    __syncthreads();
                    for (int sgi = 0; sgi < ns; ++sgi) {
                        const uint32_t j0 = sm.seg_j0[sgi], len = sm.seg_k0[sgi + 1] - sm.seg_k0[sgi];
                        for (uint32_t q = t; q < len; q += kDT) {
                            const uint32_t slot = j0 + q;
                            const uint32_t id = __float_as_uint(__ldg(&g.pos[slot].w));
                            if (id >= lo && id < hi) {
                                const uint32_t qq = atomicAdd(&sm.nw, 1u);
                                sm.v.s.gslot[qq] = slot;
                                sm.u.keys[0][qq] = ((uint64_t)id << 16) | ((uint32_t)sgi << 11) | qq;
                            }
                        }
                    }
                }
                ++wi;
                __syncthreads();
                nw = sm.nw;
            } else {
                // gather every candidate's (id, segment, gather index) key; a
                // thread's q only grows, so its segment search goes on from
                // where the last one stopped
                uint32_t sgi = 0;
                for (uint32_t q = t; q < ncand; q += kDT) {
                    while (q >= sm.seg_k0[sgi + 1]) ++sgi;
                    const uint32_t slot = sm.seg_j0[sgi] + (q - sm.seg_k0[sgi]);
                    sm.v.s.gslot[q] = slot;
                    sm.u.keys[0][q] = ((uint64_t)__float_as_uint(__ldg(&g.pos[slot].w)) << 16) | (sgi << 11) | q;
                }
                __syncthreads();
            }
            const uint64_t *sorted =
                block_bucket_sort<kDT>(sm.u.keys[0], sm.u.keys[1], sm.v.s.hist, (int)nw, k.id_bits);
            // lay the candidates out in id order over the dead sort buffers
            // (thread t takes positions t, t + kDT, ...: no bank conflicts)
            const float3 cen = make_float3(((float)cx + 0.5f) * k.side, ((float)cy + 0.5f) * k.side,
                                           ((float)cz + 0.5f) * k.side);
            uint32_t slot_r[kDenseKT], seg_r[kDenseKT];
#pragma unroll
            for (int i = 0; i < kDenseKT; ++i) {
                const int q = t + i * kDT;
                if (q < (int)nw) {
                    const uint64_t key = sorted[q];
                    slot_r[i] = sm.v.s.gslot[(uint32_t)key & 0x7ffu];
                    seg_r[i] = ((uint32_t)key >> 11) & 0x1fu;
                }
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < kDenseKT; ++i) {
                const int q = t + i * kDT;
                if (q < (int)nw) {
                    const float4 p = __ldg(g.pos + slot_r[i]);
                    const float *sh = sm.seg_s[seg_r[i]];
                    // the candidate's periodic image as the reference computes
                    // it, (float)((double)x -+ F) on each shifted axis
                    float4 im = make_float4(p.x, p.y, p.z, __uint_as_float(slot_r[i]));
                    if (sh[0] != 0.f) im.x = add_f32_f64_rn(p.x, k.Fsd, sh[0] < 0.f);
                    if (sh[1] != 0.f) im.y = add_f32_f64_rn(p.y, k.Fsd, sh[1] < 0.f);
                    if (sh[2] != 0.f) im.z = add_f32_f64_rn(p.z, k.Fsd, sh[2] < 0.f);
                    sm.u.spos[q] = im;
                    const float4 v = __ldg(g.vel + slot_r[i]);
                    sm.svx[q] = v.x;
                    sm.svy[q] = v.y;
                    sm.svz[q] = v.z;
                    const float4 cq = sm.u.spos[q];
                    reinterpret_cast<__half *>(sm.hx)[q] = __float2half_rn((cq.x - cen.x) * k.hsc);
                    reinterpret_cast<__half *>(sm.hy)[q] = __float2half_rn((cq.y - cen.y) * k.hsc);
                    reinterpret_cast<__half *>(sm.hz)[q] = __float2half_rn((cq.z - cen.z) * k.hsc);
                }
            }
            if (t == 0 && (nw & 1)) {  // pad the last pair with a candidate far out of reach
                reinterpret_cast<__half *>(sm.hx)[nw] = __float2half_rn(30000.f);
                reinterpret_cast<__half *>(sm.hy)[nw] = __float2half_rn(30000.f);
                reinterpret_cast<__half *>(sm.hz)[nw] = __float2half_rn(30000.f);
            }
            __syncthreads();
            const bool first = lo == 0, last = hi >= k.n;

            // The item's boids go in rounds of nbr (as many as the rule masks
            // and the per-boid sums hold); each boid of a round gets L lanes.
            const uint32_t words = (nw + 31) / 32, wstride = words | 1u;  // odd: boids' words in other banks
            const uint32_t pool_nbr = (uint32_t)kMaskWords / (3u * wstride);
            const uint32_t rend = min(b, rbeg + (uint32_t)kDenseRound);
            const uint32_t njobs = DIAG ? 8u : 7u;
            for (uint32_t r0 = rbeg; r0 < rend;) {
                const uint32_t nbr = min(min(rend - r0, (uint32_t)kDT), min((uint32_t)kSumsMax, pool_nbr));
                const uint32_t L = (uint32_t)kDT / nbr;               // lanes per boid
                const uint32_t csz = ((nw + L - 1) / L + 1) & ~1u;    // chunk length (even: whole pairs)
                const bool act = (uint32_t)t < nbr * L;
                const uint32_t bi = act ? (uint32_t)t % nbr : 0, l = act ? (uint32_t)t / nbr : 0;
                const uint32_t k0 = act ? min(nw, l * csz) : 0, k1 = act ? min(nw, k0 + csz) : 0;
                uint32_t *masks = sm.v.masks;
                for (uint32_t i = (uint32_t)t; i < 3 * nbr * wstride; i += kDT) masks[i] = 0;
                // the round's boids, for the filter constants and the exact tests
                for (uint32_t i = (uint32_t)t; i < nbr; i += kDT) {
                    const float4 pp = g.pos[own0 + r0 + i], vv = g.vel[own0 + r0 + i];
                    const Sight sg = make_sight(xyz(vv));
                    sm.w.a.obs[0][i] = make_float4(pp.x, pp.y, pp.z, sg.nv);
                    sm.w.a.obs[1][i] = make_float4(vv.x, vv.y, vv.z, sg.inv_nv);
                }
                __syncthreads();  // the masks are clear, the table is written
                {
                    const float4 o0 = sm.w.a.obs[0][bi], o1 = sm.w.a.obs[1][bi];
                    const float3 pi = xyz(o0), vi = xyz(o1);
                    // The filter in half precision, two candidates per instruction:
                    // it keeps every pair within the filter radius and drops only
                    // pairs whose exact v . r is negative (the bounds are in hfilt,
                    // hdot0 and hdot1); the exact tests decide the rest.
                    const __half2 bx = __float2half2_rn((pi.x - cen.x) * k.hsc);
                    const __half2 by = __float2half2_rn((pi.y - cen.y) * k.hsc);
                    const __half2 bz = __float2half2_rn((pi.z - cen.z) * k.hsc);
                    const float vt = o0.w * k.hvsc;
                    const bool pre = k.cone_pre && vt <= 1.0f;
                    const __half2 hvx = __float2half2_rn(pre ? vi.x * k.hvsc : 0.f);
                    const __half2 hvy = __float2half2_rn(pre ? vi.y * k.hvsc : 0.f);
                    const __half2 hvz = __float2half2_rn(pre ? vi.z * k.hvsc : 0.f);
                    const __half2 hf2 = __half2half2(__float2half_ru(k.hfilt));
                    const __half2 hd2 = __half2half2(pre ? __float2half_rd(-(k.hdot0 + k.hdot1 * vt))
                                                         : __ushort_as_half((unsigned short)0xfc00u));  // -inf
                    const uint32_t p0 = k0 >> 1, plen = k1 > k0 ? ((k1 + 1) >> 1) - p0 : 0;  // pairs
                    const uint32_t maxlen = __reduce_max_sync(0xffffffffu, plen);
                    const int lane = t & 31;
                    uint32_t *queue = sm.w.a.queue[t >> 5];
                    uint32_t qlen = 0;  // the same in every lane of the warp
                    // exact tests of the queued hits, every lane of the warp
                    // busy; accepted neighbours are marked in the boid's masks
                    auto flush = [&]() {
                        __syncwarp();
                        for (uint32_t e = (uint32_t)lane; e < qlen; e += 32) {
                            const uint32_t en = queue[e];
                            const uint32_t eb = en >> 11, q = en & 0x7ffu;
                            const float4 cq = sm.u.spos[q];
                            if (__float_as_uint(cq.w) == own0 + r0 + eb) continue;
                            const float4 a0 = sm.w.a.obs[0][eb], a1 = sm.w.a.obs[1][eb];
                            Sight sg;
                            sg.v = xyz(a1);
                            sg.nv = a0.w;
                            sg.inv_nv = a1.w;
                            const int f = pair_flags(xyz(a0), sg, xyz(cq), k);
                            if (!f) continue;
                            uint32_t *mb = masks + eb * wstride + (q >> 5);
                            const uint32_t bit = 1u << (q & 31);
                            if (f & 1) atomicOr(mb, bit);
                            if (f & 2) atomicOr(mb + nbr * wstride, bit);
                            if (f & 4) atomicOr(mb + 2 * nbr * wstride, bit);
                        }
                        __syncwarp();
                        qlen = 0;
                    };
                    // A lane's hits of kHitGroup iterations (two candidates
                    // each) collect in a register, then go to the warp's queue
                    // together (one scan of the lanes' counts); the queue is
                    // tested first when they would not fit.
                    constexpr uint32_t kHitGroup = kQueue / 64;
                    uint32_t hm = 0;
                    for (uint32_t it = 0; it < maxlen; ++it) {
                        const uint32_t gi = it % kHitGroup;
                        if (it < plen) {
                            const uint32_t pp = p0 + it;
                            const __half2 dx = __hsub2(sm.hx[pp], bx), dy = __hsub2(sm.hy[pp], by),
                                          dz = __hsub2(sm.hz[pp], bz);
                            const __half2 d2 = __hfma2(dz, dz, __hfma2(dy, dy, __hmul2(dx, dx)));
                            const __half2 dv = __hfma2(hvz, dz, __hfma2(hvy, dy, __hmul2(hvx, dx)));
                            const unsigned keep = __hlt2_mask(d2, hf2) & __hge2_mask(dv, hd2);
                            hm |= ((keep & 1u) | ((keep >> 15) & 2u)) << (2 * gi);
                        }
                        const bool end = it + 1 == maxlen;
                        if (gi == kHitGroup - 1 || end) {
                            const uint32_t cnt = __popc(hm);
                            uint32_t incl = cnt;
#pragma unroll
                            for (int o = 1; o < 32; o <<= 1) {
                                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                                if (lane >= o) incl += y;
                            }
                            const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
                            if (qlen + total > (uint32_t)kQueue) flush();
                            uint32_t at = qlen + incl - cnt;
                            const uint32_t q0 = 2 * (p0 + it - gi);  // the candidate of bit 0
                            while (hm) {
                                const uint32_t bb = (uint32_t)__ffs(hm) - 1;
                                hm &= hm - 1;
                                queue[at++] = (bi << 11) | (q0 + bb);
                            }
                            qlen += total;
                            if (end || qlen > (uint32_t)kQueue - 64) flush();
                        }
                    }
                }
                // the separation job's boid (at most one per thread): its
                // position from the round's table, which the sums overwrite
                float3 sep_pi = make_float3(0.f, 0.f, 0.f);
                for (uint32_t pj = (uint32_t)t; pj < 7 * nbr; pj += kDT)
                    if (pj >= 6 * nbr) sep_pi = xyz(sm.w.a.obs[0][pj - 6 * nbr]);
                __syncthreads();  // the masks are complete; the hit buffers are dead
                for (uint32_t pj = (uint32_t)t; pj < njobs * nbr; pj += kDT) {
                    const uint32_t job = pj / nbr, jb = pj - job * nbr;
                    const uint32_t js = own0 + r0 + jb;
                    const Acc *cin = first ? nullptr : o.carry + js;
                    Acc &out = sm.w.sums[jb];
                    if (job < 6) {
                        dense_sum_job(sm, masks + ((job < 3 ? 0u : 2u) * nbr + jb) * wstride, words, job, cin, out);
                    } else if (job == 6) {
                        dense_sep_job(sm, masks + (nbr + jb) * wstride, words, sep_pi, cin, out);
                    } else if (DIAG) {
                        dense_hash_job(sm, masks + jb * wstride, nbr * wstride, words, cin, out, g.pos);
                    }
                }
                __syncthreads();
                if (act && l == 0) {
                    const uint32_t s = own0 + r0 + bi;
                    Acc a = sm.w.sums[bi];
                    if (!DIAG) a.h[0] = a.h[1] = a.h[2] = 0;
                    if (last) finish_boid<DIAG>(a, g.pos[s], xyz(g.vel[s]), s, o, k);
                    else o.carry[s] = a;
                }
                __syncthreads();  // masks and sums are reused by the next round
                r0 += nbr;
            }
            if (last) break;
            lo = hi;
        }
    }
}

// ------------------------------------------------------------------ all-pairs engine

// Phase 1: a 2-D grid of (i-tile, j-tile) blocks tests every ordered pair.
// A box filter on the minimum-image offset (||dx| - F/2| > F/2 - R per axis)
// rejects almost all pairs; survivors get the exact tests and accepted
// neighbours are appended to the boid's list (unordered).  A thread's box
// hits are buffered and the whole warp runs their exact tests together once a
// buffer is nearly full (and at the end of the tile), so the rare hits do not
// stall the filter loop of the other 31 lanes, as they would inline.
constexpr int kApThreads = 128;
constexpr int kApKI = 8;                        // i per thread
constexpr int kApTileI = kApThreads * kApKI;    // 1024
constexpr int kApTileJ = 1024;
constexpr int kApHits = 24;                     // box hits buffered per thread
static_assert(kApHits > kApKI, "a j step's hits fit the buffer");

__global__ void __launch_bounds__(kApThreads)
k_ap_pairs(const float4 *__restrict__ pos, const float4 *__restrict__ vel, uint32_t *__restrict__ cnt,
           uint32_t *__restrict__ list, uint32_t cap, StepConst k)
{
    __shared__ float4 sp[kApTileJ];
    __shared__ uint16_t hits[kApHits][kApThreads];  // r << 10 | tile j
    const uint32_t n = k.n;
    const uint32_t j0 = blockIdx.y * kApTileJ;
    const uint32_t jn = min((uint32_t)kApTileJ, n - j0);
    const uint32_t ibase = blockIdx.x * kApTileI + threadIdx.x;
    for (uint32_t t = threadIdx.x; t < jn; t += kApThreads) sp[t] = pos[j0 + t];
    float3 pi[kApKI];
    const float nanf_ = __uint_as_float(0x7fffffffu);  // fails every filter test
#pragma unroll
    for (int r = 0; r < kApKI; ++r) {
        const uint32_t i = ibase + r * kApThreads;
        pi[r] = i < n ? xyz(pos[i]) : make_float3(nanf_, nanf_, nanf_);
    }
    __syncthreads();
    int nh = 0;
    // the exact tests of this thread's buffered hits (all lanes call it)
    auto flush = [&]() {
        for (int e = 0; e < nh; ++e) {
            const uint32_t en = hits[e][threadIdx.x];
            const uint32_t i = ibase + (en >> 10) * kApThreads, tj = en & 1023u, j = j0 + tj;
            if (i == j) continue;
            const float3 p = xyz(pos[i]);
            const Sight s = make_sight(xyz(vel[i]));
            const int f = pair_flags(p, s, image3(xyz(sp[tj]), p, k), k);
            if (f) {
                const uint32_t q = atomicAdd(cnt + i, 1u);
                if (q < cap) list[(size_t)i * cap + q] = j | ((uint32_t)f << 29);
            }
        }
        nh = 0;
    };
    const float h = k.halfFf, lim = k.box_lim;
    for (uint32_t t = 0; t < jn; ++t) {
        const float4 pj = sp[t];
#pragma unroll
        for (int r = 0; r < kApKI; ++r) {
            const bool nx = fabsf(fabsf(pj.x - pi[r].x) - h) > lim;
            const bool ny = fabsf(fabsf(pj.y - pi[r].y) - h) > lim;
            const bool nz = fabsf(fabsf(pj.z - pi[r].z) - h) > lim;
            if (nx && ny && nz) hits[nh++][threadIdx.x] = (uint16_t)((r << 10) | t);
        }
        if (__any_sync(0xffffffffu, nh > kApHits - kApKI)) flush();
    }
    flush();
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

cudaError_t launch_pack(const float *pos3, const float *vel3, float4 *pos4, float4 *vel4, uint32_t i0, uint32_t i1,
                        uint32_t *bad, float hi, const StepConst *bin, uint32_t *key, uint32_t *rank,
                        uint32_t *count, cudaStream_t st, uint64_t *launches)
{
    if (i1 <= i0) return cudaSuccess;
    const StepConst none{};
    k_pack<<<blocks_for(i1 - i0, 256), 256, 0, st>>>(pos3, vel3, pos4, vel4, i0, i1, bad, hi, bin ? key : nullptr,
                                                      rank, count, bin ? *bin : none);
    ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_unpack_index(const float4 *pos4, uint32_t *slot_of, uint32_t n, cudaStream_t st,
                                uint64_t *launches)
{
    if (n == 0) return cudaSuccess;
    k_unpack_index<<<blocks_for(n, 256), 256, 0, st>>>(pos4, slot_of, n);
    ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_unpack_gather(const float4 *pos4, const float4 *vel4, const uint32_t *slot_of, float *pos3,
                                 float *vel3, uint32_t i0, uint32_t i1, uint32_t n, cudaStream_t st,
                                 uint64_t *launches)
{
    if (i1 <= i0) return cudaSuccess;
    k_unpack_gather<<<blocks_for(i1 - i0, 256), 256, 0, st>>>(pos4, vel4, slot_of, pos3, vel3, i0, i1, n);
    ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_unpack(const float4 *pos4, const float4 *vel4, uint32_t *slot_of, float *pos3, float *vel3,
                          uint32_t n, cudaStream_t st, uint64_t *launches)
{
    cudaError_t e = launch_unpack_index(pos4, slot_of, n, st, launches);
    if (e != cudaSuccess) return e;
    return launch_unpack_gather(pos4, vel4, slot_of, pos3, vel3, 0, n, n, st, launches);
}

cudaError_t launch_frame(const float4 *pos4, const float4 *vel4, const float *force9, float *pframe,
                         float *vframe, int with_forces, uint32_t n, cudaStream_t st, uint64_t *launches)
{
    if (n == 0) return cudaSuccess;
    k_frame<<<blocks_for(n, 256), 256, 0, st>>>(pos4, vel4, force9, pframe, vframe, with_forces, n);
    ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_grid_keys(const StepConst &k, const float4 *pos, uint32_t *key, uint32_t *rank,
                             uint32_t *count, cudaStream_t st, uint64_t *launches, const FlockTable *ft)
{
    const uint32_t n = ft ? ft->nslots : k.n;
    if (n == 0) return cudaSuccess;
    if (ft) k_grid_keys<true><<<blocks_for(n, 256), 256, 0, st>>>(pos, key, rank, count, k, *ft);
    else k_grid_keys<false><<<blocks_for(n, 256), 256, 0, st>>>(pos, key, rank, count, k, FlockTable{});
    ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_grid_scan(const StepConst &k, const DevBuffers &b, cudaStream_t st, uint64_t *launches,
                             const FlockTable *ft)
{
    cudaError_t e = cudaMemsetAsync(b.dense_n, 0, 3 * sizeof(uint32_t), st);  // items, work queue, deferred
    if (e != cudaSuccess) return e;
    if (ft && b.defer_cnt && (e = cudaMemsetAsync(b.defer_cnt, 0, sizeof(uint32_t) * ft->count, st)) != cudaSuccess)
        return e;  // an ensemble's per-flock deferred counts
    k_grid_scan<<<b.nscan_blocks, kScanThreads, 0, st>>>(b.count, b.lstart, b.bsum, b.ticket, b.nscan_blocks);
    const uint32_t nfull = b.ncell / 4;
    const int windows = b.carry != nullptr;
    // with a side stream the classification runs beside the scatter, which
    // the caller queues next; launch_grid_force waits for it
    cudaStream_t cs = st;
    if (b.aux) {
        if ((e = cudaEventRecord(b.fork, st)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(b.aux, b.fork, 0)) != cudaSuccess) return e;
        cs = b.aux;
    }
    if (ft)
        k_grid_classify<true><<<blocks_for(nfull, 256), 256, 0, cs>>>(b.lstart, b.bsum, b.dflag,
                                                                       b.dense_list, b.dense_n, nfull, windows, k, *ft);
    else
        k_grid_classify<false><<<blocks_for(nfull, 256), 256, 0, cs>>>(b.lstart, b.bsum, b.dflag,
                                                                        b.dense_list, b.dense_n, nfull, windows, k,
                                                                        FlockTable{});
    if (b.aux && (e = cudaEventRecord(b.cjoin, b.aux)) != cudaSuccess) return e;
    *launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_grid_scatter(const StepConst &k, const DevBuffers &b, int from, bool zero_counts,
                                cudaStream_t st, uint64_t *launches, const FlockTable *ft)
{
    const uint32_t n = ft ? ft->nslots : k.n;
    if (n == 0) return cudaSuccess;
    uint32_t *cz = zero_counts ? b.count : nullptr;
    if (ft)
        k_grid_scatter<true><<<blocks_for(n, 256), 256, 0, st>>>(b.pos[from], b.vel[from], b.key, b.rank, b.lstart,
                                                                 b.bsum, b.pos[1 - from], b.vel[1 - from], cz, n, *ft);
    else
        k_grid_scatter<false><<<blocks_for(n, 256), 256, 0, st>>>(b.pos[from], b.vel[from], b.key, b.rank, b.lstart,
                                                                  b.bsum, b.pos[1 - from], b.vel[1 - from], cz, n,
                                                                  FlockTable{});
    ++*launches;
    return cudaGetLastError();
}

namespace {

// The dense kernel's shared memory exceeds the 48 KB default: opt in once
// per device and instantiation.
template <bool DIAG, bool MULTI>
cudaError_t dense_smem_opt_in()
{
    static uint64_t done = 0;  // bit per device ordinal
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev < 64 ? 1ull << dev : 0;
    if (bit && (__atomic_load_n(&done, __ATOMIC_ACQUIRE) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(k_grid_dense<DIAG, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(DenseSmem));
    if (e == cudaSuccess && bit) __atomic_fetch_or(&done, bit, __ATOMIC_RELEASE);
    return e;
}

template <bool DIAG, bool MULTI>
cudaError_t grid_force(const StepConst &k, const GridIn &g, const GridOut &o, const DevBuffers &b, unsigned nsp,
                       const FlockTable &ft, cudaStream_t st)
{
    cudaError_t e = dense_smem_opt_in<DIAG, MULTI>();
    if (e != cudaSuccess) return e;
    if (b.aux && (e = cudaStreamWaitEvent(st, b.cjoin, 0)) != cudaSuccess) return e;  // the classification
    k_grid_sparse<DIAG, MULTI><<<nsp, kRT, 0, st>>>(g, o, k, ft);
    const unsigned nmore = MULTI ? nsp : min(nsp, 2 * b.dense_grid);
    if (o.defer && b.aux) {
        // the deferred boids and the dense cells are disjoint: run them side by side
        if ((e = cudaEventRecord(b.fork, st)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(b.aux, b.fork, 0)) != cudaSuccess) return e;
        k_grid_sparse_more<DIAG, MULTI><<<nmore, kRT, 0, b.aux>>>(g, o, k, ft);
        if ((e = cudaEventRecord(b.join, b.aux)) != cudaSuccess) return e;
        k_grid_dense<DIAG, MULTI><<<b.dense_grid, kDT, sizeof(DenseSmem), st>>>(g, o, b.dense_list, b.dense_n, k, ft);
        if ((e = cudaStreamWaitEvent(st, b.join, 0)) != cudaSuccess) return e;
        return cudaGetLastError();
    }
    if (o.defer) k_grid_sparse_more<DIAG, MULTI><<<nmore, kRT, 0, st>>>(g, o, k, ft);
    k_grid_dense<DIAG, MULTI><<<b.dense_grid, kDT, sizeof(DenseSmem), st>>>(g, o, b.dense_list, b.dense_n, k, ft);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_grid_force(const StepConst &k, const DevBuffers &b, int from, bool diag, bool record_forces,
                              cudaStream_t st, uint64_t *launches, const FlockTable *ft)
{
    const uint32_t n = ft ? ft->nslots : k.n;
    if (n == 0) return cudaSuccess;
    GridIn g{b.pos[from], b.vel[from], b.lstart, b.bsum, b.dflag};
    GridOut o{};
    o.carry = static_cast<Acc *>(b.carry);
    o.wscratch = b.carry ? b.wscratch : nullptr;
    o.wcap = o.wscratch ? b.wcap : 0;
    if (b.defer && b.defer_cnt && b.carry) {
        o.defer = b.defer;
        o.defer_cnt = b.defer_cnt;
        if (b.ovf && b.ovf_n) {
            o.ovf = b.ovf;
            o.ovf_n = b.ovf_n;
        }
    }
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
    const unsigned nsp = blocks_for(n, kRT);
    const FlockTable none{};
    cudaError_t e;
    if (ft) e = diag ? grid_force<true, true>(k, g, o, b, nsp, *ft, st) : grid_force<false, true>(k, g, o, b, nsp, *ft, st);
    else e = diag ? grid_force<true, false>(k, g, o, b, nsp, none, st) : grid_force<false, false>(k, g, o, b, nsp, none, st);
    if (e == cudaSuccess) *launches += o.defer ? 3 : 2;
    return e;
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


// ------------------------------------------------------------------ ensemble statistics
//
// Order statistics of every flock of a batched ensemble, on a freshly binned
// state (sorted slots, valid cell tables).  Sums are FP64.  Per flock the
// accumulator holds kStatAcc doubles:
//   0-2  sum of unit velocities        3-5  sum of velocities
//   6-8  sum of sin(2 pi x / F)        9-11 sum of cos(2 pi x / F)
//   12-14 sum of r_hat x v_hat (about the centre of mass)
//   15   sum of capped nearest-neighbour distances
namespace {

constexpr int kStatThreads = kSlotAlign;
constexpr uint32_t kFindCap = 1u << 24;  // bound on union-find walks (far above any tree height)

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-reduce NV doubles per thread into acc[0..NV) with one atomic each.
template <int NV>
__device__ __forceinline__ void block_sum_to(const double (&v)[NV], double *acc)
{
    __shared__ double part[NV][kStatThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        const double s = warp_sum(v[i]);
        if (lane == 0) part[i][w] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < kStatThreads / 32; ++q) s += part[threadIdx.x][q];
        atomicAdd(acc + threadIdx.x, s);
    }
}

__device__ __forceinline__ uint32_t uf_find(const uint32_t *parent, uint32_t x, uint32_t *err)
{
    for (uint32_t it = 0; it < kFindCap; ++it) {
        const uint32_t p = __ldcg(parent + x);
        if (p == x) return x;
        x = p;
    }
    atomicOr(err, 1u);
    return x;
}

// Lock-free union: hook the larger root under the smaller one; a failed CAS
// means that root was hooked meanwhile, so retry from the new roots.
__device__ __forceinline__ void uf_union(uint32_t *parent, uint32_t a, uint32_t b, uint32_t *err)
{
    for (uint32_t it = 0; it < kFindCap; ++it) {
        a = uf_find(parent, a, err);
        b = uf_find(parent, b, err);
        if (a == b) return;
        const uint32_t hi = a > b ? a : b, lo = a > b ? b : a;
        const uint32_t old = atomicCAS(parent + hi, hi, lo);
        if (old == hi) return;
        a = lo;
        b = old;
    }
    atomicOr(err, 2u);
}

}  // namespace

__global__ void __launch_bounds__(kStatThreads)
k_stat_moments(const float4 *__restrict__ pos, const float4 *__restrict__ vel, FlockTable ft, double *acc,
               uint32_t *__restrict__ parent)
{
    __shared__ StepConst kf;
    load_flock(kf, ft, ft.blk_flock[blockIdx.x]);
    const uint32_t s = blockIdx.x * kStatThreads + threadIdx.x;
    parent[s] = s;
    double v[12] = {};
    if (s - kf.slot_base < kf.n) {
        const float4 p = pos[s], u = vel[s];
        const double vx = u.x, vy = u.y, vz = u.z;
        const double sp = sqrt(vx * vx + vy * vy + vz * vz);
        if (sp > 0.0) { v[0] = vx / sp; v[1] = vy / sp; v[2] = vz / sp; }
        v[3] = vx; v[4] = vy; v[5] = vz;
        const double inv = 2.0 / kf.F;
        sincospi(p.x * inv, &v[6], &v[9]);
        sincospi(p.y * inv, &v[7], &v[10]);
        sincospi(p.z * inv, &v[8], &v[11]);
    }
    block_sum_to<12>(v, acc + (size_t)kf.flock * kStatAcc);
}

// Centre of mass per flock: the periodic (circular) mean on each axis.
__global__ void k_stat_com(const double *__restrict__ acc, const StepConst *__restrict__ ks, uint32_t count,
                           double *__restrict__ com)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= count) return;
    const double *a = acc + (size_t)f * kStatAcc;
    const double F = ks[f].F;
    for (int d = 0; d < 3; ++d) {
        double c = atan2(a[6 + d], a[9 + d]) / (2.0 * 3.141592653589793) * F;
        if (c < 0.0) c += F;
        com[3 * f + d] = c;
    }
}

// Milling sum, capped nearest-neighbour distances and the union of every
// pair nearer than the link distance (the flock's cohesion sight distance),
// over the 27 full-size cells around each boid.
__global__ void __launch_bounds__(kStatThreads)
k_stat_pairs(GridIn g, FlockTable ft, const double *__restrict__ com, const float *__restrict__ link,
             double *acc, uint32_t *parent, uint32_t *err)
{
    __shared__ StepConst kf;
    load_flock(kf, ft, ft.blk_flock[blockIdx.x]);
    const StepConst &k = kf;
    const uint32_t s = blockIdx.x * kStatThreads + threadIdx.x;
    double v[4] = {};
    if (s - k.slot_base < k.n) {
        const float4 p4 = g.pos[s], u = g.vel[s];
        const float3 pi = xyz(p4);
        // r_hat x v_hat about the periodic centre of mass
        double r[3] = {pi.x - com[3 * k.flock], pi.y - com[3 * k.flock + 1], pi.z - com[3 * k.flock + 2]};
        for (int d = 0; d < 3; ++d) {
            if (r[d] > 0.5 * k.F) r[d] -= k.F;
            else if (r[d] < -0.5 * k.F) r[d] += k.F;
        }
        const double rn = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        const double vx = u.x, vy = u.y, vz = u.z;
        const double sp = sqrt(vx * vx + vy * vy + vz * vz);
        if (rn > 0.0 && sp > 0.0) {
            const double a0 = r[0] / rn, a1 = r[1] / rn, a2 = r[2] / rn;
            const double b0 = vx / sp, b1 = vy / sp, b2 = vz / sp;
            v[0] = a1 * b2 - a2 * b1;
            v[1] = a2 * b0 - a0 * b2;
            v[2] = a0 * b1 - a1 * b0;
        }
        const int cx = cell1(pi.x, k), cy = cell1(pi.y, k), cz = cell1(pi.z, k);
        const int runs = seg_runs(cx, k);
        const float lk = link[k.flock];
        float nn2 = k.side * k.side;
        for (int q = 0; q < 9 * runs; ++q) {
            const Seg sg = segment(cx, cy, cz, q, runs, k);
            const uint32_t j0 = slot_start(g.lstart, g.bsum, k.cell_base + sg.c0, k);
            const uint32_t j1 = slot_start(g.lstart, g.bsum, k.cell_base + sg.c1, k);
            for (uint32_t j = j0; j < j1; ++j) {
                if (j == s) continue;
                const float4 pj = __ldg(g.pos + j);
                const float dx = pj.x + sg.sx - pi.x, dy = pj.y + sg.sy - pi.y, dz = pj.z + sg.sz - pi.z;
                const float d2 = dx * dx + dy * dy + dz * dz;
                nn2 = fminf(nn2, d2);
                if (j > s && d2 < lk * lk) uf_union(parent, s, j, err);
            }
        }
        v[3] = sqrt((double)nn2);
    }
    block_sum_to<4>(v, acc + (size_t)k.flock * kStatAcc + 12);
}

// Component sizes: every boid adds one to its root's count.
__global__ void k_stat_roots(FlockTable ft, const uint32_t *parent, uint32_t *__restrict__ size, uint32_t *err)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ft.nslots) return;
    const StepConst &k = ft.ks[ft.blk_flock[s / kSlotAlign]];
    if (s - k.slot_base >= k.n) return;
    atomicAdd(size + uf_find(parent, s, err), 1u);
}

__global__ void k_stat_largest(FlockTable ft, const uint32_t *__restrict__ parent, const uint32_t *__restrict__ size,
                               uint32_t *__restrict__ largest)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ft.nslots) return;
    const StepConst &k = ft.ks[ft.blk_flock[s / kSlotAlign]];
    if (s - k.slot_base >= k.n || parent[s] != s) return;
    atomicMax(largest + k.flock, size[s]);
}

cudaError_t launch_ensemble_stats(const DevBuffers &b, int from, const FlockTable &ft, const float *link,
                                  double *acc, double *com, uint32_t *largest, uint32_t *err, cudaStream_t st,
                                  uint64_t *launches)
{
    const unsigned nb = ft.nslots / kStatThreads;
    uint32_t *parent = b.key, *size = b.rank;  // free between a step's binning and its rule pass
    cudaError_t e;
    if ((e = cudaMemsetAsync(acc, 0, sizeof(double) * kStatAcc * ft.count, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(largest, 0, sizeof(uint32_t) * ft.count, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(size, 0, sizeof(uint32_t) * ft.nslots, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(err, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
    k_stat_moments<<<nb, kStatThreads, 0, st>>>(b.pos[from], b.vel[from], ft, acc, parent);
    k_stat_com<<<blocks_for(ft.count, 128), 128, 0, st>>>(acc, ft.ks, ft.count, com);
    GridIn g{b.pos[from], b.vel[from], b.lstart, b.bsum, nullptr};  // k_stat_pairs reads no dense flags
    k_stat_pairs<<<nb, kStatThreads, 0, st>>>(g, ft, com, link, acc, parent, err);
    k_stat_roots<<<blocks_for(ft.nslots, 256), 256, 0, st>>>(ft, parent, size, err);
    k_stat_largest<<<blocks_for(ft.nslots, 256), 256, 0, st>>>(ft, parent, size, largest);
    *launches += 5;
    return cudaGetLastError();
}

cudaError_t grid_prepare()
{
    cudaError_t e;
    if ((e = dense_smem_opt_in<false, false>()) != cudaSuccess) return e;
    if ((e = dense_smem_opt_in<true, false>()) != cudaSuccess) return e;
    if ((e = dense_smem_opt_in<false, true>()) != cudaSuccess) return e;
    return dense_smem_opt_in<true, true>();
}

}  // namespace boidsgpu
