// boids_mlp.cu -- the sweep surrogate's network on the tensor cores.
//
// A multilayer perceptron in -> hidden -> hidden -> out with ReLU, BF16
// weights and activations and FP32 accumulation, trained with Adam on the
// mean squared error.  It maps a flock's rule parameters to its order
// statistics after a run (the ensemble's boids_ensemble_stats), so that a
// parameter sweep can be screened before the plain simulation re-runs the
// candidates it selects.  No counterpart in the reference.
//
// The forward pass's hidden-to-hidden product (rows x 256 by 256 x 256, the
// network's one square product) runs on the 5th-generation tensor cores:
// k_mlp_hidden_tc stages a 128-row tile of the activations and the whole
// weight matrix in shared memory in the canonical K-major layout, one thread
// issues tcgen05.mma (M 128, N 256, K 16) into an FP32 accumulator in tensor
// memory, and the epilogue reads it back with tcgen05.ld, adds the bias and
// writes the FP32 pre-activation and the BF16 ReLU.  The other products --
// the thin input and output layers (K or N of 8 and 4) and the backward
// pass -- are one strided GEMM kernel on mma.sync m16n8k16 (BF16 operands,
// FP32 accumulators): small, latency-bound products where a warp-level MMA
// with operands read straight from L2 is the simplest fast form.
#include "boids.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace boidsgpu {
int set_last_error(int code, const char *msg);
}

namespace {

// A read-only BF16 matrix view: element (r, c) at p[r * rs + c * cs].
struct MatB {
    const __nv_bfloat16 *p;
    long long rs, cs;
    int rows, cols;
};

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ __nv_bfloat16 at(const MatB &m, int r, int c)
{
    return (r < m.rows && c < m.cols) ? m.p[r * m.rs + c * m.cs] : __float2bfloat16_rn(0.f);
}

constexpr int kWarpsM = 4;   // warps per CTA along M (16 rows each)
constexpr int kTileN = 32;   // columns per warp (4 MMA tiles of 8)

// C = A (M x K) * B (K x N) [+ bias] [* (mask > 0)], FP32 out (row-major,
// ldc) and optionally a BF16 copy of relu(C) or C (row-major, ldb16).
__global__ void __launch_bounds__(32 * kWarpsM)
k_mlp_gemm(MatB A, MatB B, float *__restrict__ C, int ldc, __nv_bfloat16 *__restrict__ C16, int ld16,
           const float *__restrict__ bias, const float *__restrict__ mask, int ldm, int relu16)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t4 = lane & 3;
    const int r0 = (blockIdx.y * kWarpsM + warp) * 16;
    const int n0 = blockIdx.x * kTileN;
    const int M = A.rows, K = A.cols, N = B.cols;
    if (r0 >= M) return;
    float acc[4][4] = {};
    for (int kk = 0; kk < K; kk += 16) {
        const int ka = kk + 2 * t4;
        uint32_t a[4];
        a[0] = pack2(at(A, r0 + g, ka), at(A, r0 + g, ka + 1));
        a[1] = pack2(at(A, r0 + g + 8, ka), at(A, r0 + g + 8, ka + 1));
        a[2] = pack2(at(A, r0 + g, ka + 8), at(A, r0 + g, ka + 9));
        a[3] = pack2(at(A, r0 + g + 8, ka + 8), at(A, r0 + g + 8, ka + 9));
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + 8 * j + g;
            const uint32_t b0 = pack2(at(B, ka, n), at(B, ka + 1, n));
            const uint32_t b1 = pack2(at(B, ka + 8, n), at(B, ka + 9, n));
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
                : "+f"(acc[j][0]), "+f"(acc[j][1]), "+f"(acc[j][2]), "+f"(acc[j][3])
                : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int r = r0 + g + (q >= 2 ? 8 : 0);
            const int c = n0 + 8 * j + 2 * t4 + (q & 1);
            if (r >= M || c >= N) continue;
            float v = acc[j][q];
            if (bias) v += bias[c];
            if (mask && !(mask[(long long)r * ldm + c] > 0.f)) v = 0.f;
            if (C) C[(long long)r * ldc + c] = v;
            if (C16) C16[(long long)r * ld16 + c] = __float2bfloat16_rn(relu16 ? fmaxf(v, 0.f) : v);
        }
    }
}

// ------------------------------------------------------------------ hidden layer on tcgen05

// C = A W + b for A rows x 256 (BF16, row-major), W 256 x 256 (BF16, fan-in
// rows), C to FP32 (pre) and BF16 ReLU (h); 128 rows per CTA.
//
// Shared memory holds both operands K-major in 8 x 16-byte core matrices
// (8 rows of 8 consecutive K elements, 128 bytes): element (r, k) at
// ((r / 8) * 32 + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2, so core matrices
// adjacent along K are 128 bytes apart (the descriptor's leading byte offset)
// and 8-row groups 4096 bytes apart (its stride byte offset).  The weights
// arrive already in that layout, transposed (row n of the image holds
// column n of W), from k_mlp_tile_w.
constexpr int kTcM = 128, kTcN = 256, kTcK = 256;
constexpr int kTcThreads = 128;
constexpr uint32_t kTcABytes = kTcM * kTcK * 2;   // 64 KB
constexpr uint32_t kTcBBytes = kTcN * kTcK * 2;   // 128 KB
constexpr size_t kTcSmem = kTcABytes + kTcBBytes + 1024 + 64;
constexpr uint32_t kTcSpinLimit = 1u << 22;      // bounded wait on the accumulator

__device__ uint32_t g_mlp_tc_error;  // set when a tile's wait gave up (the host reports it)

__host__ __device__ constexpr uint32_t core_off(uint32_t r, uint32_t k)
{
    return ((r >> 3) * (kTcK / 8) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// The weight image: W (K x N, row-major, fan-in rows) as N rows of K, in the
// core-matrix layout above, one 16-byte row chunk per thread.
__global__ void k_mlp_tile_w(const __nv_bfloat16 *__restrict__ w, __nv_bfloat16 *__restrict__ img)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;  // chunk: (n, k8)
    if (i >= (uint32_t)(kTcN * kTcK / 8)) return;
    const uint32_t n = i / (kTcK / 8), k0 = (i % (kTcK / 8)) * 8;
    __align__(16) __nv_bfloat16 v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) v[e] = w[(size_t)(k0 + e) * kTcN + n];
    *reinterpret_cast<uint4 *>(reinterpret_cast<unsigned char *>(img) + core_off(n, k0)) =
        *reinterpret_cast<const uint4 *>(v);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    // start address, leading and stride byte offsets (all >> 4), the
    // descriptor version (0b001 at bit 46), no swizzle
    return (uint64_t)((saddr >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint32_t src_bytes)
{
    // 16 bytes global -> shared without staging in registers; src_bytes 0
    // fills the destination with zeros
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}

// One CTA per SM walks 128-row tiles: the weight image is loaded once, and
// the next tile's activations are copied in (cp.async) while the current
// tile's accumulator is read out.
__global__ void __launch_bounds__(kTcThreads, 1)
k_mlp_hidden_tc(const __nv_bfloat16 *__restrict__ a, int rows, const __nv_bfloat16 *__restrict__ wimg,
                const float *__restrict__ bias, float *__restrict__ pre, __nv_bfloat16 *__restrict__ h)
{
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char *sa = tc_smem, *sb = tc_smem + kTcABytes;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(tc_smem + kTcABytes + kTcBBytes);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(tc_smem + kTcABytes + kTcBBytes + 8);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int ntiles = (rows + kTcM - 1) / kTcM;
    const uint32_t sa_s = (uint32_t)__cvta_generic_to_shared(sa), sb_s = (uint32_t)__cvta_generic_to_shared(sb);
    // a tile's activations into shared memory (rows past the end are zero)
    auto load_a = [&](int tile) {
        const int m0 = tile * kTcM;
        for (uint32_t i = t; i < (uint32_t)(kTcM * kTcK / 8); i += kTcThreads) {
            const uint32_t r = i / (kTcK / 8), k0 = (i % (kTcK / 8)) * 8;
            const bool in = m0 + (int)r < rows;
            cp_async16(sa_s + core_off(r, k0), a + (size_t)(in ? m0 + r : 0) * kTcK + k0, in ? 16u : 0u);
        }
    };
    for (uint32_t i = t; i < kTcBBytes / 16; i += kTcThreads) cp_async16(sb_s + 16 * i, wimg + 8 * i, 16u);
    if ((int)blockIdx.x < ntiles) load_a(blockIdx.x);
    const uint32_t mbar_a = (uint32_t)__cvta_generic_to_shared(mbar);
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_a));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {  // the accumulator: 256 columns of tensor memory
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::
                         "r"((uint32_t)__cvta_generic_to_shared(tmem_slot)), "r"((uint32_t)kTcN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    // the shared-memory writes become visible to the tensor cores
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    // kind::f16: FP32 D (bit 4), BF16 A and B (bits 7, 10), both K-major,
    // N / 8 at bit 17, M / 16 at bit 24
    const uint32_t idesc =
        (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
    uint32_t phase = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        if (t == 0) {
#pragma unroll 1
            for (int kk = 0; kk < kTcK / 16; ++kk) {
                const uint64_t ad = smem_desc(sa_s + kk * 256, 128, (kTcK / 8) * 128);
                const uint64_t bd = smem_desc(sb_s + kk * 256, 128, (kTcK / 8) * 128);
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(kk));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_a)
                         : "memory");
        }
        // wait for the accumulator (bounded: a wait that gives up flags an error)
        uint32_t done = 0;
        for (uint32_t it = 0; it < kTcSpinLimit && !done; ++it)
            asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                         " selp.u32 %0, 1, 0, p;\n}\n"
                         : "=r"(done)
                         : "r"(mbar_a), "r"(phase)
                         : "memory");
        phase ^= 1u;
        done = __syncthreads_and(done);  // one decision for the whole CTA
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (!done) {
            atomicExch(&g_mlp_tc_error, 1u);
            ok = false;
            break;
        }
        // the activations' buffer is free: the next tile's copy runs under the epilogue
        const int nxt = tile + gridDim.x;
        if (nxt < ntiles) load_a(nxt);
        // epilogue: warp w reads tensor-memory lanes 32w.. (its rows), 32 columns at a time
        const int r = tile * kTcM + warp * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c = 0; c < kTcN; c += 32) {
            uint32_t v[32];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(trow + (uint32_t)c));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (r < rows) {
#pragma unroll
                for (int q = 0; q < 32; q += 8) {
                    float f[8];
                    __align__(16) __nv_bfloat16 hb[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        f[e] = __uint_as_float(v[q + e]) + __ldg(bias + c + q + e);
                        hb[e] = __float2bfloat16_rn(fmaxf(f[e], 0.f));
                    }
                    if (pre) {
                        float4 *po = reinterpret_cast<float4 *>(pre + (size_t)r * kTcN + c + q);
                        po[0] = make_float4(f[0], f[1], f[2], f[3]);
                        po[1] = make_float4(f[4], f[5], f[6], f[7]);
                    }
                    *reinterpret_cast<uint4 *>(h + (size_t)r * kTcN + c + q) = *reinterpret_cast<const uint4 *>(hb);
                }
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();  // the accumulator is read and the next activations are in place
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    (void)ok;
    asm volatile("cp.async.wait_all;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)kTcN));
    }
}

// The whole forward pass for inference, fused: 8 -> 256 -> 256 -> 4 in one
// kernel that reads x and writes y.  Per 128-row tile the CTA computes the
// first layer into shared memory (each lane keeps its 8 columns of W1 in
// registers; the tile's x is copied in ahead with cp.async), the tensor
// cores run the hidden product into one of two accumulators in tensor
// memory, and the epilogue applies bias and ReLU and folds the 256 -> 4
// output layer in registers while the next tile's product runs in the other
// accumulator.  Eight warps: warps w and w + 4 read the same accumulator
// lanes, the first the columns 0..127, the second 128..255, and their partial
// outputs meet in shared memory.  The rounding points are those of the
// unfused pass (BF16 x, h1, h2; FP32 sums).
constexpr int kTcIn = 8, kTcOut = 4;
constexpr int kTcFwdThreads = 256;
constexpr uint32_t kTcXBytes = kTcM * kTcIn * 4;  // a tile's inputs, 4 KB
constexpr size_t kTcFwdSmem = kTcABytes + kTcBBytes + 1024 + 64 +
                              sizeof(float) * (kTcN * kTcOut + kTcN + kTcOut + 2 * kTcM * kTcOut) + kTcXBytes;

__global__ void __launch_bounds__(kTcFwdThreads, 1)
k_mlp_forward_tc(const float *__restrict__ x, int rows, const __nv_bfloat16 *__restrict__ w1,
                 const float *__restrict__ b1, const __nv_bfloat16 *__restrict__ wimg, const float *__restrict__ b2,
                 const __nv_bfloat16 *__restrict__ w3, const float *__restrict__ b3, float *__restrict__ y)
{
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char *sa = tc_smem, *sb = tc_smem + kTcABytes;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(tc_smem + kTcABytes + kTcBBytes);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(tc_smem + kTcABytes + kTcBBytes + 8);
    float *sw3 = reinterpret_cast<float *>(tc_smem + kTcABytes + kTcBBytes + 64);  // W3 as float, [k][j]
    float *sb2 = sw3 + kTcN * kTcOut, *sb3 = sb2 + kTcN;
    float *ypart = sb3 + kTcOut;              // [2][kTcM][kTcOut]: the two column halves' outputs
    float *sx = ypart + 2 * kTcM * kTcOut;    // the current tile's inputs, [kTcM][kTcIn]
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int ntiles = (rows + kTcM - 1) / kTcM;
    const uint32_t sa_s = (uint32_t)__cvta_generic_to_shared(sa), sb_s = (uint32_t)__cvta_generic_to_shared(sb);
    const uint32_t sx_s = (uint32_t)__cvta_generic_to_shared(sx);
    auto load_x = [&](int tile) {  // one 16-byte chunk per thread
        static_assert(kTcXBytes / 16 == kTcFwdThreads, "a tile's inputs are one chunk per thread");
        const int m0 = tile * kTcM, r = t / 2;
        const bool in = m0 + r < rows;
        cp_async16(sx_s + 16 * t, x + (size_t)(in ? m0 + r : 0) * kTcIn + 4 * (t & 1), in ? 16u : 0u);
    };
    for (uint32_t i = t; i < kTcBBytes / 16; i += kTcFwdThreads) cp_async16(sb_s + 16 * i, wimg + 8 * i, 16u);
    if ((int)blockIdx.x < ntiles) load_x(blockIdx.x);
    for (int i = t; i < kTcN * kTcOut; i += kTcFwdThreads) sw3[i] = __bfloat162float(w3[i]);
    for (int i = t; i < kTcN; i += kTcFwdThreads) sb2[i] = b2[i];
    if (t < kTcOut) sb3[t] = b3[t];
    // this lane's 8 columns of the first layer (the same for every row it computes)
    const int k0 = lane * 8;
    float w1r[kTcIn][8], b1r[8];
#pragma unroll
    for (int i = 0; i < kTcIn; ++i)
#pragma unroll
        for (int e = 0; e < 8; ++e) w1r[i][e] = __bfloat162float(w1[i * kTcN + k0 + e]);
#pragma unroll
    for (int e = 0; e < 8; ++e) b1r[e] = b1[k0 + e];
    // the first layer of a tile (its inputs in sx) into shared memory: warp w
    // takes rows w, w + 8, ..., lane its 8 columns; rows past the end are zero
    auto layer1 = [&](int tile) {
        const int m0 = tile * kTcM;
        for (int r = warp; r < kTcM; r += kTcFwdThreads / 32) {
            __align__(16) __nv_bfloat16 hb[8];
            if (m0 + r < rows) {
                float xb[kTcIn];
#pragma unroll
                for (int i = 0; i < kTcIn; ++i) xb[i] = __bfloat162float(__float2bfloat16_rn(sx[r * kTcIn + i]));
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    float acc = 0.f;
#pragma unroll
                    for (int i = 0; i < kTcIn; ++i) acc = __fmaf_rn(xb[i], w1r[i][e], acc);
                    hb[e] = __float2bfloat16_rn(fmaxf(__fadd_rn(acc, b1r[e]), 0.f));
                }
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) hb[e] = __float2bfloat16_rn(0.f);
            }
            *reinterpret_cast<uint4 *>(sa + core_off(r, k0)) = *reinterpret_cast<const uint4 *>(hb);
        }
    };
    const uint32_t mbar_a = (uint32_t)__cvta_generic_to_shared(mbar);
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_a));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {  // two accumulators: 512 columns of tensor memory
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::
                         "r"((uint32_t)__cvta_generic_to_shared(tmem_slot)), "r"(2u * kTcN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();  // the first tile's inputs and the tables are in place
    if ((int)blockIdx.x < ntiles) layer1(blockIdx.x);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc =
        (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
    auto issue = [&](uint32_t acc_col) {  // one thread: the tile's product into the accumulator at acc_col
#pragma unroll 1
        for (int kk = 0; kk < kTcK / 16; ++kk) {
            const uint64_t ad = smem_desc(sa_s + kk * 256, 128, (kTcK / 8) * 128);
            const uint64_t bd = smem_desc(sb_s + kk * 256, 128, (kTcK / 8) * 128);
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem + acc_col),
                "l"(ad), "l"(bd), "r"(idesc), "r"(kk));
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_a)
                     : "memory");
    };
    uint32_t phase = 0, buf = 0;
    if (t == 0 && (int)blockIdx.x < ntiles) issue(0);
    const int quarter = warp & 3, half = warp >> 2;  // accumulator lanes 32 * quarter.., columns 128 * half..
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int nxt = tile + gridDim.x;
        if (nxt < ntiles) load_x(nxt);  // sx is free: this tile's first layer is done
        // wait for this tile's product (bounded: a wait that gives up flags an error)
        uint32_t done = 0;
        for (uint32_t it = 0; it < kTcSpinLimit && !done; ++it)
            asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                         " selp.u32 %0, 1, 0, p;\n}\n"
                         : "=r"(done)
                         : "r"(mbar_a), "r"(phase)
                         : "memory");
        phase ^= 1u;
        asm volatile("cp.async.wait_all;" ::: "memory");
        done = __syncthreads_and(done);  // one decision for the CTA; the next inputs are in place
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (!done) {
            atomicExch(&g_mlp_tc_error, 1u);
            break;
        }
        // the next tile's first layer into the freed buffer, and its product
        // into the other accumulator, while this tile's is read out
        if (nxt < ntiles) {
            layer1(nxt);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (t == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                issue((buf ^ 1u) * kTcN);
            }
        }
        // epilogue: bias, ReLU, BF16 and the output layer over this warp's half of the columns
        const int rl = quarter * 32 + lane;  // row within the tile
        const uint32_t trow = tmem + buf * kTcN + ((uint32_t)(quarter * 32) << 16);
        float yo[kTcOut] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
        for (int c = half * (kTcN / 2); c < (half + 1) * (kTcN / 2); c += 32) {
            uint32_t v[32];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(trow + (uint32_t)c));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int e = 0; e < 32; ++e) {
                const float hv = __bfloat162float(
                    __float2bfloat16_rn(fmaxf(__fadd_rn(__uint_as_float(v[e]), sb2[c + e]), 0.f)));
#pragma unroll
                for (int j = 0; j < kTcOut; ++j) yo[j] = __fmaf_rn(hv, sw3[(c + e) * kTcOut + j], yo[j]);
            }
        }
        *reinterpret_cast<float4 *>(ypart + (half * kTcM + rl) * kTcOut) = make_float4(yo[0], yo[1], yo[2], yo[3]);
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();  // this accumulator is read before a later tile's product reuses it
        if (half == 0) {
            const int r = tile * kTcM + rl;
            const float4 a0 = *reinterpret_cast<const float4 *>(ypart + rl * kTcOut);
            const float4 a1 = *reinterpret_cast<const float4 *>(ypart + (kTcM + rl) * kTcOut);
            if (r < rows)
                *reinterpret_cast<float4 *>(y + (size_t)r * kTcOut) =
                    make_float4(__fadd_rn(__fadd_rn(a0.x, a1.x), sb3[0]), __fadd_rn(__fadd_rn(a0.y, a1.y), sb3[1]),
                                __fadd_rn(__fadd_rn(a0.z, a1.z), sb3[2]), __fadd_rn(__fadd_rn(a0.w, a1.w), sb3[3]));
        }
        buf ^= 1u;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2u * kTcN));
    }
}

// Mean squared error over rows x cols and its gradient 2 (y - t) / (rows * cols).
__global__ void k_mlp_mse(const float *__restrict__ y, const float *__restrict__ t, int n, float scale,
                          float *__restrict__ dy, __nv_bfloat16 *__restrict__ dy16, double *loss)
{
    __shared__ double part[8];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double e2 = 0.0;
    if (i < n) {
        const float e = y[i] - t[i];
        e2 = (double)e * e;
        dy[i] = 2.f * e * scale;
        dy16[i] = __float2bfloat16_rn(2.f * e * scale);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e2 += __shfl_down_sync(0xffffffffu, e2, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = e2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w];
        atomicAdd(loss, s * scale);
    }
}

// db[c] = sum over rows of d[r][c].
__global__ void k_mlp_colsum(const float *__restrict__ d, int rows, int cols, float *__restrict__ db)
{
    const int c = blockIdx.x;
    float s = 0.f;
    for (int r = threadIdx.x; r < rows; r += blockDim.x) s += d[(long long)r * cols + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ float part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
        db[c] = t;
    }
}

// Adam on the FP32 master parameters; refreshes their BF16 copy.
__global__ void k_mlp_adam(float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                           float *__restrict__ v, __nv_bfloat16 *__restrict__ p16, long long n, float lr, float b1,
                           float b2, float c1, float c2, float eps)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = gr[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float q = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = q;
    p16[i] = __float2bfloat16_rn(q);
}

__global__ void k_to_bf16(const float *__restrict__ x, __nv_bfloat16 *__restrict__ y, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

__global__ void k_gather_rows(const float *__restrict__ src, const int *__restrict__ idx, int rows, int cols,
                              float *__restrict__ dst)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)rows * cols) return;
    const long long r = i / cols, c = i - r * cols;
    dst[i] = src[(long long)idx[r] * cols + c];
}

unsigned nb(long long n, int t) { return (unsigned)((n + t - 1) / t); }

int fail(int code, const std::string &m) { return boidsgpu::set_last_error(code, m.c_str()); }

#define MCK(call)                                                                                   \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return fail(BOIDS_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

// Parameter layout (FP32 master and BF16 copy): W1 [in x h], b1 [h],
// W2 [h x h], b2 [h], W3 [h x out], b3 [out]; W row-major (fan-in rows).
struct boids_mlp {
    int in = 0, h = 0, out = 0, device = 0;
    long long np = 0;
    long long off[6] = {};
    float *p = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *p16 = nullptr;
    long long step = 0;
    // activations for up to cap rows
    int cap = 0;
    float *x = nullptr, *t = nullptr, *pre1 = nullptr, *pre2 = nullptr, *y = nullptr, *dy = nullptr,
          *d2 = nullptr, *d1 = nullptr;
    __nv_bfloat16 *x16 = nullptr, *h1 = nullptr, *h2 = nullptr, *dy16 = nullptr, *d2_16 = nullptr, *d1_16 = nullptr;
    double *loss = nullptr;
    cudaStream_t st = nullptr;
    __nv_bfloat16 *w2img = nullptr;  // the hidden weights in the tensor-core layout (hidden width 256)
    unsigned nsm = 1;                 // SMs: the tensor-core kernel's persistent grid
};

namespace {

void free_acts(boids_mlp *m)
{
    void *q[] = {m->x, m->t, m->pre1, m->pre2, m->y, m->dy, m->d2, m->d1, m->x16, m->h1, m->h2, m->dy16, m->d2_16,
                 m->d1_16};
    for (void *p : q)
        if (p) cudaFree(p);
    m->x = m->t = m->pre1 = m->pre2 = m->y = m->dy = m->d2 = m->d1 = nullptr;
    m->x16 = m->h1 = m->h2 = m->dy16 = m->d2_16 = m->d1_16 = nullptr;
    m->cap = 0;
}

int ensure_rows(boids_mlp *m, int rows)
{
    if (rows <= m->cap) return 0;
    free_acts(m);
    const long long r = rows;
    auto A = [&](auto **p, long long n) { return cudaMalloc((void **)p, sizeof(**p) * (size_t)(n ? n : 1)); };
    if (A(&m->x, r * m->in) || A(&m->t, r * m->out) || A(&m->pre1, r * m->h) || A(&m->pre2, r * m->h) ||
        A(&m->y, r * m->out) || A(&m->dy, r * m->out) || A(&m->d2, r * m->h) || A(&m->d1, r * m->h) ||
        A(&m->x16, r * m->in) || A(&m->h1, r * m->h) || A(&m->h2, r * m->h) || A(&m->dy16, r * m->out) ||
        A(&m->d2_16, r * m->h) || A(&m->d1_16, r * m->h)) {
        cudaGetLastError();
        free_acts(m);
        return fail(BOIDS_ENOMEM, "boids_mlp: cudaMalloc of activations failed");
    }
    m->cap = rows;
    return 0;
}

void gemm(boids_mlp *m, MatB A, MatB B, float *C, int ldc, __nv_bfloat16 *C16, int ld16, const float *bias,
          const float *mask, int ldm, int relu16)
{
    dim3 grid(nb(B.cols, kTileN), nb(A.rows, 16 * kWarpsM));
    k_mlp_gemm<<<grid, 32 * kWarpsM, 0, m->st>>>(A, B, C, ldc, C16, ld16, bias, mask, ldm, relu16);
}

MatB rowmajor(const __nv_bfloat16 *p, int rows, int cols) { return MatB{p, cols, 1, rows, cols}; }
MatB transposed(const __nv_bfloat16 *p, int rows, int cols)  // the transpose of a row-major rows x cols
{
    return MatB{p, 1, rows == 0 ? 0 : cols, cols, rows};
}

// Forward pass of `rows` rows already in m->x16; output in m->y.  A hidden
// width of 256 puts the hidden-to-hidden product on the tensor cores.
void forward(boids_mlp *m, int rows, bool need_pre = true)
{
    const __nv_bfloat16 *W1 = m->p16 + m->off[0], *W2 = m->p16 + m->off[2], *W3 = m->p16 + m->off[4];
    const float *b1 = m->p + m->off[1], *b2 = m->p + m->off[3], *b3 = m->p + m->off[5];
    gemm(m, rowmajor(m->x16, rows, m->in), rowmajor(W1, m->in, m->h), m->pre1, m->h, m->h1, m->h, b1, nullptr, 0, 1);
    if (m->w2img) {
        k_mlp_tile_w<<<nb(kTcN * kTcK / 8, 256), 256, 0, m->st>>>(W2, m->w2img);
        const unsigned tiles = nb(rows, kTcM);
        k_mlp_hidden_tc<<<tiles < m->nsm ? tiles : m->nsm, kTcThreads, kTcSmem, m->st>>>(
            m->h1, rows, m->w2img, b2, need_pre ? m->pre2 : nullptr, m->h2);
    } else {
        gemm(m, rowmajor(m->h1, rows, m->h), rowmajor(W2, m->h, m->h), m->pre2, m->h, m->h2, m->h, b2, nullptr, 0,
             1);
    }
    gemm(m, rowmajor(m->h2, rows, m->h), rowmajor(W3, m->h, m->out), m->y, m->out, nullptr, 0, b3, nullptr, 0, 0);
}

// Loss and gradient of `rows` rows (targets in m->t) into m->grad.
void backward(boids_mlp *m, int rows)
{
    const __nv_bfloat16 *W2 = m->p16 + m->off[2], *W3 = m->p16 + m->off[4];
    float *gW1 = m->grad + m->off[0], *gb1 = m->grad + m->off[1], *gW2 = m->grad + m->off[2],
          *gb2 = m->grad + m->off[3], *gW3 = m->grad + m->off[4], *gb3 = m->grad + m->off[5];
    const int n = rows * m->out;
    k_mlp_mse<<<nb(n, 256), 256, 0, m->st>>>(m->y, m->t, n, 1.f / (float)n, m->dy, m->dy16, m->loss);
    // layer 3: dW3 = h2^T dy, db3 = colsum(dy), d2 = (dy W3^T) * (pre2 > 0)
    gemm(m, transposed(m->h2, rows, m->h), rowmajor(m->dy16, rows, m->out), gW3, m->out, nullptr, 0, nullptr,
         nullptr, 0, 0);
    k_mlp_colsum<<<m->out, 256, 0, m->st>>>(m->dy, rows, m->out, gb3);
    gemm(m, rowmajor(m->dy16, rows, m->out), transposed(W3, m->h, m->out), m->d2, m->h, m->d2_16, m->h, nullptr,
         m->pre2, m->h, 0);
    // layer 2
    gemm(m, transposed(m->h1, rows, m->h), rowmajor(m->d2_16, rows, m->h), gW2, m->h, nullptr, 0, nullptr, nullptr,
         0, 0);
    k_mlp_colsum<<<m->h, 256, 0, m->st>>>(m->d2, rows, m->h, gb2);
    gemm(m, rowmajor(m->d2_16, rows, m->h), transposed(W2, m->h, m->h), m->d1, m->h, m->d1_16, m->h, nullptr,
         m->pre1, m->h, 0);
    // layer 1
    gemm(m, transposed(m->x16, rows, m->in), rowmajor(m->d1_16, rows, m->h), gW1, m->h, nullptr, 0, nullptr, nullptr,
         0, 0);
    k_mlp_colsum<<<m->h, 256, 0, m->st>>>(m->d1, rows, m->h, gb1);
}

// A tensor-core tile whose wait on its accumulator gave up (the flag is
// cleared for the next call).
int tc_status(boids_mlp *m)
{
    if (!m->w2img) return 0;
    uint32_t err = 0;
    MCK(cudaMemcpyFromSymbolAsync(&err, g_mlp_tc_error, sizeof err, 0, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    if (!err) return 0;
    const uint32_t zero = 0;
    MCK(cudaMemcpyToSymbolAsync(g_mlp_tc_error, &zero, sizeof zero, 0, cudaMemcpyHostToDevice, m->st));
    return fail(BOIDS_ECUDA, "boids_mlp: a tensor-core tile's wait for its accumulator gave up");
}

int upload_rows(boids_mlp *m, const float *x, const float *t, int rows)
{
    MCK(cudaMemcpyAsync(m->x, x, sizeof(float) * (size_t)rows * m->in, cudaMemcpyHostToDevice, m->st));
    if (t) MCK(cudaMemcpyAsync(m->t, t, sizeof(float) * (size_t)rows * m->out, cudaMemcpyHostToDevice, m->st));
    k_to_bf16<<<nb((long long)rows * m->in, 256), 256, 0, m->st>>>(m->x, m->x16, (long long)rows * m->in);
    return 0;
}

// splitmix64-driven uniform in [-a, a]
float uni(uint64_t &s, float a)
{
    s += 0x9e3779b97f4a7c15ULL;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    z ^= z >> 31;
    return (float)(((double)(z >> 11) / 9007199254740992.0) * 2.0 - 1.0) * a;
}

}  // namespace

extern "C" {

int boids_mlp_create(int32_t n_in, int32_t n_hidden, int32_t n_out, uint64_t seed, int32_t device, boids_mlp **out)
{
    if (!out || n_in <= 0 || n_hidden <= 0 || n_out <= 0 || n_in > 4096 || n_hidden > 4096 || n_out > 4096)
        return fail(BOIDS_EINVAL, "boids_mlp_create: bad argument");
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return fail(BOIDS_ECUDA, "boids_mlp_create: cudaSetDevice");
    boids_mlp *m = new boids_mlp();
    m->in = n_in;
    m->h = n_hidden;
    m->out = n_out;
    m->device = device;
    const long long sz[6] = {(long long)n_in * n_hidden, n_hidden, (long long)n_hidden * n_hidden, n_hidden,
                             (long long)n_hidden * n_out, n_out};
    for (int i = 0; i < 6; ++i) {
        m->off[i] = m->np;
        m->np += sz[i];
    }
    // He-uniform weights, zero biases
    std::vector<float> h(m->np, 0.f);
    uint64_t s = seed;
    const int fan[3] = {n_in, n_hidden, n_hidden};
    for (int l = 0; l < 3; ++l) {
        const float a = std::sqrt(6.f / (float)fan[l]);
        for (long long i = 0; i < sz[2 * l]; ++i) h[m->off[2 * l] + i] = uni(s, a);
    }
    bool ok = cudaMalloc(&m->p, 4 * m->np) == cudaSuccess && cudaMalloc(&m->grad, 4 * m->np) == cudaSuccess &&
              cudaMalloc(&m->m, 4 * m->np) == cudaSuccess && cudaMalloc(&m->v, 4 * m->np) == cudaSuccess &&
              cudaMalloc(&m->p16, 2 * m->np) == cudaSuccess && cudaMalloc(&m->loss, 8) == cudaSuccess &&
              cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaMemcpy(m->p, h.data(), 4 * m->np, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(m->m, 0, 4 * m->np) == cudaSuccess && cudaMemset(m->v, 0, 4 * m->np) == cudaSuccess;
    if (ok) {
        k_to_bf16<<<nb(m->np, 256), 256, 0, m->st>>>(m->p, m->p16, m->np);
        ok = cudaStreamSynchronize(m->st) == cudaSuccess;
    }
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && nsm > 0)
        m->nsm = (unsigned)nsm;
    if (ok && n_hidden == kTcN) {  // the hidden product on the tensor cores
        ok = cudaMalloc(&m->w2img, kTcBBytes) == cudaSuccess &&
             cudaFuncSetAttribute(k_mlp_hidden_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem) ==
                 cudaSuccess &&
             cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kTcFwdSmem) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        boids_mlp_destroy(m);
        return fail(BOIDS_ENOMEM, "boids_mlp_create: device allocation failed");
    }
    *out = m;
    return BOIDS_OK;
}

void boids_mlp_destroy(boids_mlp *m)
{
    if (!m) return;
    cudaSetDevice(m->device);
    if (m->st) cudaStreamSynchronize(m->st);
    free_acts(m);
    void *q[] = {m->p, m->grad, m->m, m->v, m->p16, m->loss, m->w2img};
    for (void *p : q)
        if (p) cudaFree(p);
    if (m->st) cudaStreamDestroy(m->st);
    delete m;
}

int64_t boids_mlp_param_count(boids_mlp *m) { return m ? m->np : 0; }

int boids_mlp_get_params(boids_mlp *m, float *params)
{
    if (!m || !params) return fail(BOIDS_EINVAL, "boids_mlp_get_params: bad argument");
    cudaSetDevice(m->device);
    MCK(cudaMemcpyAsync(params, m->p, 4 * m->np, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    return BOIDS_OK;
}

int boids_mlp_set_params(boids_mlp *m, const float *params)
{
    if (!m || !params) return fail(BOIDS_EINVAL, "boids_mlp_set_params: bad argument");
    cudaSetDevice(m->device);
    MCK(cudaMemcpyAsync(m->p, params, 4 * m->np, cudaMemcpyHostToDevice, m->st));
    k_to_bf16<<<nb(m->np, 256), 256, 0, m->st>>>(m->p, m->p16, m->np);
    MCK(cudaMemsetAsync(m->m, 0, 4 * m->np, m->st));
    MCK(cudaMemsetAsync(m->v, 0, 4 * m->np, m->st));
    m->step = 0;
    MCK(cudaStreamSynchronize(m->st));
    return BOIDS_OK;
}

int boids_mlp_forward(boids_mlp *m, const float *x, int32_t rows, float *y)
{
    if (!m || (!x && rows) || (!y && rows) || rows < 0) return fail(BOIDS_EINVAL, "boids_mlp_forward: bad argument");
    if (rows == 0) return BOIDS_OK;
    cudaSetDevice(m->device);
    if (int rc = ensure_rows(m, rows)) return rc;
    if (m->w2img && m->in == kTcIn && m->out == kTcOut) {
        // the fused pass: x in, y out, one kernel after the weight image
        MCK(cudaMemcpyAsync(m->x, x, sizeof(float) * (size_t)rows * m->in, cudaMemcpyHostToDevice, m->st));
        const __nv_bfloat16 *W1 = m->p16 + m->off[0], *W2 = m->p16 + m->off[2], *W3 = m->p16 + m->off[4];
        const float *b1 = m->p + m->off[1], *b2 = m->p + m->off[3], *b3 = m->p + m->off[5];
        k_mlp_tile_w<<<nb(kTcN * kTcK / 8, 256), 256, 0, m->st>>>(W2, m->w2img);
        const unsigned tiles = nb(rows, kTcM);
        k_mlp_forward_tc<<<tiles < m->nsm ? tiles : m->nsm, kTcFwdThreads, kTcFwdSmem, m->st>>>(
            m->x, rows, W1, b1, m->w2img, b2, W3, b3, m->y);
    } else {
        if (int rc = upload_rows(m, x, nullptr, rows)) return rc;
        forward(m, rows, false);  // inference: the backward pass's pre-activations are not needed
    }
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(y, m->y, sizeof(float) * (size_t)rows * m->out, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    return tc_status(m);
}

int boids_mlp_gradient(boids_mlp *m, const float *x, const float *t, int32_t rows, float *grad, double *loss)
{
    if (!m || !x || !t || !grad || rows <= 0) return fail(BOIDS_EINVAL, "boids_mlp_gradient: bad argument");
    cudaSetDevice(m->device);
    if (int rc = ensure_rows(m, rows)) return rc;
    if (int rc = upload_rows(m, x, t, rows)) return rc;
    MCK(cudaMemsetAsync(m->loss, 0, 8, m->st));
    forward(m, rows);
    backward(m, rows);
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(grad, m->grad, 4 * m->np, cudaMemcpyDeviceToHost, m->st));
    double l = 0;
    MCK(cudaMemcpyAsync(&l, m->loss, 8, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    if (loss) *loss = l;
    return tc_status(m);
}

int boids_mlp_train(boids_mlp *m, const float *x, const float *t, int32_t rows, int32_t epochs, int32_t batch,
                    float lr, uint64_t shuffle_seed, double *last_epoch_loss)
{
    if (!m || !x || !t || rows <= 0 || epochs < 0 || batch <= 0)
        return fail(BOIDS_EINVAL, "boids_mlp_train: bad argument");
    cudaSetDevice(m->device);
    if (batch > rows) batch = rows;
    if (int rc = ensure_rows(m, rows + batch)) return rc;
    // the whole set stays resident: rows [0, rows) of x/t; batches are gathered behind it
    float *X = m->x, *T = m->t;
    MCK(cudaMemcpyAsync(X, x, sizeof(float) * (size_t)rows * m->in, cudaMemcpyHostToDevice, m->st));
    MCK(cudaMemcpyAsync(T, t, sizeof(float) * (size_t)rows * m->out, cudaMemcpyHostToDevice, m->st));
    int *d_idx = nullptr;
    float *bx = nullptr, *bt = nullptr;
    if (cudaMalloc(&d_idx, sizeof(int) * rows) != cudaSuccess ||
        cudaMalloc(&bx, sizeof(float) * (size_t)batch * m->in) != cudaSuccess ||
        cudaMalloc(&bt, sizeof(float) * (size_t)batch * m->out) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_idx);
        cudaFree(bx);
        return fail(BOIDS_ENOMEM, "boids_mlp_train: cudaMalloc failed");
    }
    std::vector<int> idx(rows);
    for (int i = 0; i < rows; ++i) idx[i] = i;
    uint64_t s = shuffle_seed;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    double epoch_loss = 0.0;
    int rc = 0;
    float *keep_x = m->x, *keep_t = m->t;
    for (int ep = 0; ep < epochs && !rc; ++ep) {
        for (int i = rows - 1; i > 0; --i) {  // Fisher-Yates
            s += 0x9e3779b97f4a7c15ULL;
            uint64_t z = s;
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
            z ^= z >> 31;
            const int j = (int)(z % (uint64_t)(i + 1));
            std::swap(idx[i], idx[j]);
        }
        if (cudaMemcpyAsync(d_idx, idx.data(), sizeof(int) * rows, cudaMemcpyHostToDevice, m->st) != cudaSuccess ||
            cudaMemsetAsync(m->loss, 0, 8, m->st) != cudaSuccess) {
            rc = fail(BOIDS_ECUDA, "boids_mlp_train: copy failed");
            break;
        }
        int nbatch = 0;
        for (int b0 = 0; b0 < rows; b0 += batch, ++nbatch) {
            const int r = std::min(batch, rows - b0);
            k_gather_rows<<<nb((long long)r * m->in, 256), 256, 0, m->st>>>(keep_x, d_idx + b0, r, m->in, bx);
            k_gather_rows<<<nb((long long)r * m->out, 256), 256, 0, m->st>>>(keep_t, d_idx + b0, r, m->out, bt);
            // the forward/backward buffers read x/t from m->x/m->t: point them at the batch
            m->x = bx;
            m->t = bt;
            k_to_bf16<<<nb((long long)r * m->in, 256), 256, 0, m->st>>>(bx, m->x16, (long long)r * m->in);
            forward(m, r);
            backward(m, r);
            m->x = keep_x;
            m->t = keep_t;
            ++m->step;
            const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
            k_mlp_adam<<<nb(m->np, 256), 256, 0, m->st>>>(m->p, m->grad, m->m, m->v, m->p16, m->np, lr, b1, b2, c1,
                                                         c2, eps);
        }
        double l = 0;
        if (cudaMemcpyAsync(&l, m->loss, 8, cudaMemcpyDeviceToHost, m->st) != cudaSuccess ||
            cudaStreamSynchronize(m->st) != cudaSuccess) {
            rc = fail(BOIDS_ECUDA, std::string("boids_mlp_train: ") + cudaGetErrorString(cudaGetLastError()));
            break;
        }
        epoch_loss = l / nbatch;
    }
    if (!rc && cudaGetLastError() != cudaSuccess) rc = fail(BOIDS_ECUDA, "boids_mlp_train: kernel launch failed");
    if (!rc) rc = tc_status(m);
    cudaFree(d_idx);
    cudaFree(bx);
    cudaFree(bt);
    if (last_epoch_loss) *last_epoch_loss = epoch_loss;
    return rc;
}

}  // extern "C"
