// mlp.cu -- the learned warm start of the Jacobi solve (no reference counterpart).
//
// A 7 -> 64 -> 64 -> 1 ReLU network maps per-particle features of the first
// density pass (neighbour count, density ratio, kernel width, the plain Jacobi
// lambda, velocity divergence, the previous substep's applied lambda sum and its
// neighbour mean) to an initial lambda that replaces the plain one in the first
// position update.  Weights are BF16 on the tensor cores with FP32
// accumulation: inference with tcgen05.mma into TMEM (k_mlp_tc); training
// (k_mlp_grad) runs the per-row forward and backward on mma.sync m16n8k16 and the two
// weight-gradient GEMMs, sums over the CTA's rows, as one tcgen05.mma into TMEM; the
// master copy is FP32.
//
// Parameter vector (FP32), offsets in floats:
//   0 mu[8]  8 inv_sigma[8]  16 W1[64][8]  528 b1[64]  592 W2[64][64]  4688 b2[64]
//   4752 w3[64]  4816 b3  4817 y_scale  4818 y_mean  4819 omega_max  4820 min_neighbors
//   4821..4823 reserved                                 (4824 floats, 4801 trained)
//
// Two guards of the solver hook (not used by the network itself):
//   omega_max > 0 bounds the learned lambda to a per-particle over-relaxation of
//   the plain one: lambda_hat in [omega_max * lambda, lambda] where the plain
//   lambda is negative, 0 elsewhere;
//   a particle with fewer than min_neighbors neighbours keeps the plain lambda
//   (spray and thin sheets, where an over-push can separate a pair for good).
//
// Fragment layouts of mma.m16n8k16 (lane = 4 g + q):
//   A 16x16 row: a0 (g, 2q..2q+1) a1 (g+8, 2q..) a2 (g, 2q+8..) a3 (g+8, 2q+8..)
//   B 16x8 col:  b0 (k = 2q..2q+1, n = g)  b1 (k = 2q+8.., n = g)
//   C 16x8:      c0,c1 (g, 2q..2q+1)  c2,c3 (g+8, 2q..2q+1)
// so the accumulators of n-tiles 2s and 2s+1 are exactly the A fragment of k-step s
// of the next layer.
#include <cuda_bf16.h>

#include <algorithm>

#include "apbf_internal.cuh"

namespace apbf {

constexpr int kP_MU = 0, kP_IS = 8, kP_W1 = 16, kP_B1 = 528, kP_W2 = 592, kP_B2 = 4688, kP_W3 = 4752, kP_B3 = 4816,
              kP_YS = 4817, kP_YM = 4818, kP_OM = 4819, kP_NMIN = 4820, kP_N = 4824;
constexpr int kH = 64;          // hidden width
constexpr int kF = 8;           // feature slots (7 used)
constexpr int kRowsWarp = 32;   // rows per warp (two m16 tiles)
constexpr int kWarps = 4;
constexpr int kRowsCta = kRowsWarp * kWarps;
constexpr int kLd = 72;         // bf16 row stride of 64-wide tiles in shared memory (bank-conflict free)

namespace {

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Shared-memory copy of the weights in BF16.
struct SmemW {
    __nv_bfloat16 w1[kH * 16];   // [n][16]: features 0..7, zeros 8..15
    __nv_bfloat16 w2[kH * kLd];  // [n][k]
    __nv_bfloat16 w2t[kH * kLd]; // [k][n]
    float b1[kH], b2[kH], w3[kH];
    float mu[kF], is[kF];
    float b3, ys, ym, om, nmin;
};

__device__ void load_weights(SmemW &w, const float *__restrict__ P) {
    for (int t = threadIdx.x; t < kH * 16; t += blockDim.x) {
        const int n = t / 16, f = t % 16;
        w.w1[t] = __float2bfloat16_rn(f < kF ? P[kP_W1 + n * kF + f] : 0.0f);
    }
    for (int t = threadIdx.x; t < kH * kH; t += blockDim.x) {
        const int n = t / kH, k = t % kH;
        const __nv_bfloat16 v = __float2bfloat16_rn(P[kP_W2 + t]);
        w.w2[n * kLd + k] = v;
        w.w2t[k * kLd + n] = v;
    }
    for (int t = threadIdx.x; t < kH; t += blockDim.x) {
        w.b1[t] = P[kP_B1 + t];
        w.b2[t] = P[kP_B2 + t];
        w.w3[t] = P[kP_W3 + t];
    }
    for (int t = threadIdx.x; t < kF; t += blockDim.x) {
        w.mu[t] = P[kP_MU + t];
        w.is[t] = P[kP_IS + t];
    }
    if (threadIdx.x == 0) {
        w.b3 = P[kP_B3];
        w.ys = P[kP_YS];
        w.ym = P[kP_YM];
        w.om = P[kP_OM];
        w.nmin = P[kP_NMIN];
    }
}

// Activations of one warp: two m16 tiles of 32 rows.
struct Acts {
    uint32_t x[2][4];     // A fragments of the normalised features (k 0..15)
    float h1[2][8][4];    // relu(layer 1), C layout
    float h2[2][8][4];    // relu(layer 2), C layout
    float y[2][2];        // output of rows g and g+8 of each tile (normalised space)
};

__device__ __forceinline__ void forward_warp(const SmemW &w, const float *__restrict__ X, uint32_t row0, uint32_t nrows,
                                             Acts &A) {
    const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const uint32_t r0 = row0 + 16 * t + g, r1 = r0 + 8;
        float x00 = 0.f, x01 = 0.f, x10 = 0.f, x11 = 0.f;
        if (r0 < nrows) {
            x00 = (X[(size_t)r0 * kF + 2 * q] - w.mu[2 * q]) * w.is[2 * q];
            x01 = (X[(size_t)r0 * kF + 2 * q + 1] - w.mu[2 * q + 1]) * w.is[2 * q + 1];
        }
        if (r1 < nrows) {
            x10 = (X[(size_t)r1 * kF + 2 * q] - w.mu[2 * q]) * w.is[2 * q];
            x11 = (X[(size_t)r1 * kF + 2 * q + 1] - w.mu[2 * q + 1]) * w.is[2 * q + 1];
        }
        A.x[t][0] = pack_bf16(x00, x01);
        A.x[t][1] = pack_bf16(x10, x11);
        A.x[t][2] = 0u;
        A.x[t][3] = 0u;
    }
    // layer 1
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int n = 8 * j + g;
        const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&w.w1[n * 16 + 2 * q]);
        const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&w.w1[n * 16 + 8 + 2 * q]);
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            float d[4] = {w.b1[8 * j + 2 * q], w.b1[8 * j + 2 * q + 1], w.b1[8 * j + 2 * q], w.b1[8 * j + 2 * q + 1]};
            mma16816(d, A.x[t], b0, b1);
#pragma unroll
            for (int e = 0; e < 4; ++e) A.h1[t][j][e] = fmaxf(d[e], 0.0f);
        }
    }
    // layer 2
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        uint32_t a[4][4];
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            a[s][0] = pack_bf16(A.h1[t][2 * s][0], A.h1[t][2 * s][1]);
            a[s][1] = pack_bf16(A.h1[t][2 * s][2], A.h1[t][2 * s][3]);
            a[s][2] = pack_bf16(A.h1[t][2 * s + 1][0], A.h1[t][2 * s + 1][1]);
            a[s][3] = pack_bf16(A.h1[t][2 * s + 1][2], A.h1[t][2 * s + 1][3]);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = 8 * j + g;
            float d[4] = {w.b2[8 * j + 2 * q], w.b2[8 * j + 2 * q + 1], w.b2[8 * j + 2 * q], w.b2[8 * j + 2 * q + 1]};
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&w.w2[n * kLd + 16 * s + 2 * q]);
                const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&w.w2[n * kLd + 16 * s + 8 + 2 * q]);
                mma16816(d, a[s], b0, b1);
            }
#pragma unroll
            for (int e = 0; e < 4; ++e) A.h2[t][j][e] = fmaxf(d[e], 0.0f);
        }
        // layer 3: y = h2 . w3 + b3 over the quad's 16 columns, then across the quad
        float y0 = 0.f, y1 = 0.f;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float wa = w.w3[8 * j + 2 * q], wb = w.w3[8 * j + 2 * q + 1];
            y0 += A.h2[t][j][0] * wa + A.h2[t][j][1] * wb;
            y1 += A.h2[t][j][2] * wa + A.h2[t][j][3] * wb;
        }
        y0 += __shfl_xor_sync(0xffffffffu, y0, 1);
        y0 += __shfl_xor_sync(0xffffffffu, y0, 2);
        y1 += __shfl_xor_sync(0xffffffffu, y1, 1);
        y1 += __shfl_xor_sync(0xffffffffu, y1, 2);
        A.y[t][0] = y0 + w.b3;
        A.y[t][1] = y1 + w.b3;
    }
}

// ---- inference on the 5th-generation tensor cores (tcgen05, accumulators in TMEM) ----
//
// A CTA of 128 threads runs tiles of 128 rows; thread t owns row t.  The operands
// of the two hidden layers sit in shared memory in the canonical K-major layout
// without swizzle: 8-row x 16-byte core matrices, K-adjacent cores 128 B apart
// (leading byte offset), 8-row groups 16 B x K apart (stride byte offset).  One
// thread issues tcgen05.mma (M 128, N 64, K 16 per instruction, BF16 in, FP32
// accumulators in 64 TMEM columns that both layers reuse), tcgen05.commit arrives
// on an mbarrier, and every warp reads its 32 TMEM lanes back with tcgen05.ld.
// Bias, ReLU, the 64 -> 1 output layer and the solver's guards run on the CUDA
// cores in FP32.  Waits are bounded: a wait that gives up marks the outputs NaN
// (and the status word, in the solver hook) and the kernel frees its TMEM.

constexpr int kTcRows = 128;
constexpr uint32_t kTcCols = 64;  // TMEM columns per CTA
constexpr uint32_t kTcIdesc = (1u << 4)                // D: FP32
                              | (1u << 7) | (1u << 10)  // A, B: BF16
                              | ((64u >> 3) << 17)      // N = 64
                              | ((128u >> 4) << 24);    // M = 128; A and B K-major

// The network as the kernel keeps it in shared memory: BF16 weights in the operand
// layout and the FP32 vectors.  Built once per parameter vector (k_mlp_pack) so
// that a CTA fetches it with one bulk copy.
struct TcImage {
    unsigned char w1[kH * 16 * 2];  // B of layer 1: N 64 x K 16
    unsigned char w2[kH * kH * 2];  // B of layer 2: N 64 x K 64
    float b1[kH], b2[kH], w3[kH], mu[kF], is[kF];
    float b3, ys, ym, om, nmin, pad[3];
};
static_assert(sizeof(TcImage) % 16 == 0, "bulk copies move multiples of 16 bytes");
constexpr uint32_t kTcImageBytes = sizeof(TcImage);
constexpr size_t kTcA1 = (sizeof(TcImage) + 1023) / 1024 * 1024;

struct __align__(1024) TcSmem {
    TcImage img;
    unsigned char pad_[kTcA1 - sizeof(TcImage)];
    unsigned char a1[kTcRows * 16 * 2];  // A of layer 1: M 128 x K 16 (normalised features)
    unsigned char a2[kTcRows * kH * 2];  // A of layer 2: M 128 x K 64 (relu(layer 1))
    unsigned long long bar;              // MMA completion
    unsigned long long bar_w;            // arrival of the weight image
    uint32_t tmem;
};

// Byte offset of element (row, k) of a K-major operand with K columns.
__device__ __forceinline__ uint32_t core_off(uint32_t row, uint32_t k, uint32_t K) {
    return (row >> 3) * (K * 16u) + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start, leading and stride byte offsets (>> 4),
// the descriptor version bit 46, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(const void *p, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((smem_u32(p) & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(kTcIdesc), "r"(accumulate));
}
__device__ __forceinline__ void tc_mma_id(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate,
                                          uint32_t idesc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void tc_commit(unsigned long long *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Bounded wait for the mbarrier phase `parity`.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity) {
    const uint32_t b = smem_u32(bar);
    for (uint32_t it = 0; it < (1u << 20); ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(b), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 16 FP32 columns of this thread's TMEM lane; the wait is tied to the registers so
// that no use is scheduled before the load has completed.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Builds the image from the FP32 parameter vector, thread t of nt.
__device__ __forceinline__ void build_image(TcImage &img, const float *__restrict__ P, int t0, int nt) {
    for (int t = t0; t < kH * 16; t += nt) {
        const int n = t >> 4, k = t & 15;
        *reinterpret_cast<__nv_bfloat16 *>(img.w1 + core_off(n, k, 16)) =
            __float2bfloat16_rn(k < kF ? P[kP_W1 + n * kF + k] : 0.0f);
    }
    for (int t = t0; t < kH * kH; t += nt) {
        const int n = t >> 6, k = t & 63;
        *reinterpret_cast<__nv_bfloat16 *>(img.w2 + core_off(n, k, kH)) = __float2bfloat16_rn(P[kP_W2 + t]);
    }
    for (int t = t0; t < kH; t += nt) {
        img.b1[t] = P[kP_B1 + t];
        img.b2[t] = P[kP_B2 + t];
        img.w3[t] = P[kP_W3 + t];
    }
    for (int t = t0; t < kF; t += nt) {
        img.mu[t] = P[kP_MU + t];
        img.is[t] = P[kP_IS + t];
    }
    if (t0 == 0) {
        img.b3 = P[kP_B3];
        img.ys = P[kP_YS];
        img.ym = P[kP_YM];
        img.om = P[kP_OM];
        img.nmin = P[kP_NMIN];
        img.pad[0] = img.pad[1] = img.pad[2] = 0.0f;
    }
}

__global__ void k_mlp_pack(const float *__restrict__ P, TcImage *img) { build_image(*img, P, threadIdx.x, blockDim.x); }

struct TcOut {
    // MODE 0: out[r] = the network's output in physical units
    float *out;
    // MODE 1 (the solver hook): lambda_hat with the guards replaces the plain lambda in
    // the solve record, the packed record and the self shift
    const float4 *selfdir;
    float4 *rec;
    int4 *pk;
    int4 *shift;
    Status *st;
};

// image != null: the weights arrive by one bulk copy (cp.async.bulk) of the packed
// image; else every CTA builds them from the FP32 parameters.
template <int MODE>
__global__ void __launch_bounds__(kTcRows) k_mlp_tc(const float *__restrict__ P, const TcImage *image,
                                                    const float *__restrict__ X, uint32_t nrows, const uint32_t *d_len,
                                                    int early_exit, TcOut o) {
    __shared__ TcSmem sm;
    if (MODE == 1 && early_exit && *(volatile const uint32_t *)&o.st->converged) return;  // uniform
    const uint32_t n = MODE == 1 ? d_len[kLenParticles] : nrows;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&sm.bar)) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&sm.bar_w)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (image) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&sm.bar_w)),
                         "r"(kTcImageBytes)
                         : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(&sm.img)),
                "l"(image), "r"(kTcImageBytes), "r"(smem_u32(&sm.bar_w))
                : "memory");
        }
    }
    if (!image) build_image(sm.img, P, tid, blockDim.x);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    bool ok = true;
    unsigned long long *pending = &sm.bar_w;  // the barrier of a wait that gave up, and its phase
    uint32_t pending_parity = 0;
    if (image) ok = __syncthreads_and(mbar_wait(&sm.bar_w, 0u)) != 0;  // the weights are in
    const uint32_t tmem = sm.tmem;
    const uint32_t lane_tmem = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's 32 lanes
    const uint64_t a1 = tc_desc(sm.a1, 128u, 256u), b1 = tc_desc(sm.img.w1, 128u, 256u);
    uint32_t phase = 0;
    for (uint32_t base = blockIdx.x * kTcRows; base < n && ok; base += gridDim.x * kTcRows) {
        const uint32_t r = base + tid;
        const bool valid = r < n;
        // layer 1 operand: the normalised features (slots 8..15 zero)
        float x[kF];
#pragma unroll
        for (int f = 0; f < kF; ++f) x[f] = valid ? (X[(size_t)r * kF + f] - sm.img.mu[f]) * sm.img.is[f] : 0.0f;
        uint4 lo;
        lo.x = pack_bf16(x[0], x[1]);
        lo.y = pack_bf16(x[2], x[3]);
        lo.z = pack_bf16(x[4], x[5]);
        lo.w = pack_bf16(x[6], x[7]);
        *reinterpret_cast<uint4 *>(sm.a1 + core_off(tid, 0, 16)) = lo;
        *reinterpret_cast<uint4 *>(sm.a1 + core_off(tid, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            tc_mma(tmem, a1, b1, 0u);
            tc_commit(&sm.bar);
        }
        ok = __syncthreads_and(mbar_wait(&sm.bar, phase)) != 0;
        if (!ok) {
            pending = &sm.bar;
            pending_parity = phase;
            break;
        }
        phase ^= 1u;
        tc_fence_after();
        // relu(layer 1 + b1) -> the layer-2 operand
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float v[16];
            tmem_ld16(lane_tmem + 16u * c, v);
            uint4 h0, h1;
            h0.x = pack_bf16(fmaxf(v[0] + sm.img.b1[16 * c + 0], 0.f), fmaxf(v[1] + sm.img.b1[16 * c + 1], 0.f));
            h0.y = pack_bf16(fmaxf(v[2] + sm.img.b1[16 * c + 2], 0.f), fmaxf(v[3] + sm.img.b1[16 * c + 3], 0.f));
            h0.z = pack_bf16(fmaxf(v[4] + sm.img.b1[16 * c + 4], 0.f), fmaxf(v[5] + sm.img.b1[16 * c + 5], 0.f));
            h0.w = pack_bf16(fmaxf(v[6] + sm.img.b1[16 * c + 6], 0.f), fmaxf(v[7] + sm.img.b1[16 * c + 7], 0.f));
            h1.x = pack_bf16(fmaxf(v[8] + sm.img.b1[16 * c + 8], 0.f), fmaxf(v[9] + sm.img.b1[16 * c + 9], 0.f));
            h1.y = pack_bf16(fmaxf(v[10] + sm.img.b1[16 * c + 10], 0.f), fmaxf(v[11] + sm.img.b1[16 * c + 11], 0.f));
            h1.z = pack_bf16(fmaxf(v[12] + sm.img.b1[16 * c + 12], 0.f), fmaxf(v[13] + sm.img.b1[16 * c + 13], 0.f));
            h1.w = pack_bf16(fmaxf(v[14] + sm.img.b1[16 * c + 14], 0.f), fmaxf(v[15] + sm.img.b1[16 * c + 15], 0.f));
            *reinterpret_cast<uint4 *>(sm.a2 + core_off(tid, 16 * c, kH)) = h0;
            *reinterpret_cast<uint4 *>(sm.a2 + core_off(tid, 16 * c + 8, kH)) = h1;
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                tc_mma(tmem, tc_desc(sm.a2 + 256 * k, 128u, 1024u), tc_desc(sm.img.w2 + 256 * k, 128u, 1024u),
                       k > 0 ? 1u : 0u);
            tc_commit(&sm.bar);
        }
        ok = __syncthreads_and(mbar_wait(&sm.bar, phase)) != 0;
        if (!ok) {
            pending = &sm.bar;
            pending_parity = phase;
            break;
        }
        phase ^= 1u;
        tc_fence_after();
        // layer 3 on the CUDA cores: y = relu(layer 2 + b2) . w3 + b3
        float y = sm.img.b3;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float v[16];
            tmem_ld16(lane_tmem + 16u * c, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) y += fmaxf(v[i] + sm.img.b2[16 * c + i], 0.0f) * sm.img.w3[16 * c + i];
        }
        tc_fence_before();  // this tile's TMEM reads are done before the next tile's MMA
        if (!valid) continue;
        if (MODE == 0) {
            o.out[r] = y * sm.img.ys + sm.img.ym;
        } else {
            float lam = y * sm.img.ys + sm.img.ym;
            const float l0 = X[(size_t)r * kF + 3];  // the plain lambda of this pass
            if (sm.img.om > 0.0f) lam = l0 < 0.0f ? fminf(fmaxf(lam, sm.img.om * l0), l0) : 0.0f;
            if (X[(size_t)r * kF] < sm.img.nmin) lam = l0;  // too few neighbours: the plain lambda
            lam = fminf(lam, 0.0f);
            float4 rc = o.rec[r];
            rc.x = lam;
            o.rec[r] = rc;
            o.pk[r].w = __float_as_int(lam);
            const float4 sd = o.selfdir[r];  // selfGrad (xyz), inverse mass (w)
            int4 sh = make_int4(0, 0, 0, 0);
            if (lam < 0.0f) {
                const float sc = lam * sd.w * APBF_FIX;
                sh.x = f2i(sd.x * sc);
                sh.y = f2i(sd.y * sc);
                sh.z = f2i(sd.z * sc);
            }
            sh.w = o.shift[r].w;  // the density pass's deferred-filter flag
            o.shift[r] = sh;
        }
    }
    if (!ok) {
        // a copy or an MMA that did not complete in time: its results are not used; wait
        // (bounded) for it before the TMEM is freed, and report
        mbar_wait(pending, pending_parity);
        if (tid == 0) {
            if (MODE == 1) set_flag(o.st, APBF_FLAG_SPIN_LIMIT);
        }
        if (MODE == 0)
            for (uint32_t r = blockIdx.x * kTcRows + tid; r < n; r += gridDim.x * kTcRows) o.out[r] = __int_as_float(0x7fc00000);
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
    }
}

// Persistent grid: a few CTAs per SM, each loading the weights once.
static int tc_grid(uint32_t rows) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
    }
    const uint32_t tiles = (rows + kTcRows - 1) / kTcRows;
    const uint32_t cap = (uint32_t)sms * 6u;  // 6 x 64 TMEM columns of 512 per SM
    return (int)std::max(1u, std::min(tiles, cap));
}

// Weight gradients as one GEMM on the tensor cores: D (M 128 x N 80, FP32 in TMEM)
// = A B^T summed over the CTA's 128 rows (K), A = [dH2^T; dH1^T] (rows 0..63: the
// hidden-2 deltas, 64..127: the hidden-1 deltas) and B = [h1^T; x^T] (rows 0..63:
// relu(layer 1), 64..79: the 16 feature slots, 8..15 zero), both K-major in the
// canonical layout without swizzle.  Rows 0..63, columns 0..63 of D are dW2; rows
// 64..127, columns 64..71 are dW1 (the off-diagonal blocks are not used).
constexpr uint32_t kGradN = 80;
constexpr uint32_t kGradCols = 128;  // TMEM columns: a power of two >= kGradN
constexpr uint32_t kGradIdesc = (1u << 4)                   // D: FP32
                                | (1u << 7) | (1u << 10)     // A, B: BF16
                                | ((kGradN >> 3) << 17)      // N = 80
                                | ((128u >> 4) << 24);       // M = 128; A and B K-major
constexpr size_t kGradOffA = (sizeof(SmemW) + 1023) / 1024 * 1024;
constexpr size_t kGradOffB = kGradOffA + (size_t)128 * kRowsCta * 2;
constexpr size_t kGradOffR = kGradOffB + (size_t)kGradN * kRowsCta * 2;
constexpr size_t kGradOffBar = kGradOffR + (size_t)kWarps * (3 * kH + 2) * sizeof(float);
constexpr size_t kGradSmem = kGradOffBar + 16;
static_assert(kRowsCta == 128, "the weight-gradient GEMM takes K = 128 rows per CTA");

// Training: forward + backward of one CTA's 128 rows; the CTA's gradient (sum over
// its rows of d loss / d param) goes to partials[blockIdx.x][param];
// partials[..][kP_N - 1] holds the CTA's weighted sum of squared errors.  Loss =
// mean over the batch of w(e) e^2 with e = y - t in the normalised space and
// w = over_weight where e < 0 (a lambda more negative than the target: a larger
// push than the plain solve made), 1 elsewhere -- an expectile regression that,
// for over_weight > 1, keeps the prediction below the target where it is uncertain.
__global__ void __launch_bounds__(kRowsCta) k_mlp_grad(const float *__restrict__ P, const float *__restrict__ X,
                                                        const float *__restrict__ T, uint32_t nrows,
                                                        float over_weight, float *__restrict__ partials) {
    extern __shared__ __align__(1024) unsigned char smem[];
    SmemW &w = *reinterpret_cast<SmemW *>(smem);
    unsigned char *ga = smem + kGradOffA;  // A of the weight-gradient GEMM (M 128 x K 128)
    unsigned char *gb = smem + kGradOffB;  // B (N 80 x K 128)
    float(*red)[3 * kH + 2] = reinterpret_cast<float(*)[3 * kH + 2]>(smem + kGradOffR);  // per warp
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem + kGradOffBar);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + kGradOffBar + 8);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kGradCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        tc_fence_before();
    }
    load_weights(w, P);
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    auto put = [](unsigned char *op, int row, int k, float v) {
        *reinterpret_cast<__nv_bfloat16 *>(op + core_off((uint32_t)row, (uint32_t)k, kRowsCta)) = __float2bfloat16_rn(v);
    };
    const uint32_t base = blockIdx.x * kRowsCta;
    const uint32_t row0 = base + warp * kRowsWarp;
    const float inv_b = 1.0f / (float)nrows;
    Acts A;
    forward_warp(w, X, row0, nrows, A);

    float db1[8][2], db2[8][2], dw3[8][2];
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int c = 0; c < 2; ++c) db1[j][c] = db2[j][c] = dw3[j][c] = 0.0f;
    float db3 = 0.0f, sse = 0.0f;
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const uint32_t r0 = row0 + 16 * t + g, r1 = r0 + 8;
        const float e0 = r0 < nrows ? A.y[t][0] - T[r0] : 0.0f;
        const float e1 = r1 < nrows ? A.y[t][1] - T[r1] : 0.0f;
        const float w0 = e0 < 0.0f ? over_weight : 1.0f, w1 = e1 < 0.0f ? over_weight : 1.0f;
        const float dy0 = 2.0f * (w0 * e0) * inv_b, dy1 = 2.0f * (w1 * e1) * inv_b;
        if (q == 0) {
            sse += w0 * e0 * e0 + w1 * e1 * e1;
            db3 += dy0 + dy1;
        }
        // dH2 = dy w3 relu'(h2); dw3 += dy h2; db2 += dH2
        float dh2[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float wa = w.w3[8 * j + 2 * q], wb = w.w3[8 * j + 2 * q + 1];
            dh2[j][0] = A.h2[t][j][0] > 0.0f ? dy0 * wa : 0.0f;
            dh2[j][1] = A.h2[t][j][1] > 0.0f ? dy0 * wb : 0.0f;
            dh2[j][2] = A.h2[t][j][2] > 0.0f ? dy1 * wa : 0.0f;
            dh2[j][3] = A.h2[t][j][3] > 0.0f ? dy1 * wb : 0.0f;
            dw3[j][0] += dy0 * A.h2[t][j][0] + dy1 * A.h2[t][j][2];
            dw3[j][1] += dy0 * A.h2[t][j][1] + dy1 * A.h2[t][j][3];
            db2[j][0] += dh2[j][0] + dh2[j][2];
            db2[j][1] += dh2[j][1] + dh2[j][3];
        }
        // dH1 = dH2 W2 relu'(h1)  (B operand from the transposed copy)
        uint32_t a[4][4];
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            a[s][0] = pack_bf16(dh2[2 * s][0], dh2[2 * s][1]);
            a[s][1] = pack_bf16(dh2[2 * s][2], dh2[2 * s][3]);
            a[s][2] = pack_bf16(dh2[2 * s + 1][0], dh2[2 * s + 1][1]);
            a[s][3] = pack_bf16(dh2[2 * s + 1][2], dh2[2 * s + 1][3]);
        }
        float dh1[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = 8 * j + g;  // output column = W2 input index k
            float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&w.w2t[n * kLd + 16 * s + 2 * q]);
                const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&w.w2t[n * kLd + 16 * s + 8 + 2 * q]);
                mma16816(d, a[s], b0, b1);
            }
#pragma unroll
            for (int e = 0; e < 4; ++e) dh1[j][e] = A.h1[t][j][e] > 0.0f ? d[e] : 0.0f;
            db1[j][0] += dh1[j][0] + dh1[j][2];
            db1[j][1] += dh1[j][1] + dh1[j][3];
        }
        // the operands of the weight-gradient GEMM: local row = K index
        const int lr0 = warp * kRowsWarp + 16 * t + g, lr1 = lr0 + 8;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c0 = 8 * j + 2 * q, c1 = c0 + 1;
            put(ga, c0, lr0, dh2[j][0]);
            put(ga, c1, lr0, dh2[j][1]);
            put(ga, c0, lr1, dh2[j][2]);
            put(ga, c1, lr1, dh2[j][3]);
            put(ga, kH + c0, lr0, dh1[j][0]);
            put(ga, kH + c1, lr0, dh1[j][1]);
            put(ga, kH + c0, lr1, dh1[j][2]);
            put(ga, kH + c1, lr1, dh1[j][3]);
            put(gb, c0, lr0, A.h1[t][j][0]);
            put(gb, c1, lr0, A.h1[t][j][1]);
            put(gb, c0, lr1, A.h1[t][j][2]);
            put(gb, c1, lr1, A.h1[t][j][3]);
        }
        // normalised features (A fragment a0/a1 hold columns 2q, 2q+1 of rows g, g+8),
        // slots 8..15 zero
        const __nv_bfloat162 x0 = *reinterpret_cast<const __nv_bfloat162 *>(&A.x[t][0]);
        const __nv_bfloat162 x1 = *reinterpret_cast<const __nv_bfloat162 *>(&A.x[t][1]);
        const auto putb = [&](int row, int k, __nv_bfloat16 v) {
            *reinterpret_cast<__nv_bfloat16 *>(gb + core_off((uint32_t)(kH + row), (uint32_t)k, kRowsCta)) = v;
        };
        putb(2 * q, lr0, x0.x);
        putb(2 * q + 1, lr0, x0.y);
        putb(2 * q, lr1, x1.x);
        putb(2 * q + 1, lr1, x1.y);
        putb(2 * q + 8, lr0, __float2bfloat16_rn(0.0f));
        putb(2 * q + 9, lr0, __float2bfloat16_rn(0.0f));
        putb(2 * q + 8, lr1, __float2bfloat16_rn(0.0f));
        putb(2 * q + 9, lr1, __float2bfloat16_rn(0.0f));
    }
    // warp reductions of the vector gradients over the 8 row groups (lanes with equal q)
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int off = 4; off < 32; off <<= 1) {
                db1[j][c] += __shfl_xor_sync(0xffffffffu, db1[j][c], off);
                db2[j][c] += __shfl_xor_sync(0xffffffffu, db2[j][c], off);
                dw3[j][c] += __shfl_xor_sync(0xffffffffu, dw3[j][c], off);
            }
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        db3 += __shfl_xor_sync(0xffffffffu, db3, off);
        sse += __shfl_xor_sync(0xffffffffu, sse, off);
    }
    if (g == 0) {
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                red[warp][8 * j + 2 * q + c] = db1[j][c];
                red[warp][kH + 8 * j + 2 * q + c] = db2[j][c];
                red[warp][2 * kH + 8 * j + 2 * q + c] = dw3[j][c];
            }
    }
    if (lane == 0) {
        red[warp][3 * kH] = db3;
        red[warp][3 * kH + 1] = sse;
    }
    __syncthreads();
    float *out = partials + (size_t)blockIdx.x * kP_N;
    for (int t = threadIdx.x; t < 3 * kH + 2; t += blockDim.x) {
        float v = 0.0f;
        for (int k = 0; k < kWarps; ++k) v += red[k][t];  // fixed order
        if (t < kH) out[kP_B1 + t] = v;
        else if (t < 2 * kH) out[kP_B2 + t - kH] = v;
        else if (t < 3 * kH) out[kP_W3 + t - 2 * kH] = v;
        else if (t == 3 * kH) out[kP_B3] = v;
        else out[kP_N - 1] = v;
    }
    // dW2 and dW1 on the tensor cores: one thread issues the 8 K-steps of 16 rows,
    // the commit arrives on the mbarrier, and thread t reads row t of D from its lane
    fence_async_smem();  // the operands written above, for the tensor core's proxy
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < kRowsCta / 16; ++k)
            tc_mma_id(tmem, tc_desc(ga + 256 * k, 128u, kRowsCta * 16u), tc_desc(gb + 256 * k, 128u, kRowsCta * 16u),
                      k > 0 ? 1u : 0u, kGradIdesc);
        tc_commit(bar);
    }
    const bool ok = __syncthreads_and(mbar_wait(bar, 0u)) != 0;
    const int tr = threadIdx.x;  // row of D (its TMEM lane)
    const uint32_t lane_tmem = tmem + ((uint32_t)(warp * 32) << 16);
    if (ok) {
        tc_fence_after();
        if (warp < 2) {  // rows 0..63: dW2[tr][0..63]
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float v[16];
                tmem_ld16(lane_tmem + 16u * c, v);
#pragma unroll
                for (int i = 0; i < 16; ++i) out[kP_W2 + tr * kH + 16 * c + i] = v[i];
            }
        } else {  // rows 64..127, columns 64..71: dW1[tr - 64][0..7]
            float v[16];
            tmem_ld16(lane_tmem + 64u, v);
#pragma unroll
            for (int f = 0; f < kF; ++f) out[kP_W1 + (tr - kH) * kF + f] = v[f];
        }
    } else {
        // the MMA did not complete in time: wait (bounded) before the TMEM is freed, and
        // mark the weight gradients NaN (the loss and the parameters show it)
        mbar_wait(bar, 0u);
        for (int t = tr; t < kH * kH; t += blockDim.x) out[kP_W2 + t] = __int_as_float(0x7fc00000);
        for (int t = tr; t < kH * kF; t += blockDim.x) out[kP_W1 + t] = __int_as_float(0x7fc00000);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kGradCols) : "memory");
    }
}

// Fixed-order sum of the CTA gradients, then Adam on the trained parameters.
__global__ void k_mlp_adam(float *P, float *m, float *v, const float *__restrict__ partials, int ctas, float lr,
                           float b1p, float b2p, float *grad_out, float *loss_out, uint32_t nrows) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kP_N) return;
    float gsum = 0.0f;
    for (int c = 0; c < ctas; ++c) gsum += partials[(size_t)c * kP_N + t];
    if (t == kP_N - 1) {
        if (loss_out) *loss_out = gsum / (float)nrows;
        return;
    }
    const bool trained = t >= kP_W1 && t <= kP_B3;
    if (grad_out) grad_out[t] = trained ? gsum : 0.0f;
    if (!trained || lr == 0.0f) return;
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    const float mt = beta1 * m[t] + (1.0f - beta1) * gsum;
    const float vt = beta2 * v[t] + (1.0f - beta2) * gsum * gsum;
    m[t] = mt;
    v[t] = vt;
    P[t] -= lr * (mt / (1.0f - b1p)) / (sqrtf(vt / (1.0f - b2p)) + eps);
}

}  // namespace

static_assert(kP_N == kMlpParams, "parameter vector size");

apbf_status mlp_forward(const float *P, const float *X, uint32_t nrows, float *out, cudaStream_t s) {
    if (nrows == 0) return APBF_OK;
    TcOut o = {};
    o.out = out;
    k_mlp_tc<0><<<tc_grid(nrows), kTcRows, 0, s>>>(P, nullptr, X, nrows, nullptr, 0, o);
    APBF_CUDA(cudaGetLastError());
    return APBF_OK;
}

apbf_status mlp_train_step(float *P, float *m, float *v, float *partials, const float *X, const float *T,
                           uint32_t nrows, float lr, float over_weight, uint32_t step, float *grad_out,
                           float *loss_out, cudaStream_t s) {
    if (nrows == 0) return APBF_OK;
    const uint32_t ctas = (nrows + kRowsCta - 1) / kRowsCta;
    APBF_CUDA(cudaMemsetAsync(partials, 0, (size_t)ctas * kP_N * sizeof(float), s));
    static bool attr_set = false;
    if (!attr_set) {
        APBF_CUDA(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem));
        attr_set = true;
    }
    k_mlp_grad<<<ctas, kRowsCta, kGradSmem, s>>>(P, X, T, nrows, over_weight, partials);
    APBF_CUDA(cudaGetLastError());
    const float b1p = powf(0.9f, (float)(step + 1)), b2p = powf(0.999f, (float)(step + 1));
    k_mlp_adam<<<(kP_N + 255) / 256, 256, 0, s>>>(P, m, v, partials, (int)ctas, lr, b1p, b2p, grad_out, loss_out,
                                                   nrows);
    APBF_CUDA(cudaGetLastError());
    return APBF_OK;
}

uint32_t mlp_partials_floats(uint32_t nrows) { return ((nrows + kRowsCta - 1) / kRowsCta) * (uint32_t)kP_N; }

apbf_status mlp_pack(const float *P, void *image, cudaStream_t s) {
    k_mlp_pack<<<1, 256, 0, s>>>(P, reinterpret_cast<TcImage *>(image));
    APBF_CUDA(cudaGetLastError());
    return APBF_OK;
}

size_t mlp_image_bytes() { return sizeof(TcImage); }

apbf_status mlp_lambda(apbf_ctx *ctx, cudaStream_t s, bool early_exit) {
    TcOut o = {};
    o.selfdir = ctx->selfdir;
    o.rec = ctx->solve_rec;
    o.pk = ctx->solve_pk;
    o.shift = ctx->shift;
    o.st = ctx->status;
    APBF_BEFORE_LAUNCH(ctx, s, "k_mlp_tc");
    k_mlp_tc<1><<<tc_grid(ctx->cfg.particle_capacity), kTcRows, 0, s>>>(
        ctx->mlp_params, reinterpret_cast<const TcImage *>(ctx->mlp_image), ctx->features, 0u, ctx->d_len,
        early_exit ? 1 : 0, o);
    APBF_AFTER_LAUNCH(ctx, s, "k_mlp_tc");
    return APBF_OK;
}

}  // namespace apbf
