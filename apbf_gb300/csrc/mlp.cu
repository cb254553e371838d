// mlp.cu -- the learned warm start of the Jacobi solve (no reference counterpart).
//
// A 7 -> 64 -> 64 -> 1 ReLU network maps per-particle features of the first
// density pass (neighbour count, density ratio, kernel width, the plain Jacobi
// lambda, velocity divergence, the previous substep's applied lambda sum and its
// neighbour mean) to an initial lambda that replaces the plain one in the first
// position update.  Weights are BF16 on the tensor cores with FP32
// accumulation (mma.sync m16n8k16); the master copy is FP32.
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
constexpr int kLdT = kRowsCta + 8;  // bf16 row stride of transposed [64][128] tiles

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

// Inference over a batch: out[r] = y(r) in physical units (y * y_scale + y_mean).
__global__ void __launch_bounds__(kRowsCta) k_mlp_forward(const float *__restrict__ P, const float *__restrict__ X,
                                                           uint32_t nrows, float *__restrict__ out) {
    __shared__ SmemW w;
    load_weights(w, P);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    for (uint32_t base = blockIdx.x * kRowsCta; base < nrows; base += gridDim.x * kRowsCta) {
        const uint32_t row0 = base + warp * kRowsWarp;
        Acts A;
        forward_warp(w, X, row0, nrows, A);
        if (q == 0) {
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                const uint32_t r0 = row0 + 16 * t + g, r1 = r0 + 8;
                if (r0 < nrows) out[r0] = A.y[t][0] * w.ys + w.ym;
                if (r1 < nrows) out[r1] = A.y[t][1] * w.ys + w.ym;
            }
        }
    }
}

// The learned first correction: lambda_hat from the features of the first
// density pass replaces the plain lambda in the solve record and in the self
// shift (incompressibility_2.comp:106-109 with lambda_hat).
__global__ void __launch_bounds__(kRowsCta) k_mlp_lambda(const float *__restrict__ P, const float *__restrict__ X,
                                                          const float4 *__restrict__ selfdir, float4 *rec, int4 *pk,
                                                          int4 *shift,
                                                          const uint32_t *d_len, const Status *st, int early_exit) {
    if (early_exit && *(volatile const uint32_t *)&st->converged) return;
    __shared__ SmemW w;
    load_weights(w, P);
    __syncthreads();
    const uint32_t n = d_len[kLenParticles];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    for (uint32_t base = blockIdx.x * kRowsCta; base < n; base += gridDim.x * kRowsCta) {
        const uint32_t row0 = base + warp * kRowsWarp;
        Acts A;
        forward_warp(w, X, row0, n, A);
        // quad lane q writes row g of tile q/2 (q even: row g, odd: row g+8)
#pragma unroll
        for (int t = 0; t < 2; ++t)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (q != 2 * t + h) continue;
                const uint32_t r = row0 + 16 * t + g + 8 * h;
                if (r >= n) continue;
                float lam = A.y[t][h] * w.ys + w.ym;
                const float l0 = X[(size_t)r * kF + 3];  // the plain lambda of this pass
                if (w.om > 0.0f) lam = l0 < 0.0f ? fminf(fmaxf(lam, w.om * l0), l0) : 0.0f;
                if (X[(size_t)r * kF] < w.nmin) lam = l0;  // too few neighbours: the plain lambda
                lam = fminf(lam, 0.0f);
                float4 rc = rec[r];
                rc.x = lam;
                rec[r] = rc;
                pk[r].w = __float_as_int(lam);
                const float4 sd = selfdir[r];  // selfGrad (xyz), inverse mass (w)
                int4 sh = make_int4(0, 0, 0, 0);
                if (lam < 0.0f) {
                    const float sc = lam * sd.w * APBF_FIX;
                    sh.x = f2i(sd.x * sc);
                    sh.y = f2i(sd.y * sc);
                    sh.z = f2i(sd.z * sc);
                }
                sh.w = shift[r].w;  // the density pass's deferred-filter flag
                shift[r] = sh;
            }
    }
}

constexpr size_t kGradOffT = (sizeof(SmemW) + 15) / 16 * 16;
constexpr size_t kGradSmem = kGradOffT + (size_t)(3 * kH + 16) * kLdT * sizeof(__nv_bfloat16) +
                             (size_t)kWarps * (3 * kH + 2) * sizeof(float);

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
    extern __shared__ __align__(16) unsigned char smem[];
    SmemW &w = *reinterpret_cast<SmemW *>(smem);
    __nv_bfloat16 *dh2t = reinterpret_cast<__nv_bfloat16 *>(smem + kGradOffT);   // [n][row]
    __nv_bfloat16 *h1t = dh2t + kH * kLdT;                                        // [k][row]
    __nv_bfloat16 *dh1t = h1t + kH * kLdT;                                        // [n][row]
    __nv_bfloat16 *xt = dh1t + kH * kLdT;                                         // [f][row]
    float(*red)[3 * kH + 2] = reinterpret_cast<float(*)[3 * kH + 2]>(xt + 16 * kLdT);  // per warp
    load_weights(w, P);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
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
        // stage transposed tiles for the weight-gradient GEMMs
        const int lr0 = warp * kRowsWarp + 16 * t + g, lr1 = lr0 + 8;  // local rows
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c0 = 8 * j + 2 * q, c1 = c0 + 1;
            dh2t[c0 * kLdT + lr0] = __float2bfloat16_rn(dh2[j][0]);
            dh2t[c1 * kLdT + lr0] = __float2bfloat16_rn(dh2[j][1]);
            dh2t[c0 * kLdT + lr1] = __float2bfloat16_rn(dh2[j][2]);
            dh2t[c1 * kLdT + lr1] = __float2bfloat16_rn(dh2[j][3]);
            h1t[c0 * kLdT + lr0] = __float2bfloat16_rn(A.h1[t][j][0]);
            h1t[c1 * kLdT + lr0] = __float2bfloat16_rn(A.h1[t][j][1]);
            h1t[c0 * kLdT + lr1] = __float2bfloat16_rn(A.h1[t][j][2]);
            h1t[c1 * kLdT + lr1] = __float2bfloat16_rn(A.h1[t][j][3]);
            dh1t[c0 * kLdT + lr0] = __float2bfloat16_rn(dh1[j][0]);
            dh1t[c1 * kLdT + lr0] = __float2bfloat16_rn(dh1[j][1]);
            dh1t[c0 * kLdT + lr1] = __float2bfloat16_rn(dh1[j][2]);
            dh1t[c1 * kLdT + lr1] = __float2bfloat16_rn(dh1[j][3]);
        }
        // normalised features (A fragment a0/a1 hold columns 2q, 2q+1 of rows g, g+8)
        const __nv_bfloat162 x0 = *reinterpret_cast<const __nv_bfloat162 *>(&A.x[t][0]);
        const __nv_bfloat162 x1 = *reinterpret_cast<const __nv_bfloat162 *>(&A.x[t][1]);
        xt[(2 * q) * kLdT + lr0] = x0.x;
        xt[(2 * q + 1) * kLdT + lr0] = x0.y;
        xt[(2 * q) * kLdT + lr1] = x1.x;
        xt[(2 * q + 1) * kLdT + lr1] = x1.y;
        xt[(2 * q + 8) * kLdT + lr0] = __float2bfloat16_rn(0.0f);
        xt[(2 * q + 9) * kLdT + lr0] = __float2bfloat16_rn(0.0f);
        xt[(2 * q + 8) * kLdT + lr1] = __float2bfloat16_rn(0.0f);
        xt[(2 * q + 9) * kLdT + lr1] = __float2bfloat16_rn(0.0f);
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
    // dW2[n][k] = sum_r dH2[r][n] h1[r][k]: warp w owns rows n of m-tile w
    {
        const int m0 = 16 * warp;
        float acc[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
        for (int s = 0; s < kRowsCta / 16; ++s) {
            uint32_t a[4];
            a[0] = *reinterpret_cast<const uint32_t *>(&dh2t[(m0 + g) * kLdT + 16 * s + 2 * q]);
            a[1] = *reinterpret_cast<const uint32_t *>(&dh2t[(m0 + g + 8) * kLdT + 16 * s + 2 * q]);
            a[2] = *reinterpret_cast<const uint32_t *>(&dh2t[(m0 + g) * kLdT + 16 * s + 8 + 2 * q]);
            a[3] = *reinterpret_cast<const uint32_t *>(&dh2t[(m0 + g + 8) * kLdT + 16 * s + 8 + 2 * q]);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int k = 8 * j + g;
                const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&h1t[k * kLdT + 16 * s + 2 * q]);
                const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&h1t[k * kLdT + 16 * s + 8 + 2 * q]);
                mma16816(acc[j], a, b0, b1);
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c = 8 * j + 2 * q;
            out[kP_W2 + (m0 + g) * kH + c] = acc[j][0];
            out[kP_W2 + (m0 + g) * kH + c + 1] = acc[j][1];
            out[kP_W2 + (m0 + g + 8) * kH + c] = acc[j][2];
            out[kP_W2 + (m0 + g + 8) * kH + c + 1] = acc[j][3];
        }
    }
    // dW1[n][f] = sum_r dH1[r][n] x[r][f]
    {
        const int m0 = 16 * warp;
        float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int s = 0; s < kRowsCta / 16; ++s) {
            uint32_t a[4];
            a[0] = *reinterpret_cast<const uint32_t *>(&dh1t[(m0 + g) * kLdT + 16 * s + 2 * q]);
            a[1] = *reinterpret_cast<const uint32_t *>(&dh1t[(m0 + g + 8) * kLdT + 16 * s + 2 * q]);
            a[2] = *reinterpret_cast<const uint32_t *>(&dh1t[(m0 + g) * kLdT + 16 * s + 8 + 2 * q]);
            a[3] = *reinterpret_cast<const uint32_t *>(&dh1t[(m0 + g + 8) * kLdT + 16 * s + 8 + 2 * q]);
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int f = 8 * j + g;
                const uint32_t b0 = *reinterpret_cast<const uint32_t *>(&xt[f * kLdT + 16 * s + 2 * q]);
                const uint32_t b1 = *reinterpret_cast<const uint32_t *>(&xt[f * kLdT + 16 * s + 8 + 2 * q]);
                mma16816(acc[j], a, b0, b1);
            }
        }
        // only features 0..7 are parameters (tile j = 0)
        const int c = 2 * q;
        out[kP_W1 + (m0 + g) * kF + c] = acc[0][0];
        out[kP_W1 + (m0 + g) * kF + c + 1] = acc[0][1];
        out[kP_W1 + (m0 + g + 8) * kF + c] = acc[0][2];
        out[kP_W1 + (m0 + g + 8) * kF + c + 1] = acc[0][3];
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
    const uint32_t ctas = (nrows + kRowsCta - 1) / kRowsCta;
    k_mlp_forward<<<ctas < 4096u ? ctas : 4096u, kRowsCta, 0, s>>>(P, X, nrows, out);
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

apbf_status mlp_lambda(apbf_ctx *ctx, cudaStream_t s, bool early_exit) {
    const uint32_t cap = ctx->cfg.particle_capacity;
    const uint32_t ctas = (cap + kRowsCta - 1) / kRowsCta;
    APBF_BEFORE_LAUNCH(ctx, s, "k_mlp_lambda");
    k_mlp_lambda<<<ctas < 2048u ? ctas : 2048u, kRowsCta, 0, s>>>(ctx->mlp_params, ctx->features, ctx->selfdir,
                                                                  ctx->solve_rec, ctx->solve_pk, ctx->shift, ctx->d_len,
                                                                  ctx->status, early_exit ? 1 : 0);
    APBF_AFTER_LAUNCH(ctx, s, "k_mlp_lambda");
    return APBF_OK;
}

}  // namespace apbf
