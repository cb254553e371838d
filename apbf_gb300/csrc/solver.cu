// solver.cu -- incompressibility::apply (source/incompressibility.cpp:12-45), one
// Jacobi iteration in two gather passes instead of the reference's four
// dispatches with per-pair integer atomics:
//
//  k_density_lambda (particle i, over its own row):  incompressibility_0.comp
//    (self density) + incompressibility_1.comp (density, weighted gradient and
//    squared-gradient sums, as 2^18 fixed-point integers) + incompressibility_2.comp
//    (lambda, boundariness, self shift) + the boundariness filter of
//    incompressibility_3.comp:41-46,60.  Writes lambda, the self shift, the
//    per-particle Gauss constants and the density-error partials (64-bit
//    fixed-point integers, turned into the FP64 mean by the last block).
//  k_delta (particle j, over the particles whose rows contain j):
//    incompressibility_3.comp:62-66 as a gather: x_j += sum_i int(gradW_ij * lambda_i * 2^18)
//    plus the self shift, into the other position buffer.
//
// The per-pair integer terms are computed by the same code from the same inputs
// as the scatter form, and integer addition is associative, so the gather is
// bit-identical to the atomic scatter.  Gradients are recomputed in k_delta
// rather than stored (the reference writes 16 bytes per pair).
#include <algorithm>
#include <cstddef>
#include <type_traits>

#include "apbf_internal.cuh"

namespace apbf {
namespace {

// Contraction-proof dot product: k_density_lambda and k_delta must evaluate
// bit-identical gradients for the same pair.
__device__ __forceinline__ float dot3x(float3 a, float3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}

// The boundariness filter of incompressibility_3.comp:41-46,60 for the Gauss
// kernel, whose gradient points along -d: the pair (i, j) at offset d = x_j - x_i
// clears a non-zero boundariness of i when -normalize(gradW) . ed > 0.6 with
// ed = -normalize(gradient sum of i).  Explicit rounding: the density pass and the
// position pass (which takes the test over when rows are symmetric) must agree.
__device__ __forceinline__ bool filter_dir(int32_t gx, int32_t gy, int32_t gz, float3 &ed) {
    const float3 gi = make_float3((float)gx, (float)gy, (float)gz);
    const float gl = __fsqrt_rn(dot3x(gi, gi));
    if (!(gl > 0.0f)) return false;
    ed = make_float3(-__fdiv_rn(gi.x, gl), -__fdiv_rn(gi.y, gl), -__fdiv_rn(gi.z, gl));
    return true;
}
__device__ __forceinline__ bool gauss_filter_hit(float3 ed, float3 d) {
    const float r2 = dot3x(d, d);
    if (r2 < 1.0e-8f) return false;  // zero gradient: normalize() gives NaN, no filter
    return -dot3x(ed, d) > __fmul_rn(0.6f, __fsqrt_rn(r2));
}

struct PassA {
    const int4 *pos;
    const float *inv_mass;
    const float *radius;
    const float *kw;
    float *bness;
    const uint32_t *count;
    const uint32_t *idx;
    uint32_t stride;
    float *lambda;  // non-null (debug): the pass's lambda
    int4 *shift;
    float4 *rec;  // per particle: lambda, Gauss ivd, Gauss norm, kernel width (read by k_delta)
    int4 *pk;     // per particle: position xyz and the applied lambda (read by k_delta when widths are uniform)
    float2 *kc;   // per particle: Gauss constants of its width, ivd 2^-36 and norm (read by k_delta when widths differ)
    uint32_t *dbg_dens;
    int4 *dbg_grad;
    uint32_t *dbg_sq;
    long long *partials;  // per block: the two error sums in 2^-24 fixed point, kernel-width bits min << 32 | max
    const uint32_t *d_len;
    Status *st;
    double *red_out;     // [2], [3]: mean compression / absolute error of this pass
    float *features;     // non-null: the 8 features of this pass (first pass of a substep)
    float4 *selfdir;     // non-null with features: self-shift direction and inverse mass
    const float4 *vel;   // velocities, for the divergence feature
    const float *lam_prev;  // lambda_prev: the previous substep's sum at pass 0, this substep's after
    int projected;          // 1: pull-back allowed (passes after the first of a warm-started substep)
    int loop_offset;        // >= 0: solve loop pass number = st->pass_index + loop_offset
    uint32_t max_passes;    // loop passes from this number on are skipped
    int4 *filt;             // non-null: Gauss filter deferred to the position pass when rows are symmetric
    float target;        // > 0: set st->converged when the error is at most this
    int early_exit;      // skip the pass when st->converged is set
    float rmin3;  // pow(2 * smallestTargetRadius, 3)
    int hk, gk, method, update_b;
    float b_speed, b_sgl_factor, b_up_factor;
};

// Gauss constants in the units of the unscaled fixed-point offset D (2^18 per
// reference unit): the exponent scale ivd 2^-36 (r^2 = |D|^2 2^-36), the height
// norm, and the gradient factor 2 ln2 ivd 2^-18 (kernels.glsl:112-123 with r = D 2^-18).
struct GaussPair {
    float ivd36, norm, k2;
};
__device__ __forceinline__ GaussPair gauss_pair(float ivd36, float norm) {
    // k2 = round(ivd ln2) 2^-17: the factor 2 of the gradient and the 2^-18 of r = D 2^-18
    return {ivd36, norm, ivd36 * (0.693147180559945309f * 0x1p19f)};
}
__device__ __forceinline__ GaussPair gauss_pair(KConst c) { return gauss_pair(c.ivd * 0x1p-36f, c.norm); }
__device__ __forceinline__ float3 udiff(int4 from, int4 to) {
    return make_float3((float)wadd(to.x, -from.x), (float)wadd(to.y, -from.y), (float)wadd(to.z, -from.z));
}

// The Gauss height and gradient of the offset D = to - from in fixed-point units.
// Every product is the FP32 rounding of the reference-unit product (fdiff, r2,
// kernel_gradient's -2 ivd W r) scaled by a power of two, which is exact in the
// normal range: the terms equal the reference-unit evaluation bit for bit, except
// for gradients far below one fixed-point unit of any sum (subnormal intermediates).
__device__ __forceinline__ void gauss_terms_r2(float3 D, float r2, const GaussPair &k, float &W, float3 &g) {
    W = exp2f(r2 * k.ivd36) * k.norm;
    if (r2 < 1.0e-8f * 0x1p36f) {  // dist < 0.0001 reference units
        g = make_float3(0.f, 0.f, 0.f);
        return;
    }
    const float s = W * k.k2;
    g = make_float3(s * D.x, s * D.y, s * D.z);
}
__device__ __forceinline__ void gauss_terms(float3 D, const GaussPair &k, float &W, float3 &g) {
    gauss_terms_r2(D, dot3x(D, D), k, W, g);
}

// gauss_filter_hit for the offset x_j - x_i = -D, D in fixed-point units and
// r2 = |D|^2.  Every quantity is the reference-unit one times a power of two, and
// none is subnormal (|D| components are 0 or >= 1, those of ed 0 or >= 2^-32), so
// the decision is gauss_filter_hit's bit for bit.
__device__ __forceinline__ bool gauss_filter_hit_fixed(float3 ed, float3 D, float r2) {
    if (r2 < 1.0e-8f * 0x1p36f) return false;
    return dot3x(ed, D) > __fmul_rn(0.6f, __fsqrt_rn(r2));
}

template <bool GAUSS>
__device__ __forceinline__ void pair_terms(int hk, int gk, float3 d, float kw, KConst c, float &W, float3 &g) {
    float r2 = dot3x(d, d);
    if (GAUSS) {
        W = gauss_height(r2, c);
        g = kernel_gradient(1, d, r2, kw, c, W);
    } else {
        W = kernel_height(hk, r2, kw, c);
        float Wg = gk == 1 ? (hk == 1 ? W : gauss_height(r2, c)) : 0.0f;
        g = kernel_gradient(gk, d, r2, kw, c, Wg);
    }
}

// Fixed-order (deterministic) sum of per-block partial pairs with one block of
// blockDim.x (a power of two, at most 256) threads: thread t sums partials t,
// t + blockDim.x, ... in order, then a fixed tree.
__device__ __forceinline__ void block_sum2(const double *partials, int blocks, double &t1, double &t2) {
    __shared__ double s1[256], s2[256];
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < blocks; k += blockDim.x) {
        a += ((volatile const double *)partials)[2 * k];
        b += ((volatile const double *)partials)[2 * k + 1];
    }
    s1[threadIdx.x] = a;
    s2[threadIdx.x] = b;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if ((int)threadIdx.x < off) {
            s1[threadIdx.x] += s1[threadIdx.x + off];
            s2[threadIdx.x] += s2[threadIdx.x + off];
        }
        __syncthreads();
    }
    t1 = s1[0];
    t2 = s2[0];
}

// Mean density error terms: per particle in 2^-24 fixed point (the FP32 ratio
// times 2^24 is exact; ratios of 128 and more saturate), summed as 64-bit
// integers.  Integer sums are order-free, so the mean is deterministic without
// FP64 arithmetic per particle (GB300's FP64 pipe is a small fraction of its FP32
// rate).  NaN counts as saturated, so a NaN state never converges.
constexpr float kErrScale = 16777216.0f;
__device__ __forceinline__ long long err_fix(float x) {
    return x != x ? 0x7fffffffll : (long long)__float2int_rn(__fmul_rn(x, kErrScale));
}

// Sums of the per-block integer error partials and the min / max of the
// per-block kernel-width bits (partials of three words per block).
__device__ __forceinline__ void block_reduce_partials(const long long *partials, int blocks, long long &t1,
                                                      long long &t2, uint32_t &kmin, uint32_t &kmax) {
    __shared__ long long s1[32], s2[32];
    __shared__ uint32_t s3[32], s4[32];
    long long a = 0, b = 0;
    uint32_t lo = 0xffffffffu, hi = 0u;
    for (int k = threadIdx.x; k < blocks; k += blockDim.x) {
        a += ((volatile const long long *)partials)[3 * k];
        b += ((volatile const long long *)partials)[3 * k + 1];
        const unsigned long long w = (unsigned long long)((volatile const long long *)partials)[3 * k + 2];
        lo = min(lo, (uint32_t)(w >> 32));
        hi = max(hi, (uint32_t)w);
    }
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if ((threadIdx.x & 31) == 0) {
        s1[threadIdx.x >> 5] = a;
        s2[threadIdx.x >> 5] = b;
        s3[threadIdx.x >> 5] = lo;
        s4[threadIdx.x >> 5] = hi;
    }
    __syncthreads();
    t1 = 0;
    t2 = 0;
    kmin = 0xffffffffu;
    kmax = 0u;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
        t1 += s1[k];
        t2 += s2[k];
        kmin = min(kmin, s3[k]);
        kmax = max(kmax, s4[k]);
    }
}

constexpr int kUnroll = 4;

// L threads per particle ("lanes"): lane s of a particle's group takes row
// entries s, s + L, ...; the group's integer sums are then combined by shuffles.
// Wrapping integer sums are order-free, so every L gives the same density,
// gradient and squared-gradient sums bit for bit.
template <int L, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}
template <int L>
__device__ __forceinline__ int32_t group_wsum(int32_t v) {
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1) v = wadd(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}

// XTRA: the warm-start features or the centre-of-mass boundariness sums
// (method 1) are gathered too; the common pass is compiled without them.
// Per-thread partial results of a density pass: the two error sums (2^-24 fixed
// point) and the range of the kernel-width bits.
struct PassSums {
    long long e1 = 0, e2 = 0;
    uint32_t kwlo = 0xffffffffu, kwhi = 0u;
};

// One particle (row i_raw, lane sub of its group of L) of a density pass:
// incompressibility_0..2 and the boundariness filter of incompressibility_3.
// Every lane of the group must call it (group shuffles).
template <bool GAUSS, int L, bool XTRA>
__device__ __forceinline__ void density_one(const PassA &a, const int4 *__restrict__ pos, uint32_t i_raw, uint32_t n,
                                            uint32_t sub, bool defer, bool write_rec, PassSums &ps) {
    {
        const bool valid = i_raw < n;
        const uint32_t i = valid ? i_raw : 0u;
        const int4 p = pos[i];
        const float kw = a.kw[i];
        const KConst c = gauss_consts(kw);
        const GaussPair gp = gauss_pair(c);
        uint32_t dens = 0u;
        int32_t gx = 0, gy = 0, gz = 0;
        uint32_t sq = 0;
        int32_t cx = 0, cy = 0, cz = 0, cw = 0;
        const uint32_t cnt = valid ? a.count[i] : 0u;
        // loaded with the particle's other data, so that they are not one more round
        // trip after the neighbour loop
        const float im = a.inv_mass[i], radius = a.radius[i];
        float b = a.bness[i];
        const uint32_t *row = a.idx + i;
        const bool feat = XTRA && a.features != nullptr;
        const float4 vi = feat ? a.vel[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        float div = 0.0f;  // sum_j m_j (v_j - v_i) . gradW_ij  (velocity divergence x density)
        float nprev = 0.0f;  // sum_j lambda_prev_j (the neighbours' previous-substep lambda sums)
        // Batches of kUnroll pairs per lane, software-pipelined: the neighbour gathers
        // of a batch go out with the row entries of the next, then the arithmetic, so
        // a batch costs one memory latency instead of two.
        uint32_t jj[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const uint32_t k = sub + u * L;
            jj[u] = k < cnt ? row[(size_t)k * a.stride] : i;
        }
        for (uint32_t k0 = sub; k0 < cnt; k0 += L * kUnroll) {
            int4 qq[kUnroll];
            uint32_t jn[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) qq[u] = pos[jj[u]];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const uint32_t k = k0 + (L * kUnroll) + u * L;
                jn[u] = k < cnt ? row[(size_t)k * a.stride] : i;
            }
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                if (k0 + u * L >= cnt) break;
                const int4 q = qq[u];
                // the neighbour's mass rides in position.w (x / invMassN = x * mass)
                const float mjf = __int_as_float(q.w) * APBF_FIX;  // neighbour mass x 2^18
                float W;
                float3 g;
                if (GAUSS)
                    gauss_terms(udiff(p, q), gp, W, g);
                else
                    pair_terms<false>(a.hk, a.gk, fdiff(p, q), kw, c, W, g);
                dens += f2u(W * mjf);
                gx = wadd(gx, f2i(g.x * mjf));
                gy = wadd(gy, f2i(g.y * mjf));
                gz = wadd(gz, f2i(g.z * mjf));
                sq += f2u(dot3x(g, g) * mjf);
                if (feat) {
                    const float4 vj = a.vel[jj[u]];
                    div += __int_as_float(q.w) * ((vj.x - vi.x) * g.x + (vj.y - vi.y) * g.y + (vj.z - vi.z) * g.z);
                    nprev += a.lam_prev[jj[u]];
                }
                if (XTRA && a.method == 1) {  // incompressibility_1.comp:62-68
                    const float den = kw * APBF_FIX / mjf;
                    cx = wadd(cx, f2i((float)wadd(q.x, -p.x) / den));
                    cy = wadd(cy, f2i((float)wadd(q.y, -p.y) / den));
                    cz = wadd(cz, f2i((float)wadd(q.z, -p.z) / den));
                    cw = wadd(cw, f2i(mjf));
                }
            }
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) jj[u] = jn[u];
        }
        if (L > 1) {
            dens = group_sum<L>(dens);
            sq = group_sum<L>(sq);
            gx = group_wsum<L>(gx);
            gy = group_wsum<L>(gy);
            gz = group_wsum<L>(gz);
            if (feat) {
                div = group_sum<L>(div);
                nprev = group_sum<L>(nprev);
            }
            if (XTRA && a.method == 1) {
                cx = group_wsum<L>(cx);
                cy = group_wsum<L>(cy);
                cz = group_wsum<L>(cz);
                cw = group_wsum<L>(cw);
            }
        }
        if (!valid || sub != 0) return;
        const float W0 = GAUSS ? c.norm : kernel_height(a.hk, 0.0f, kw, c);
        dens += f2u(W0 / im * APBF_FIX);  // incompressibility_0.comp:32-45 (the self term)
        // incompressibility_2.comp:77-109
        const float r2x = 2.0f * radius;
        const float ird = (r2x * r2x * r2x) * im;
        const float density = (float)dens * APBF_INV_FIX;
        const float3 wgs = make_float3((float)gx * APBF_INV_FIX, (float)gy * APBF_INV_FIX, (float)gz * APBF_INV_FIX);
        float sqs = (float)sq * APBF_INV_FIX;
        const float wgsq = dot3x(wgs, wgs);
        const float sgl = sqrtf(wgsq) * ird;
        sqs += wgsq * im;
        const float under = 1.0f - density * ird;
        if (a.update_b) {
            float bn;
            if (XTRA && a.method == 1) {
                float tm = (float)cw * APBF_INV_FIX + 1.0f / im;
                float3 cv = make_float3((float)cx, (float)cy, (float)cz);
                bn = sqrtf(dot3x(cv, cv)) / (APBF_FIX * tm) * a.b_sgl_factor;
            } else {
                bn = sgl * kw * a.b_sgl_factor + fmaxf(0.0f, under) * a.b_up_factor;
            }
            bn = bn >= 1.0f ? 1.0f : 0.0f;
            float step = bn - b;
            b = b + fminf(a.b_speed, fmaxf(-a.b_speed, step));
            b = fminf(1.0f, b);
        }
        float lam = under / (ird * ird * (sqs + 0.01f));
        lam /= a.rmin3 / ird * im;
        if (a.lambda) a.lambda[i] = lam;
        // The lambda this pass applies: the reference applies only pushes (lambda < 0,
        // incompressibility_2.comp:106, incompressibility_3.comp:63).  Projected mode
        // (warm-started solve) also applies a pull-back lambda > 0 where earlier passes
        // of this substep pushed, up to their sum, so that an over-push is undone; the
        // density that pull-back would restore counts as error.
        float applied = lam < 0.0f ? lam : 0.0f;
        float pull = 0.0f;
        if (a.projected && lam > 0.0f) {
            applied = fminf(lam, -a.lam_prev[i]);  // lam_prev: the sum applied so far (<= 0)
            if (applied > 0.0f) pull = under * (applied / lam);
            else applied = 0.0f;
        }
        if (write_rec) a.rec[i] = make_float4(applied, c.ivd, c.norm, kw);
        else if (GAUSS) a.kc[i] = make_float2(gp.ivd36, gp.norm);
        a.pk[i] = make_int4(p.x, p.y, p.z, __float_as_int(applied));
        ps.kwlo = min(ps.kwlo, __float_as_uint(kw));
        ps.kwhi = max(ps.kwhi, __float_as_uint(kw));
        if (feat) {
            float *fo = a.features + (size_t)i * 8;
            fo[0] = (float)cnt;
            fo[1] = density * ird - 1.0f;
            fo[2] = kw / radius;
            fo[3] = lam;
            fo[4] = density > 0.0f ? div / density : 0.0f;
            fo[5] = a.lam_prev[i];
            fo[6] = cnt ? nprev / (float)cnt : 0.0f;
            fo[7] = 0.0f;
            a.selfdir[i] = make_float4(-wgs.x * ird, -wgs.y * ird, -wgs.z * ird, im);
        }
        int4 sh = make_int4(0, 0, 0, 0);
        if (applied != 0.0f) {
            const float sc = applied * im * APBF_FIX;
            sh.x = f2i(-wgs.x * ird * sc);
            sh.y = f2i(-wgs.y * ird * sc);
            sh.z = f2i(-wgs.z * ird * sc);
        } else if (!(lam >= 0.0f)) {
            set_flag(a.st, APBF_FLAG_NONFINITE);  // NaN lambda: no shift (int(NaN) = 0)
        }
        // incompressibility_3.comp:41-46,60: filter (only changes a non-zero boundariness);
        // deferred, it is recorded for particles with boundariness, flagged in shift.w
        if (defer) {
            if (b > 0.0f) {
                a.filt[i] = make_int4(gx, gy, gz, 1);
                sh.w = 1;
            }
        } else if (a.method == 2 && b > 0.0f) {
            float3 ed;
            if (GAUSS && filter_dir(gx, gy, gz, ed)) {
                // batches of kUnroll neighbours in row order, software-pipelined as the
                // sums above (the first hit ends the test, as in the plain loop)
                uint32_t fj[kUnroll];
#pragma unroll
                for (int u = 0; u < kUnroll; ++u) fj[u] = (uint32_t)u < cnt ? row[(size_t)u * a.stride] : i;
                bool hit = false;
                for (uint32_t k0 = 0; k0 < cnt && !hit; k0 += kUnroll) {
                    int4 fq[kUnroll];
                    uint32_t fn[kUnroll];
#pragma unroll
                    for (int u = 0; u < kUnroll; ++u) fq[u] = pos[fj[u]];
#pragma unroll
                    for (int u = 0; u < kUnroll; ++u) {
                        const uint32_t k = k0 + kUnroll + u;
                        fn[u] = k < cnt ? row[(size_t)k * a.stride] : i;
                    }
#pragma unroll
                    for (int u = 0; u < kUnroll; ++u) {
                        if (hit || k0 + u >= cnt) break;
                        hit = gauss_filter_hit(ed, fdiff(p, fq[u]));
                    }
#pragma unroll
                    for (int u = 0; u < kUnroll; ++u) fj[u] = fn[u];
                }
                if (hit) b = 0.0f;
            } else if (!GAUSS && filter_dir(gx, gy, gz, ed)) {
                for (uint32_t k = 0; k < cnt; ++k) {
                    const uint32_t j = a.idx[(size_t)k * a.stride + i];
                    const float3 d = fdiff(p, pos[j]);
                    {
                        float W;
                        float3 g;
                        pair_terms<GAUSS>(a.hk, a.gk, d, kw, c, W, g);
                        float l = sqrtf(dot3x(g, g));
                        if (!(l > 0.0f)) continue;
                        float dd = ed.x * (g.x / l) + ed.y * (g.y / l) + ed.z * (g.z / l);
                        if (dd > 0.6f) {
                            b = 0.0f;
                            break;
                        }
                    }
                }
            }
        }
        a.shift[i] = sh;
        a.bness[i] = b;
        const float ratio = __fmaf_rn(density, ird, -1.0f);  // one rounding of the exact product - 1
        ps.e1 += err_fix(ratio > 0.0f ? ratio : pull);
        ps.e2 += err_fix(fabsf(ratio));
        if (a.dbg_dens) {
            a.dbg_dens[i] = dens;
            a.dbg_grad[i] = make_int4(gx, gy, gz, 0);
            a.dbg_sq[i] = sq;
        }
    }
}

// Block sums of the per-thread PassSums, valid in thread 0.
__device__ __forceinline__ PassSums block_pass_sums(PassSums ps) {
    __shared__ long long s1[8], s2[8];
    __shared__ uint32_t s3[8], s4[8];
    for (int off = 16; off > 0; off >>= 1) {
        ps.e1 += __shfl_down_sync(0xffffffffu, ps.e1, off);
        ps.e2 += __shfl_down_sync(0xffffffffu, ps.e2, off);
    }
    ps.kwlo = __reduce_min_sync(0xffffffffu, ps.kwlo);
    ps.kwhi = __reduce_max_sync(0xffffffffu, ps.kwhi);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s1[w] = ps.e1;
        s2[w] = ps.e2;
        s3[w] = ps.kwlo;
        s4[w] = ps.kwhi;
    }
    __syncthreads();
    PassSums t;
    if (threadIdx.x == 0) {
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            t.e1 += s1[k];
            t.e2 += s2[k];
            t.kwlo = min(t.kwlo, s3[k]);
            t.kwhi = max(t.kwhi, s4[k]);
        }
    }
    __syncthreads();  // the shared arrays may be reused by the next call
    return t;
}

// The end of a density pass, once all its sums are in (one thread): mean errors,
// width uniformity, pass counter and the convergence flag for the passes that follow.
__device__ __forceinline__ void finish_pass(const PassA &a, uint32_t n, long long t1, long long t2) {
    const double inv = 1.0 / (double)kErrScale;
    const double m1 = n ? (double)t1 * inv / n : 0.0, m2 = n ? (double)t2 * inv / n : 0.0;
    a.red_out[2] = m1;
    a.red_out[3] = m2;
    a.st->density_passes += 1u;
    if (a.target > 0.0f && m1 <= (double)a.target) {
        a.st->converged = 1u;  // the remaining passes of the substep are skipped
        a.st->converged_substeps += 1u;
    }
}

template <bool GAUSS, int L, bool XTRA>
__global__ void __launch_bounds__(256, GAUSS ? 4 : 3) k_density_lambda(PassA a) {
    const bool skip = (a.early_exit && *(volatile uint32_t *)&a.st->converged) ||
                      (a.loop_offset >= 0 && a.st->pass_index + (uint32_t)a.loop_offset >= a.max_passes);
    // With symmetric rows or union rows the Gauss filter runs in this pass's position
    // update, which gathers over the same neighbours anyway; filter_tag tells it whether to.
    const bool defer = GAUSS && a.filt && a.method == 2 &&
                       (a.st->range_min == a.st->range_max || a.st->union_rows != 0u);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st->filter_tag = (!skip && defer) ? 1u : 0u;
    if (skip) return;  // uniform over the grid
    const uint32_t n = a.d_len[kLenParticles];
    const uint32_t sub = threadIdx.x % L;
    // passes after the first: the widths' uniformity of the first pass still holds
    // the position update of the Gauss kernel gathers the packed records and widths;
    // the other kernels gather the solve records, written every pass
    const bool write_rec = !GAUSS;
    PassSums ps;
    // the block iterates as a whole (uniform trip count: the group shuffles need every lane)
    const uint32_t gpb = blockDim.x / L;
    for (uint32_t base = blockIdx.x * gpb; base < n; base += gridDim.x * gpb)
        density_one<GAUSS, L, XTRA>(a, a.pos, base + threadIdx.x / L, n, sub, defer, write_rec, ps);
    const PassSums bs = block_pass_sums(ps);
    __shared__ bool s_last;
    if (threadIdx.x == 0) {
        const long long t1 = bs.e1, t2 = bs.e2;
        const uint32_t lo = bs.kwlo, hi = bs.kwhi;
        a.partials[3 * blockIdx.x] = t1;
        a.partials[3 * blockIdx.x + 1] = t2;
        a.partials[3 * blockIdx.x + 2] = (long long)(((unsigned long long)lo << 32) | hi);
        __threadfence();
        s_last = atomicAdd(&a.st->done_blocks, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    // the last block: sum of all partials, error and convergence flag for the
    // passes that follow
    __threadfence();
    long long t1, t2;
    uint32_t kmin, kmax;
    block_reduce_partials(a.partials, gridDim.x, t1, t2, kmin, kmax);
    if (threadIdx.x == 0) {
        a.st->done_blocks = 0u;
        a.st->kw_uniform = kmin == kmax ? 1u : 0u;  // the position update may gather the packed records
        finish_pass(a, n, t1, t2);
    }
}

struct PassB {
    const int4 *pos;
    int4 *pos_out;
    const float4 *rec;
    const int4 *pk;   // the density pass's packed records (position, applied lambda)
    const float2 *kc;  // the density pass's Gauss constants per particle
    const float *kw;
    const int4 *shift;
    const float *radius;
    const float4 *bmin, *bmax, *rot;
    uint32_t nboxes;  // > 0: box collision of the next iteration applied to the output
    const uint32_t *count;
    const uint32_t *idx;
    const uint32_t *rcount;
    const uint32_t *ridx;
    uint32_t stride;
    const uint32_t *d_len;
    const Status *st;
    int gk;
    int early_exit;  // converged: copy the positions unchanged (the buffers swap regardless)
    float *lam_prev;  // prev_mode / acc_mode (0 off, 1 reset, 2 add): accumulate the lambda
    float *lam_acc;   // this pass applied (rec.x: the learned one in a learned pass)
    int prev_mode, acc_mode;
    int loop_offset;      // >= 0: solve loop pass number = st->pass_index + loop_offset
    uint32_t max_passes;  // loop passes from this number on copy through; box after all but the last
    const int4 *filt;     // the density pass's deferred Gauss filter (gradient sum, boundariness > 0)
    float *bness;
};

__device__ __forceinline__ void accumulate(float *dst, int mode, uint32_t j, float v) {
    if (mode == 1) dst[j] = v;
    else if (mode == 2) dst[j] += v;
}

// One neighbour's term of a position update: int(gradW_ij * lambda_i * 2^18) per
// axis (incompressibility_3.comp:62-66) for the neighbour's record q (position,
// and for the Gauss kernel the applied lambda in w), its Gauss constants kci (as
// the density pass computed them from its width) or solve record rr.  PACKED (every
// width equal): j's own constants cj.  The main row and the correction rows use this
// one function, so a term subtracted again cancels exactly.
// The Gauss term of the offset D = x_j - x_i (fixed-point units) with r2 = |D|^2.
__device__ __forceinline__ int3 gauss_delta(float3 D, float r2, float lam, const GaussPair &k) {
    float W;
    float3 g;
    gauss_terms_r2(D, r2, k, W, g);
    const float sc = lam * APBF_FIX;
    return make_int3(f2i(g.x * sc), f2i(g.y * sc), f2i(g.z * sc));
}

template <bool GAUSS, bool PACKED>
__device__ __forceinline__ int3 pair_delta(const PassB &a, int4 q, float lam, float2 kci, float4 rr, int4 p,
                                           const GaussPair &gpj) {
    if (GAUSS) {
        const float3 D = udiff(q, p);
        return gauss_delta(D, dot3x(D, D), lam, PACKED ? gpj : gauss_pair(kci.x, kci.y));
    }
    float3 g;
    {
        KConst c;
        c.ivd = rr.y;
        c.norm = rr.z;
        const float3 d = fdiff(q, p);
        const float r2 = dot3x(d, d);
        g = kernel_gradient(a.gk, d, r2, rr.w, c, a.gk == 1 ? gauss_height(r2, c) : 0.0f);
    }
    const float sc = lam * APBF_FIX;
    return make_int3(f2i(g.x * sc), f2i(g.y * sc), f2i(g.z * sc));
}

// Sum over particle j's row of the neighbours' terms (incompressibility_3.comp:62-66
// as a gather) and the deferred boundariness filter over the row's first fcnt
// entries.  PACKED: the neighbours' packed records (position, applied lambda) with
// j's own Gauss constants cj (every width equal); GAUSS otherwise: the packed
// records and the neighbours' Gauss constants; other kernels: the solve records
// and the positions.
template <bool GAUSS, int L, bool PACKED>
__device__ __forceinline__ int3 delta_row(const PassB &a, const int4 *__restrict__ pos, const uint32_t *row, uint32_t cnt,
                                          uint32_t fcnt, uint32_t j, uint32_t sub, int4 p, const GaussPair &cj,
                                          bool fil, float3 ed, bool &hit, int4 start) {
    int32_t ax = start.x, ay = start.y, az = start.z;
    // software-pipelined as in density_one: the gathers of a batch go out with the
    // row entries of the next
    // Entries are masked to their index bits: rows the search tuner leaves behind may be
    // correction rows read as transposed ones (flag bit 31), and no entry may address
    // beyond the lists (the index bits of every valid entry are the entry itself).
    uint32_t ii[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
        const uint32_t k = sub + u * L;
        ii[u] = k < cnt ? row[(size_t)k * a.stride] & ~kNoDelta : j;
    }
    for (uint32_t k0 = sub; k0 < cnt; k0 += L * kUnroll) {
        float4 rr[kUnroll];
        int4 qq[kUnroll];
        float2 kk[kUnroll];
        uint32_t in_[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            if (PACKED) {
                qq[u] = a.pk[ii[u]];
            } else if (GAUSS) {
                qq[u] = a.pk[ii[u]];
                kk[u] = a.kc[ii[u]];
            } else {
                rr[u] = a.rec[ii[u]];
                qq[u] = pos[ii[u]];
            }
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const uint32_t k = k0 + (L * kUnroll) + u * L;
            in_[u] = k < cnt ? row[(size_t)k * a.stride] & ~kNoDelta : j;
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const float lam = k0 + u * L < cnt ? (PACKED || GAUSS ? __int_as_float(qq[u].w) : rr[u].x) : 0.0f;
            int3 t;
            if (GAUSS) {
                // the deferred filter (Gauss only) shares the offset and its square with the term
                const bool ftest = fil && !hit && k0 + u * L < fcnt;
                if (lam == 0.0f && !ftest) continue;
                const float3 D = udiff(qq[u], p);
                const float r2 = dot3x(D, D);
                if (ftest) hit = gauss_filter_hit_fixed(ed, D, r2);
                if (lam == 0.0f) continue;  // the applied lambda (incompressibility_3.comp:63); padding lanes
                t = gauss_delta(D, r2, lam, PACKED ? cj : gauss_pair(kk[u].x, kk[u].y));
            } else {
                if (lam == 0.0f) continue;
                t = pair_delta<false, false>(a, qq[u], lam, kk[u], rr[u], p, cj);
            }
            ax = wadd(ax, t.x);
            ay = wadd(ay, t.y);
            az = wadd(az, t.z);
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) ii[u] = in_[u];
    }
    return make_int3(ax, ay, az);
}

// Particle j's correction row (radii that differ, neighborhood.cu): terms of
// entries flagged kNoDelta subtracted (j holds them, their radius does not reach
// j), the others added (they hold j, j's radius does not reach them).  Lane sub of
// the group of L takes entries sub, sub + L, ...
template <bool GAUSS, int L, bool PACKED>
__device__ __forceinline__ int3 delta_corrections(const PassB &a, const int4 *__restrict__ pos, uint32_t m, uint32_t j,
                                                  uint32_t sub, int4 p, const GaussPair &cj, int3 acc) {
    for (uint32_t k = sub; k < m; k += L) {
        const uint32_t e = a.ridx[(size_t)k * a.stride + j];
        const uint32_t i = e & ~kNoDelta;
        float4 rr = make_float4(0.f, 0.f, 0.f, 0.f);
        int4 q;
        float2 kci = make_float2(0.f, 0.f);
        if (PACKED || GAUSS) {
            q = a.pk[i];
            if (!PACKED) kci = a.kc[i];
        } else {
            rr = a.rec[i];
            q = pos[i];
        }
        const float lam = PACKED || GAUSS ? __int_as_float(q.w) : rr.x;
        if (lam == 0.0f) continue;
        const int3 t = pair_delta<GAUSS, PACKED>(a, q, lam, kci, rr, p, cj);
        if (e & kNoDelta) {
            acc.x = wadd(acc.x, -t.x);
            acc.y = wadd(acc.y, -t.y);
            acc.z = wadd(acc.z, -t.z);
        } else {
            acc.x = wadd(acc.x, t.x);
            acc.y = wadd(acc.y, t.y);
            acc.z = wadd(acc.z, t.z);
        }
    }
    return acc;
}

// One particle (row j_raw, lane sub of its group of L) of a position update:
// incompressibility_3 as a gather, the deferred filter, the next iteration's box
// collision (nboxes > 0) and the lambda bookkeeping.  Every lane of the group
// must call it (group shuffles).
template <bool GAUSS, int L>
__device__ __forceinline__ void delta_one(const PassB &a, const int4 *__restrict__ pos, int4 *pos_out, uint32_t j_raw,
                                          uint32_t n, uint32_t sub, bool packed, bool filter, const uint32_t *cnt_arr,
                                          const uint32_t *idx_arr, bool corr, uint32_t nboxes) {
    {
        const bool valid = j_raw < n;
        const uint32_t j = valid ? j_raw : 0u;
        const int4 p = pos[j];
        // j's Gauss constants as the density pass stored them
        const float2 kcj = GAUSS ? a.kc[j] : make_float2(0.f, 0.f);
        const GaussPair cj = gauss_pair(kcj.x, kcj.y);
        int32_t ax, ay, az;
        const uint32_t cnt = valid ? cnt_arr[j] : 0u;
        const uint32_t *row = idx_arr + j;
        // the self shift (incompressibility_2.comp:106-109); w flags a deferred filter
        const int4 shj = valid ? a.shift[j] : make_int4(0, 0, 0, 0);
        float3 ed = make_float3(0.f, 0.f, 0.f);
        bool fil = false, hit = false;  // this particle's deferred filter, and whether a neighbour cleared it
        uint32_t fcnt = 0;              // the filter's entries: j's own neighbours, the row's prefix
        if (filter && shj.w != 0) {
            const int4 fj = a.filt[j];
            fil = filter_dir(fj.x, fj.y, fj.z, ed);
            fcnt = a.count[j];
        }
        // the sums start from the self shift on the first lane: wrapping integer sums
        // are order-free, and the load is in flight with the particle's other data
        const int4 sh = sub == 0 ? shj : make_int4(0, 0, 0, 0);
        const float rj = a.radius[j];
        int3 acc = packed ? delta_row<GAUSS, L, true>(a, pos, row, cnt, fcnt, j, sub, p, cj, fil, ed, hit, sh)
                          : delta_row<GAUSS, L, false>(a, pos, row, cnt, fcnt, j, sub, p, cj, fil, ed, hit, sh);
        if (corr) {  // the correction row (radii that differ): usually empty
            const uint32_t m = valid ? a.rcount[j] : 0u;
            if (m) acc = packed ? delta_corrections<GAUSS, L, true>(a, pos, m, j, sub, p, cj, acc)
                                : delta_corrections<GAUSS, L, false>(a, pos, m, j, sub, p, cj, acc);
        }
        ax = acc.x;
        ay = acc.y;
        az = acc.z;
        if (L > 1) {
            ax = group_wsum<L>(ax);
            ay = group_wsum<L>(ay);
            az = group_wsum<L>(az);
            if (filter) {
                int h = hit ? 1 : 0;
#pragma unroll
                for (int off = L / 2; off > 0; off >>= 1) h |= __shfl_xor_sync(0xffffffffu, h, off);
                hit = h != 0;
            }
        }
        if (!valid || sub != 0) return;
        if (hit) a.bness[j] = 0.0f;
        int4 out = make_int4(wadd(p.x, ax), wadd(p.y, ay), wadd(p.z, az), p.w);
        if (nboxes) out = box_push(out, rj, j, a.bmin, a.bmax, a.rot, nboxes);
        pos_out[j] = out;
        if (a.prev_mode | a.acc_mode) {
            const float lj = __int_as_float(a.pk[j].w);  // applied (learned) lambda
            accumulate(a.lam_prev, a.prev_mode, j, lj);
            accumulate(a.lam_acc, a.acc_mode, j, lj);
        }
    }
}

// A converged pass (no position update) of particle j: the deferred filter still
// belongs to it, the positions are copied through and nothing is applied.
__device__ __forceinline__ void delta_skip_filter(const PassB &a, const int4 *__restrict__ pos, uint32_t j) {
    if (!a.shift[j].w) return;
    const int4 fj = a.filt[j];
    float3 ed;
    if (!filter_dir(fj.x, fj.y, fj.z, ed)) return;
    const int4 p = pos[j];
    for (uint32_t k = 0; k < a.count[j]; ++k)
        if (gauss_filter_hit(ed, fdiff(p, pos[a.idx[(size_t)k * a.stride + j]]))) {
            a.bness[j] = 0.0f;
            break;
        }
}
__device__ __forceinline__ void delta_skip_copy(const PassB &a, uint32_t j) {
    a.pos_out[j] = a.pos[j];
    accumulate(a.lam_prev, a.prev_mode, j, 0.0f);  // nothing applied in this pass
    accumulate(a.lam_acc, a.acc_mode, j, 0.0f);
}

template <bool GAUSS, int L>
__global__ void __launch_bounds__(256, 4) k_delta(PassB a) {
    const uint32_t n = a.d_len[kLenParticles];
    bool skip = a.early_exit && *(volatile const uint32_t *)&a.st->converged;
    uint32_t nboxes = a.nboxes;
    if (a.loop_offset >= 0) {
        const uint32_t pass = a.st->pass_index + (uint32_t)a.loop_offset;
        skip = skip || pass >= a.max_passes;
        if (pass + 1u >= a.max_passes) nboxes = 0u;  // no box collision after the last iteration
    }
    // the density pass of this pass deferred the Gauss filter to here (symmetric rows)
    const bool filter = GAUSS && *(volatile const uint32_t *)&a.st->filter_tag != 0u;
    if (skip) {
        if (filter)  // converged: no position update, but the filter still belongs to this pass
            for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
                delta_skip_filter(a, a.pos, j);
        for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
            delta_skip_copy(a, j);
        return;
    }
    // Rows: symmetric (equal radii) or with correction rows (the green search with
    // radii that differ): the particle's own row; transposed rows otherwise.
    const bool sym = a.st->range_min == a.st->range_max;
    const bool corr = !sym && a.st->union_rows != 0u;
    // Equal kernel widths (same bits): every neighbour's Gauss constants are this
    // particle's, so one 16-byte record (position, applied lambda) per neighbour is
    // gathered instead of the solve record and the position.
    const bool packed = GAUSS && a.st->kw_uniform != 0u;
    const uint32_t *cnt_arr = sym || corr ? a.count : a.rcount;
    const uint32_t *idx_arr = sym || corr ? a.idx : a.ridx;
    const uint32_t sub = threadIdx.x % L;
    const uint32_t gpb = blockDim.x / L;
    for (uint32_t base = blockIdx.x * gpb; base < n; base += gridDim.x * gpb)
        delta_one<GAUSS, L>(a, a.pos, a.pos_out, base + threadIdx.x / L, n, sub, packed, filter, cnt_arr, idx_arr,
                            corr, nboxes);
}

// ---- the solve loop as one persistent cooperative kernel ----

struct LoopArgs {
    int4 *pos_a;          // positions before the first loop pass; the final positions end here
    int4 *pos_b;          // the other position buffer
    uint32_t first;       // number of the first loop pass
    uint32_t max_passes;  // passes from this number on do not run
    uint32_t nboxes;      // boxes of the next iteration's collision (none after the last pass)
    int defer;            // the density pass may leave the Gauss filter to the position phase (rows symmetric)
};

constexpr uint32_t kBarrierSpins = 1u << 22;  // x __nanosleep(64): a few hundred ms at most

// Grid barrier of a cooperative launch (every block resident).  The last block to
// arrive finishes the density pass when fin is set (one thread, all partial sums
// in) and releases the others; a wait that exceeds kBarrierSpins sets
// APBF_FLAG_SPIN_LIMIT and returns false, after which the block leaves the kernel
// (the blocks still waiting give up in turn, so every wait ends).
__device__ __forceinline__ bool grid_barrier(Status *st, uint32_t &gen, const PassA *fin, uint32_t n) {
    __syncthreads();
    __shared__ uint32_t s_ok;
    if (threadIdx.x == 0) {
        uint32_t ok = 1u;
        __threadfence();
        const uint32_t arrived = atomicAdd(&st->bar_arrive, 1u) + 1u;
        if (arrived == gridDim.x) {
            if (fin) {
                const unsigned long long t1 = *(volatile unsigned long long *)&st->loop_e1;
                const unsigned long long t2 = *(volatile unsigned long long *)&st->loop_e2;
                st->loop_e1 = 0ull;
                st->loop_e2 = 0ull;
                finish_pass(*fin, n, (long long)t1, (long long)t2);
            }
            st->bar_arrive = 0u;
            __threadfence();
            atomicAdd(&st->bar_gen, 1u);  // release
        } else {
            uint32_t spins = 0;
            bool inject;
            const uint32_t limit = wait_limit(st, kBarrierSpins, inject);
            while (inject || *(volatile uint32_t *)&st->bar_gen == gen) {
                if (++spins > limit) {
                    set_flag(st, APBF_FLAG_SPIN_LIMIT);
                    st->spin_where = 3u;
                    ok = 0u;
                    break;
                }
                __nanosleep(64);
            }
            __threadfence();
        }
        s_ok = ok;
    }
    __syncthreads();
    ++gen;
    return s_ok != 0u;
}

// Jacobi passes first .. max_passes-1 of a substep (or until a density pass meets
// the error target) in one launch: per pass, the density phase (density_one for
// every particle, error sums by integer atomics), a grid barrier whose last block
// finishes the pass, the position phase (delta_one) and a second barrier.  The
// per-particle arithmetic is the two-kernel form's own, so the results are
// identical; what goes away is two launches per pass and their ramp-up and drain.
// The widths' uniformity is the one pass 0 found (widths do not change within a
// substep).
template <bool GAUSS>
__global__ void __launch_bounds__(256, 4) k_solve_loop(PassA a, PassB b, LoopArgs l) {
    Status *st = a.st;
    if (a.early_exit && *(volatile uint32_t *)&st->converged) return;  // pass 0 met the target: no loop pass
    uint32_t gen = *(volatile uint32_t *)&st->bar_gen;  // read before this block's first arrival
    const uint32_t n = a.d_len[kLenParticles];
    const bool sym = st->range_min == st->range_max;
    const bool corr = !sym && st->union_rows != 0u;
    // with symmetric rows or correction rows the Gauss filter runs in the position phase
    // (as k_density_lambda decides)
    const bool defer = l.defer != 0 && (sym || corr);
    const bool packed = GAUSS && st->kw_uniform != 0u;
    const uint32_t *cnt_arr = sym || corr ? b.count : b.rcount;
    const uint32_t *idx_arr = sym || corr ? b.idx : b.ridx;
    const uint32_t T = gridDim.x * blockDim.x, t0 = blockIdx.x * blockDim.x + threadIdx.x;
    int4 *cur = l.pos_a, *nxt = l.pos_b;
    for (uint32_t pass = l.first; pass < l.max_passes; ++pass) {
        PassSums ps;
        for (uint32_t i = t0; i < n; i += T) density_one<GAUSS, 1, false>(a, cur, i, n, 0u, defer, !GAUSS, ps);
        const PassSums bs = block_pass_sums(ps);
        if (threadIdx.x == 0) {
            atomicAdd(&st->loop_e1, (unsigned long long)bs.e1);
            atomicAdd(&st->loop_e2, (unsigned long long)bs.e2);
        }
        if (!grid_barrier(st, gen, &a, n)) return;
        if (*(volatile uint32_t *)&st->converged != 0u) {
            // converged: no position update (the positions stay in cur), the deferred
            // filter still belongs to this pass
            for (uint32_t j = t0; j < n; j += T) {
                if (defer) delta_skip_filter(b, cur, j);
                accumulate(b.lam_prev, b.prev_mode, j, 0.0f);
            }
            break;
        }
        const uint32_t nb = pass + 1u < l.max_passes ? l.nboxes : 0u;
        for (uint32_t j = t0; j < n; j += T)
            delta_one<GAUSS, 1>(b, cur, nxt, j, n, 0u, packed, defer, cnt_arr, idx_arr, corr, nb);
        if (!grid_barrier(st, gen, nullptr, n)) return;
        int4 *t = cur;
        cur = nxt;
        nxt = t;
    }
    if (cur != l.pos_a)  // an odd number of updates: bring the positions back to the caller's buffer
        for (uint32_t j = t0; j < n; j += T) l.pos_a[j] = cur[j];
}

// ---- the solve loops of a batch of scenes as one persistent cooperative kernel ----

// One scene of a batched solve: its pass arguments, its two position buffers and
// its loop limits (LoopArgs per scene).
struct BatchScene {
    PassA a;
    PassB b;
    LoopArgs l;
};

struct BatchSync {
    uint32_t bar_arrive;  // blocks arrived at the current grid barrier
    uint32_t bar_gen;     // grid barriers released so far
    uint32_t pad[2];
};

// Grid barrier of the batched solve (bounded like grid_barrier).  fin: the last
// block to arrive finishes the density pass of every scene that ran one (its
// threads one scene each: error means from the scenes' integer sums, convergence).
__device__ __forceinline__ bool batch_barrier(BatchSync *sy, uint32_t &gen, const BatchScene *tab, uint32_t S,
                                              unsigned long long *acc, const uint32_t *s_n, const uint8_t *s_run,
                                              bool fin) {
    __syncthreads();
    __shared__ uint32_t s_last, s_ok;
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&sy->bar_arrive, 1u) + 1u == gridDim.x ? 1u : 0u;
        s_ok = 1u;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        if (fin)
            for (uint32_t sc = threadIdx.x; sc < S; sc += blockDim.x) {
                if (!s_run[sc]) continue;
                const unsigned long long t1 = *(volatile unsigned long long *)&acc[2 * sc];
                const unsigned long long t2 = *(volatile unsigned long long *)&acc[2 * sc + 1];
                acc[2 * sc] = 0ull;
                acc[2 * sc + 1] = 0ull;
                finish_pass(tab[sc].a, s_n[sc], (long long)t1, (long long)t2);
            }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            sy->bar_arrive = 0u;
            __threadfence();
            atomicAdd(&sy->bar_gen, 1u);  // release
        }
    } else if (threadIdx.x == 0) {
        uint32_t spins = 0;
        bool inject;
        const uint32_t limit = wait_limit(tab[0].a.st, kBarrierSpins, inject);
        while (inject || *(volatile uint32_t *)&sy->bar_gen == gen) {
            if (++spins > limit) {
                for (uint32_t sc = 0; sc < S; ++sc) {
                    set_flag(tab[sc].a.st, APBF_FLAG_SPIN_LIMIT);
                    tab[sc].a.st->spin_where = 4u;
                }
                s_ok = 0u;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
    }
    __syncthreads();
    ++gen;
    return s_ok != 0u;
}

constexpr uint32_t kBatchScenes = 256;  // scenes per batched solve (a finishing thread each)

// Jacobi passes 1.. of every scene in the table (each until its own error target or
// pass limit), the scenes' particles cut into units of one block: per pass the
// density phase of every running scene, a grid barrier whose last block finishes
// those scenes' passes, the position phase, a second barrier.  The per-particle
// arithmetic is density_one / delta_one, as in the per-scene forms, so each scene
// ends bit-identical to a solve of its own.
__global__ void __launch_bounds__(256, 4) k_solve_batch(const BatchScene *__restrict__ tab, uint32_t S,
                                                        BatchSync *sy, unsigned long long *acc) {
    __shared__ uint32_t s_n[kBatchScenes], s_unit[kBatchScenes + 1], s_max[kBatchScenes];
    __shared__ uint8_t s_run[kBatchScenes], s_conv[kBatchScenes], s_upd[kBatchScenes], s_done[kBatchScenes];
    __shared__ uint8_t s_defer[kBatchScenes], s_packed[kBatchScenes], s_sym[kBatchScenes];
    __shared__ uint32_t s_maxpass;
    uint32_t gen = *(volatile uint32_t *)&sy->bar_gen;  // read before this block's first arrival
    for (uint32_t sc = threadIdx.x; sc < S; sc += blockDim.x) {
        const BatchScene &b = tab[sc];
        const Status *st = b.a.st;
        s_n[sc] = b.a.d_len[kLenParticles];
        s_max[sc] = b.l.max_passes;
        // rows: 1 symmetric, 2 own rows with correction rows, 0 transposed
        s_sym[sc] = st->range_min == st->range_max ? 1 : (st->union_rows != 0u ? 2 : 0);
        s_defer[sc] = (b.l.defer != 0 && s_sym[sc] != 0) ? 1 : 0;
        s_packed[sc] = st->kw_uniform != 0u ? 1 : 0;
        s_done[sc] = (b.a.early_exit && *(volatile const uint32_t *)&st->converged) ? 1 : 0;  // pass 0 met the target
        s_upd[sc] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // units of blockDim particles per scene, and the largest pass limit
        uint32_t u = 0, mp = 0;
        for (uint32_t sc = 0; sc < S; ++sc) {
            s_unit[sc] = u;
            u += (s_n[sc] + blockDim.x - 1) / blockDim.x;
            mp = max(mp, s_max[sc]);
        }
        s_unit[S] = u;
        s_maxpass = mp;
    }
    __syncthreads();
    const uint32_t units = s_unit[S];
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t pass = 1; pass < s_maxpass; ++pass) {
        bool any = false;
        for (uint32_t sc = 0; sc < S; ++sc) any = any || (!s_done[sc] && pass < s_max[sc]);
        if (!any) break;  // uniform: every block holds the same flags
        __syncthreads();
        for (uint32_t sc = threadIdx.x; sc < S; sc += blockDim.x) s_run[sc] = (!s_done[sc] && pass < s_max[sc]) ? 1 : 0;
        __syncthreads();
        // density phase
        for (uint32_t u = blockIdx.x; u < units; u += gridDim.x) {
            uint32_t lo = 0, hi = S;  // the scene of unit u: s_unit[sc] <= u < s_unit[sc + 1]
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (s_unit[mid] <= u) lo = mid;
                else hi = mid;
            }
            const uint32_t sc = lo;
            if (!s_run[sc]) continue;  // uniform over the block
            const BatchScene &bs = tab[sc];
            const int4 *cur = (s_upd[sc] & 1u) ? bs.l.pos_b : bs.l.pos_a;
            const uint32_t i = (u - s_unit[sc]) * blockDim.x + threadIdx.x;
            PassSums ps;
            density_one<true, 1, false>(bs.a, cur, i, s_n[sc], 0u, s_defer[sc] != 0, false, ps);
            long long e1 = ps.e1, e2 = ps.e2;
            for (int off = 16; off > 0; off >>= 1) {
                e1 += __shfl_down_sync(0xffffffffu, e1, off);
                e2 += __shfl_down_sync(0xffffffffu, e2, off);
            }
            if (lane == 0 && (e1 | e2)) {
                atomicAdd(&acc[2 * sc], (unsigned long long)e1);
                atomicAdd(&acc[2 * sc + 1], (unsigned long long)e2);
            }
        }
        if (!batch_barrier(sy, gen, tab, S, acc, s_n, s_run, true)) return;
        for (uint32_t sc = threadIdx.x; sc < S; sc += blockDim.x)
            s_conv[sc] = (s_run[sc] && *(volatile const uint32_t *)&tab[sc].a.st->converged) ? 1 : 0;
        __syncthreads();
        // position phase
        for (uint32_t u = blockIdx.x; u < units; u += gridDim.x) {
            uint32_t lo = 0, hi = S;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (s_unit[mid] <= u) lo = mid;
                else hi = mid;
            }
            const uint32_t sc = lo;
            if (!s_run[sc]) continue;
            const BatchScene &bs = tab[sc];
            const PassB &b = bs.b;
            const int4 *cur = (s_upd[sc] & 1u) ? bs.l.pos_b : bs.l.pos_a;
            int4 *nxt = (s_upd[sc] & 1u) ? bs.l.pos_a : bs.l.pos_b;
            const uint32_t j = (u - s_unit[sc]) * blockDim.x + threadIdx.x;
            if (s_conv[sc]) {  // converged: the deferred filter of this pass, nothing applied
                if (j < s_n[sc]) {
                    if (s_defer[sc]) delta_skip_filter(b, cur, j);
                    accumulate(b.lam_prev, b.prev_mode, j, 0.0f);
                }
                continue;
            }
            const uint32_t nb = pass + 1u < s_max[sc] ? bs.l.nboxes : 0u;
            const uint32_t *cnt_arr = s_sym[sc] ? b.count : b.rcount;
            const uint32_t *idx_arr = s_sym[sc] ? b.idx : b.ridx;
            delta_one<true, 1>(b, cur, nxt, j, s_n[sc], 0u, s_packed[sc] != 0, s_defer[sc] != 0, cnt_arr, idx_arr,
                               s_sym[sc] == 2, nb);
        }
        if (!batch_barrier(sy, gen, tab, S, acc, s_n, s_run, false)) return;
        for (uint32_t sc = threadIdx.x; sc < S; sc += blockDim.x) {
            if (!s_run[sc]) continue;
            if (s_conv[sc]) s_done[sc] = 1;
            else s_upd[sc] = (uint8_t)(s_upd[sc] + 1);
        }
        __syncthreads();
    }
    // scenes that end after an odd number of updates: positions back to their pos_a
    for (uint32_t u = blockIdx.x; u < units; u += gridDim.x) {
        uint32_t lo = 0, hi = S;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_unit[mid] <= u) lo = mid;
            else hi = mid;
        }
        const uint32_t sc = lo;
        if (!(s_upd[sc] & 1u)) continue;
        const uint32_t j = (u - s_unit[sc]) * blockDim.x + threadIdx.x;
        if (j < s_n[sc]) tab[sc].l.pos_a[j] = tab[sc].l.pos_b[j];
    }
}

__global__ void k_mass_volume(const float *inv_mass, const float *radius, const uint32_t *d_len, double *partials) {
    const uint32_t n = d_len[kLenParticles];
    double m = 0.0, v = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        m += 1.0 / (double)inv_mass[i];
        double r = radius[i];
        v += r * r * r;
    }
    __shared__ double s1[8], s2[8];
    for (int off = 16; off > 0; off >>= 1) {
        m += __shfl_down_sync(0xffffffffu, m, off);
        v += __shfl_down_sync(0xffffffffu, v, off);
    }
    if ((threadIdx.x & 31) == 0) {
        s1[threadIdx.x >> 5] = m;
        s2[threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t1 = 0.0, t2 = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            t1 += s1[k];
            t2 += s2[k];
        }
        partials[2 * blockIdx.x] = t1;
        partials[2 * blockIdx.x + 1] = t2;
    }
}

__global__ void __launch_bounds__(256) k_finalize_mass(const double *partials, int blocks, double *out) {
    double t1, t2;
    block_sum2(partials, blocks, t1, t2);
    if (threadIdx.x == 0) {
        out[0] = t1;
        out[1] = t2;
    }
}

}  // namespace

// Calls f with std::integral_constant<int, L> for the tuned lanes per particle.
template <typename F>
void launch_lanes(int lanes, F &&f) {
    switch (lanes) {
        case 2: f(std::integral_constant<int, 2>()); break;
        case 4: f(std::integral_constant<int, 4>()); break;
        case 8: f(std::integral_constant<int, 8>()); break;
        default: f(std::integral_constant<int, 1>()); break;
    }
}

// Kernel arguments of the density pass (PassA) and the position update (PassB)
// for the context's current buffers and the solve options.
static PassA make_pass_a(apbf_ctx *ctx, const SolveOpts &o) {
    const bool converge = o.converge, projected = o.projected;
    const int feature_mode = o.feature_mode, prev_mode = o.prev_mode;
    FluidBufs &f = ctx->fl[ctx->fcur];
    const apbf_settings &st = ctx->settings;
    PassA a;
    a.pos = f.pos;
    a.inv_mass = f.inv_mass;
    a.radius = f.radius;
    a.kw = f.kernel_width;
    a.bness = f.boundariness;
    a.count = ctx->nb_count;
    a.idx = ctx->nb_idx;
    a.stride = ctx->row_stride;
    a.lambda = ctx->debug ? ctx->lambda : nullptr;
    a.shift = ctx->shift;
    a.rec = ctx->solve_rec;
    a.pk = ctx->solve_pk;
    a.kc = ctx->solve_kc;
    a.dbg_dens = ctx->debug ? ctx->dbg_density : nullptr;
    a.dbg_grad = ctx->dbg_grad;
    a.dbg_sq = ctx->dbg_sq;
    a.partials = reinterpret_cast<long long *>(ctx->red_partials);
    a.d_len = ctx->d_len;
    a.st = ctx->status;
    a.red_out = ctx->red_out;
    a.target = converge ? st.density_error_target : 0.0f;
    a.early_exit = converge ? 1 : 0;
    a.features = feature_mode ? ctx->features : nullptr;
    a.selfdir = ctx->selfdir;
    a.vel = f.vel;
    a.lam_prev = f.lambda_prev;
    a.projected = projected && prev_mode == 2 ? 1 : 0;
    a.loop_offset = o.loop_offset;
    a.max_passes = o.max_passes;
    a.filt = ctx->tuning.filter_in_density ? nullptr : ctx->filt;
    const float rm2 = 2.0f * st.smallest_target_radius;
    a.rmin3 = rm2 * rm2 * rm2;
    a.hk = st.height_kernel_id;
    a.gk = st.gradient_kernel_id;
    a.method = st.boundariness_calculation_method;
    a.update_b = st.update_boundariness;
    a.b_speed = st.boundariness_adaption_speed;
    a.b_sgl_factor = st.boundariness_self_grad_length_factor;
    a.b_up_factor = st.boundariness_underpressure_factor;
    return a;
}

static PassB make_pass_b(apbf_ctx *ctx, const SolveOpts &o) {
    FluidBufs &f = ctx->fl[ctx->fcur];
    FluidBufs &alt = ctx->fl[ctx->fcur ^ 1];
    const apbf_settings &st = ctx->settings;
    PassB b;
    b.pos = f.pos;
    b.pos_out = alt.pos;
    b.rec = ctx->solve_rec;
    b.pk = ctx->solve_pk;
    b.kc = ctx->solve_kc;
    b.kw = f.kernel_width;
    b.shift = ctx->shift;
    b.radius = f.radius;
    b.bmin = ctx->box_min;
    b.bmax = ctx->box_max;
    b.rot = ctx->box_rot;
    b.nboxes = o.box_after ? ctx->n_boxes : 0u;
    b.count = ctx->nb_count;
    b.idx = ctx->nb_idx;
    b.rcount = ctx->rev_count;
    b.ridx = ctx->rev_idx;
    b.stride = ctx->row_stride;
    b.d_len = ctx->d_len;
    b.st = ctx->status;
    b.gk = st.gradient_kernel_id;
    b.early_exit = o.converge ? 1 : 0;
    b.lam_prev = f.lambda_prev;
    b.lam_acc = ctx->lam_acc;
    b.prev_mode = o.prev_mode;
    b.acc_mode = o.acc_mode;
    b.loop_offset = o.loop_offset;
    b.max_passes = o.max_passes;
    b.filt = ctx->filt;
    b.bness = f.boundariness;
    return b;
}

apbf_status incompressibility(apbf_ctx *ctx, cudaStream_t s, const SolveOpts &o) {
    const bool converge = o.converge, learned = o.learned;
    const uint32_t cap = ctx->cfg.particle_capacity;
    FluidBufs &f = ctx->fl[ctx->fcur];
    FluidBufs &alt = ctx->fl[ctx->fcur ^ 1];
    const apbf_settings &st = ctx->settings;
    const bool gauss = st.height_kernel_id == 1 && st.gradient_kernel_id == 1;
    const PassA a = make_pass_a(ctx, o);
    const int g = ctx->red_blocks;
    const int lanes = ctx->tuning.gather_lanes;
    const int pb = ctx->tuning.pass_block == 128 ? 128 : 256;
    const int bps = (int)std::min(8u, std::max(1u, ctx->tuning.pass_blocks_per_sm));
    // the error reduction has one partial per block: at most red_blocks blocks
    const int ga = std::min(g, grid_for(ctx, (uint32_t)std::min<uint64_t>((uint64_t)cap * lanes, 0xffffffffu), pb, bps));
    const bool xtra = a.features != nullptr || a.method == 1;
    APBF_BEFORE_LAUNCH(ctx, s, "k_density_lambda");
    launch_lanes(lanes, [&](auto lc) {
        constexpr int Lc = decltype(lc)::value;
        if (gauss && xtra)
            k_density_lambda<true, Lc, true><<<ga, pb, 0, s>>>(a);
        else if (gauss)
            k_density_lambda<true, Lc, false><<<ga, pb, 0, s>>>(a);
        else
            k_density_lambda<false, Lc, true><<<ga, pb, 0, s>>>(a);
    });
    APBF_AFTER_LAUNCH(ctx, s, "k_density_lambda");

    if (learned) {  // the network's lambda replaces the plain one in this update
        apbf_status r = mlp_lambda(ctx, s, converge);
        if (r != APBF_OK) return r;
    }
    const PassB b = make_pass_b(ctx, o);
    APBF_BEFORE_LAUNCH(ctx, s, "k_delta");
    const int gd = grid_for(ctx, (uint32_t)std::min<uint64_t>((uint64_t)cap * lanes, 0xffffffffu), pb, bps);
    launch_lanes(lanes, [&](auto lc) {
        constexpr int Lc = decltype(lc)::value;
        if (gauss)
            k_delta<true, Lc><<<gd, pb, 0, s>>>(b);
        else
            k_delta<false, Lc><<<gd, pb, 0, s>>>(b);
    });
    APBF_AFTER_LAUNCH(ctx, s, "k_delta");
    // the updated positions now live in the alternate buffer: swap position buffers
    int4 *tmp = f.pos;
    f.pos = alt.pos;
    alt.pos = tmp;
    return APBF_OK;
}

bool solve_persistent_eligible(const apbf_ctx *ctx, const SolveOpts &o) {
    const apbf_settings &st = ctx->settings;
    return ctx->persistent_solve && ctx->coop_blocks > 0 && !ctx->in_batch && st.height_kernel_id == 1 &&
           st.gradient_kernel_id == 1 &&
           st.boundariness_calculation_method != 1 && !o.feature_mode && !o.learned && !o.acc_mode &&
           !ctx->debug && !ctx->prof_on && o.max_passes >= 2;
}

apbf_status solve_persistent(apbf_ctx *ctx, cudaStream_t s, const SolveOpts &o) {
    if (!solve_persistent_eligible(ctx, o)) return APBF_ERR_INVALID_ARG;
    SolveOpts q = o;
    q.loop_offset = -1;
    q.box_after = true;  // decided per pass in the kernel
    PassA a = make_pass_a(ctx, q);
    PassB b = make_pass_b(ctx, q);
    a.features = nullptr;
    LoopArgs l;
    l.pos_a = ctx->fl[ctx->fcur].pos;
    l.pos_b = ctx->fl[ctx->fcur ^ 1].pos;
    l.first = 1u;
    l.max_passes = o.max_passes;
    l.nboxes = ctx->n_boxes;
    l.defer = (a.filt && a.method == 2) ? 1 : 0;
    // barrier counters and pass sums start from zero on every launch
    APBF_CUDA(cudaMemsetAsync(&ctx->status->bar_arrive, 0,
                              offsetof(Status, loop_e2) + sizeof(unsigned long long) - offsetof(Status, bar_arrive), s));
    const uint32_t want = (ctx->cfg.particle_capacity + 255u) / 256u;
    const uint32_t grid = std::max(1u, std::min((uint32_t)ctx->coop_blocks, want));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    APBF_BEFORE_LAUNCH(ctx, s, "k_solve_loop");
    APBF_CUDA(cudaLaunchKernelEx(&cfg, k_solve_loop<true>, a, b, l));
    APBF_AFTER_LAUNCH(ctx, s, "k_solve_loop");
    return APBF_OK;
}

// Resident blocks of the persistent solve kernel (0: cooperative launches are
// not available), computed once per context.
int solve_persistent_blocks(int device, int num_sms) {
    int coop = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess || !coop) return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_loop<true>, 256, 0) != cudaSuccess) return 0;
    return per_sm * num_sms;
}

bool batch_solve_eligible(const apbf_ctx *ctx, const SolveOpts &o) {
    const apbf_settings &st = ctx->settings;
    return ctx->coop_blocks > 0 && st.height_kernel_id == 1 && st.gradient_kernel_id == 1 &&
           st.boundariness_calculation_method != 1 && !o.feature_mode && !o.learned && !o.acc_mode && !ctx->debug &&
           !ctx->prof_on && o.max_passes >= 2;
}

size_t batch_scene_bytes() { return sizeof(BatchScene); }
size_t batch_sync_bytes() { return sizeof(BatchSync); }
uint32_t batch_max_scenes() { return kBatchScenes; }

void batch_scene_fill(apbf_ctx *ctx, const SolveOpts &o, void *entry) {
    SolveOpts q = o;
    q.loop_offset = -1;
    q.box_after = true;  // decided per pass in the kernel
    BatchScene &e = *reinterpret_cast<BatchScene *>(entry);
    e.a = make_pass_a(ctx, q);
    e.a.features = nullptr;
    e.b = make_pass_b(ctx, q);
    e.l.pos_a = ctx->fl[ctx->fcur].pos;
    e.l.pos_b = ctx->fl[ctx->fcur ^ 1].pos;
    e.l.first = 1u;
    e.l.max_passes = o.max_passes;
    e.l.nboxes = ctx->n_boxes;
    e.l.defer = (e.a.filt && e.a.method == 2) ? 1 : 0;
}

apbf_status solve_batch_launch(const void *d_table, uint32_t n_scenes, void *d_sync, unsigned long long *d_acc,
                               int grid, cudaStream_t s) {
    if (n_scenes == 0 || n_scenes > kBatchScenes || grid <= 0) return APBF_ERR_INVALID_ARG;
    APBF_CUDA(cudaMemsetAsync(d_sync, 0, sizeof(BatchSync), s));
    APBF_CUDA(cudaMemsetAsync(d_acc, 0, (size_t)2 * n_scenes * sizeof(unsigned long long), s));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    APBF_CUDA(cudaLaunchKernelEx(&cfg, k_solve_batch, reinterpret_cast<const BatchScene *>(d_table), n_scenes,
                                 reinterpret_cast<BatchSync *>(d_sync), d_acc));
    return APBF_OK;
}

int solve_batch_blocks(int device, int num_sms) {
    int coop = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess || !coop) return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_batch, 256, 0) != cudaSuccess) return 0;
    return per_sm * num_sms;
}

apbf_status reduce_fp64(apbf_ctx *ctx, double out[4], cudaStream_t s) {
    FluidBufs &f = ctx->fl[ctx->fcur];
    const int g = ctx->red_blocks;
    // red_out[2..3] hold the error of the last density pass (its last block wrote them)
    APBF_BEFORE_LAUNCH(ctx, s, "k_mass_volume");
    k_mass_volume<<<g, kBlock, 0, s>>>(f.inv_mass, f.radius, ctx->d_len, ctx->red_partials + 4 * g);
    APBF_AFTER_LAUNCH(ctx, s, "k_mass_volume");
    APBF_BEFORE_LAUNCH(ctx, s, "k_finalize_mass");
    k_finalize_mass<<<1, 256, 0, s>>>(ctx->red_partials + 4 * g, g, ctx->red_out);
    APBF_AFTER_LAUNCH(ctx, s, "k_finalize_mass");
    APBF_CUDA(cudaMemcpyAsync(out, ctx->red_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    APBF_CUDA(cudaStreamSynchronize(s));
    return APBF_OK;
}

namespace {
// Appends (features, sum of min(0, lambda)) of the particles to the caller's
// sample buffers, in particle order, up to their capacity.
__global__ void k_record_append(const float *feat, const float *acc, const uint32_t *d_len, float *out_f,
                                float *out_t, uint32_t cap, uint32_t *count) {
    const uint32_t n = d_len[kLenParticles];
    const uint32_t base = *count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t r = base + i;
        if (r >= cap) break;
        for (int k = 0; k < 8; ++k) out_f[(size_t)r * 8 + k] = feat[(size_t)i * 8 + k];
        out_t[r] = acc[i];
    }
}
__global__ void k_record_count(const uint32_t *d_len, uint32_t cap, uint32_t *count) {
    const uint32_t v = *count + d_len[kLenParticles];
    *count = v < cap ? v : cap;
}
}  // namespace

apbf_status record_samples(apbf_ctx *ctx, cudaStream_t s) {
    const uint32_t cap = ctx->cfg.particle_capacity;
    APBF_BEFORE_LAUNCH(ctx, s, "k_record_append");
    k_record_append<<<grid_for(ctx, cap), kBlock, 0, s>>>(ctx->features, ctx->lam_acc, ctx->d_len, ctx->rec_features,
                                                         ctx->rec_targets, ctx->rec_capacity, ctx->rec_count);
    APBF_AFTER_LAUNCH(ctx, s, "k_record_append");
    APBF_BEFORE_LAUNCH(ctx, s, "k_record_count");
    k_record_count<<<1, 1, 0, s>>>(ctx->d_len, ctx->rec_capacity, ctx->rec_count);
    APBF_AFTER_LAUNCH(ctx, s, "k_record_count");
    return APBF_OK;
}

}  // namespace apbf
