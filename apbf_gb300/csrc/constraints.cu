// constraints.cu -- the reference's further constraint operators on the same
// particle and neighbour lists, with plain FP32 arithmetic: this translation unit
// is compiled with -fmad=false, so every operation rounds on its own, in the
// written order, as the oracle's C restatement does.
//
//  sphere_collision::apply (source/sphere_collision.cpp:19-31): sphere_collision.comp:42-58
//  inter_particle_collision::apply (source/inter_particle_collision.cpp:10-18):
//      inter_particle_collision.comp:25-51, a Jacobi step (reads the old positions,
//      adds the shifts to a copy)
//  glue::applyNewGlue / glue::apply (source/glue.cpp:38-60): generate_glue.comp:24-46,
//      glue.comp:32-55
//
// The reference appends glue with an atomic counter (unordered); here the glue
// list is in row order (particle, then its row), compacted by a prefix sum.  The
// position shifts are integer atomic adds as in the reference: integer sums do not
// depend on their order, so the results are deterministic (glue entries read the
// positions before the pass, see k_glue_apply).
#include "apbf_internal.cuh"

namespace apbf {
namespace {

__device__ __forceinline__ float fract_p(float x) { return x - floorf(x); }

// shadertoy 4djSRW hash11 (MIT licence), as in sphere_collision.comp:24-30
__device__ __forceinline__ float hash11(float p) {
    p = fract_p(p * 0.1031f);
    p *= p + 33.33f;
    p *= p + p;
    return fract_p(p);
}

__global__ void k_sphere_collision(int4 *pos, const float *radius, const uint32_t *d_len, float3 c, float R,
                                   int hollow) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += gridDim.x * blockDim.x) {
        const int4 ip = pos[id];
        float px = (float)ip.x / 262144.0f, py = (float)ip.y / 262144.0f, pz = (float)ip.z / 262144.0f;
        const float r = radius[id];
        const float dir = hollow ? -1.0f : 1.0f;
        const float off = dir * (r + hash11((float)id * py + px + pz) * 0.05f);
        const float rx = px - c.x, ry = py - c.y, rz = pz - c.z;
        const float d = sqrtf(rx * rx + ry * ry + rz * rz);
        const float target = R + off;
        if ((d < target) == (hollow != 0)) continue;
        const float s = target / d;
        px = c.x + rx * s;
        py = c.y + ry * s;
        pz = c.z + rz * s;
        pos[id] = make_int4(f2i(px * 262144.0f), f2i(py * 262144.0f), f2i(pz * 262144.0f), ip.w);
    }
}

// Each ordered pair (i, j) of the rows is solved by particle i when i has the
// larger radius, or the same radius and the larger index (the reference's "once
// per pair" rule); the shifts go to both particles.
__global__ void k_inter_particle_collision(const int4 *__restrict__ old_pos, int4 *new_pos, const float *radius,
                                           const float *inv_mass, const uint32_t *count, const uint32_t *idx,
                                           uint32_t stride, const uint32_t *d_len) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t cnt = count[i];
        const int4 p = old_pos[i];
        const float r = radius[i], im = inv_mass[i];
        for (uint32_t k = 0; k < cnt; ++k) {
            const uint32_t j = idx[(size_t)k * stride + i];
            const float rN = radius[j];
            if (rN > r || (rN == r && j >= i)) continue;
            const int4 q = old_pos[j];
            const float dx = (float)wadd(q.x, -p.x), dy = (float)wadd(q.y, -p.y), dz = (float)wadd(q.z, -p.z);
            const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
            const float ce = dist - (r + rN) * 262144.0f;
            if (ce >= 0.0f) continue;
            const float imN = inv_mass[j];
            const float scalar = ce / (im + imN);
            const float a = im * scalar / dist, b = -imN * scalar / dist;
            atomicAdd(&new_pos[i].x, f2i(a * dx));
            atomicAdd(&new_pos[i].y, f2i(a * dy));
            atomicAdd(&new_pos[i].z, f2i(a * dz));
            atomicAdd(&new_pos[j].x, f2i(b * dx));
            atomicAdd(&new_pos[j].y, f2i(b * dy));
            atomicAdd(&new_pos[j].z, f2i(b * dz));
        }
    }
}

// generate_glue.comp:30-45: glue the pair (i, j) of the rows when j has the smaller
// radius, or the same radius and the larger index, and the gap is at most 2 r_i.
__device__ __forceinline__ bool glue_pair(const int4 *pos, const float *radius, uint32_t i, uint32_t j, int4 p,
                                          float r, uint32_t *dist_out) {
    const float rN = radius[j];
    if (rN > r || (rN == r && i >= j)) return false;
    const int4 q = pos[j];
    const float dx = (float)wadd(q.x, -p.x) / 262144.0f, dy = (float)wadd(q.y, -p.y) / 262144.0f,
                dz = (float)wadd(q.z, -p.z) / 262144.0f;
    const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
    const float gap = dist - r - rN;
    if (gap > 2.0f * r) return false;
    *dist_out = f2u(dist * 262144.0f);
    return true;
}

__global__ void k_glue_count(const int4 *pos, const float *radius, const uint32_t *count, const uint32_t *idx,
                             uint32_t stride, const uint32_t *d_len, uint32_t *per_particle) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 p = pos[i];
        const float r = radius[i];
        uint32_t c = 0, d;
        for (uint32_t k = 0; k < count[i]; ++k)
            if (glue_pair(pos, radius, i, idx[(size_t)k * stride + i], p, r, &d)) ++c;
        per_particle[i] = c;
    }
}

__global__ void k_glue_write(const int4 *pos, const float *radius, const uint32_t *count, const uint32_t *idx,
                             uint32_t stride, const uint32_t *d_len, const uint32_t *scan, uint32_t cap,
                             uint32_t *g0, uint32_t *g1, uint32_t *gd, uint32_t *glen, Status *st) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 p = pos[i];
        const float r = radius[i];
        uint32_t o = i ? scan[i - 1] : 0u;  // inclusive scan -> first slot of particle i
        uint32_t d;
        for (uint32_t k = 0; k < count[i]; ++k) {
            const uint32_t j = idx[(size_t)k * stride + i];
            if (!glue_pair(pos, radius, i, j, p, r, &d)) continue;
            if (o < cap) {
                g0[o] = i;
                g1[o] = j;
                gd[o] = d;
            }
            ++o;
        }
        if (i == n - 1) {
            const uint32_t total = scan[i];
            if (total > cap) set_flag(st, APBF_FLAG_TRANSFER_OVERFLOW);
            *glen = total < cap ? total : cap;
        }
    }
    if (n == 0 && blockIdx.x == 0 && threadIdx.x == 0) *glen = 0u;
}

// glue.comp reads the positions it updates (a race between entries that share a
// particle); here every entry reads the positions before the pass and adds to a
// copy, a Jacobi step like inter_particle_collision.
__global__ void k_glue_apply(const int4 *__restrict__ old_pos, int4 *pos, const float *inv_mass, const uint32_t *g0,
                             const uint32_t *g1, const uint32_t *gd, const uint32_t *glen, float stability) {
    const uint32_t m = *glen;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const uint32_t a = g0[k], b = g1[k];
        const int4 p0 = old_pos[a], p1 = old_pos[b];
        const float im0 = inv_mass[a], im1 = inv_mass[b];
        const float dx = (float)wadd(p1.x, -p0.x), dy = (float)wadd(p1.y, -p0.y), dz = (float)wadd(p1.z, -p0.z);
        const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
        const float ce = dist - (float)gd[k];
        const float scalar = stability * ce / ((im0 + im1) * dist);
        atomicAdd(&pos[a].x, f2i(im0 * scalar * dx));
        atomicAdd(&pos[a].y, f2i(im0 * scalar * dy));
        atomicAdd(&pos[a].z, f2i(im0 * scalar * dz));
        atomicAdd(&pos[b].x, f2i(-im1 * scalar * dx));
        atomicAdd(&pos[b].y, f2i(-im1 * scalar * dy));
        atomicAdd(&pos[b].z, f2i(-im1 * scalar * dz));
    }
}

__global__ void k_glue_remap(uint32_t *g0, uint32_t *g1, const uint32_t *glen, const uint32_t *inv_perm,
                             const uint32_t *d_len, Status *st) {
    const uint32_t m = *glen, n = d_len[kLenParticles];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const uint32_t a = g0[k], b = g1[k];
        if (a >= n || b >= n) {
            set_flag(st, APBF_FLAG_NONFINITE);
            continue;
        }
        g0[k] = inv_perm[a];
        g1[k] = inv_perm[b];
    }
}

}  // namespace

apbf_status glue_remap(apbf_ctx *ctx, cudaStream_t s) {
    if (!ctx->glue_cap) return APBF_OK;
    APBF_BEFORE_LAUNCH(ctx, s, "k_glue_remap");
    k_glue_remap<<<grid_for(ctx, ctx->glue_cap), kBlock, 0, s>>>(ctx->glue0, ctx->glue1, ctx->glue_len, ctx->inv_perm,
                                                               ctx->d_len, ctx->status);
    APBF_AFTER_LAUNCH(ctx, s, "k_glue_remap");
    return APBF_OK;
}

}  // namespace apbf

using namespace apbf;

extern "C" apbf_status apbf_sphere_collision_apply(apbf_ctx *ctx, const float center[3], float radius, int hollow,
                                                   void *stream) {
    if (!ctx || !center) return APBF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    FluidBufs &f = ctx->fl[ctx->fcur];
    APBF_BEFORE_LAUNCH(ctx, s, "k_sphere_collision");
    k_sphere_collision<<<grid_for(ctx, ctx->cfg.particle_capacity), kBlock, 0, s>>>(
        f.pos, f.radius, ctx->d_len, make_float3(center[0], center[1], center[2]), radius, hollow ? 1 : 0);
    APBF_AFTER_LAUNCH(ctx, s, "k_sphere_collision");
    return APBF_OK;
}

extern "C" apbf_status apbf_inter_particle_collision_apply(apbf_ctx *ctx, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t cap = ctx->cfg.particle_capacity;
    FluidBufs &f = ctx->fl[ctx->fcur];
    FluidBufs &alt = ctx->fl[ctx->fcur ^ 1];
    // the new positions start as a copy of the old ones (inter_particle_collision.cpp:15-17)
    APBF_CUDA(cudaMemcpyAsync(alt.pos, f.pos, (size_t)cap * sizeof(int4), cudaMemcpyDeviceToDevice, s));
    APBF_BEFORE_LAUNCH(ctx, s, "k_inter_particle_collision");
    k_inter_particle_collision<<<grid_for(ctx, cap), kBlock, 0, s>>>(f.pos, alt.pos, f.radius, f.inv_mass,
                                                                    ctx->nb_count, ctx->nb_idx, ctx->row_stride,
                                                                    ctx->d_len);
    APBF_AFTER_LAUNCH(ctx, s, "k_inter_particle_collision");
    int4 *t = f.pos;
    f.pos = alt.pos;
    alt.pos = t;
    return APBF_OK;
}

extern "C" apbf_status apbf_glue_generate(apbf_ctx *ctx, uint32_t capacity, void *stream) {
    if (!ctx || !capacity) return APBF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t cap = ctx->cfg.particle_capacity;
    if (capacity > ctx->glue_cap) {  // the glue list grows on demand, like a gpu_list request
        APBF_CUDA(cudaStreamSynchronize(s));
        cudaFree(ctx->glue0);
        cudaFree(ctx->glue1);
        cudaFree(ctx->glue_d);
        ctx->glue0 = ctx->glue1 = ctx->glue_d = nullptr;
        ctx->glue_cap = 0;
        APBF_CUDA(cudaMalloc(&ctx->glue0, (size_t)capacity * 4));
        APBF_CUDA(cudaMalloc(&ctx->glue1, (size_t)capacity * 4));
        APBF_CUDA(cudaMalloc(&ctx->glue_d, (size_t)capacity * 4));
        if (!ctx->glue_len) APBF_CUDA(cudaMalloc(&ctx->glue_len, 4));
        ctx->glue_cap = capacity;
        ctx->graph_version++;
    }
    FluidBufs &f = ctx->fl[ctx->fcur];
    APBF_BEFORE_LAUNCH(ctx, s, "k_glue_count");
    k_glue_count<<<grid_for(ctx, cap), kBlock, 0, s>>>(f.pos, f.radius, ctx->nb_count, ctx->nb_idx, ctx->row_stride,
                                                      ctx->d_len, ctx->scan_tmp);
    APBF_AFTER_LAUNCH(ctx, s, "k_glue_count");
    apbf_status r = prefix_sum_device(ctx, ctx->scan_tmp, ctx->d_len + kLenParticles, cap, s);
    if (r != APBF_OK) return r;
    APBF_BEFORE_LAUNCH(ctx, s, "k_glue_write");
    k_glue_write<<<grid_for(ctx, cap), kBlock, 0, s>>>(f.pos, f.radius, ctx->nb_count, ctx->nb_idx, ctx->row_stride,
                                                      ctx->d_len, ctx->scan_tmp, ctx->glue_cap, ctx->glue0, ctx->glue1,
                                                      ctx->glue_d, ctx->glue_len, ctx->status);
    APBF_AFTER_LAUNCH(ctx, s, "k_glue_write");
    return APBF_OK;
}

extern "C" apbf_status apbf_glue_apply(apbf_ctx *ctx, float stability, float elasticity, void *stream) {
    (void)elasticity;  // unused by the reference too (glue.comp:21, "TODO delete overstretched glue")
    if (!ctx) return APBF_ERR_INVALID_ARG;
    if (!ctx->glue_cap) return APBF_OK;
    cudaStream_t s = (cudaStream_t)stream;
    FluidBufs &f = ctx->fl[ctx->fcur];
    FluidBufs &alt = ctx->fl[ctx->fcur ^ 1];
    APBF_CUDA(cudaMemcpyAsync(alt.pos, f.pos, (size_t)ctx->cfg.particle_capacity * sizeof(int4),
                              cudaMemcpyDeviceToDevice, s));
    APBF_BEFORE_LAUNCH(ctx, s, "k_glue_apply");
    k_glue_apply<<<grid_for(ctx, ctx->glue_cap), kBlock, 0, s>>>(f.pos, alt.pos, f.inv_mass, ctx->glue0, ctx->glue1,
                                                               ctx->glue_d, ctx->glue_len, stability);
    APBF_AFTER_LAUNCH(ctx, s, "k_glue_apply");
    int4 *t = f.pos;
    f.pos = alt.pos;
    alt.pos = t;
    return APBF_OK;
}

extern "C" apbf_status apbf_glue_get_view(apbf_ctx *ctx, uint32_t **p0, uint32_t **p1, uint32_t **dist,
                                          uint32_t **d_length, uint32_t *capacity) {
    if (!ctx || !p0 || !p1 || !dist || !d_length || !capacity) return APBF_ERR_INVALID_ARG;
    *p0 = ctx->glue0;
    *p1 = ctx->glue1;
    *dist = ctx->glue_d;
    *d_length = ctx->glue_len;
    *capacity = ctx->glue_cap;
    return APBF_OK;
}
