// glue.cu -- substep stages whose reference arithmetic is plain FP32 (no
// transcendental functions), computed here with every operation rounded on its
// own: this translation unit is compiled with -fmad=false, so results are
// bit-identical to an IEEE FP32 evaluation in the written order.
//
//  velocity_handling::apply (source/velocity_handling.cpp:15-31):
//    infer_velocity.comp:30-31, apply_acceleration.comp:26-27, apply_velocity.comp:29-30
//  box_collision::apply (source/box_collision.cpp:12-24): box_collision.comp:35-60
//  kernel width from boundary distance (source/pool.cpp:77-80):
//    uint_to_float_with_indexed_lower_bound.comp:31-45
#include "apbf_internal.cuh"

namespace apbf {
namespace {

__global__ void k_velocity(FluidBufs f, const uint32_t *d_len, float inv_den, float3 acc_dt, float sc) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int4 p = f.pos[i];
        const int4 bk = f.pos_backup[i];
        float4 v = f.vel[i];
        v.x = (float)wadd(p.x, -bk.x) / inv_den;
        v.y = (float)wadd(p.y, -bk.y) / inv_den;
        v.z = (float)wadd(p.z, -bk.z) / inv_den;
        f.pos_backup[i] = p;
        v.x = v.x + acc_dt.x;
        v.y = v.y + acc_dt.y;
        v.z = v.z + acc_dt.z;
        p.x = wadd(p.x, f2i(v.x * sc));
        p.y = wadd(p.y, f2i(v.y * sc));
        p.z = wadd(p.z, f2i(v.z * sc));
        f.vel[i] = v;
        f.pos[i] = p;
    }
}

__global__ void k_backup(FluidBufs f, const uint32_t *d_len) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        f.pos_backup[i] = f.pos[i];
}

__global__ void k_box_collision(int4 *pos, const float *radius, const uint32_t *d_len, const float4 *bmin,
                                const float4 *bmax, uint32_t nb) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += gridDim.x * blockDim.x)
        pos[id] = box_push(pos[id], radius[id], id, bmin, bmax, nb);
}

__device__ __forceinline__ float move_towards_geo(float old_v, float new_v, float step) {
    float dir = new_v > old_v ? 1.0f : (new_v < old_v ? -1.0f : 0.0f);
    float result = old_v * (1.0f + step * dir);
    bool reached = (old_v < new_v) != (result < new_v);
    return reached ? new_v : result;
}

__global__ void k_kw_from_bd(FluidBufs f, const uint32_t *d_len, float factor, float speed) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float value = (float)f.boundary_distance[i] * factor;
        float lb = f.radius[i] * 4.0f;
        value = move_towards_geo(f.kernel_width[i], value, speed);
        f.kernel_width[i] = fmaxf(value, lb);
    }
}

}  // namespace

apbf_status velocity_handling(apbf_ctx *ctx, float dt, const float accel[3], cudaStream_t s) {
    FluidBufs &f = ctx->fl[ctx->fcur];
    const int g = grid_for(ctx, ctx->cfg.particle_capacity);
    if (dt == 0.0f) {
        APBF_BEFORE_LAUNCH(ctx, s, "k_backup");
        k_backup<<<g, kBlock, 0, s>>>(f, ctx->d_len);
        APBF_AFTER_LAUNCH(ctx, s, "k_backup");
        return APBF_OK;
    }
    const float inv_den = ctx->last_dt * 262144.0f;
    const float3 acc = make_float3(accel[0] * dt, accel[1] * dt, accel[2] * dt);
    const float sc = dt * 262144.0f;
    APBF_BEFORE_LAUNCH(ctx, s, "k_velocity");
    k_velocity<<<g, kBlock, 0, s>>>(f, ctx->d_len, inv_den, acc, sc);
    APBF_AFTER_LAUNCH(ctx, s, "k_velocity");
    ctx->last_dt = dt;
    return APBF_OK;
}

apbf_status box_collision(apbf_ctx *ctx, cudaStream_t s) {
    if (ctx->n_boxes == 0) return APBF_OK;
    FluidBufs &f = ctx->fl[ctx->fcur];
    APBF_BEFORE_LAUNCH(ctx, s, "k_box_collision");
    k_box_collision<<<grid_for(ctx, ctx->cfg.particle_capacity), kBlock, 0, s>>>(f.pos, f.radius, ctx->d_len,
                                                                                  ctx->box_min, ctx->box_max,
                                                                                  ctx->n_boxes);
    APBF_AFTER_LAUNCH(ctx, s, "k_box_collision");
    return APBF_OK;
}

apbf_status kw_from_boundary_distance(apbf_ctx *ctx, cudaStream_t s) {
    FluidBufs &f = ctx->fl[ctx->fcur];
    const float factor = ctx->settings.target_radius_scale_factor / 262144.0f;
    APBF_BEFORE_LAUNCH(ctx, s, "k_kw_from_bd");
    k_kw_from_bd<<<grid_for(ctx, ctx->cfg.particle_capacity), kBlock, 0, s>>>(f, ctx->d_len, factor,
                                                                               ctx->settings.kernel_width_adaption_speed);
    APBF_AFTER_LAUNCH(ctx, s, "k_kw_from_bd");
    return APBF_OK;
}

}  // namespace apbf
