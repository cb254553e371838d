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

// ---- emitter (no reference counterpart) ----
// 32-bit integer hash (a SplitMix64-style finaliser on the 64-bit mix of the inputs)
__device__ __forceinline__ uint32_t emit_hash(uint32_t seed, uint64_t layer, uint32_t cell, uint32_t axis) {
    uint64_t z = ((uint64_t)seed << 32) ^ (layer * 0x9E3779B97F4A7C15ull) ^ ((uint64_t)cell << 2) ^ axis;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (uint32_t)(z >> 32);
}

// One thread: which layers cross the emission plane during this substep, how many
// particles fit, and the new length.  state: [0] T, [1] emitted, [2] first layer,
// [3] count, [4] old length, [5] T at the start of the substep.
__global__ void k_emit_plan(double *state, uint32_t *d_len, Status *st, apbf_emitter e, double dt, uint32_t cap) {
    const double T = state[0];
    const double layer_dt = __ddiv_rn(2.0 * (double)e.radius, (double)e.speed);
    const uint64_t l0 = (uint64_t)ceil(__ddiv_rn(T, layer_dt));
    const uint64_t l1 = (uint64_t)ceil(__ddiv_rn(__dadd_rn(T, dt), layer_dt));
    const uint64_t per_layer = (uint64_t)e.nx * e.nz;
    uint64_t want = (l1 - l0) * per_layer;
    const uint64_t emitted = (uint64_t)state[1];
    if (e.max_particles && emitted + want > e.max_particles) want = e.max_particles > emitted ? e.max_particles - emitted : 0;
    const uint32_t n = d_len[kLenParticles];
    const uint64_t room = cap > n ? cap - n : 0;
    if (want > room) {
        set_flag(st, APBF_FLAG_PARTICLE_OVERFLOW);
        want = room;
    }
    state[0] = __dadd_rn(T, dt);
    state[1] = (double)(emitted + want);
    state[2] = (double)l0;
    state[3] = (double)want;
    state[4] = (double)n;
    state[5] = T;
    d_len[kLenParticles] = n + (uint32_t)want;
}

// Appends the planned particles after the old length, in (layer, i, j) order.
__global__ void k_emit(FluidBufs f, const double *state, apbf_emitter e, float inv_mass, int32_t backup_dy) {
    const uint64_t l0 = (uint64_t)state[2], count = (uint64_t)state[3];
    const uint32_t n0 = (uint32_t)state[4];
    const double Ts = state[5];
    const uint32_t per_layer = e.nx * e.nz;
    const double layer_dt = __ddiv_rn(2.0 * (double)e.radius, (double)e.speed);
    const float jr = __fmul_rn(e.jitter, e.radius);
    for (uint64_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t layer = l0 + k / per_layer;
        const uint32_t cell = (uint32_t)(k % per_layer), ci = cell / e.nz, cj = cell % e.nz;
        float jit[3];
        for (uint32_t a = 0; a < 3; ++a) {
            const float u = (float)(emit_hash(e.seed, layer, cell, a) >> 8) * 5.9604644775390625e-8f;  // [0, 1)
            jit[a] = __fmul_rn(__fsub_rn(__fmul_rn(2.0f, u), 1.0f), jr);
        }
        // above the plane by (t_l - T) * speed at the start of the substep
        const double t_l = __dmul_rn((double)layer, layer_dt);
        const float dy = (float)__dmul_rn(__dsub_rn(t_l, Ts), (double)e.speed);
        const float x = __fadd_rn(__fadd_rn(e.origin[0], __fmul_rn((float)(2u * ci + 1u), e.radius)), jit[0]);
        const float y = __fadd_rn(__fadd_rn(e.origin[1], dy), jit[1]);
        const float z = __fadd_rn(__fadd_rn(e.origin[2], __fmul_rn((float)(2u * cj + 1u), e.radius)), jit[2]);
        const int4 p = make_int4(f2i(__fmul_rn(x, 262144.0f)), f2i(__fmul_rn(y, 262144.0f)),
                                 f2i(__fmul_rn(z, 262144.0f)), 0);
        const uint32_t id = n0 + (uint32_t)k;
        f.pos[id] = p;
        f.pos_backup[id] = make_int4(p.x, wadd(p.y, backup_dy), p.z, 0);  // velocity (0, -speed, 0) inferred
        f.vel[id] = make_float4(0.0f, -e.speed, 0.0f, 0.0f);
        f.inv_mass[id] = inv_mass;
        f.radius[id] = e.radius;
        f.transferring[id] = 0u;
        f.target_radius[id] = e.radius;
        f.kernel_width[id] = __fmul_rn(e.radius, 4.0f);
        f.boundariness[id] = 1.0f;
        f.boundary_distance[id] = (uint32_t)__fmul_rn(e.radius, 262144.0f);
        f.lambda_prev[id] = 0.0f;
    }
}

__global__ void k_backup(FluidBufs f, const uint32_t *d_len) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        f.pos_backup[i] = f.pos[i];
}

__global__ void k_box_collision(int4 *pos, const float *radius, const uint32_t *d_len, const float4 *bmin,
                                const float4 *bmax, const float4 *rot, uint32_t nb) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += gridDim.x * blockDim.x)
        pos[id] = box_push(pos[id], radius[id], id, bmin, bmax, rot, nb);
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

apbf_status emit(apbf_ctx *ctx, float dt, cudaStream_t s) {
    const apbf_emitter &e = ctx->emitter;
    if (!e.enabled || dt <= 0.0f) return APBF_OK;
    FluidBufs &f = ctx->fl[ctx->fcur];
    APBF_BEFORE_LAUNCH(ctx, s, "k_emit_plan");
    k_emit_plan<<<1, 1, 0, s>>>(ctx->emit_state, ctx->d_len, ctx->status, e, (double)dt, ctx->cfg.particle_capacity);
    APBF_AFTER_LAUNCH(ctx, s, "k_emit_plan");
    const int32_t backup_dy = f2i_host(e.speed * ctx->last_dt * 262144.0f);
    APBF_BEFORE_LAUNCH(ctx, s, "k_emit");
    k_emit<<<grid_for(ctx, e.nx * e.nz * 4u), kBlock, 0, s>>>(f, ctx->emit_state, e, ctx->emit_inv_mass, backup_dy);
    APBF_AFTER_LAUNCH(ctx, s, "k_emit");
    return APBF_OK;
}

apbf_status box_collision(apbf_ctx *ctx, cudaStream_t s) {
    if (ctx->n_boxes == 0) return APBF_OK;
    FluidBufs &f = ctx->fl[ctx->fcur];
    APBF_BEFORE_LAUNCH(ctx, s, "k_box_collision");
    k_box_collision<<<grid_for(ctx, ctx->cfg.particle_capacity), kBlock, 0, s>>>(f.pos, f.radius, ctx->d_len,
                                                                                  ctx->box_min, ctx->box_max,
                                                                                  ctx->box_rot,
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
