// tune.cu -- launch-shape tuning of a context on its current particle state.
//
// The reference fixes its workgroup sizes in the shaders; here the number of
// threads per particle of the two gather passes of the Jacobi solve (density +
// lambda, position update) is picked by timing each candidate on the context's
// own neighbour rows, so the choice follows the scene's neighbour counts.  The
// particle state is saved before and restored after, so tuning leaves the
// simulation unchanged; the results of the passes do not depend on the choice.
#include "apbf_internal.cuh"

namespace apbf {

static apbf_status time_shape(apbf_ctx *ctx, cudaStream_t s, const apbf_tuning &t, int reps, float *ms_out) {
    ctx->tuning = t;
    SolveOpts o;  // plain pass: no early stop, no features, no lambda bookkeeping
    for (int k = 0; k < 2; ++k) {  // warm-up (one pair keeps the buffer roles)
        apbf_status r = incompressibility(ctx, s, o);
        if (r != APBF_OK) return r;
    }
    cudaEvent_t a, b;
    APBF_CUDA(cudaEventCreate(&a));
    APBF_CUDA(cudaEventCreate(&b));
    APBF_CUDA(cudaEventRecord(a, s));
    for (int k = 0; k < 2 * reps; ++k) {
        apbf_status r = incompressibility(ctx, s, o);
        if (r != APBF_OK) return r;
    }
    APBF_CUDA(cudaEventRecord(b, s));
    APBF_CUDA(cudaEventSynchronize(b));
    float ms = 0.0f;
    APBF_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms_out = ms / (2.0f * reps);
    return APBF_OK;
}

}  // namespace apbf

using namespace apbf;

extern "C" apbf_status apbf_set_tuning(apbf_ctx *ctx, const apbf_tuning *t) {
    if (!ctx || !t) return APBF_ERR_INVALID_ARG;
    const uint32_t l = t->gather_lanes;
    if ((l != 1 && l != 2 && l != 4 && l != 8) || (t->pass_block != 128 && t->pass_block != 256) ||
        t->pass_blocks_per_sm < 1 || t->pass_blocks_per_sm > 8 || t->build_tiled > 2) {
        set_error("apbf_set_tuning: gather_lanes 1, 2, 4 or 8; pass_block 128 or 256; pass_blocks_per_sm 1..8; "
                  "build_tiled 0, 1 or 2");
        return APBF_ERR_INVALID_ARG;
    }
    ctx->tuning = *t;
    ctx->graph_version++;
    return APBF_OK;
}

extern "C" apbf_status apbf_get_tuning(apbf_ctx *ctx, apbf_tuning *t) {
    if (!ctx || !t) return APBF_ERR_INVALID_ARG;
    *t = ctx->tuning;
    return APBF_OK;
}

extern "C" apbf_status apbf_autotune(apbf_ctx *ctx, void *stream, apbf_tuning *chosen, float *pass_ms) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t cap = ctx->cfg.particle_capacity;
    FluidBufs &f = ctx->fl[ctx->fcur];
    // save what the passes change: positions, boundariness, the status block
    int4 *pos_save = nullptr;
    float *b_save = nullptr;
    Status *st_save = nullptr;
    apbf_status r = APBF_OK;
    if (cudaMalloc(&pos_save, cap * sizeof(int4)) != cudaSuccess || cudaMalloc(&b_save, cap * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&st_save, sizeof(Status)) != cudaSuccess) {
        cudaFree(pos_save);
        cudaFree(b_save);
        cudaFree(st_save);
        set_error("apbf_autotune: out of device memory for the state snapshot");
        return APBF_ERR_CUDA;
    }
    int4 *pos_cur = f.pos;
    cudaMemcpyAsync(pos_save, pos_cur, cap * sizeof(int4), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(b_save, f.boundariness, cap * sizeof(float), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(st_save, ctx->status, sizeof(Status), cudaMemcpyDeviceToDevice, s);
    const bool prof = ctx->prof_on;
    ctx->prof_on = false;
    const apbf_tuning before = ctx->tuning;
    const int lanes[4] = {1, 2, 4, 8}, blocks[2] = {128, 256}, per_sm[3] = {2, 4, 8};
    constexpr int kCands = 24;
    float best_ms = 0.0f, times[kCands] = {};
    apbf_tuning best_t = before;
    int best = -1;
    for (int c = 0; c < kCands && r == APBF_OK; ++c) {
        apbf_tuning t = before;
        t.gather_lanes = (uint32_t)lanes[c / 6];
        t.pass_block = (uint32_t)blocks[(c / 3) % 2];
        t.pass_blocks_per_sm = (uint32_t)per_sm[c % 3];
        r = time_shape(ctx, s, t, 4, &times[c]);
        // restore the positions after every candidate (pairs of passes keep the roles)
        if (f.pos != pos_cur) r = r == APBF_OK ? APBF_ERR_CUDA : r;
        cudaMemcpyAsync(pos_cur, pos_save, cap * sizeof(int4), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(f.boundariness, b_save, cap * sizeof(float), cudaMemcpyDeviceToDevice, s);
        if (r == APBF_OK && (best < 0 || times[c] < best_ms)) {
            best = c;
            best_ms = times[c];
            best_t = t;
        }
    }
    cudaMemcpyAsync(ctx->status, st_save, sizeof(Status), cudaMemcpyDeviceToDevice, s);
    cudaStreamSynchronize(s);
    cudaFree(pos_save);
    cudaFree(b_save);
    cudaFree(st_save);
    ctx->prof_on = prof;
    if (r != APBF_OK) {
        ctx->tuning = before;
        return r;
    }
    ctx->tuning = best_t;
    ctx->graph_version++;
    if (chosen) *chosen = ctx->tuning;
    if (pass_ms)
        for (int c = 0; c < kCands; ++c) pass_ms[c] = times[c];
    return APBF_OK;
}
