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
    const uint32_t db = t->sort_digit_bits;
    if ((l != 1 && l != 2 && l != 4 && l != 8) || (t->pass_block != 128 && t->pass_block != 256) ||
        t->pass_blocks_per_sm < 1 || t->pass_blocks_per_sm > 8 || t->reserved0 != 0 ||
        (db != 0 && (db < 6 || db > 8)) || t->search_log2res > ctx->cfg.max_log2res) {
        set_error("apbf_set_tuning: gather_lanes 1, 2, 4 or 8; pass_block 128 or 256; pass_blocks_per_sm 1..8; "
                  "reserved0 0; sort_digit_bits 0, 6, 7 or 8; search_log2res 0..max_log2res");
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

// ---- the neighbour search: sort digit width and search grid ----

namespace apbf {
namespace {

struct EventTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    EventTimer() {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~EventTimer() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    float ms(cudaStream_t s) {
        cudaEventSynchronize(b);
        float t = 0.0f;
        cudaEventElapsedTime(&t, a, b);
        return t;
    }
};

}  // namespace
}  // namespace apbf

// Times the radix sort of the search on the keys of the current particle order for
// 6-, 7- and 8-bit digits (the same order each), then the whole neighbour search of
// apbf_substep on grids of 2^(L-1), 2^L and 2^(L+1) cells per axis (within
// max_log2res; the same neighbour sets) with the chosen sort, keeps the fastest of
// each and restores the particle state, the transfer list, the status block and the
// buffer roles after every search it ran.  The search's rows and cell ranges are
// left from the last candidate: the next substep searches anew.
extern "C" apbf_status apbf_autotune_search(apbf_ctx *ctx, void *stream, apbf_tuning *chosen, float *ms) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    if (ctx->scene.log2res < 1) {
        set_error("apbf_autotune_search: call apbf_set_scene first");
        return APBF_ERR_INVALID_ARG;
    }
    if (ctx->glue_cap) {
        set_error("apbf_autotune_search: not with a glue list (the search remaps it)");
        return APBF_ERR_INVALID_ARG;
    }
    cudaSetDevice(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t cap = ctx->cfg.particle_capacity, tcap = ctx->cfg.transfer_capacity;
    const apbf_tuning before = ctx->tuning;
    const uint32_t L0 = before.search_log2res ? before.search_log2res : ctx->scene.log2res;
    const HostState hs = host_state(ctx);
    uint32_t *tmp_k = nullptr, *tmp_v = nullptr, *tr_save = nullptr;
    Status *st_save = nullptr;
    if (cudaMalloc(&tmp_k, cap * 4) != cudaSuccess || cudaMalloc(&tmp_v, cap * 4) != cudaSuccess ||
        cudaMalloc(&tr_save, (size_t)tcap * 8) != cudaSuccess || cudaMalloc(&st_save, sizeof(Status)) != cudaSuccess) {
        cudaFree(tmp_k);
        cudaFree(tmp_v);
        cudaFree(tr_save);
        cudaFree(st_save);
        set_error("apbf_autotune_search: out of device memory for the snapshot");
        return APBF_ERR_CUDA;
    }
    const TransferBufs &tr = ctx->tr[ctx->tcur];
    cudaMemcpyAsync(tr_save, tr.source, (size_t)tcap * 4, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(tr_save + tcap, tr.target, (size_t)tcap * 4, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(st_save, ctx->status, sizeof(Status), cudaMemcpyDeviceToDevice, s);
    const bool prof = ctx->prof_on;
    ctx->prof_on = false;
    apbf_status r = APBF_OK;
    float t_sort[3] = {0.f, 0.f, 0.f}, t_grid[3] = {0.f, 0.f, 0.f};
    EventTimer ev;
    // (1) digit width
    uint32_t best_bits = 8u;
    for (int c = 0; c < 3 && r == APBF_OK; ++c) {
        ctx->tuning.sort_digit_bits = 6u + (uint32_t)c;
        r = sort_pairs_device(ctx, ctx->sorted_keys, ctx->perm, ctx->d_len + kLenParticles, cap, 3u * L0, tmp_k, tmp_v,
                              s);  // warm-up
        cudaEventRecord(ev.a, s);
        for (int k = 0; k < 4 && r == APBF_OK; ++k)
            r = sort_pairs_device(ctx, ctx->sorted_keys, ctx->perm, ctx->d_len + kLenParticles, cap, 3u * L0, tmp_k,
                                  tmp_v, s);
        cudaEventRecord(ev.b, s);
        t_sort[c] = ev.ms(s) / 4.0f;
        if (r == APBF_OK && t_sort[c] < t_sort[best_bits - 6u]) best_bits = 6u + (uint32_t)c;
    }
    // (2) search grid
    const apbf_settings &st = ctx->settings;
    const float scale = (st.basic_pbf || st.base_kernel_width_on_boundary_distance) ? 1.0f : 1.5f;
    const bool spread = !st.basic_pbf && !st.base_kernel_width_on_boundary_distance;  // as apbf_substep searches
    uint32_t best_L = L0;
    float best_t = 0.0f;
    ctx->tuning.sort_digit_bits = best_bits;
    for (int c = 0; c < 3 && r == APBF_OK; ++c) {
        const int L = (int)L0 - 1 + c;
        if (L < 1 || L > (int)ctx->cfg.max_log2res) continue;
        float tot = 0.0f;
        for (int k = 0; k < 3 && r == APBF_OK; ++k) {  // one warm-up, two timed
            cudaEventRecord(ev.a, s);
            r = neighborhood_green(ctx, scale, ctx->scene.min_pos, ctx->scene.max_pos, (uint32_t)L, s, false, !spread);
            cudaEventRecord(ev.b, s);
            const float t = ev.ms(s);
            if (k > 0) tot += t;
            // the state as before: buffer roles, transfer list, status
            set_host_state(ctx, hs);
            cudaMemcpyAsync(tr.source, tr_save, (size_t)tcap * 4, cudaMemcpyDeviceToDevice, s);
            cudaMemcpyAsync(tr.target, tr_save + tcap, (size_t)tcap * 4, cudaMemcpyDeviceToDevice, s);
            cudaMemcpyAsync(ctx->status, st_save, sizeof(Status), cudaMemcpyDeviceToDevice, s);
        }
        t_grid[c] = tot / 2.0f;
        if (r == APBF_OK && (best_t == 0.0f || t_grid[c] < best_t)) {
            best_t = t_grid[c];
            best_L = (uint32_t)L;
        }
    }
    cudaStreamSynchronize(s);
    cudaFree(tmp_k);
    cudaFree(tmp_v);
    cudaFree(tr_save);
    cudaFree(st_save);
    ctx->prof_on = prof;
    ctx->tuning = before;
    if (r != APBF_OK) return r;
    ctx->tuning.sort_digit_bits = best_bits;
    ctx->tuning.search_log2res = best_L == ctx->scene.log2res ? 0u : best_L;
    ctx->graph_version++;
    if (chosen) *chosen = ctx->tuning;
    if (ms) {
        for (int c = 0; c < 3; ++c) ms[c] = t_sort[c];
        for (int c = 0; c < 3; ++c) ms[3 + c] = t_grid[c];
    }
    return APBF_OK;
}
