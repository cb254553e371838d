// graph.cu -- the Jacobi passes of a substep as one graph launch.
//
// The reference records solverIterations (box collision + incompressibility)
// dispatches per substep (source/pool.cpp:92-95).  With a density-error target
// the number of passes a substep needs is only known on the device, so launching
// the maximum count from the host costs two kernel launches per skipped pass.
// Here passes 1.. of a substep are one CUDA graph: a while-conditional node whose
// body runs two passes (A -> B, B -> A, so the buffer roles are the same on every
// run) and a one-thread kernel that advances the device pass counter and keeps the
// loop going while no pass met the target and passes remain.  Passes past the
// last one inside a body run copy the positions through, as a converged pass does.
//
// Kernel arguments are captured by value, so a graph is specific to the buffer
// roles at capture time (current fluid set, current position buffer), the pass
// limit and the solve modes; up to four are cached per context and every change of
// settings or boxes drops them.
#include "apbf_internal.cuh"

namespace apbf {

namespace {

__global__ void k_loop_init(Status *st) { st->pass_index = 1u; }

__global__ void k_loop_next(cudaGraphConditionalHandle h, Status *st, uint32_t max_passes) {
    const uint32_t next = st->pass_index + 2u;
    st->pass_index = next;
    st->loop_iters += 1u;
    const uint32_t go = (*(volatile uint32_t *)&st->converged == 0u && next < max_passes) ? 1u : 0u;
    cudaGraphSetConditional(h, go);
}

void release(SolveGraph &g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
    g = SolveGraph();
}

}  // namespace

void destroy_solve_graphs(apbf_ctx *ctx) {
    for (auto &g : ctx->solve_graphs) release(g);
    ctx->solve_graph_next = 0;
}

static apbf_status build_solve_graph(apbf_ctx *ctx, const SolveOpts &o, SolveGraph &out) {
    if (!ctx->capture_stream) APBF_CUDA(cudaStreamCreateWithFlags(&ctx->capture_stream, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    APBF_CUDA(cudaGraphCreate(&g, 0));
    out.graph = g;
    cudaGraphConditionalHandle h;
    APBF_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault));
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    APBF_CUDA(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p));
    cudaGraph_t body = p.conditional.phGraph_out[0];

    // record the body's launches into it (nothing runs while capturing)
    cudaStream_t cs = ctx->capture_stream;
    APBF_CUDA(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    ctx->capturing = true;
    apbf_status r = APBF_OK;
    for (int k = 0; k < 2 && r == APBF_OK; ++k) {
        SolveOpts q = o;
        q.loop_offset = k;
        q.box_after = true;  // decided per pass on the device
        r = incompressibility(ctx, cs, q);
    }
    if (r == APBF_OK) {
        k_loop_next<<<1, 1, 0, cs>>>(h, ctx->status, o.max_passes);
        if (cudaGetLastError() != cudaSuccess) r = APBF_ERR_CUDA;
    }
    ctx->capturing = false;
    cudaGraph_t captured = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &captured);
    if (r != APBF_OK) return r;
    if (e != cudaSuccess) return cuda_check(e, "cudaStreamEndCapture (solve loop body)");
    size_t nodes = 0;
    APBF_CUDA(cudaGraphGetNodes(body, nullptr, &nodes));
    ctx->loop_launches_per_iter = nodes;
    APBF_CUDA(cudaGraphInstantiate(&out.exec, g, 0));
    return APBF_OK;
}

apbf_status solve_loop(apbf_ctx *ctx, cudaStream_t s, const SolveOpts &o) {
    const FluidBufs &f = ctx->fl[ctx->fcur];
    const unsigned long long key[4] = {
        ((unsigned long long)ctx->fcur << 32) | o.max_passes,
        (unsigned long long)(uintptr_t)f.pos,
        (unsigned long long)((o.converge ? 1 : 0) | (o.projected ? 2 : 0) | (o.prev_mode << 2)),
        ctx->graph_version};
    SolveGraph *hit = nullptr;
    for (auto &g : ctx->solve_graphs)
        if (g.exec && g.key[0] == key[0] && g.key[1] == key[1] && g.key[2] == key[2] && g.key[3] == key[3]) hit = &g;
    if (!hit) {
        SolveGraph &slot = ctx->solve_graphs[ctx->solve_graph_next];
        ctx->solve_graph_next = (ctx->solve_graph_next + 1) % kSolveGraphs;
        release(slot);
        int4 *pos_before = ctx->fl[ctx->fcur].pos;
        apbf_status r = build_solve_graph(ctx, o, slot);
        if (r != APBF_OK) {
            release(slot);
            return r;
        }
        if (ctx->fl[ctx->fcur].pos != pos_before) {  // two captured passes swap the buffers twice
            release(slot);
            set_error("solve loop: buffer roles changed during capture");
            return APBF_ERR_CUDA;
        }
        for (int k = 0; k < 4; ++k) slot.key[k] = key[k];
        hit = &slot;
    }
    APBF_BEFORE_LAUNCH(ctx, s, "k_loop_init");
    k_loop_init<<<1, 1, 0, s>>>(ctx->status);
    APBF_AFTER_LAUNCH(ctx, s, "k_loop_init");
    APBF_CUDA(cudaGraphLaunch(hit->exec, s));
    return APBF_OK;
}

}  // namespace apbf
