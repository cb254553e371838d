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
#include <vector>

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

// Records the loop body (two passes + the loop-condition kernel) into `body` on
// stream cs (which must not be capturing anything else).
static apbf_status capture_loop_body(apbf_ctx *ctx, cudaStream_t cs, cudaGraph_t body, cudaGraphConditionalHandle h,
                                     const SolveOpts &o) {
    APBF_CUDA(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    const bool was = ctx->capturing;
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
    ctx->capturing = was;
    cudaGraph_t captured = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &captured);
    if (r != APBF_OK) return r;
    if (e != cudaSuccess) return cuda_check(e, "cudaStreamEndCapture (solve loop body)");
    size_t nodes = 0;
    APBF_CUDA(cudaGraphGetNodes(body, nullptr, &nodes));
    ctx->loop_launches_per_iter = nodes;
    return APBF_OK;
}

// Adds a while-conditional node (default: enter) to graph g after deps; returns
// the node, its handle and its body graph.
static apbf_status add_loop_node(cudaGraph_t g, const cudaGraphNode_t *deps, const cudaGraphEdgeData *edges,
                                 size_t ndeps, cudaGraphNode_t *node, cudaGraphConditionalHandle *h,
                                 cudaGraph_t *body) {
    APBF_CUDA(cudaGraphConditionalHandleCreate(h, g, 1u, cudaGraphCondAssignDefault));
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = *h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    APBF_CUDA(cudaGraphAddNode(node, g, deps, edges, ndeps, &p));
    *body = p.conditional.phGraph_out[0];
    return APBF_OK;
}

static apbf_status ensure_streams(apbf_ctx *ctx) {
    if (!ctx->capture_stream) APBF_CUDA(cudaStreamCreateWithFlags(&ctx->capture_stream, cudaStreamNonBlocking));
    if (!ctx->capture_stream2) APBF_CUDA(cudaStreamCreateWithFlags(&ctx->capture_stream2, cudaStreamNonBlocking));
    return APBF_OK;
}

static apbf_status build_solve_graph(apbf_ctx *ctx, const SolveOpts &o, SolveGraph &out) {
    apbf_status r = ensure_streams(ctx);
    if (r != APBF_OK) return r;
    APBF_CUDA(cudaGraphCreate(&out.graph, 0));
    cudaGraphNode_t node;
    cudaGraphConditionalHandle h;
    cudaGraph_t body;
    r = add_loop_node(out.graph, nullptr, nullptr, 0, &node, &h, &body);
    if (r != APBF_OK) return r;
    r = capture_loop_body(ctx, ctx->capture_stream, body, h, o);
    if (r != APBF_OK) return r;
    APBF_CUDA(cudaGraphInstantiate(&out.exec, out.graph, 0));
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

apbf_status solve_loop_captured(apbf_ctx *ctx, cudaStream_t s, const SolveOpts &o) {
    apbf_status r = ensure_streams(ctx);
    if (r != APBF_OK) return r;
    k_loop_init<<<1, 1, 0, s>>>(ctx->status);
    APBF_CUDA(cudaGetLastError());
    cudaStreamCaptureStatus cst;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edges = nullptr;
    size_t nd = 0;
    APBF_CUDA(cudaStreamGetCaptureInfo(s, &cst, nullptr, &g, &deps, &edges, &nd));
    if (cst != cudaStreamCaptureStatusActive) {
        set_error("solve loop: stream is not capturing");
        return APBF_ERR_CUDA;
    }
    cudaGraphNode_t node;
    cudaGraphConditionalHandle h;
    cudaGraph_t body;
    r = add_loop_node(g, deps, edges, nd, &node, &h, &body);
    if (r != APBF_OK) return r;
    int4 *pos_before = ctx->fl[ctx->fcur].pos;
    r = capture_loop_body(ctx, ctx->capture_stream2, body, h, o);
    if (r != APBF_OK) return r;
    if (ctx->fl[ctx->fcur].pos != pos_before) {
        set_error("solve loop: buffer roles changed during capture");
        return APBF_ERR_CUDA;
    }
    APBF_CUDA(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    return APBF_OK;
}

// ---- whole substeps ------------------------------------------------------------

// Everything a substep changes on the host: the roles of the double-buffered
// lists (current set, swapped position and boundary-distance arrays) and last_dt.
HostState host_state(const apbf_ctx *ctx) {
    HostState h;
    std::memcpy(h.fl, ctx->fl, sizeof(h.fl));
    std::memcpy(h.tr, ctx->tr, sizeof(h.tr));
    h.old_bd = ctx->old_bd;
    h.fcur = ctx->fcur;
    h.tcur = ctx->tcur;
    h.last_dt = ctx->last_dt;
    return h;
}

void set_host_state(apbf_ctx *ctx, const HostState &h) {
    std::memcpy(ctx->fl, h.fl, sizeof(h.fl));
    std::memcpy(ctx->tr, h.tr, sizeof(h.tr));
    ctx->old_bd = h.old_bd;
    ctx->fcur = h.fcur;
    ctx->tcur = h.tcur;
    ctx->last_dt = h.last_dt;
}

unsigned long long substep_mode_bits(const apbf_ctx *ctx) {
    return (unsigned long long)ctx->warm_start | ((unsigned long long)ctx->track_lambda << 8) |
           ((unsigned long long)ctx->mlp_loaded << 9);
}

static unsigned long long count_kernel_nodes(cudaGraph_t g) {
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return 0;
    std::vector<cudaGraphNode_t> nodes(n);
    if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return 0;
    unsigned long long k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

static void release(SubstepGraph &g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
    g = SubstepGraph();
}

void destroy_substep_graphs(apbf_ctx *ctx) {
    for (auto &g : ctx->substep_graphs) release(g);
    ctx->substep_graph_next = 0;
}

apbf_status substep_graph(apbf_ctx *ctx, float dt, cudaStream_t s) {
    const HostState before = host_state(ctx);
    const unsigned long long mode = substep_mode_bits(ctx);
    for (auto &g : ctx->substep_graphs) {
        if (g.exec && g.before == before && g.dt == dt && g.version == ctx->graph_version && g.mode == mode) {
            APBF_CUDA(cudaGraphLaunch(g.exec, s));
            set_host_state(ctx, g.after);
            ctx->launches += g.kernels;
            return APBF_OK;
        }
    }
    apbf_status r = ensure_streams(ctx);
    if (r != APBF_OK) return r;
    SubstepGraph &slot = ctx->substep_graphs[ctx->substep_graph_next];
    ctx->substep_graph_next = (ctx->substep_graph_next + 1) % kSubstepGraphs;
    release(slot);
    cudaStream_t cs = ctx->capture_stream;
    APBF_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
    ctx->capturing = true;
    r = substep_body(ctx, dt, cs, true);
    ctx->capturing = false;
    cudaError_t e = cudaStreamEndCapture(cs, &slot.graph);
    if (r == APBF_OK && e != cudaSuccess) r = cuda_check(e, "cudaStreamEndCapture (substep)");
    if (r == APBF_OK && cudaGraphInstantiate(&slot.exec, slot.graph, 0) != cudaSuccess)
        r = cuda_check(cudaGetLastError(), "cudaGraphInstantiate (substep)");
    if (r != APBF_OK) {
        release(slot);
        set_host_state(ctx, before);  // nothing ran
        return r;
    }
    slot.before = before;
    slot.after = host_state(ctx);
    slot.dt = dt;
    slot.version = ctx->graph_version;
    slot.mode = mode;
    slot.kernels = count_kernel_nodes(slot.graph);
    APBF_CUDA(cudaGraphLaunch(slot.exec, s));
    ctx->launches += slot.kernels;
    return APBF_OK;
}

}  // namespace apbf

// ---- batches of contexts: one graph whose parallel branches are their substeps ----

using namespace apbf;

struct apbf_batch {
    std::vector<apbf_ctx *> ctx;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    // batched solve: the scenes' passes 1.. in one persistent cooperative launch
    int persistent = 0;  // apbf_batch_set_persistent_solve
    int coop_grid = 0;                   // resident grid of that kernel (0: not available)
    void *d_table = nullptr;             // device table of the scenes (one entry per context)
    void *d_sync = nullptr;              // its grid barrier
    unsigned long long *d_acc = nullptr; // the scenes' error sums
    cudaEvent_t solved = nullptr;
    std::vector<cudaEvent_t> pre;
    struct Entry {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        std::vector<HostState> before, after;
        std::vector<unsigned long long> version, mode, kernels;
        float dt = 0.0f;
        void *h_table = nullptr;  // pinned host copy of the scene table this graph uploads
    };
    Entry cache[kSubstepGraphs];
    int next = 0;
};

static void release(apbf_batch::Entry &e) {
    if (e.exec) cudaGraphExecDestroy(e.exec);
    if (e.graph) cudaGraphDestroy(e.graph);
    if (e.h_table) cudaFreeHost(e.h_table);
    e = apbf_batch::Entry();
}

extern "C" apbf_status apbf_batch_create(apbf_ctx *const *ctxs, uint32_t n, apbf_batch **out) {
    if (!ctxs || !n || !out) return APBF_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n; ++i) {
        if (!ctxs[i] || ctxs[i]->device != ctxs[0]->device) {
            set_error("apbf_batch_create: null context or contexts on different devices");
            return APBF_ERR_INVALID_ARG;
        }
        for (uint32_t j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) {
                set_error("apbf_batch_create: a context appears twice");
                return APBF_ERR_INVALID_ARG;
            }
    }
    cudaSetDevice(ctxs[0]->device);
    apbf_batch *b = new apbf_batch();
    b->ctx.assign(ctxs, ctxs + n);
    b->join.resize(n, nullptr);
    b->pre.resize(n, nullptr);
    bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->solved, cudaEventDisableTiming) == cudaSuccess;
    for (uint32_t i = 0; ok && i < n; ++i)
        ok = cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->pre[i], cudaEventDisableTiming) == cudaSuccess &&
             ensure_streams(ctxs[i]) == APBF_OK;
    if (ok && n <= batch_max_scenes()) {
        b->coop_grid = solve_batch_blocks(ctxs[0]->device, ctxs[0]->num_sms);
        if (b->coop_grid > 0)
            ok = cudaMalloc(&b->d_table, (size_t)n * batch_scene_bytes()) == cudaSuccess &&
                 cudaMalloc(&b->d_sync, batch_sync_bytes()) == cudaSuccess &&
                 cudaMalloc((void **)&b->d_acc, (size_t)2 * n * sizeof(unsigned long long)) == cudaSuccess;
    }
    if (!ok) {
        apbf_batch_destroy(b);
        set_error("apbf_batch_create: stream or event creation failed");
        return APBF_ERR_CUDA;
    }
    *out = b;
    return APBF_OK;
}

extern "C" apbf_status apbf_batch_destroy(apbf_batch *b) {
    if (!b) return APBF_ERR_INVALID_ARG;
    for (auto &e : b->cache) release(e);
    for (auto ev : b->join)
        if (ev) cudaEventDestroy(ev);
    for (auto ev : b->pre)
        if (ev) cudaEventDestroy(ev);
    if (b->solved) cudaEventDestroy(b->solved);
    if (b->d_table) cudaFree(b->d_table);
    if (b->d_sync) cudaFree(b->d_sync);
    if (b->d_acc) cudaFree(b->d_acc);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return APBF_OK;
}

extern "C" apbf_status apbf_batch_set_persistent_solve(apbf_batch *b, int enable) {
    if (!b) return APBF_ERR_INVALID_ARG;
    b->persistent = enable ? 1 : 0;
    for (auto &e : b->cache) release(e);
    return APBF_OK;
}

extern "C" apbf_status apbf_batch_substep(apbf_batch *b, float dt, void *stream) {
    if (!b) return APBF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = b->ctx.size();
    bool graphable = true;
    for (auto *c : b->ctx) {
        if (c->scene.log2res < 1) {
            set_error("apbf_batch_substep: call apbf_set_scene on every context first");
            return APBF_ERR_INVALID_ARG;
        }
        graphable = graphable && !c->prof_on && !c->debug && c->rec_iterations == 0 &&
                    c->settings.solver_iterations >= 2 && c->use_graphs >= 1;
    }
    if (!graphable) {  // tracing, debugging or recording: one context after the other
        for (auto *c : b->ctx) {
            apbf_status r = apbf_substep(c, dt, stream);
            if (r != APBF_OK) return r;
        }
        return APBF_OK;
    }
    std::vector<HostState> before(n);
    std::vector<unsigned long long> version(n), mode(n);
    for (size_t i = 0; i < n; ++i) {
        before[i] = host_state(b->ctx[i]);
        version[i] = b->ctx[i]->graph_version;
        mode[i] = substep_mode_bits(b->ctx[i]);
    }
    for (auto &e : b->cache) {
        if (e.exec && e.dt == dt && e.before == before && e.version == version && e.mode == mode) {
            APBF_CUDA(cudaGraphLaunch(e.exec, s));
            for (size_t i = 0; i < n; ++i) {
                set_host_state(b->ctx[i], e.after[i]);
                b->ctx[i]->launches += e.kernels[i];
            }
            return APBF_OK;
        }
    }
    apbf_batch::Entry &e = b->cache[b->next];
    b->next = (b->next + 1) % kSubstepGraphs;
    release(e);
    const bool batched = b->persistent && b->coop_grid > 0;
    if (batched) APBF_CUDA(cudaMallocHost(&e.h_table, n * batch_scene_bytes()));  // before the capture
    apbf_status r = APBF_OK;
    APBF_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed));
    APBF_CUDA(cudaEventRecord(b->fork, b->stream));
    e.kernels.assign(n, 0);
    // Each context's substep up to its first Jacobi pass as a parallel branch; passes
    // 1.. of every context that qualifies in one batched persistent launch; then the
    // rest of each substep as a branch again.  Contexts that do not qualify run their
    // whole substep in their branch.
    std::vector<SolveOpts> opts(n);
    std::vector<uint8_t> deferred(n, 0);
    for (size_t i = 0; i < n && r == APBF_OK; ++i) {
        apbf_ctx *c = b->ctx[i];
        cudaStream_t cs = c->capture_stream;
        if (cudaStreamWaitEvent(cs, b->fork, 0) != cudaSuccess) {
            r = APBF_ERR_CUDA;
            break;
        }
        c->capturing = true;
        c->in_batch = true;  // parallel branches: no persistent solve of their own
        bool d = false;
        r = substep_body(c, dt, cs, true, batched ? &opts[i] : nullptr, &d);
        c->in_batch = false;
        deferred[i] = d ? 1 : 0;
        if (!d) c->capturing = false;
        cudaEvent_t ev = d ? b->pre[i] : b->join[i];
        if (r == APBF_OK &&
            (cudaEventRecord(ev, cs) != cudaSuccess || cudaStreamWaitEvent(b->stream, ev, 0) != cudaSuccess))
            r = APBF_ERR_CUDA;
    }
    uint32_t m = 0;
    for (size_t i = 0; i < n && r == APBF_OK; ++i)
        if (deferred[i])
            batch_scene_fill(b->ctx[i], opts[i], static_cast<char *>(e.h_table) + (size_t)m++ * batch_scene_bytes());
    if (r == APBF_OK && m > 0) {
        if (cudaMemcpyAsync(b->d_table, e.h_table, (size_t)m * batch_scene_bytes(), cudaMemcpyHostToDevice,
                            b->stream) != cudaSuccess)
            r = APBF_ERR_CUDA;
        if (r == APBF_OK) r = solve_batch_launch(b->d_table, m, b->d_sync, b->d_acc, b->coop_grid, b->stream);
        if (r == APBF_OK && cudaEventRecord(b->solved, b->stream) != cudaSuccess) r = APBF_ERR_CUDA;
        for (size_t i = 0; i < n && r == APBF_OK; ++i) {
            if (!deferred[i]) continue;
            apbf_ctx *c = b->ctx[i];
            cudaStream_t cs = c->capture_stream;
            if (cudaStreamWaitEvent(cs, b->solved, 0) != cudaSuccess) {
                r = APBF_ERR_CUDA;
                break;
            }
            r = substep_post(c, cs);
            c->capturing = false;
            if (r == APBF_OK && (cudaEventRecord(b->join[i], cs) != cudaSuccess ||
                                 cudaStreamWaitEvent(b->stream, b->join[i], 0) != cudaSuccess))
                r = APBF_ERR_CUDA;
        }
    }
    for (auto *c : b->ctx) c->capturing = false;
    cudaError_t ce = cudaStreamEndCapture(b->stream, &e.graph);
    if (r == APBF_OK && ce != cudaSuccess) r = cuda_check(ce, "cudaStreamEndCapture (batch)");
    if (r == APBF_OK && cudaGraphInstantiate(&e.exec, e.graph, 0) != cudaSuccess)
        r = cuda_check(cudaGetLastError(), "cudaGraphInstantiate (batch)");
    if (r != APBF_OK) {
        release(e);
        for (size_t i = 0; i < n; ++i) set_host_state(b->ctx[i], before[i]);
        if (r == APBF_ERR_CUDA) set_error("apbf_batch_substep: capture failed");
        return r;
    }
    e.before = before;
    e.after.resize(n);
    for (size_t i = 0; i < n; ++i) e.after[i] = host_state(b->ctx[i]);
    e.version = version;
    e.mode = mode;
    e.dt = dt;
    // kernel nodes per context: counted on the whole graph, shared out evenly for the
    // launch counters (the branches have the same stage sequence)
    const unsigned long long total = count_kernel_nodes(e.graph);
    for (size_t i = 0; i < n; ++i) e.kernels[i] = total / n;
    APBF_CUDA(cudaGraphLaunch(e.exec, s));
    for (size_t i = 0; i < n; ++i) b->ctx[i]->launches += e.kernels[i];
    return APBF_OK;
}
