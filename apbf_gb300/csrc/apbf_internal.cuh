// apbf_internal.cuh -- context layout and device helpers shared by the CUDA sources.
//
// Data layout in HBM (structure of arrays, one entry per particle, particle order
// = Morton cell order after every neighbourhood search):
//   position / pos_backup  int4   (x, y, z, pad) in 2^18 fixed point
//   velocity               float4
//   inverse_mass, radius, target_radius, kernel_width, boundariness   float
//   transferring, boundary_distance                                   uint32
// Two complete attribute sets exist (cur / alt); a reorder gathers cur -> alt and
// swaps, the Jacobi position update ping-pongs the position buffers.
// Neighbour rows are column-major: index[k * row_stride + i] (k < count[i]), so a
// warp of consecutive particles reads one 128-byte line per k.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>
#include <string>
#include <vector>

#include "../../include/apbf_gb300.h"

#define APBF_FIX 262144.0f
#define APBF_INV_FIX (1.0f / 262144.0f)

namespace apbf {

constexpr int kBlock = 256;
// Correction-row entry flag (neighborhood.cu): the entry is in the row owner's own
// neighbour row but the entry's radius does not reach the owner, so the position
// update subtracts its term again; the entry's index is the low 31 bits.
constexpr uint32_t kNoDelta = 0x80000000u;
constexpr uint32_t kSpinLimit = 1u << 22;  // bounded device-side waits

struct FluidBufs {
    int4 *pos;
    float4 *vel;
    float *inv_mass;
    float *radius;
    int4 *pos_backup;
    uint32_t *transferring;
    float *target_radius;
    float *kernel_width;
    float *boundariness;
    uint32_t *boundary_distance;
    float *lambda_prev;  // sum of the lambdas applied in the particle's last substep (warm-start feature)
};

struct TransferBufs {
    uint32_t *source;
    uint32_t *target;
    float *time_left;
};

// Device status block (one allocation, zeroed by apbf_get_status(clear=1)).
struct Status {
    uint32_t flags;
    uint32_t required_neighbors;
    uint32_t required_transfers;
    uint32_t required_particles;
    unsigned long long range_min;  // smallest fixed-point search radius of the last search
    unsigned long long range_max;
    uint32_t symmetric;            // 1 if every search radius was equal (rows are symmetric)
    uint32_t spin_where;
    uint32_t density_passes;       // density passes executed (not skipped after convergence)
    uint32_t converged;            // set by a density pass whose error met the target
    uint32_t done_blocks;          // last-block counter of the density pass reduction
    uint32_t converged_substeps;   // substeps in which a density pass met the target
    uint32_t pass_index;           // solve loop graph: index of the first pass of the current body run
    uint32_t loop_iters;           // solve loop graph: body runs since the context was created
    uint32_t filter_tag;           // 1: this pass's density kernel left the boundariness filter to k_delta
    uint32_t union_rows;           // 1: the reverse-row arrays hold correction rows (see neighborhood.cu)
    uint32_t wait_limit;           // spins of a bounded device wait before it gives up (0: the wait's default);
                                   // bit 31: the waits treat their awaited flag as never set (failure tests)
    uint32_t kw_uniform;           // 1: every kernel width of this density pass had the same bits
    uint32_t bar_arrive;           // persistent solve: blocks arrived at the current grid barrier
    uint32_t bar_gen;              // persistent solve: grid barriers released so far
    unsigned long long loop_e1;    // persistent solve: error sums of the current pass (2^-24 fixed point)
    unsigned long long loop_e2;
};

// Device length block.
enum LenSlot : uint32_t {
    kLenParticles = 0,
    kLenTransfers = 1,
    kLenSplits = 2,
    kLenDelParticles = 3,
    kLenDelTransfers = 4,
    kLenMerges = 5,
    kLenScratch = 6,
    kLenSlots = 16
};

// Per-particle Gauss-kernel constants computed once per density pass and reused
// by the position-update pass (so both evaluate bit-identical gradients).
struct KConst {
    float ivd;   // -invDoubleVariance * log2(e) (kernels.glsl:87), the exponent scale of exp2
    float norm;  // pow(invDoubleVarianceWithoutPi, D/2) (kernels.glsl:88)
};

struct Ctx;

// Sort scratch sizes.
constexpr int kSortItems = 16;
constexpr int kSortWarps = 8;
constexpr int kSortTile = kSortItems * 32 * kSortWarps;  // 4096 keys per tile

}  // namespace apbf

namespace apbf {
// One timed kernel launch: CUDA events recorded on the launching stream.
struct ProfSlot {
    const char *name;
    cudaEvent_t a, b;
};

// One instantiated solve loop (graph.cu): a while-conditional graph node whose
// body runs two Jacobi passes and decides on the device whether to go on.
struct SolveGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long key[4] = {0, 0, 0, 0};
};
constexpr int kSolveGraphs = 4;

// Host-side roles of the context's buffers; a substep moves them from one value to
// the next, and a captured substep graph is valid for one starting value.
struct HostState {
    FluidBufs fl[2];
    TransferBufs tr[2];
    uint32_t *old_bd = nullptr;
    int fcur = 0, tcur = 0;
    float last_dt = 0.0f;
    bool operator==(const HostState &o) const {
        return std::memcmp(fl, o.fl, sizeof(fl)) == 0 && std::memcmp(tr, o.tr, sizeof(tr)) == 0 &&
               old_bd == o.old_bd && fcur == o.fcur && tcur == o.tcur && last_dt == o.last_dt;
    }
};

// One instantiated whole-substep graph (graph.cu).
struct SubstepGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    HostState before, after;
    float dt = 0.0f;
    unsigned long long version = 0, mode = 0;
    unsigned long long kernels = 0;  // kernel nodes outside the solve loop body
};
constexpr int kSubstepGraphs = 8;  // the buffer roles of an adaptive scene cycle with a period of up to 6
}  // namespace apbf

struct apbf_ctx {
    apbf_config cfg;
    apbf_settings settings;
    apbf_scene scene;
    int device = 0;
    int num_sms = 152;
    float last_dt = 1.0f;  // velocity_handling.h:17
    uint32_t row_stride = 0;

    apbf::FluidBufs fl[2];
    apbf::TransferBufs tr[2];
    int fcur = 0;
    int tcur = 0;
    uint32_t *d_len = nullptr;

    uint32_t *nb_count = nullptr;
    uint32_t *nb_idx = nullptr;
    uint32_t *rev_count = nullptr;
    uint32_t *rev_idx = nullptr;
    unsigned long long *d_pairs = nullptr;

    uint32_t *keys[2] = {nullptr, nullptr};
    uint32_t *vals[2] = {nullptr, nullptr};
    uint32_t *sort_hist = nullptr;         // 4 passes x 256
    uint32_t *sort_status = nullptr;       // tiles x 256
    uint32_t *sort_counters = nullptr;     // tile counters per pass
    uint32_t sort_tiles = 0;
    uint32_t *sorted_keys = nullptr;       // result of the last neighbourhood sort
    uint32_t *perm = nullptr;              // new id -> old id of the last reorder
    uint32_t *inv_perm = nullptr;
    uint32_t *cell_start = nullptr;
    uint32_t *cell_end = nullptr;
    ulonglong2 *pos_code = nullptr;        // per particle: 96-bit position code {bits 0-63, bits 64-95}
    int4 *srec = nullptr;                  // per particle: search record (position xyz, fixed-point radius)
    int search_method = APBF_NEIGHBORHOOD_GREEN;  // the substep's neighbour search

    float *lambda = nullptr;
    int4 *shift = nullptr;
    float4 *solve_rec = nullptr;   // per particle: lambda, Gauss constants (ivd, norm), kernel width
    int4 *solve_pk = nullptr;      // per particle: position (xyz) and applied lambda (w, float bits)
    float2 *solve_kc = nullptr;    // per particle: Gauss constants (ivd, norm) of its kernel width
    int4 *filt = nullptr;          // per particle: gradient sum and boundariness > 0, for the deferred filter
    // learned warm start
    float *mlp_params = nullptr;   // FP32 parameter vector (mlp.cu)
    unsigned char *mlp_image = nullptr;  // its packed BF16 form for the tensor-core inference (mlp.cu)
    float *features = nullptr;     // per particle: 8 features of the first density pass
    float4 *selfdir = nullptr;     // per particle: self-shift direction (xyz), inverse mass (w)
    float *lam_acc = nullptr;      // per particle: sum of min(0, lambda) over the recorded iterations
    int warm_start = 0;            // APBF_WARM_* bits: learned first update, projected later passes
    int track_lambda = 0;          // 1: keep lambda_prev (set once recording or the warm start is used)
    int mlp_loaded = 0;
    // recording of training samples (armed for one apbf_substep)
    uint32_t rec_iterations = 0;
    float *rec_features = nullptr;
    float *rec_targets = nullptr;
    uint32_t rec_capacity = 0;
    uint32_t *rec_count = nullptr;
    uint32_t *dbg_density = nullptr;
    int4 *dbg_grad = nullptr;
    uint32_t *dbg_sq = nullptr;

    // adaptive scratch
    uint32_t *ukw = nullptr;
    uint32_t *min_nd = nullptr;
    uint32_t *nearest = nullptr;
    uint32_t *old_bd = nullptr;
    uint32_t *proposal = nullptr;  // per particle: packed proposal kind
    uint32_t *claim = nullptr;     // proposal list (particle ids in index order)
    uint32_t *owner = nullptr;     // per particle: smallest claimant slot, all ones between calls
    uint32_t *decided = nullptr;
    uint32_t *flag_scan = nullptr;
    uint32_t *list_a = nullptr;
    uint32_t *list_b = nullptr;
    uint32_t *scan_tmp = nullptr;
    uint32_t *t_keep = nullptr;    // per transfer: kept after particle_transfer
    uint32_t *t_scan = nullptr;    // per transfer: inclusive scan of t_keep

    double *red_partials = nullptr;
    double *red_out = nullptr;
    int red_blocks = 0;

    float4 *box_min = nullptr;
    float4 *box_max = nullptr;
    float4 *box_rot = nullptr;  // 3 rows per box; row 0 .w != 0 marks an oriented box
    uint32_t n_boxes = 0;
    uint32_t n_aabb = 0;        // boxes set by apbf_set_boxes (the oriented ones follow)
    apbf_emitter emitter = {};  // emitter.enabled == 0: none
    uint32_t *glue0 = nullptr, *glue1 = nullptr, *glue_d = nullptr, *glue_len = nullptr;  // glue list (constraints.cu)
    uint32_t glue_cap = 0;
    uint32_t *le_buf = nullptr;  // list services' scratch (listedit.cu), allocated on first use
    float emit_inv_mass = 0.0f;
    double *emit_state = nullptr;  // device: [0] stream time T, [1] particles emitted, [2..3] this substep's plan

    apbf::Status *status = nullptr;
    uint32_t n_cells_log2_alloc = 0;
    int debug = 0;
    std::vector<void *> owned;  // every device allocation, freed by apbf_destroy

    // tracing: per-launch events when enabled, launch counter always
    bool prof_on = false;
    std::vector<apbf::ProfSlot> prof;
    size_t prof_used = 0;
    unsigned long long prof_dropped = 0;
    unsigned long long launches = 0;
    apbf::ProfSlot *prof_open = nullptr;
    bool capturing = false;        // launches go into a graph being built: not counted

    apbf_tuning tuning = {1u, 256u, 8u, 0u, 0u, 0u, 0u, 0u};  // launch shapes (apbf_set_tuning / apbf_autotune)

    // solve loop graphs (graph.cu)
    int use_graphs = 1;
    int persistent_solve = 0;  // passes 1.. as one persistent cooperative kernel (apbf_set_persistent_solve)
    int coop_blocks = 0;       // its resident grid (0: cooperative launches unavailable)
    bool in_batch = false;     // being captured as one branch of a batch graph
    unsigned long long graph_version = 1;  // bumped by every change captured by value
    apbf::SolveGraph solve_graphs[apbf::kSolveGraphs];
    int solve_graph_next = 0;
    cudaStream_t capture_stream = nullptr;
    cudaStream_t capture_stream2 = nullptr;  // solve loop bodies captured inside a substep capture
    unsigned long long loop_launches_per_iter = 0;  // kernel nodes per body run
    apbf::SubstepGraph substep_graphs[apbf::kSubstepGraphs];
    int substep_graph_next = 0;

    // caller-owned lists (apbf_bind_lists): the context's own buffers while bound, and
    // the caller's length words
    bool bound = false;
    apbf::FluidBufs own_fl[2];
    apbf::TransferBufs own_tr[2];
    uint32_t *own_nb_count = nullptr, *own_nb_idx = nullptr;
    uint32_t *ext_len_particles = nullptr, *ext_len_transfers = nullptr;
};

namespace apbf {

void set_error(const std::string &msg);
apbf_status cuda_check(cudaError_t e, const char *what);
#define APBF_CUDA(call)                                              \
    do {                                                             \
        cudaError_t _e = (call);                                     \
        if (_e != cudaSuccess) return apbf::cuda_check(_e, #call);   \
    } while (0)
#define APBF_LAUNCH_CHECK(what)                                      \
    do {                                                             \
        cudaError_t _e = cudaGetLastError();                         \
        if (_e != cudaSuccess) return apbf::cuda_check(_e, what);    \
    } while (0)

// Kernel-launch bookkeeping: every launch is counted; when tracing is on, a
// pair of events is recorded around it on the launching stream.
inline void before_launch(apbf_ctx *c, cudaStream_t s, const char *name) {
    if (c->capturing) return;
    ++c->launches;
    c->prof_open = nullptr;
    if (!c->prof_on) return;
    if (c->prof_used >= c->prof.size()) {
        ++c->prof_dropped;
        return;
    }
    ProfSlot *slot = &c->prof[c->prof_used++];
    slot->name = name;
    cudaEventRecord(slot->a, s);
    c->prof_open = slot;
}
inline void after_launch(apbf_ctx *c, cudaStream_t s) {
    if (c->capturing) return;
    if (c->prof_open) cudaEventRecord(c->prof_open->b, s);
    c->prof_open = nullptr;
}
#define APBF_BEFORE_LAUNCH(ctx, stream, name) apbf::before_launch((ctx), (stream), (name))
#define APBF_AFTER_LAUNCH(ctx, stream, what)                         \
    do {                                                             \
        apbf::after_launch((ctx), (stream));                         \
        cudaError_t _e = cudaGetLastError();                         \
        if (_e != cudaSuccess) return apbf::cuda_check(_e, what);    \
    } while (0)

// While the caller's lists are bound (apbf_bind_lists), a stage call copies the
// caller's length words into the context's length block before its work and back
// after it, stream-ordered: the kernels read every length from that one block.
struct BoundLengths {
    apbf_ctx *c;
    cudaStream_t s;
    apbf_status status = APBF_OK;
    BoundLengths(apbf_ctx *ctx, cudaStream_t stream) : c(ctx), s(stream) {
        if (!c || !c->bound) return;
        cudaError_t e = cudaMemcpyAsync(c->d_len + kLenParticles, c->ext_len_particles, sizeof(uint32_t),
                                        cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->d_len + kLenTransfers, c->ext_len_transfers, sizeof(uint32_t),
                                cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) status = cuda_check(e, "copy of the bound lists' lengths");
    }
    ~BoundLengths() {
        if (!c || !c->bound || status != APBF_OK) return;
        cudaMemcpyAsync(c->ext_len_particles, c->d_len + kLenParticles, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(c->ext_len_transfers, c->d_len + kLenTransfers, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
    }
};
#define APBF_BOUND_LENGTHS(ctx, stream)                          \
    apbf::BoundLengths _bound_lengths((ctx), (stream));          \
    if (_bound_lengths.status != APBF_OK) return _bound_lengths.status

inline int grid_for(const apbf_ctx *ctx, uint32_t n, int block = kBlock, int per_sm = 8) {
    uint64_t need = ((uint64_t)n + block - 1) / block;
    uint64_t cap = (uint64_t)ctx->num_sms * per_sm;
    if (need < 1) need = 1;
    return (int)(need < cap ? need : cap);
}

// float -> int32 truncating toward zero, saturating, NaN -> 0 (rule C4), on the host
inline int32_t f2i_host(float x) {
    if (!(x == x)) return 0;
    if (x >= 2147483647.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int32_t)(-2147483647 - 1);
    return (int32_t)x;
}

// ---- host-side stage launchers (defined in the .cu files) ----
apbf_status emit(apbf_ctx *ctx, float dt, cudaStream_t s);  // glue.cu
// neighborhood.cu: gather by ctx->perm; with `search` also the search records for range scale `scale`
apbf_status reorder_particles(apbf_ctx *ctx, cudaStream_t s, bool search = false, float scale = 0.0f);
apbf_status glue_remap(apbf_ctx *ctx, cudaStream_t s);      // constraints.cu: glue ids follow a reorder
apbf_status sort_pairs_device(apbf_ctx *ctx, const uint32_t *keys_in, const uint32_t *vals_in, const uint32_t *d_count,
                              uint32_t max_count, uint32_t key_bits, uint32_t *keys_out, uint32_t *vals_out,
                              cudaStream_t s);
apbf_status prefix_sum_device(apbf_ctx *ctx, uint32_t *d_values, const uint32_t *d_count, uint32_t max_count,
                              cudaStream_t s);
// corrections = false: no correction rows (the substep prunes and transposes the rows
// next, spread_kernel_width)
apbf_status neighborhood_green(apbf_ctx *ctx, float range_scale, const float minp[3], const float maxp[3],
                               uint32_t log2res, cudaStream_t s, bool fuse_box = false, bool corrections = true);
apbf_status neighborhood_binary_search(apbf_ctx *ctx, float range_scale, cudaStream_t s,
                                       bool fuse_box = false);  // neighborhood_bs.cu
apbf_status velocity_handling(apbf_ctx *ctx, float dt, const float accel[3], cudaStream_t s);
apbf_status box_collision(apbf_ctx *ctx, cudaStream_t s);
// feature_mode: 0 none, 1 write features + self-shift direction; acc_mode: 0 none,
// 1 lam_acc = min(0, lambda), 2 lam_acc += min(0, lambda); learned: the first
// position update takes lambda from the network.
// Options of one Jacobi pass (density + lambda, then position update).
struct SolveOpts {
    bool box_after = false;   // box collision of the next iteration applied to this pass's output
    bool converge = false;    // density_error_target > 0: skip the pass once a pass met it
    int feature_mode = 0;     // 1: write the warm-start features (first pass of a substep)
    int acc_mode = 0;         // lam_acc: 0 off, 1 reset, 2 add the applied lambda (recorded passes)
    bool learned = false;     // the network's lambda replaces the computed one in this update
    int prev_mode = 0;        // lambda_prev: 0 off, 1 reset, 2 add the applied lambda
    bool projected = false;   // with prev_mode 2: pull-back up to the substep's accumulated push
    bool later_pass = false;  // not the first pass of a substep (the widths' uniformity is known)
    int loop_offset = -1;     // >= 0: a pass of the solve loop graph, number = pass_index + offset;
    uint32_t max_passes = 0;  //   skipped from max_passes on, box after it unless it is the last
};
apbf_status incompressibility(apbf_ctx *ctx, cudaStream_t s, const SolveOpts &o = SolveOpts());
// Passes 1.. of a substep as one persistent cooperative kernel with grid barriers
// between the density and position phases; APBF_ERR_INVALID_ARG when the solve
// does not qualify (then the caller uses the per-pass or graph forms).
apbf_status solve_persistent(apbf_ctx *ctx, cudaStream_t s, const SolveOpts &o);
bool solve_persistent_eligible(const apbf_ctx *ctx, const SolveOpts &o);
int solve_persistent_blocks(int device, int num_sms);
// The solve loops of a batch of scenes as one persistent cooperative kernel over a
// device table of scenes (solver.cu): eligibility, table entry size and filling,
// launch, resident grid.
bool batch_solve_eligible(const apbf_ctx *ctx, const SolveOpts &o);
size_t batch_scene_bytes();
size_t batch_sync_bytes();
uint32_t batch_max_scenes();
void batch_scene_fill(apbf_ctx *ctx, const SolveOpts &o, void *entry);
apbf_status solve_batch_launch(const void *d_table, uint32_t n_scenes, void *d_sync, unsigned long long *d_acc,
                               int grid, cudaStream_t s);
int solve_batch_blocks(int device, int num_sms);
// Passes 1.. of a substep as one graph launch (a device-side while loop).
apbf_status solve_loop(apbf_ctx *ctx, cudaStream_t s, const SolveOpts &o);
// The same loop as a conditional node of the graph that stream s is capturing.
apbf_status solve_loop_captured(apbf_ctx *ctx, cudaStream_t s, const SolveOpts &o);
void destroy_solve_graphs(apbf_ctx *ctx);
void destroy_substep_graphs(apbf_ctx *ctx);
// Whole substeps as graphs (graph.cu): one context, or a batch of contexts as the
// parallel branches of one graph.
// defer_loop non-null: when the substep's passes 1.. qualify for a batched solve,
// the body stops after the first pass, fills *defer_loop, sets *deferred and leaves
// the passes and substep_post to the caller.
apbf_status substep_body(apbf_ctx *ctx, float dt, cudaStream_t s, bool capture, SolveOpts *defer_loop = nullptr,
                         bool *deferred = nullptr);
apbf_status substep_post(apbf_ctx *ctx, cudaStream_t s);
bool substep_graph_eligible(const apbf_ctx *ctx);
apbf_status substep_graph(apbf_ctx *ctx, float dt, cudaStream_t s);
HostState host_state(const apbf_ctx *ctx);
void set_host_state(apbf_ctx *ctx, const HostState &h);
unsigned long long substep_mode_bits(const apbf_ctx *ctx);
constexpr int kMlpParams = 4824;  // floats of the warm-start parameter vector (mlp.cu)
apbf_status mlp_forward(const float *P, const float *X, uint32_t nrows, float *out, cudaStream_t s);
apbf_status mlp_train_step(float *P, float *m, float *v, float *partials, const float *X, const float *T,
                           uint32_t nrows, float lr, float over_weight, uint32_t step, float *grad_out,
                           float *loss_out, cudaStream_t s);
uint32_t mlp_partials_floats(uint32_t nrows);
apbf_status mlp_lambda(apbf_ctx *ctx, cudaStream_t s, bool early_exit);
// Packs a parameter vector into the inference kernel's shared-memory image
// (mlp_image_bytes() bytes, 16-byte aligned).
apbf_status mlp_pack(const float *P, void *image, cudaStream_t s);
size_t mlp_image_bytes();
apbf_status record_samples(apbf_ctx *ctx, cudaStream_t s);
apbf_status kw_from_boundary_distance(apbf_ctx *ctx, cudaStream_t s);
apbf_status spread_kernel_width(apbf_ctx *ctx, cudaStream_t s);
apbf_status update_transfers(apbf_ctx *ctx, cudaStream_t s);
apbf_status particle_transfer(apbf_ctx *ctx, float dt, cudaStream_t s);
apbf_status reduce_fp64(apbf_ctx *ctx, double out[4], cudaStream_t s);
apbf_status export_pairs(apbf_ctx *ctx, uint32_t *d_pairs, uint32_t cap, uint32_t *d_length, cudaStream_t s);
apbf_status build_reverse_rows(apbf_ctx *ctx, cudaStream_t s);

// ---- device helpers ----
#ifdef __CUDACC__

// GLSL int()/uint(): truncate toward zero, saturate, NaN -> 0 (cvt.rzi.sat semantics).
__device__ __forceinline__ int32_t f2i(float x) { return __float2int_rz(x); }
__device__ __forceinline__ uint32_t f2u(float x) { return __float2uint_rz(x); }
__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

__device__ __forceinline__ void set_flag(Status *st, uint32_t f) { atomicOr(&st->flags, f); }

// Spin bound of a bounded wait and whether the wait ignores its flag (set by
// apbf_set_wait_limit to test the failure path without a fault or a hang).
constexpr uint32_t kWaitInject = 0x80000000u;
__device__ __forceinline__ uint32_t wait_limit(const Status *st, uint32_t dflt, bool &inject) {
    const uint32_t v = *(volatile const uint32_t *)&st->wait_limit;
    inject = (v & kWaitInject) != 0u;
    const uint32_t l = v & ~kWaitInject;
    return l ? l : dflt;
}

// Bits of a 10-bit value spread to every third bit (Morton interleave).
__device__ __host__ __forceinline__ uint32_t spread3(uint32_t x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}
// calculate_position_hash.comp:29-36: bit i of axis d -> bit 3i + d.
__device__ __host__ __forceinline__ uint32_t morton3(uint32_t cx, uint32_t cy, uint32_t cz) {
    return spread3(cx) | (spread3(cy) << 1) | (spread3(cz) << 2);
}

// Canonical cell of a fixed-point coordinate: clamp(floor((x - lo) * 2^L / (hi - lo))).
__device__ __forceinline__ uint32_t cell_coord(long long x, long long lo, long long hi, uint32_t L) {
    const long long cells = 1ll << L;
    if (x <= lo) return 0u;
    if (x >= hi) return (uint32_t)(cells - 1);
    long long c = ((x - lo) << L) / (hi - lo);
    return (uint32_t)(c > cells - 1 ? cells - 1 : c);
}

// Fixed-point difference as reference units: vec3(posN - pos) / POS_RESOLUTION.
__device__ __forceinline__ float3 fdiff(int4 from, int4 to) {
    return make_float3((float)wadd(to.x, -from.x) * APBF_INV_FIX, (float)wadd(to.y, -from.y) * APBF_INV_FIX,
                       (float)wadd(to.z, -from.z) * APBF_INV_FIX);
}

__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

constexpr float kPiF = 3.14159265f;  // kernels.glsl:1

// Gauss constants of a kernel width (kernels.glsl:84-89, 104) in closed form:
// height = 0.6 / (kw/2)^3, ivw = height^(2/3) = 0.6^(2/3) (2/kw)^2 and
// norm = ivw^(3/2) = height (the reference's two pow() calls, without them).
__device__ __forceinline__ KConst gauss_consts(float kw) {
    KConst c;
    const float inv_half = 2.0f / kw;
    const float ivw = 0.71137866089801251f * (inv_half * inv_half);
    c.ivd = -(ivw * kPiF) * 1.44269504088896341f;
    c.norm = 0.6f * (inv_half * inv_half * inv_half);
    return c;
}

// exp(-r2 * ivd) * norm as exp2 of a pre-scaled exponent (ivd holds -ivd * log2(e)).
__device__ __forceinline__ float gauss_height(float r2, KConst c) { return exp2f(r2 * c.ivd) * c.norm; }

// kernel_height (kernels.glsl:99-110).  r2 = dot(r, r).
__device__ __forceinline__ float kernel_height(int kid, float r2, float h, KConst c) {
    switch (kid) {
    case 1: return gauss_height(r2, c);
    case 0: {
        float dist = sqrtf(r2);
        if (dist > h) return 0.0f;
        float q = dist / h, k = 8.0f / (kPiF * h * h * h);
        if (q <= 0.5f) { float q2 = q * q; return k * (6.0f * q * q2 - 6.0f * q2 + 1.0f); }
        float m = 1.0f - q;
        return k * (2.0f * m * m * m);
    }
    case 2: {
        float h2 = h * h;
        if (r2 > h2) return 0.0f;
        float d = h2 - r2, h3 = h * h * h;
        return 315.0f * (d * d * d) / (64.0f * kPiF * (h3 * h3 * h3));
    }
    case 3: {
        float height = 3.0f / (kPiF * h * h * h);
        return fmaxf(0.0f, (1.0f - sqrtf(r2) / h) * height);
    }
    case 4: {
        float dist = sqrtf(r2);
        float a = 15.0f / (2.0f * kPiF * (h * h * h * h * h));
        if (dist >= h) return 0.0f;
        return a * (h - dist) * (h - dist);
    }
    default: return 0.0f;
    }
}

// kernel_gradient (kernels.glsl:112-123).  For Gauss, Wg is the Gauss height at r.
__device__ __forceinline__ float3 kernel_gradient(int kid, float3 r, float r2, float h, KConst c, float Wg) {
    switch (kid) {
    case 1: {
        if (r2 < 1.0e-8f) return make_float3(0.f, 0.f, 0.f);  // dist < 0.0001
        // -W * 2 * dist * ivd * normalize(r) = -2 ivd W r, with ivd = -c.ivd / log2(e)
        float s = Wg * 2.0f * (c.ivd * 0.693147180559945309f);
        return make_float3(s * r.x, s * r.y, s * r.z);
    }
    case 0: {
        float dist = sqrtf(r2);
        if (dist > h || dist < 0.0001f) return make_float3(0.f, 0.f, 0.f);
        float q = dist / h, l = 48.0f / (kPiF * h * h * h);
        float s = q <= 0.5f ? l * q * (3.0f * q - 2.0f) : l * (-(1.0f - q) * (1.0f - q));
        float inv = 1.0f / (dist * h);
        return make_float3(s * (r.x * inv), s * (r.y * inv), s * (r.z * inv));
    }
    case 2: {
        float dist = sqrtf(r2);
        if (dist > h || dist < 0.0001f) return make_float3(0.f, 0.f, 0.f);
        float h3 = h * h * h, m = h - dist;
        float s = -45.0f * m * m / (kPiF * h3 * h3);
        return make_float3(s * (r.x / dist), s * (r.y / dist), s * (r.z / dist));
    }
    case 3: {
        float dist = sqrtf(r2);
        float st = 3.0f / (kPiF * h * h * h * h);
        if (dist > h || dist < 0.0001f) return make_float3(0.f, 0.f, 0.f);
        float s = st / dist;
        return make_float3(-r.x * s, -r.y * s, -r.z * s);
    }
    case 4: {
        float dist = sqrtf(r2);
        if (dist > h || dist < 0.0001f) return make_float3(0.f, 0.f, 0.f);
        float a = 15.0f / (2.0f * kPiF * (h * h * h * h * h));
        float s = -2.0f * a * fmaxf(0.0f, h - dist) / dist;
        return make_float3(s * r.x, s * r.y, s * r.z);
    }
    default: return make_float3(0.f, 0.f, 0.f);
    }
}

// ---- box collision (box_collision.comp:19-60), every operation rounded on its
// own so that any translation unit reproduces the FP32 evaluation exactly ----
__device__ __forceinline__ float fract_rn(float x) { return __fsub_rn(x, floorf(x)); }

__device__ __forceinline__ float3 hash31_rn(float p) {  // shadertoy 4djSRW hash31 (MIT licence)
    float3 q = make_float3(fract_rn(__fmul_rn(p, 0.1031f)), fract_rn(__fmul_rn(p, 0.1030f)),
                           fract_rn(__fmul_rn(p, 0.0973f)));
    float t = __fmul_rn(q.x, __fadd_rn(q.y, 33.33f));
    t = __fadd_rn(t, __fmul_rn(q.y, __fadd_rn(q.z, 33.33f)));
    t = __fadd_rn(t, __fmul_rn(q.z, __fadd_rn(q.x, 33.33f)));
    q.x = __fadd_rn(q.x, t);
    q.y = __fadd_rn(q.y, t);
    q.z = __fadd_rn(q.z, t);
    return make_float3(fract_rn(__fmul_rn(__fadd_rn(q.x, q.y), q.z)), fract_rn(__fmul_rn(__fadd_rn(q.x, q.z), q.y)),
                       fract_rn(__fmul_rn(__fadd_rn(q.y, q.z), q.x)));
}

// Canonical search radius: floor(kw * scale * 2^18) from the FP32 inputs, clamped
// below 2^31 (positions are int32, so no distance needs more).
__device__ __forceinline__ long long range_fixed(float kw, float scale) {
    double r = (double)kw * (double)scale * 262144.0;
    if (!(r >= 0.0)) return -1;
    if (r > 2147483647.0) r = 2147483647.0;
    return (long long)floor(r);
}

// |b - a|^2 <= R^2 exactly.  Once every |d| <= R < 2^31 is known, each square is
// one 32x32 -> 64-bit multiply and the sum cannot overflow 64 bits.
__device__ __forceinline__ bool within(int4 a, int4 b, long long R) {
    long long dx = (long long)b.x - a.x, dy = (long long)b.y - a.y, dz = (long long)b.z - a.z;
    dx = dx < 0 ? -dx : dx;
    dy = dy < 0 ? -dy : dy;
    dz = dz < 0 ? -dz : dz;
    if (dx > R || dy > R || dz > R) return false;
    const uint32_t ux = (uint32_t)dx, uy = (uint32_t)dy, uz = (uint32_t)dz, ur = (uint32_t)R;
    unsigned long long s = (unsigned long long)ux * ux + (unsigned long long)uy * uy + (unsigned long long)uz * uz;
    return s <= (unsigned long long)ur * ur;
}


// box_collision.comp:35-57 on one box in the box's own frame: (qx, qy, qz) is the
// particle position relative to the frame, [lo, hi] the box; the box is grown by the
// radius and by the hash jitter h1 / h2, and the particle is moved out through the
// nearest face of whichever corner is closer.  Returns whether it moved.
__device__ __forceinline__ bool push_out(float &qx, float &qy, float &qz, float3 lo, float3 hi, float r, float3 h1,
                                         float3 h2) {
    float tx0 = __fsub_rn(__fsub_rn(__fsub_rn(lo.x, r), __fmul_rn(h1.x, 0.05f)), qx);
    float ty0 = __fsub_rn(__fsub_rn(__fsub_rn(lo.y, r), __fmul_rn(h1.y, 0.05f)), qy);
    float tz0 = __fsub_rn(__fsub_rn(__fsub_rn(lo.z, r), __fmul_rn(h1.z, 0.05f)), qz);
    float tx1 = __fsub_rn(__fadd_rn(__fadd_rn(hi.x, r), __fmul_rn(h2.x, 0.05f)), qx);
    float ty1 = __fsub_rn(__fadd_rn(__fadd_rn(hi.y, r), __fmul_rn(h2.y, 0.05f)), qy);
    float tz1 = __fsub_rn(__fadd_rn(__fadd_rn(hi.z, r), __fmul_rn(h2.z, 0.05f)), qz);
    // smallestComponent(-toMin) and smallestComponent(toMax), box_collision.comp:27-33
    {
        const float vx = -tx0, vy = -ty0, vz = -tz0;
        const bool b1 = vx <= vy, b2 = vx <= vz, b3 = vy <= vz;
        tx0 = __fmul_rn(tx0, (b1 && b2) ? 1.0f : 0.0f);
        ty0 = __fmul_rn(ty0, (!b1 && b3) ? 1.0f : 0.0f);
        tz0 = __fmul_rn(tz0, (!b2 && !b3) ? 1.0f : 0.0f);
    }
    {
        const bool b1 = tx1 <= ty1, b2 = tx1 <= tz1, b3 = ty1 <= tz1;
        tx1 = __fmul_rn(tx1, (b1 && b2) ? 1.0f : 0.0f);
        ty1 = __fmul_rn(ty1, (!b1 && b3) ? 1.0f : 0.0f);
        tz1 = __fmul_rn(tz1, (!b2 && !b3) ? 1.0f : 0.0f);
    }
    const float dmin = -__fadd_rn(__fadd_rn(tx0, ty0), tz0);
    const float dmax = __fadd_rn(__fadd_rn(tx1, ty1), tz1);
    if (dmin <= 0.0f || dmax <= 0.0f) return false;
    if (dmin < dmax) {
        qx = __fadd_rn(qx, tx0);
        qy = __fadd_rn(qy, ty0);
        qz = __fadd_rn(qz, tz0);
    } else {
        qx = __fadd_rn(qx, tx1);
        qy = __fadd_rn(qy, ty1);
        qz = __fadd_rn(qz, tz1);
    }
    return true;
}

__device__ __forceinline__ float dot3_rn(float4 a, float x, float y, float z) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, x), __fmul_rn(a.y, y)), __fmul_rn(a.z, z));
}

// True when push_out cannot move a particle at q whatever the jitter: some axis d
// has q_d < fl(fl(lo_d - r) - c) or q_d >= fl(fl(hi_d + r) + c), c = 0.0500001 >=
// every 0.05 * h with h in [0, 1).  Rounding is monotone, so then q_d <= the
// jittered lower threshold (or >= the upper one), the selected component of
// -toMin (toMax) is <= 0 and push_out returns false.  Only for finite thresholds
// below 1e30, where every component push_out forms is finite.
__device__ __forceinline__ bool box_clear(float qx, float qy, float qz, float3 lo, float3 hi, float r) {
    const float c = 0.0500001f;
    const float b0x = __fsub_rn(__fsub_rn(lo.x, r), c), b0y = __fsub_rn(__fsub_rn(lo.y, r), c),
                b0z = __fsub_rn(__fsub_rn(lo.z, r), c);
    const float b1x = __fadd_rn(__fadd_rn(hi.x, r), c), b1y = __fadd_rn(__fadd_rn(hi.y, r), c),
                b1z = __fadd_rn(__fadd_rn(hi.z, r), c);
    const float m = fmaxf(fmaxf(fmaxf(fabsf(b0x), fabsf(b0y)), fmaxf(fabsf(b0z), fabsf(b1x))),
                          fmaxf(fabsf(b1y), fabsf(b1z)));
    if (!(m < 1.0e30f)) return false;
    return qx < b0x || qy < b0y || qz < b0z || qx >= b1x || qy >= b1y || qz >= b1z;
}

// Pushes one particle (sorted id `id`, radius r) out of every box.  Box k is
// axis-aligned ([bmin, bmax], as in the reference) unless rot[3k].w != 0: then it
// is oriented, bmin = its centre, bmax = its half extents and rot[3k..3k+2] the
// rows of its rotation (local axis i = row i), and the same push runs in its frame.
// The jitter hashes depend only on the id and the current position: they are
// computed for the first box that may push and kept until a push moves the particle,
// and boxes that box_clear rules out skip them (same results, box by box).
__device__ __forceinline__ int4 box_push(int4 ip, float r, uint32_t id, const float4 *__restrict__ bmin,
                                         const float4 *__restrict__ bmax, const float4 *__restrict__ rot,
                                         uint32_t nb) {
    if (nb == 0) return ip;
    // vec3(position) / POS_RESOLUTION: a division by 2^18 is the exact product with 2^-18
    float px = __fmul_rn((float)ip.x, 0x1p-18f), py = __fmul_rn((float)ip.y, 0x1p-18f),
          pz = __fmul_rn((float)ip.z, 0x1p-18f);
    const float fid = (float)id;
    float3 h1 = make_float3(0.f, 0.f, 0.f), h2 = h1;
    bool have = false;
    for (uint32_t k = 0; k < nb; ++k) {
        const float4 lo = bmin[k], hi = bmax[k];
        const float4 r0 = rot[3 * k];
        if (r0.w == 0.0f) {
            const float3 l3 = make_float3(lo.x, lo.y, lo.z), u3 = make_float3(hi.x, hi.y, hi.z);
            if (box_clear(px, py, pz, l3, u3, r)) continue;
            if (!have) {
                h1 = hash31_rn(__fsub_rn(__fsub_rn(__fmul_rn(fid, px), py), pz));
                h2 = hash31_rn(__fadd_rn(__fadd_rn(__fmul_rn(fid, py), px), pz));
                have = true;
            }
            if (push_out(px, py, pz, l3, u3, r, h1, h2)) have = false;
            continue;
        }
        const float4 r1 = rot[3 * k + 1], r2 = rot[3 * k + 2];
        const float dx = __fsub_rn(px, lo.x), dy = __fsub_rn(py, lo.y), dz = __fsub_rn(pz, lo.z);
        float qx = dot3_rn(r0, dx, dy, dz), qy = dot3_rn(r1, dx, dy, dz), qz = dot3_rn(r2, dx, dy, dz);
        const float3 nh = make_float3(-hi.x, -hi.y, -hi.z), u3 = make_float3(hi.x, hi.y, hi.z);
        if (box_clear(qx, qy, qz, nh, u3, r)) continue;
        if (!have) {
            h1 = hash31_rn(__fsub_rn(__fsub_rn(__fmul_rn(fid, px), py), pz));
            h2 = hash31_rn(__fadd_rn(__fadd_rn(__fmul_rn(fid, py), px), pz));
            have = true;
        }
        if (!push_out(qx, qy, qz, nh, u3, r, h1, h2)) continue;
        have = false;
        // back to the world frame: p = centre + R^T q
        px = __fadd_rn(lo.x, __fadd_rn(__fadd_rn(__fmul_rn(r0.x, qx), __fmul_rn(r1.x, qy)), __fmul_rn(r2.x, qz)));
        py = __fadd_rn(lo.y, __fadd_rn(__fadd_rn(__fmul_rn(r0.y, qx), __fmul_rn(r1.y, qy)), __fmul_rn(r2.y, qz)));
        pz = __fadd_rn(lo.z, __fadd_rn(__fadd_rn(__fmul_rn(r0.z, qx), __fmul_rn(r1.z, qy)), __fmul_rn(r2.z, qz)));
    }
    return make_int4(f2i(__fmul_rn(px, 262144.0f)), f2i(__fmul_rn(py, 262144.0f)), f2i(__fmul_rn(pz, 262144.0f)), ip.w);
}

#endif  // __CUDACC__

}  // namespace apbf
