// capi.cu -- the extern "C" boundary declared in include/apbf_gb300.h: context
// lifetime, list access, stage dispatch and the whole-substep driver.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "apbf_internal.cuh"

namespace apbf {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

apbf_status cuda_check(cudaError_t e, const char *what) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return APBF_ERR_CUDA;
}

namespace {

template <typename T>
apbf_status dalloc(T **p, size_t count, std::vector<void *> &owned) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) return cuda_check(e, "cudaMalloc");
    owned.push_back((void *)*p);
    return APBF_OK;
}

}  // namespace

// gpu_list::set_length from a host value, stream-ordered (no synchronisation).
__global__ void k_set_length(uint32_t *d_len, uint32_t slot, uint32_t v) { d_len[slot] = v; }

// Host <-> device copy of the particle lists in one launch.  Each field is a byte
// range of a multiple of 4 bytes; host ranges are page-locked host memory that the
// GPU addresses directly (pointers from cudaPointerGetAttributes), so the loads or
// stores of this kernel cross the CPU-GPU link while the device side is HBM.  One
// grid row (blockIdx.y) per field; 16-byte units where both ends are 16-byte aligned.
struct CopyField {
    char *dst;
    const char *src;
    unsigned long long bytes;
    int vec16;
};
constexpr int kMaxCopyFields = 11;
struct CopyList {
    CopyField f[kMaxCopyFields];
};

__global__ void __launch_bounds__(256) k_copy_fields(CopyList list) {
    const CopyField fd = list.f[blockIdx.y];
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long done = 0;
    if (fd.vec16) {
        const unsigned long long n16 = fd.bytes >> 4;
        const uint4 *src = reinterpret_cast<const uint4 *>(fd.src);
        uint4 *dst = reinterpret_cast<uint4 *>(fd.dst);
        // four independent 16-byte loads in flight per thread: the link's latency is long
        for (unsigned long long i = t; i < n16; i += 4 * stride) {
            uint4 v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i + u * stride < n16) v[u] = src[i + u * stride];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i + u * stride < n16) dst[i + u * stride] = v[u];
        }
        done = n16 << 4;
    }
    const unsigned long long n4 = (fd.bytes - done) >> 2;
    const uint32_t *src = reinterpret_cast<const uint32_t *>(fd.src + done);
    uint32_t *dst = reinterpret_cast<uint32_t *>(fd.dst + done);
    for (unsigned long long i = t; i < n4; i += 4 * stride) {
        uint32_t v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u * stride < n4) v[u] = src[i + u * stride];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u * stride < n4) dst[i + u * stride] = v[u];
    }
}

// The device address of page-locked host memory at `p`, or nullptr when `p` is
// ordinary (pageable) host memory or not host memory at all.
void *mapped_host(const void *p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // clears the error of an unknown pointer
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Copies `nf` fields of `n` particles (bytes per particle each) between host and
// device: one k_copy_fields launch for the page-locked host arrays, cudaMemcpyAsync
// for the others.  to_device: host -> device.
apbf_status copy_fluid_fields(apbf_ctx *ctx, void *const *dev, void *const *host, const size_t *bpp, int nf, size_t n,
                              bool to_device, cudaStream_t s) {
    CopyList list = {};
    int nk = 0;
    size_t largest = 0;
    for (int k = 0; k < nf; ++k) {
        if (!host[k] || !n) continue;
        const size_t bytes = n * bpp[k];
        void *mh = mapped_host(host[k]);
        if (!mh) {
            APBF_CUDA(to_device ? cudaMemcpyAsync(dev[k], host[k], bytes, cudaMemcpyHostToDevice, s)
                                : cudaMemcpyAsync(host[k], dev[k], bytes, cudaMemcpyDeviceToHost, s));
            continue;
        }
        CopyField &fd = list.f[nk++];
        fd.dst = static_cast<char *>(to_device ? dev[k] : mh);
        fd.src = static_cast<const char *>(to_device ? mh : dev[k]);
        fd.bytes = bytes;
        fd.vec16 = ((reinterpret_cast<uintptr_t>(fd.dst) | reinterpret_cast<uintptr_t>(fd.src)) & 15u) == 0;
        largest = bytes > largest ? bytes : largest;
    }
    if (nk) {
        const size_t units = (largest + 15) / 16;
        const unsigned gx = (unsigned)std::max<size_t>(1, std::min<size_t>((units + 1023) / 1024,
                                                                           (size_t)ctx->num_sms * 2));
        APBF_BEFORE_LAUNCH(ctx, s, "k_copy_fields");
        k_copy_fields<<<dim3(gx, (unsigned)nk), 256, 0, s>>>(list);
        APBF_AFTER_LAUNCH(ctx, s, "k_copy_fields");
    }
    return APBF_OK;
}
}  // namespace apbf

using namespace apbf;

extern "C" {

uint32_t apbf_abi_version(void) { return APBF_ABI_VERSION; }

const char *apbf_last_error(void) { return apbf::g_last_error.c_str(); }

// Reference defaults, source/settings.cpp:5-31 (3D).
void apbf_default_settings(apbf_settings *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->height_kernel_id = 1;
    o->gradient_kernel_id = 1;
    o->merge = 1;
    o->split = 1;
    o->base_kernel_width_on_target_radius = 1;
    o->base_kernel_width_on_boundary_distance = 1;
    o->update_target_radius = 1;
    o->update_boundariness = 1;
    o->boundariness_calculation_method = 2;
    o->basic_pbf = 0;
    o->solver_iterations = 3;
    o->boundariness_adaption_speed = 0.5f;
    o->kernel_width_adaption_speed = 0.01f;
    o->boundariness_self_grad_length_factor = 2.0f;
    o->boundariness_underpressure_factor = 4.0f;
    o->merge_duration = 2.0f;
    o->split_duration = 0.0f;
    o->smallest_target_radius = 1.0f;
    o->target_radius_offset = 10.0f;
    o->target_radius_scale_factor = 0.3f;
}

apbf_status apbf_destroy(apbf_ctx *ctx) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    for (auto &p : ctx->prof) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    destroy_solve_graphs(ctx);
    destroy_substep_graphs(ctx);
    cudaFree(ctx->glue0);
    cudaFree(ctx->glue1);
    cudaFree(ctx->glue_d);
    cudaFree(ctx->glue_len);
    cudaFree(ctx->le_buf);
    if (ctx->capture_stream) cudaStreamDestroy(ctx->capture_stream);
    if (ctx->capture_stream2) cudaStreamDestroy(ctx->capture_stream2);
    for (void *p : ctx->owned) cudaFree(p);
    delete ctx;
    return APBF_OK;
}

apbf_status apbf_create(const apbf_config *cfg, apbf_ctx **out) {
    if (!cfg || !out) return APBF_ERR_INVALID_ARG;
    *out = nullptr;
    if (cfg->particle_capacity == 0 || cfg->particle_capacity >= (1u << 28) || cfg->max_neighbors == 0 ||
        cfg->max_log2res < 1 || cfg->max_log2res > 9) {
        set_error("apbf_create: invalid capacities (particles in [1, 2^28), max_neighbors > 0, max_log2res in [1, 9])");
        return APBF_ERR_INVALID_ARG;
    }
    apbf_ctx *ctx = new (std::nothrow) apbf_ctx();
    if (!ctx) return APBF_ERR_INVALID_ARG;
    ctx->cfg = *cfg;
    if (ctx->cfg.transfer_capacity == 0) ctx->cfg.transfer_capacity = APBF_MAX_TRANSFERS;
    apbf_default_settings(&ctx->settings);
    std::memset(&ctx->scene, 0, sizeof(ctx->scene));
    ctx->device = cfg->device;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) {
        delete ctx;
        return cuda_check(e, "cudaSetDevice");
    }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const uint32_t cap = cfg->particle_capacity;
    const uint32_t tcap = ctx->cfg.transfer_capacity;
    ctx->row_stride = (cap + 31u) & ~31u;
    auto &o = ctx->owned;
    apbf_status r = APBF_OK;
#define A(ptr, count)                                  \
    do {                                               \
        r = dalloc(&(ptr), (size_t)(count), o);        \
        if (r != APBF_OK) {                            \
            apbf_destroy(ctx);                         \
            return r;                                  \
        }                                              \
    } while (0)
    for (int k = 0; k < 2; ++k) {
        FluidBufs &f = ctx->fl[k];
        A(f.pos, cap);
        A(f.vel, cap);
        A(f.inv_mass, cap);
        A(f.radius, cap);
        A(f.pos_backup, cap);
        A(f.transferring, cap);
        A(f.target_radius, cap);
        A(f.kernel_width, cap);
        A(f.boundariness, cap);
        A(f.boundary_distance, cap);
        A(f.lambda_prev, cap);
        TransferBufs &t = ctx->tr[k];
        A(t.source, tcap);
        A(t.target, tcap);
        A(t.time_left, tcap);
    }
    A(ctx->d_len, kLenSlots);
    A(ctx->nb_count, cap);
    A(ctx->rev_count, cap);
    A(ctx->nb_idx, (size_t)ctx->row_stride * cfg->max_neighbors);
    A(ctx->rev_idx, (size_t)ctx->row_stride * cfg->max_neighbors);
    A(ctx->d_pairs, 1);
    for (int k = 0; k < 2; ++k) {
        A(ctx->keys[k], cap);
        A(ctx->vals[k], cap);
    }
    ctx->sort_tiles = (cap + kSortTile - 1) / kSortTile;
    A(ctx->sort_hist, 4 * 256);
    A(ctx->sort_counters, 8);
    A(ctx->sort_status, (size_t)4 * ctx->sort_tiles * 256);
    A(ctx->sorted_keys, cap);
    A(ctx->perm, cap);
    A(ctx->inv_perm, cap);
    A(ctx->scan_tmp, cap);
    A(ctx->t_keep, tcap);
    A(ctx->t_scan, tcap);
    const size_t ncells = (size_t)1 << (3 * cfg->max_log2res);
    A(ctx->cell_start, ncells);
    A(ctx->cell_end, ncells);
    A(ctx->pos_code, cap);
    A(ctx->srec, cap);
    ctx->n_cells_log2_alloc = cfg->max_log2res;
    A(ctx->lambda, cap);
    A(ctx->shift, cap);
    A(ctx->solve_rec, cap);
    A(ctx->solve_pk, cap);
    A(ctx->solve_kc, cap);
    A(ctx->filt, cap);
    A(ctx->mlp_params, kMlpParams);
    A(ctx->mlp_image, mlp_image_bytes());
    A(ctx->features, (size_t)cap * 8);
    A(ctx->selfdir, cap);
    A(ctx->lam_acc, cap);
    A(ctx->dbg_density, cap);
    A(ctx->dbg_grad, cap);
    A(ctx->dbg_sq, cap);
    A(ctx->ukw, cap);
    A(ctx->min_nd, cap);
    A(ctx->nearest, cap);
    A(ctx->old_bd, cap);
    A(ctx->proposal, cap);
    A(ctx->claim, cap);
    A(ctx->owner, cap);
    A(ctx->decided, cap);
    A(ctx->flag_scan, cap);
    A(ctx->list_a, cap);
    A(ctx->list_b, cap);
    ctx->red_blocks = grid_for(ctx, cap, kBlock, 8);
    ctx->coop_blocks = solve_persistent_blocks(ctx->device, ctx->num_sms);
    A(ctx->red_partials, (size_t)6 * ctx->red_blocks);
    A(ctx->red_out, 4);
    A(ctx->box_min, APBF_MAX_BOXES);
    A(ctx->box_max, APBF_MAX_BOXES);
    A(ctx->box_rot, 3 * APBF_MAX_BOXES);
    A(ctx->emit_state, 8);
    A(ctx->status, 1);
#undef A
    cudaMemset(ctx->d_len, 0, kLenSlots * sizeof(uint32_t));
    cudaMemset(ctx->status, 0, sizeof(Status));
    cudaMemset(ctx->red_out, 0, 4 * sizeof(double));
    cudaMemset(ctx->nb_count, 0, (size_t)cap * sizeof(uint32_t));
    cudaMemset(ctx->owner, 0xff, (size_t)cap * sizeof(uint32_t));
    for (int k = 0; k < 2; ++k) {
        cudaMemset(ctx->fl[k].pos, 0, (size_t)cap * sizeof(int4));
        cudaMemset(ctx->fl[k].pos_backup, 0, (size_t)cap * sizeof(int4));
        cudaMemset(ctx->fl[k].vel, 0, (size_t)cap * sizeof(float4));
        cudaMemset(ctx->fl[k].lambda_prev, 0, (size_t)cap * sizeof(float));
        cudaMemset(ctx->fl[k].transferring, 0, (size_t)cap * sizeof(uint32_t));
    }
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        apbf_destroy(ctx);
        return cuda_check(e, "apbf_create");
    }
    *out = ctx;
    return APBF_OK;
}

apbf_status apbf_set_settings(apbf_ctx *ctx, const apbf_settings *s) {
    if (!ctx || !s) return APBF_ERR_INVALID_ARG;
    if (s->height_kernel_id < 0 || s->height_kernel_id > 4 || s->gradient_kernel_id < 0 || s->gradient_kernel_id > 4 ||
        s->boundariness_calculation_method < 0 || s->boundariness_calculation_method > 2 || s->solver_iterations < 0) {
        set_error("apbf_set_settings: kernel ids in [0, 4], boundariness method in [0, 2], iterations >= 0");
        return APBF_ERR_INVALID_ARG;
    }
    ctx->settings = *s;
    ctx->graph_version++;  // solve loop graphs hold settings by value
    return APBF_OK;
}

apbf_status apbf_set_scene(apbf_ctx *ctx, const apbf_scene *scene) {
    if (!ctx || !scene) return APBF_ERR_INVALID_ARG;
    if (scene->log2res < 1 || scene->log2res > ctx->cfg.max_log2res) {
        set_error("apbf_set_scene: log2res must be in [1, max_log2res]");
        return APBF_ERR_INVALID_ARG;
    }
    ctx->scene = *scene;
    return APBF_OK;
}

apbf_status apbf_set_boxes(apbf_ctx *ctx, const float *bmin, const float *bmax, uint32_t n) {
    if (!ctx || n > APBF_MAX_BOXES || (n && (!bmin || !bmax))) return APBF_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (n) {
        APBF_CUDA(cudaMemcpy(ctx->box_min, bmin, n * sizeof(float4), cudaMemcpyHostToDevice));
        APBF_CUDA(cudaMemcpy(ctx->box_max, bmax, n * sizeof(float4), cudaMemcpyHostToDevice));
        std::vector<float4> zero(3 * (size_t)n, make_float4(0.f, 0.f, 0.f, 0.f));  // axis-aligned
        APBF_CUDA(cudaMemcpy(ctx->box_rot, zero.data(), zero.size() * sizeof(float4), cudaMemcpyHostToDevice));
    }
    ctx->n_boxes = n;
    ctx->n_aabb = n;
    ctx->graph_version++;
    return APBF_OK;
}

apbf_status apbf_set_emitter(apbf_ctx *ctx, const apbf_emitter *e) {
    if (!ctx || !e) return APBF_ERR_INVALID_ARG;
    if (e->enabled && (!(e->radius > 0.0f) || !(e->speed > 0.0f) || e->nx == 0 || e->nz == 0 || !(e->jitter >= 0.0f) ||
                       (uint64_t)e->nx * e->nz > 0xffffffu)) {
        set_error("apbf_set_emitter: radius and speed > 0, 1 <= nx * nz <= 2^24, jitter >= 0");
        return APBF_ERR_INVALID_ARG;
    }
    cudaSetDevice(ctx->device);
    ctx->emitter = *e;
    const double d = 2.0 * (double)e->radius;
    ctx->emit_inv_mass = (float)(1.0 / (d * d * d));
    APBF_CUDA(cudaMemset(ctx->emit_state, 0, 8 * sizeof(double)));
    ctx->graph_version++;
    return APBF_OK;
}

apbf_status apbf_set_oriented_boxes(apbf_ctx *ctx, const float *center, const float *half, const float *quat,
                                    uint32_t n) {
    if (!ctx || ctx->n_aabb + n > APBF_MAX_BOXES || (n && (!center || !half || !quat))) return APBF_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    std::vector<float4> c(n), h(n), rot(3 * (size_t)n);
    for (uint32_t k = 0; k < n; ++k) {
        const double qx = quat[4 * k], qy = quat[4 * k + 1], qz = quat[4 * k + 2], qw = quat[4 * k + 3];
        const double nq = std::sqrt(qx * qx + qy * qy + qz * qz + qw * qw);
        if (!(nq > 0.0) || !(half[4 * k] >= 0.0f) || !(half[4 * k + 1] >= 0.0f) || !(half[4 * k + 2] >= 0.0f)) {
            set_error("apbf_set_oriented_boxes: zero quaternion or negative half extent");
            return APBF_ERR_INVALID_ARG;
        }
        const double x = qx / nq, y = qy / nq, z = qz / nq, w = qw / nq;
        // rows of R^T, i.e. the box's local axes in world coordinates (R rotates local -> world)
        const double m[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w)},
                                {2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w)},
                                {2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)}};
        for (int r = 0; r < 3; ++r)
            rot[3 * k + r] = make_float4((float)m[r][0], (float)m[r][1], (float)m[r][2], r == 0 ? 1.0f : 0.0f);
        c[k] = make_float4(center[4 * k], center[4 * k + 1], center[4 * k + 2], 0.0f);
        h[k] = make_float4(half[4 * k], half[4 * k + 1], half[4 * k + 2], 0.0f);
    }
    const uint32_t o = ctx->n_aabb;
    if (n) {
        APBF_CUDA(cudaMemcpy(ctx->box_min + o, c.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
        APBF_CUDA(cudaMemcpy(ctx->box_max + o, h.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
        APBF_CUDA(cudaMemcpy(ctx->box_rot + 3 * o, rot.data(), rot.size() * sizeof(float4), cudaMemcpyHostToDevice));
    }
    ctx->n_boxes = o + n;
    ctx->graph_version++;
    return APBF_OK;
}

apbf_status apbf_get_box_rotations(apbf_ctx *ctx, float *rot_out, uint32_t n) {
    if (!ctx || !rot_out || n > ctx->n_boxes) return APBF_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    APBF_CUDA(cudaMemcpy(rot_out, ctx->box_rot, 3 * (size_t)n * sizeof(float4), cudaMemcpyDeviceToHost));
    return APBF_OK;
}

apbf_status apbf_set_debug(apbf_ctx *ctx, int enable) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    ctx->debug = enable ? 1 : 0;
    ctx->graph_version++;
    return APBF_OK;
}

apbf_status apbf_set_solve_graph(apbf_ctx *ctx, int mode) {
    if (!ctx || mode < 0 || mode > 2) return APBF_ERR_INVALID_ARG;
    ctx->use_graphs = mode;
    destroy_solve_graphs(ctx);
    destroy_substep_graphs(ctx);
    return APBF_OK;
}

apbf_status apbf_set_persistent_solve(apbf_ctx *ctx, int enable) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    if (enable && ctx->coop_blocks <= 0) {
        set_error("apbf_set_persistent_solve: the device has no cooperative launches");
        return APBF_ERR_INVALID_ARG;
    }
    ctx->persistent_solve = enable ? 1 : 0;
    ctx->graph_version++;
    destroy_solve_graphs(ctx);
    destroy_substep_graphs(ctx);
    return APBF_OK;
}

apbf_status apbf_fluid_get_view(apbf_ctx *ctx, apbf_fluid_view *o) {
    if (!ctx || !o) return APBF_ERR_INVALID_ARG;
    const FluidBufs &f = ctx->fl[ctx->fcur];
    o->capacity = ctx->cfg.particle_capacity;
    o->d_length = ctx->bound ? ctx->ext_len_particles : ctx->d_len + kLenParticles;
    o->position = (int32_t *)f.pos;
    o->velocity = (float *)f.vel;
    o->inverse_mass = f.inv_mass;
    o->radius = f.radius;
    o->pos_backup = (int32_t *)f.pos_backup;
    o->transferring = f.transferring;
    o->target_radius = f.target_radius;
    o->kernel_width = f.kernel_width;
    o->boundariness = f.boundariness;
    o->boundary_distance = f.boundary_distance;
    return APBF_OK;
}

apbf_status apbf_transfers_get_view(apbf_ctx *ctx, apbf_transfers_view *o) {
    if (!ctx || !o) return APBF_ERR_INVALID_ARG;
    const TransferBufs &t = ctx->tr[ctx->tcur];
    o->capacity = ctx->cfg.transfer_capacity;
    o->d_length = ctx->bound ? ctx->ext_len_transfers : ctx->d_len + kLenTransfers;
    o->source = t.source;
    o->target = t.target;
    o->time_left = t.time_left;
    return APBF_OK;
}

apbf_status apbf_neighbors_get_view(apbf_ctx *ctx, apbf_neighbors_view *o) {
    if (!ctx || !o) return APBF_ERR_INVALID_ARG;
    o->row_stride = ctx->row_stride;
    o->max_per_row = ctx->cfg.max_neighbors;
    o->count = ctx->nb_count;
    o->index = ctx->nb_idx;
    o->d_total = ctx->d_pairs;
    return APBF_OK;
}

apbf_status apbf_neighbors_get_reverse_view(apbf_ctx *ctx, apbf_neighbors_view *o, uint32_t *union_rows,
                                            void *stream) {
    if (!ctx || !o) return APBF_ERR_INVALID_ARG;
    o->row_stride = ctx->row_stride;
    o->max_per_row = ctx->cfg.max_neighbors;
    o->count = ctx->rev_count;
    o->index = ctx->rev_idx;
    o->d_total = ctx->d_pairs;
    if (union_rows) {
        Status hs;
        cudaStream_t s = (cudaStream_t)stream;
        APBF_CUDA(cudaMemcpyAsync(&hs, ctx->status, sizeof(Status), cudaMemcpyDeviceToHost, s));
        APBF_CUDA(cudaStreamSynchronize(s));
        *union_rows = hs.range_min == hs.range_max ? 2u : hs.union_rows;
    }
    return APBF_OK;
}

apbf_status apbf_set_lengths(apbf_ctx *ctx, uint32_t np, uint32_t nt, void *stream) {
    if (!ctx || np > ctx->cfg.particle_capacity || nt > ctx->cfg.transfer_capacity) {
        set_error("apbf_set_lengths: length above capacity");
        return APBF_ERR_INVALID_ARG;
    }
    uint32_t v[2] = {np, nt};
    cudaStream_t s = (cudaStream_t)stream;
    APBF_CUDA(cudaMemcpyAsync(ctx->d_len, v, sizeof(v), cudaMemcpyHostToDevice, s));
    if (ctx->bound) {
        APBF_CUDA(cudaMemcpyAsync(ctx->ext_len_particles, ctx->d_len + kLenParticles, 4, cudaMemcpyDeviceToDevice, s));
        APBF_CUDA(cudaMemcpyAsync(ctx->ext_len_transfers, ctx->d_len + kLenTransfers, 4, cudaMemcpyDeviceToDevice, s));
    }
    // a new state has no lambda history (the warm start's previous-substep feature)
    APBF_CUDA(cudaMemsetAsync(ctx->fl[ctx->fcur].lambda_prev, 0, (size_t)ctx->cfg.particle_capacity * sizeof(float), s));
    APBF_CUDA(cudaStreamSynchronize(s));
    return APBF_OK;
}

// Bytes per particle of the lists in apbf_host_fluid order.
static const size_t kFluidFieldBytes[11] = {16, 16, 4, 4, 16, 4, 4, 4, 4, 4, 4};

apbf_status apbf_fluid_write(apbf_ctx *ctx, const apbf_host_fluid *in, uint32_t count, void *stream) {
    if (!ctx || !in) return APBF_ERR_INVALID_ARG;
    if (count > ctx->cfg.particle_capacity) {
        set_error("apbf_fluid_write: count above the particle capacity");
        return APBF_ERR_INVALID_ARG;
    }
    cudaSetDevice(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    const FluidBufs &f = ctx->fl[ctx->fcur];
    void *const dev[] = {f.pos, f.vel, f.inv_mass, f.radius, f.pos_backup, f.transferring, f.target_radius,
                         f.kernel_width, f.boundariness, f.boundary_distance, f.lambda_prev};
    void *const host[] = {in->position,      in->velocity,    in->inverse_mass,      in->radius,
                          in->pos_backup,    in->transferring, in->target_radius,    in->kernel_width,
                          in->boundariness,  in->boundary_distance, in->lambda_prev};
    apbf_status r = apbf::copy_fluid_fields(ctx, dev, host, kFluidFieldBytes, 11, count, true, s);
    if (r != APBF_OK) return r;
    APBF_BEFORE_LAUNCH(ctx, s, "k_set_length");
    apbf::k_set_length<<<1, 1, 0, s>>>(ctx->d_len, kLenParticles, count);
    APBF_AFTER_LAUNCH(ctx, s, "k_set_length");
    return APBF_OK;
}

apbf_status apbf_fluid_read(apbf_ctx *ctx, apbf_host_fluid *out, uint32_t max_count, uint32_t *h_count, void *stream) {
    if (!ctx || !out || !h_count) return APBF_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    const FluidBufs &f = ctx->fl[ctx->fcur];
    const size_t n = std::min(max_count, ctx->cfg.particle_capacity);
    APBF_CUDA(cudaMemcpyAsync(h_count, ctx->d_len + kLenParticles, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    void *const dev[] = {f.pos, f.vel, f.inv_mass, f.radius, f.pos_backup, f.transferring, f.target_radius,
                         f.kernel_width, f.boundariness, f.boundary_distance, f.lambda_prev};
    void *const host[] = {out->position, out->velocity, out->inverse_mass, out->radius, out->pos_backup,
                          out->transferring, out->target_radius, out->kernel_width, out->boundariness,
                          out->boundary_distance, out->lambda_prev};
    return apbf::copy_fluid_fields(ctx, dev, host, kFluidFieldBytes, 11, n, false, s);
}

apbf_status apbf_get_lengths(apbf_ctx *ctx, uint32_t *np, uint32_t *nt, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    uint32_t v[2];
    cudaStream_t s = (cudaStream_t)stream;
    if (ctx->bound) {
        APBF_CUDA(cudaMemcpyAsync(v, ctx->ext_len_particles, 4, cudaMemcpyDeviceToHost, s));
        APBF_CUDA(cudaMemcpyAsync(v + 1, ctx->ext_len_transfers, 4, cudaMemcpyDeviceToHost, s));
    } else {
        APBF_CUDA(cudaMemcpyAsync(v, ctx->d_len, sizeof(v), cudaMemcpyDeviceToHost, s));
    }
    APBF_CUDA(cudaStreamSynchronize(s));
    if (np) *np = v[0];
    if (nt) *nt = v[1];
    return APBF_OK;
}

apbf_status apbf_velocity_handling_apply(apbf_ctx *ctx, float dt, const float acc[3], void *stream) {
    if (!ctx || !acc) return APBF_ERR_INVALID_ARG;
    APBF_BOUND_LENGTHS(ctx, (cudaStream_t)stream);
    return velocity_handling(ctx, dt, acc, (cudaStream_t)stream);
}

apbf_status apbf_neighborhood_green_apply(apbf_ctx *ctx, float range_scale, const float minp[3], const float maxp[3],
                                          uint32_t log2res, void *stream) {
    if (!ctx || !minp || !maxp) return APBF_ERR_INVALID_ARG;
    APBF_BOUND_LENGTHS(ctx, (cudaStream_t)stream);
    return neighborhood_green(ctx, range_scale, minp, maxp, log2res, (cudaStream_t)stream);
}

apbf_status apbf_box_collision_apply(apbf_ctx *ctx, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    APBF_BOUND_LENGTHS(ctx, (cudaStream_t)stream);
    return box_collision(ctx, (cudaStream_t)stream);
}

apbf_status apbf_incompressibility_apply(apbf_ctx *ctx, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    APBF_BOUND_LENGTHS(ctx, (cudaStream_t)stream);
    return incompressibility(ctx, (cudaStream_t)stream);
}

apbf_status apbf_kernel_width_from_boundary_distance_apply(apbf_ctx *ctx, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    APBF_BOUND_LENGTHS(ctx, (cudaStream_t)stream);
    return kw_from_boundary_distance(ctx, (cudaStream_t)stream);
}

apbf_status apbf_spread_kernel_width_apply(apbf_ctx *ctx, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    APBF_BOUND_LENGTHS(ctx, (cudaStream_t)stream);
    return spread_kernel_width(ctx, (cudaStream_t)stream);
}

apbf_status apbf_update_transfers_apply(apbf_ctx *ctx, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    APBF_BOUND_LENGTHS(ctx, (cudaStream_t)stream);
    return update_transfers(ctx, (cudaStream_t)stream);
}

apbf_status apbf_particle_transfer_apply(apbf_ctx *ctx, float dt, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    APBF_BOUND_LENGTHS(ctx, (cudaStream_t)stream);
    return particle_transfer(ctx, dt, (cudaStream_t)stream);
}

// pool::update (source/pool.cpp:67-106).
}  // extern "C"

namespace apbf {
// The body of pool::update (pool.cpp:67-106) on stream s.  capture: s is being
// captured into a substep graph, so the solve loop becomes a conditional node of
// that graph instead of a launch of its own.
apbf_status substep_body(apbf_ctx *ctx, float dt, cudaStream_t s, bool capture, SolveOpts *defer_loop,
                         bool *deferred) {
    if (deferred) *deferred = false;
    const apbf_settings &st = ctx->settings;
    apbf_status r = emit(ctx, dt, s);  // new particles first (no reference counterpart)
    if (r != APBF_OK) return r;
    r = velocity_handling(ctx, dt, ctx->scene.acceleration, s);
    if (r != APBF_OK) return r;
    const bool adaptive = !st.basic_pbf;
    if (adaptive && (st.merge || st.split)) {
        r = particle_transfer(ctx, dt, s);
        if (r != APBF_OK) return r;
    }
    if (adaptive && st.base_kernel_width_on_boundary_distance) {
        r = kw_from_boundary_distance(ctx, s);
        if (r != APBF_OK) return r;
    }
    const float scale = (st.basic_pbf || st.base_kernel_width_on_boundary_distance) ? 1.0f : 1.5f;
    // The box pass of each Jacobi iteration (pool.cpp:92-95) is fused into the kernel
    // before it: the neighbour-row build for the first iteration (not when
    // spread_kernel_width must still see the pre-box positions), the position
    // update of the previous iteration for the others.
    const bool spread = adaptive && !st.base_kernel_width_on_boundary_distance;
    const bool fuse_first = st.solver_iterations > 0 && !spread;
    if (ctx->search_method == APBF_NEIGHBORHOOD_BINARY_SEARCH)
        r = neighborhood_binary_search(ctx, scale, s, fuse_first);
    else
        r = neighborhood_green(ctx, scale, ctx->scene.min_pos, ctx->scene.max_pos,
                               ctx->tuning.search_log2res ? ctx->tuning.search_log2res : ctx->scene.log2res, s,
                               fuse_first, !spread);
    if (r != APBF_OK) return r;
    if (spread) {
        r = spread_kernel_width(ctx, s);
        if (r != APBF_OK) return r;
    }
    const bool converge = st.density_error_target > 0.0f;
    // cleared even without a target: the solve loop graph's condition reads it, and a
    // flag left by an earlier substep that had a target would end the loop early
    APBF_CUDA(cudaMemsetAsync(&ctx->status->converged, 0, sizeof(uint32_t), s));
    const bool recording = ctx->rec_iterations > 0;
    const bool learned = (ctx->warm_start & APBF_WARM_LEARNED) && ctx->mlp_loaded;
    const bool projected = (ctx->warm_start & APBF_WARM_PROJECTED) != 0;
    const bool track = ctx->track_lambda != 0;
    // Passes 1.. as one graph launch whose while loop stops on the device (at
    // convergence or after solver_iterations passes), instead of one launch pair per
    // possible pass; not while tracing, debugging or recording.
    const bool loop_graph = ctx->use_graphs && !ctx->prof_on && !ctx->debug && !recording &&
                            st.solver_iterations >= 2;
    for (int it = 0; it < st.solver_iterations; ++it) {
        if (it == 0 && !fuse_first) {
            r = box_collision(ctx, s);
            if (r != APBF_OK) return r;
        }
        SolveOpts o;
        o.box_after = it + 1 < st.solver_iterations;
        o.later_pass = it > 0;
        o.converge = converge;
        o.feature_mode = it == 0 && (learned || recording) ? 1 : 0;
        o.acc_mode = recording && (uint32_t)it < ctx->rec_iterations ? (it == 0 ? 1 : 2) : 0;
        o.learned = learned && it == 0;
        o.prev_mode = track ? (it == 0 ? 1 : 2) : 0;
        o.projected = projected;
        if (it == 1 && st.solver_iterations >= 2 && !recording) {
            SolveOpts q = o;
            q.max_passes = (uint32_t)st.solver_iterations;
            if (defer_loop && deferred && batch_solve_eligible(ctx, q)) {  // passes 1.. in the batch's launch
                *defer_loop = q;
                *deferred = true;
                return APBF_OK;
            }
            if (solve_persistent_eligible(ctx, q)) {  // passes 1.. in one persistent launch
                r = solve_persistent(ctx, s, q);
                if (r != APBF_OK) return r;
                break;
            }
        }
        if (it == 1 && loop_graph) {
            o.max_passes = (uint32_t)st.solver_iterations;
            r = capture ? solve_loop_captured(ctx, s, o) : solve_loop(ctx, s, o);
            if (r != APBF_OK) return r;
            break;
        }
        r = incompressibility(ctx, s, o);
        if (r != APBF_OK) return r;
    }
    return substep_post(ctx, s);
}

// The end of a substep after its Jacobi passes: sample recording, update_transfers.
apbf_status substep_post(apbf_ctx *ctx, cudaStream_t s) {
    const apbf_settings &st = ctx->settings;
    const bool adaptive = !st.basic_pbf;
    const bool recording = ctx->rec_iterations > 0;
    apbf_status r = APBF_OK;
    if (recording) {
        if (st.solver_iterations > 0) {
            r = record_samples(ctx, s);
            if (r != APBF_OK) return r;
        }
        ctx->rec_iterations = 0;  // armed for one substep
    }
    if (adaptive) {
        r = update_transfers(ctx, s);
        if (r != APBF_OK) return r;
    }
    return APBF_OK;
}

bool substep_graph_eligible(const apbf_ctx *ctx) {
    return ctx->use_graphs == 2 && !ctx->prof_on && !ctx->debug && ctx->rec_iterations == 0 &&
           ctx->settings.solver_iterations >= 2;
}
}  // namespace apbf

extern "C" {

apbf_status apbf_substep(apbf_ctx *ctx, float dt, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    if (ctx->scene.log2res < 1) {
        set_error("apbf_substep: call apbf_set_scene first");
        return APBF_ERR_INVALID_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    APBF_BOUND_LENGTHS(ctx, s);
    if (substep_graph_eligible(ctx)) return substep_graph(ctx, dt, s);
    return substep_body(ctx, dt, s, false);
}

apbf_status apbf_reduce_fp64(apbf_ctx *ctx, double out[4], void *stream) {
    if (!ctx || !out) return APBF_ERR_INVALID_ARG;
    APBF_BOUND_LENGTHS(ctx, (cudaStream_t)stream);
    return reduce_fp64(ctx, out, (cudaStream_t)stream);
}

namespace {
bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0u; }
}  // namespace

apbf_status apbf_bind_lists(apbf_ctx *ctx, const apbf_fluid_view fluid[2], const apbf_transfers_view transfers[2],
                            const apbf_neighbors_view *nb) {
    if (!ctx || !fluid || !transfers || !nb) return APBF_ERR_INVALID_ARG;
    if (ctx->bound) {
        set_error("apbf_bind_lists: lists already bound (apbf_unbind_lists first)");
        return APBF_ERR_INVALID_ARG;
    }
    for (int k = 0; k < 2; ++k) {
        const apbf_fluid_view &f = fluid[k];
        const apbf_transfers_view &t = transfers[k];
        const bool ok_f = f.capacity >= ctx->cfg.particle_capacity && f.d_length && f.d_length == fluid[0].d_length &&
                          f.position && f.velocity && f.inverse_mass && f.radius && f.pos_backup && f.transferring &&
                          f.target_radius && f.kernel_width && f.boundariness && f.boundary_distance &&
                          aligned16(f.position) && aligned16(f.velocity) && aligned16(f.pos_backup);
        const bool ok_t = t.capacity >= ctx->cfg.transfer_capacity && t.d_length &&
                          t.d_length == transfers[0].d_length && t.source && t.target && t.time_left;
        if (!ok_f || !ok_t) {
            set_error("apbf_bind_lists: two list sets with every attribute, capacities of at least the context's, one "
                      "length word per list, 16-byte aligned int4/float4 arrays");
            return APBF_ERR_INVALID_ARG;
        }
    }
    if (nb->row_stride != ctx->row_stride || nb->max_per_row < ctx->cfg.max_neighbors || !nb->count || !nb->index) {
        set_error("apbf_bind_lists: neighbour rows need the context's row_stride (apbf_neighbors_get_view) and at "
                  "least its max_neighbors entries per row");
        return APBF_ERR_INVALID_ARG;
    }
    APBF_CUDA(cudaSetDevice(ctx->device));
    APBF_CUDA(cudaDeviceSynchronize());  // no work of the context may still use its own lists
    for (int k = 0; k < 2; ++k) {
        ctx->own_fl[k] = ctx->fl[k];
        ctx->own_tr[k] = ctx->tr[k];
        FluidBufs &d = ctx->fl[k];
        const apbf_fluid_view &f = fluid[k];
        d.pos = (int4 *)f.position;
        d.vel = (float4 *)f.velocity;
        d.inv_mass = f.inverse_mass;
        d.radius = f.radius;
        d.pos_backup = (int4 *)f.pos_backup;
        d.transferring = f.transferring;
        d.target_radius = f.target_radius;
        d.kernel_width = f.kernel_width;
        d.boundariness = f.boundariness;
        d.boundary_distance = f.boundary_distance;  // lambda_prev stays the context's (warm-start history)
        ctx->tr[k].source = transfers[k].source;
        ctx->tr[k].target = transfers[k].target;
        ctx->tr[k].time_left = transfers[k].time_left;
    }
    ctx->fcur = 0;
    ctx->tcur = 0;
    ctx->own_nb_count = ctx->nb_count;
    ctx->own_nb_idx = ctx->nb_idx;
    ctx->nb_count = nb->count;
    ctx->nb_idx = nb->index;
    ctx->ext_len_particles = fluid[0].d_length;
    ctx->ext_len_transfers = transfers[0].d_length;
    destroy_substep_graphs(ctx);  // captured with the context's own buffers
    destroy_solve_graphs(ctx);
    ctx->graph_version++;
    ctx->bound = true;
    return APBF_OK;
}

apbf_status apbf_unbind_lists(apbf_ctx *ctx) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    if (!ctx->bound) return APBF_OK;
    APBF_CUDA(cudaSetDevice(ctx->device));
    APBF_CUDA(cudaDeviceSynchronize());
    for (int k = 0; k < 2; ++k) {
        ctx->fl[k] = ctx->own_fl[k];
        ctx->tr[k] = ctx->own_tr[k];
    }
    ctx->fcur = 0;
    ctx->tcur = 0;
    ctx->nb_count = ctx->own_nb_count;
    ctx->nb_idx = ctx->own_nb_idx;
    destroy_substep_graphs(ctx);
    destroy_solve_graphs(ctx);
    ctx->graph_version++;
    ctx->bound = false;
    return APBF_OK;
}

apbf_status apbf_set_wait_limit(apbf_ctx *ctx, uint32_t limit, int inject) {
    if (!ctx || (limit & kWaitInject)) {
        set_error("apbf_set_wait_limit: limit must be below 2^31");
        return APBF_ERR_INVALID_ARG;
    }
    const uint32_t v = limit | (inject ? kWaitInject : 0u);
    APBF_CUDA(cudaSetDevice(ctx->device));
    APBF_CUDA(cudaMemcpy(&ctx->status->wait_limit, &v, sizeof(v), cudaMemcpyHostToDevice));
    return APBF_OK;
}

apbf_status apbf_get_status(apbf_ctx *ctx, apbf_status_info *out, int clear, void *stream) {
    if (!ctx || !out) return APBF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    Status hs;
    unsigned long long pairs = 0;
    APBF_CUDA(cudaMemcpyAsync(&hs, ctx->status, sizeof(Status), cudaMemcpyDeviceToHost, s));
    APBF_CUDA(cudaMemcpyAsync(&pairs, ctx->d_pairs, sizeof(pairs), cudaMemcpyDeviceToHost, s));
    APBF_CUDA(cudaStreamSynchronize(s));
    out->flags = hs.flags;
    out->required_neighbors = hs.required_neighbors;
    out->required_transfers = hs.required_transfers;
    out->required_particles = hs.required_particles;
    out->pairs = pairs;
    out->density_passes = hs.density_passes;
    out->converged_substeps = hs.converged_substeps;
    out->spin_where = hs.spin_where;
    out->reserved = 0;
    if (clear) {
        Status z = hs;
        z.flags = 0;
        z.required_neighbors = z.required_transfers = z.required_particles = 0;
        z.spin_where = 0;
        z.density_passes = 0;
        z.converged_substeps = 0;
        APBF_CUDA(cudaMemcpyAsync(ctx->status, &z, sizeof(Status), cudaMemcpyHostToDevice, s));
        APBF_CUDA(cudaStreamSynchronize(s));
    }
    if (hs.flags & APBF_FLAG_SPIN_LIMIT) return APBF_ERR_SPIN_LIMIT;
    if (hs.flags & (APBF_FLAG_NEIGHBOR_OVERFLOW | APBF_FLAG_TRANSFER_OVERFLOW | APBF_FLAG_PARTICLE_OVERFLOW |
                    APBF_FLAG_GRID_OVERFLOW))
        return APBF_ERR_CAPACITY;
    if (hs.flags & APBF_FLAG_NONFINITE) return APBF_ERR_NONFINITE;
    return APBF_OK;
}

apbf_status apbf_export_pairs(apbf_ctx *ctx, uint32_t *d_pairs, uint32_t cap, uint32_t *d_length, void *stream) {
    if (!ctx || !d_pairs || !d_length) return APBF_ERR_INVALID_ARG;
    return export_pairs(ctx, d_pairs, cap, d_length, (cudaStream_t)stream);
}

apbf_status apbf_debug_incompressibility(apbf_ctx *ctx, uint32_t *d_density, int32_t *d_grad4, uint32_t *d_sq,
                                         float *d_lambda, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = ctx->cfg.particle_capacity;
    if (d_density) APBF_CUDA(cudaMemcpyAsync(d_density, ctx->dbg_density, n * 4, cudaMemcpyDeviceToDevice, s));
    if (d_grad4) APBF_CUDA(cudaMemcpyAsync(d_grad4, ctx->dbg_grad, n * 16, cudaMemcpyDeviceToDevice, s));
    if (d_sq) APBF_CUDA(cudaMemcpyAsync(d_sq, ctx->dbg_sq, n * 4, cudaMemcpyDeviceToDevice, s));
    if (d_lambda) APBF_CUDA(cudaMemcpyAsync(d_lambda, ctx->lambda, n * 4, cudaMemcpyDeviceToDevice, s));
    return APBF_OK;
}

apbf_status apbf_debug_sort(apbf_ctx *ctx, uint32_t *d_perm, uint32_t *d_keys, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = ctx->cfg.particle_capacity;
    if (d_perm) APBF_CUDA(cudaMemcpyAsync(d_perm, ctx->perm, n * 4, cudaMemcpyDeviceToDevice, s));
    if (d_keys) APBF_CUDA(cudaMemcpyAsync(d_keys, ctx->sorted_keys, n * 4, cudaMemcpyDeviceToDevice, s));
    return APBF_OK;
}

apbf_status apbf_profile_enable(apbf_ctx *ctx, int enable, uint32_t capacity) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (enable && capacity > ctx->prof.size()) {
        size_t old = ctx->prof.size();
        ctx->prof.resize(capacity);
        for (size_t i = old; i < capacity; ++i) {
            APBF_CUDA(cudaEventCreate(&ctx->prof[i].a));
            APBF_CUDA(cudaEventCreate(&ctx->prof[i].b));
            ctx->prof[i].name = "";
        }
    }
    ctx->prof_on = enable != 0;
    ctx->prof_used = 0;
    ctx->prof_dropped = 0;
    return APBF_OK;
}

apbf_status apbf_profile_read(apbf_ctx *ctx, apbf_kernel_time *out, uint32_t cap, uint32_t *n_out,
                              unsigned long long *dropped, void *stream) {
    if (!ctx || (!out && cap) || !n_out) return APBF_ERR_INVALID_ARG;
    APBF_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    std::vector<apbf_kernel_time> agg;
    for (size_t i = 0; i < ctx->prof_used; ++i) {
        float ms = 0.0f;
        APBF_CUDA(cudaEventElapsedTime(&ms, ctx->prof[i].a, ctx->prof[i].b));
        const char *nm = ctx->prof[i].name;
        size_t k = 0;
        for (; k < agg.size(); ++k)
            if (std::strncmp(agg[k].name, nm, sizeof(agg[k].name)) == 0) break;
        if (k == agg.size()) {
            apbf_kernel_time t;
            std::memset(&t, 0, sizeof(t));
            std::strncpy(t.name, nm, sizeof(t.name) - 1);
            agg.push_back(t);
        }
        agg[k].launches++;
        agg[k].total_ms += ms;
    }
    uint32_t m = (uint32_t)std::min<size_t>(agg.size(), cap);
    for (uint32_t k = 0; k < m; ++k) out[k] = agg[k];
    *n_out = m;
    if (dropped) *dropped = ctx->prof_dropped;
    ctx->prof_used = 0;
    ctx->prof_dropped = 0;
    return APBF_OK;
}

apbf_status apbf_launch_count(apbf_ctx *ctx, unsigned long long *out) {
    if (!ctx || !out) return APBF_ERR_INVALID_ARG;
    // kernels run by solve loop graphs: the body's kernel nodes per loop iteration
    uint32_t iters = 0;
    cudaSetDevice(ctx->device);
    APBF_CUDA(cudaMemcpy(&iters, &ctx->status->loop_iters, sizeof(iters), cudaMemcpyDeviceToHost));
    *out = ctx->launches + (unsigned long long)iters * ctx->loop_launches_per_iter;
    return APBF_OK;
}

apbf_status apbf_mlp_param_count(uint32_t *out) {
    if (!out) return APBF_ERR_INVALID_ARG;
    *out = (uint32_t)kMlpParams;
    return APBF_OK;
}

apbf_status apbf_mlp_partials_size(uint32_t n_samples, uint32_t *out_floats) {
    if (!out_floats) return APBF_ERR_INVALID_ARG;
    *out_floats = mlp_partials_floats(n_samples);
    return APBF_OK;
}

apbf_status apbf_mlp_load(apbf_ctx *ctx, const float *d_params, void *stream) {
    if (!ctx || !d_params) return APBF_ERR_INVALID_ARG;
    APBF_CUDA(cudaMemcpyAsync(ctx->mlp_params, d_params, kMlpParams * sizeof(float), cudaMemcpyDeviceToDevice,
                              (cudaStream_t)stream));
    apbf_status r = mlp_pack(ctx->mlp_params, ctx->mlp_image, (cudaStream_t)stream);
    if (r != APBF_OK) return r;
    ctx->mlp_loaded = 1;
    return APBF_OK;
}

apbf_status apbf_set_warm_start(apbf_ctx *ctx, int mode) {
    if (!ctx || (mode & ~(APBF_WARM_LEARNED | APBF_WARM_PROJECTED))) return APBF_ERR_INVALID_ARG;
    if ((mode & APBF_WARM_LEARNED) && !ctx->mlp_loaded) {
        set_error("apbf_set_warm_start: load the network with apbf_mlp_load first");
        return APBF_ERR_INVALID_ARG;
    }
    ctx->warm_start = mode;
    if (mode) ctx->track_lambda = 1;
    return APBF_OK;
}

apbf_status apbf_record_samples(apbf_ctx *ctx, uint32_t iterations, float *d_features, float *d_targets,
                                uint32_t capacity, uint32_t *d_count) {
    if (!ctx || !iterations || !d_features || !d_targets || !d_count) return APBF_ERR_INVALID_ARG;
    ctx->rec_iterations = iterations;
    ctx->rec_features = d_features;
    ctx->rec_targets = d_targets;
    ctx->rec_capacity = capacity;
    ctx->rec_count = d_count;
    ctx->track_lambda = 1;
    return APBF_OK;
}

apbf_status apbf_mlp_forward(const float *d_params, const float *d_features, uint32_t n, float *d_out, void *stream) {
    if (!d_params || (n && (!d_features || !d_out))) return APBF_ERR_INVALID_ARG;
    return mlp_forward(d_params, d_features, n, d_out, (cudaStream_t)stream);
}

apbf_status apbf_mlp_train_step(float *d_params, float *d_m, float *d_v, float *d_partials, const float *d_features,
                                const float *d_targets, uint32_t n, float lr, float over_weight, uint32_t step,
                                float *d_grad, float *d_loss, void *stream) {
    if (!d_params || !d_m || !d_v || !d_partials || (n && (!d_features || !d_targets)) || !(over_weight > 0.0f)) {
        set_error("apbf_mlp_train_step: null buffer or over_weight <= 0");
        return APBF_ERR_INVALID_ARG;
    }
    return mlp_train_step(d_params, d_m, d_v, d_partials, d_features, d_targets, n, lr, over_weight, step, d_grad,
                          d_loss, (cudaStream_t)stream);
}

static uint32_t bit_length(uint32_t v) {
    uint32_t b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

apbf_status apbf_sort_pairs(apbf_ctx *ctx, const uint32_t *d_keys, const uint32_t *d_values, const uint32_t *d_count,
                            uint32_t max_count, uint32_t value_upper_bound, uint32_t *d_out_keys,
                            uint32_t *d_out_values, void *stream) {
    if (!ctx || !d_keys || !d_values || !d_count || !d_out_keys || !d_out_values) return APBF_ERR_INVALID_ARG;
    if (max_count > ctx->cfg.particle_capacity) {
        set_error("apbf_sort_pairs: max_count above the context's particle capacity");
        return APBF_ERR_INVALID_ARG;
    }
    return sort_pairs_device(ctx, d_keys, d_values, d_count, max_count, bit_length(value_upper_bound), d_out_keys,
                             d_out_values, (cudaStream_t)stream);
}

apbf_status apbf_prefix_sum(apbf_ctx *ctx, uint32_t *d_values, const uint32_t *d_count, uint32_t max_count,
                            void *stream) {
    if (!ctx || !d_values || !d_count) return APBF_ERR_INVALID_ARG;
    if (max_count > ctx->cfg.particle_capacity) {
        set_error("apbf_prefix_sum: max_count above the context's particle capacity");
        return APBF_ERR_INVALID_ARG;
    }
    return prefix_sum_device(ctx, d_values, d_count, max_count, (cudaStream_t)stream);
}

}  // extern "C"
