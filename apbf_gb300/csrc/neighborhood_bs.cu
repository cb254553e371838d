// neighborhood_bs.cu -- neighborhood_binary_search::apply
// (source/neighborhood_binary_search.cpp:22-75), the reference's default search
// (shaders/cpu_gpu_shared_config.h:5).
//
//  1. k_code_word + sort_pairs_device, three times: stable sort of the particles by
//     the 96-bit interleave of their raw coordinates, least significant 32-bit word
//     first, so that ties keep the list order (neighborhood_binary_search.cpp:43-47,
//     calculate_position_code.comp:22-72).
//  2. reorder_particles: gather every attribute, remap the transfer and glue lists
//     (neighborhood_binary_search.cpp:49-50).
//  3. k_sorted_codes: the codes of the sorted particles (:52-56).
//  4. k_bs_rows: per particle, the 27 cells of edge 2^k around its own cell; each
//     cell's particles are one run of the sorted codes, found by a lower-bound search
//     (neighborhood_binary_search.comp:186-275).
//
// Canonical rules where the reference's arithmetic is not exact:
//  * the level k is the smallest with 2^k >= R, R the canonical fixed-point search
//    radius floor(kw * scale * 2^18) of the Green search, instead of
//    ceil(log2(range * 2^18)) in FP32 (comp:188): exact, and still cells at least R
//    wide, so the 27 cells hold every particle within R;
//  * the neighbour predicate is the Green search's exact integer one,
//    |x_j - x_i|^2 <= R^2, instead of an FP32 distance (comp:271);
//  * the lower bound is searched over the whole sorted list: the reference's
//    block-local shortcut (comp:104-108) can start inside a run of equal codes
//    that begins in an earlier block;
//  * at k = 31 each axis has two cells, so the offsets -1 and +1 name the same cell;
//    it is scanned once (the reference scans it twice and lists those neighbours
//    twice).
#include "apbf_internal.cuh"

namespace apbf {
namespace {

// Bits 0..20 of v moved to bits 0, 3, 6, ..., 60.
__device__ __forceinline__ unsigned long long spread21(uint32_t v) {
    unsigned long long x = v & 0x1fffffu;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

// Code bit 3b + a is bit b of axis a (x = 0, y = 1, z = 2), the coordinates taken as
// uint32 (calculate_position_code.comp:22-62).  .x holds code bits 0-63, .y bits 64-95.
__device__ __forceinline__ ulonglong2 code96(uint32_t x, uint32_t y, uint32_t z) {
    const unsigned long long lo = spread21(x) | spread21(y) << 1 | spread21(z) << 2;
    const unsigned long long t = spread21(x >> 21) | spread21(y >> 21) << 1 | spread21(z >> 21) << 2;
    return make_ulonglong2(lo | t << 63, t >> 1);
}

__device__ __forceinline__ bool less96(ulonglong2 a, ulonglong2 b) {
    return a.y < b.y || (a.y == b.y && a.x < b.x);
}

__device__ __forceinline__ uint32_t code_word(ulonglong2 c, uint32_t w) {
    return w == 0 ? (uint32_t)c.x : (w == 1 ? (uint32_t)(c.x >> 32) : (uint32_t)c.y);
}

// keys[k] = word w of the code of particle o, vals[k] = o, with o = order[k] (k when
// order is null).
__global__ void k_code_word(const int4 *__restrict__ pos, const uint32_t *d_len, uint32_t w,
                            const uint32_t *__restrict__ order, uint32_t *__restrict__ keys,
                            uint32_t *__restrict__ vals) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t o = order ? order[k] : k;
        const int4 p = pos[o];
        keys[k] = code_word(code96((uint32_t)p.x, (uint32_t)p.y, (uint32_t)p.z), w);
        if (vals) vals[k] = o;
    }
}

__global__ void k_sorted_codes(const int4 *__restrict__ pos, const uint32_t *d_len, ulonglong2 *__restrict__ code) {
    const uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 p = pos[i];
        code[i] = code96((uint32_t)p.x, (uint32_t)p.y, (uint32_t)p.z);
    }
}

__global__ void k_bs_reset(Status *st, unsigned long long *total) {
    st->range_min = 0xffffffffffffffffull;
    st->range_max = 0ull;
    *total = 0ull;
}

// First index j in [0, n) with code[j] >= t (n when none), searched outward from
// `hint` with doubling steps and then bisected: cells near a particle are mostly
// near it in the sorted order.
__device__ __forceinline__ uint32_t lower_bound96(const ulonglong2 *__restrict__ code, uint32_t n, uint32_t hint,
                                                  ulonglong2 t) {
    uint32_t lo, hi;  // the answer lies in [lo, hi]
    if (less96(code[hint], t)) {
        uint32_t a = hint, step = 1;  // code[a] < t
        for (;;) {
            const uint32_t b = step <= n - 1 - a ? a + step : n;  // index to probe, or n
            if (b >= n) {
                lo = a + 1;
                hi = n;
                break;
            }
            if (!less96(code[b], t)) {
                lo = a + 1;
                hi = b;
                break;
            }
            a = b;
            step <<= 1;
        }
    } else {
        uint32_t b = hint, step = 1;  // code[b] >= t
        for (;;) {
            if (b == 0) {
                lo = hi = 0;
                break;
            }
            const uint32_t a = b > step ? b - step : 0;
            if (less96(code[a], t)) {
                lo = a + 1;
                hi = b;
                break;
            }
            b = a;
            step <<= 1;
        }
    }
    while (lo < hi) {  // bisect: code[hi] >= t (or hi == n), code[lo - 1] < t
        const uint32_t mid = lo + (hi - lo) / 2;
        if (less96(code[mid], t))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

struct BsArgs {
    const int4 *pos;
    int4 *pos_box;  // when non-null: receives box_collision(pos) (the first Jacobi iteration's box pass)
    const ulonglong2 *code;
    const float *range;
    const float *radius;
    const float4 *bmin, *bmax, *rot;
    uint32_t nboxes;
    float scale;
    const uint32_t *d_len;
    uint32_t stride, maxn;
    uint32_t *count, *idx;
    unsigned long long *total;
    Status *st;
};

// neighborhood_binary_search.comp:180-275, one thread per particle.
__global__ void __launch_bounds__(256) k_bs_rows(BsArgs a) {
    const uint32_t n = a.d_len[kLenParticles];
    unsigned long long local = 0;
    long long rmin = 0x7fffffffffffffffll, rmax = -1;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 p = a.pos[i];
        const long long R = range_fixed(a.range[i], a.scale);
        uint32_t c = 0;
        if (R < 0) {
            set_flag(a.st, APBF_FLAG_NONFINITE);  // NaN or negative kernel width: no neighbours
        } else {
            rmin = R < rmin ? R : rmin;
            rmax = R > rmax ? R : rmax;
            // level: smallest k with 2^k >= R (R < 2^31, so k <= 31)
            const uint32_t k = R <= 1 ? 0u : 32u - (uint32_t)__clz((uint32_t)(R - 1));
            const uint32_t d3 = 3u * k;  // the code bits below the cell
            const ulonglong2 m96 = make_ulonglong2(d3 >= 64 ? ~0ull : (1ull << d3) - 1ull,
                                                   d3 > 64 ? (1ull << (d3 - 64)) - 1ull : 0ull);
            const uint32_t top = k == 31 ? 1u : 2u;  // at k = 31 the offset +1 is the offset -1
            const uint32_t ux = (uint32_t)p.x >> k, uy = (uint32_t)p.y >> k, uz = (uint32_t)p.z >> k;
            for (uint32_t dz = 0; dz <= top; ++dz)
                for (uint32_t dy = 0; dy <= top; ++dy)
                    for (uint32_t dx = 0; dx <= top; ++dx) {
                        // the corner of the cell, wrapping modulo 2^32 like the code arithmetic
                        const ulonglong2 first = code96((ux + dx - 1u) << k, (uy + dy - 1u) << k, (uz + dz - 1u) << k);
                        const ulonglong2 last = make_ulonglong2(first.x | m96.x, first.y | m96.y);
                        for (uint32_t j = lower_bound96(a.code, n, i, first); j < n; ++j) {
                            if (less96(last, a.code[j])) break;
                            if (j == i || !within(p, a.pos[j], R)) continue;
                            if (c < a.maxn) a.idx[(size_t)c * a.stride + i] = j;
                            ++c;
                        }
                    }
        }
        if (c > a.maxn) {
            set_flag(a.st, APBF_FLAG_NEIGHBOR_OVERFLOW);
            atomicMax(&a.st->required_neighbors, c);
        }
        a.count[i] = c < a.maxn ? c : a.maxn;
        local += c < a.maxn ? c : a.maxn;
        if (a.pos_box) a.pos_box[i] = box_push(p, a.radius[i], i, a.bmin, a.bmax, a.rot, a.nboxes);
    }
    for (int off = 16; off > 0; off >>= 1) {
        local += __shfl_down_sync(0xffffffffu, local, off);
        const long long a2 = __shfl_down_sync(0xffffffffu, rmin, off);
        const long long c2 = __shfl_down_sync(0xffffffffu, rmax, off);
        rmin = a2 < rmin ? a2 : rmin;
        rmax = c2 > rmax ? c2 : rmax;
    }
    if ((threadIdx.x & 31) == 0) {
        if (local) atomicAdd(a.total, local);
        if (rmax >= 0) {
            atomicMin(&a.st->range_min, (unsigned long long)rmin);
            atomicMax(&a.st->range_max, (unsigned long long)rmax);
        }
    }
}

}  // namespace

apbf_status neighborhood_binary_search(apbf_ctx *ctx, float range_scale, cudaStream_t s, bool fuse_box) {
    const uint32_t cap = ctx->cfg.particle_capacity;
    const int g = grid_for(ctx, cap);
    // three stable passes, least significant word first
    for (uint32_t w = 0; w < 3; ++w) {
        const FluidBufs &cur = ctx->fl[ctx->fcur];
        APBF_BEFORE_LAUNCH(ctx, s, "k_code_word");
        k_code_word<<<g, kBlock, 0, s>>>(cur.pos, ctx->d_len, w, w ? ctx->perm : nullptr, ctx->keys[0],
                                         ctx->vals[0]);
        APBF_AFTER_LAUNCH(ctx, s, "k_code_word");
        apbf_status r = sort_pairs_device(ctx, ctx->keys[0], ctx->vals[0], ctx->d_len + kLenParticles, cap, 32u,
                                          ctx->sorted_keys, ctx->perm, s);
        if (r != APBF_OK) return r;
    }
    apbf_status r = reorder_particles(ctx, s);
    if (r != APBF_OK) return r;
    FluidBufs &f = ctx->fl[ctx->fcur];
    APBF_BEFORE_LAUNCH(ctx, s, "k_sorted_codes");
    k_sorted_codes<<<g, kBlock, 0, s>>>(f.pos, ctx->d_len, ctx->pos_code);
    APBF_AFTER_LAUNCH(ctx, s, "k_sorted_codes");
    APBF_BEFORE_LAUNCH(ctx, s, "k_bs_reset");
    k_bs_reset<<<1, 1, 0, s>>>(ctx->status, ctx->d_pairs);
    APBF_AFTER_LAUNCH(ctx, s, "k_bs_reset");
    FluidBufs &spare = ctx->fl[ctx->fcur ^ 1];
    BsArgs a;
    a.pos = f.pos;
    a.pos_box = fuse_box ? spare.pos : nullptr;
    a.code = ctx->pos_code;
    a.range = f.kernel_width;
    a.radius = f.radius;
    a.bmin = ctx->box_min;
    a.bmax = ctx->box_max;
    a.rot = ctx->box_rot;
    a.nboxes = ctx->n_boxes;
    a.scale = range_scale;
    a.d_len = ctx->d_len;
    a.stride = ctx->row_stride;
    a.maxn = ctx->cfg.max_neighbors;
    a.count = ctx->nb_count;
    a.idx = ctx->nb_idx;
    a.total = ctx->d_pairs;
    a.st = ctx->status;
    APBF_BEFORE_LAUNCH(ctx, s, "k_bs_rows");
    k_bs_rows<<<grid_for(ctx, cap, kBlock, 8), kBlock, 0, s>>>(a);
    APBF_AFTER_LAUNCH(ctx, s, "k_bs_rows");
    if (fuse_box) {  // the box-collided positions are the current ones now
        int4 *t = f.pos;
        f.pos = spare.pos;
        spare.pos = t;
    }
    return build_reverse_rows(ctx, s);
}

}  // namespace apbf

using namespace apbf;

extern "C" {

apbf_status apbf_neighborhood_binary_search_apply(apbf_ctx *ctx, float range_scale, void *stream) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    return neighborhood_binary_search(ctx, range_scale, (cudaStream_t)stream);
}

apbf_status apbf_calculate_position_code(apbf_ctx *ctx, const uint32_t *d_index_list, uint32_t code_section,
                                         uint32_t *d_out, void *stream) {
    if (!ctx || !d_out || code_section > 2) {
        set_error("calculate_position_code: needs an output and a code section in 0..2");
        return APBF_ERR_INVALID_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const FluidBufs &f = ctx->fl[ctx->fcur];
    APBF_BEFORE_LAUNCH(ctx, s, "k_code_word");
    k_code_word<<<grid_for(ctx, ctx->cfg.particle_capacity), kBlock, 0, s>>>(f.pos, ctx->d_len, code_section,
                                                                              d_index_list, d_out, nullptr);
    APBF_AFTER_LAUNCH(ctx, s, "k_code_word");
    return APBF_OK;
}

apbf_status apbf_set_neighborhood_search(apbf_ctx *ctx, int method) {
    if (!ctx) return APBF_ERR_INVALID_ARG;
    if (method != APBF_NEIGHBORHOOD_GREEN && method != APBF_NEIGHBORHOOD_BINARY_SEARCH) {
        set_error("set_neighborhood_search: the method is APBF_NEIGHBORHOOD_GREEN or APBF_NEIGHBORHOOD_BINARY_SEARCH");
        return APBF_ERR_INVALID_ARG;
    }
    if (method != ctx->search_method) ctx->graph_version++;  // captured substeps hold the search
    ctx->search_method = method;
    return APBF_OK;
}

}  // extern "C"
