// listedit.cu -- the reference's list-edit engine as device services on plain
// device arrays (gpu_list / indexed_list, source/gpu_list.h and indexed_list.h):
// apply an edit list, build the edit list of a deletion or a duplication, remap an
// index list after its hidden list was edited, append one list to another.  The
// substep uses its own fused forms of these; the services are for other callers.
//
// The reference remaps index lists with atomic_swap.comp chains and an atomic
// counter in generate_new_index_and_edit_list.comp, so the order of the result is
// not defined; here it is canonical (rule C8): by new hidden index, then by the
// old position in the index list -- obtained with the stable radix sort, so the
// results are deterministic and equal the oracle's.
#include <algorithm>

#include "apbf_internal.cuh"

namespace apbf {
namespace {

__global__ void k_le_apply(const uint32_t *__restrict__ src, uint32_t stride, const uint32_t *__restrict__ edit,
                           const uint32_t *d_len, uint32_t max_len, uint32_t *__restrict__ dst) {
    const uint32_t m = d_len ? min(*d_len, max_len) : max_len;
    const uint64_t words = (uint64_t)m * stride;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < words; w += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t e = w / stride, o = w % stride;
        dst[w] = src[(uint64_t)edit[e] * stride + o];
    }
}

__global__ void k_le_fill(uint32_t *a, uint32_t n, uint32_t v) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}

__global__ void k_le_mark(const uint32_t *del, const uint32_t *d_del_len, uint32_t max_del, uint32_t n_hidden,
                          uint32_t *flags) {
    const uint32_t m = min(*d_del_len, max_del);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x)
        if (del[k] < n_hidden) flags[del[k]] = 0u;
}

// find_value_changes.comp:15-28 on the inclusive scan of the survivor flags
__global__ void k_le_survivors(const uint32_t *scan, uint32_t n_hidden, uint32_t *edit, uint32_t *d_edit_len) {
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n_hidden; id += gridDim.x * blockDim.x) {
        const uint32_t cur = scan[id], prev = id ? scan[id - 1] : 0u;
        if (cur != prev) edit[prev] = id;
        if (id == n_hidden - 1) *d_edit_len = cur;
    }
    if (n_hidden == 0 && blockIdx.x == 0 && threadIdx.x == 0) *d_edit_len = 0u;
}

__global__ void k_le_keys(const uint32_t *list, const uint32_t *d_len, uint32_t max_len, uint32_t n_hidden,
                          uint32_t *keys, uint32_t *vals) {
    const uint32_t m = min(*d_len, max_len);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < max_len; p += gridDim.x * blockDim.x) {
        keys[p] = p < m && list[p] < n_hidden ? list[p] : n_hidden;  // out of range: sorted last, ignored
        vals[p] = p;
    }
}

// [start, end) of every hidden id in the sorted keys (find_value_ranges.comp)
__global__ void k_le_ranges(const uint32_t *skeys, const uint32_t *d_len, uint32_t max_len, uint32_t n_hidden,
                            uint32_t *start, uint32_t *end) {
    const uint32_t m = min(*d_len, max_len);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < m; p += gridDim.x * blockDim.x) {
        const uint32_t cur = skeys[p], prev = p ? skeys[p - 1] : 0xffffffffu;
        if (cur >= n_hidden) continue;
        if (p == 0 || cur != prev) start[cur] = p;
        if (p == m - 1 || skeys[p + 1] != cur) end[cur] = p + 1;
    }
}

__global__ void k_le_counts(const uint32_t *edit, const uint32_t *d_edit_len, uint32_t max_edit, uint32_t n_hidden,
                            const uint32_t *start, const uint32_t *end, uint32_t *cnt) {
    const uint32_t m = min(*d_edit_len, max_edit);
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < max_edit; e += gridDim.x * blockDim.x) {
        const uint32_t h = e < m ? edit[e] : n_hidden;
        cnt[e] = h < n_hidden ? end[h] - start[h] : 0u;
    }
}

__global__ void k_le_emit(const uint32_t *edit, const uint32_t *d_edit_len, uint32_t max_edit, uint32_t n_hidden,
                          const uint32_t *start, const uint32_t *scan, const uint32_t *spos, uint32_t out_cap,
                          uint32_t *out, uint32_t *new_edit, uint32_t *d_out_len, uint32_t *d_required) {
    const uint32_t m = min(*d_edit_len, max_edit);
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x) {
        const uint32_t h = edit[e];
        const uint32_t c = scan[e] - (e ? scan[e - 1] : 0u);
        const uint32_t o = scan[e] - c;
        for (uint32_t t = 0; t < c; ++t) {
            if (o + t >= out_cap) break;
            out[o + t] = e;
            if (new_edit) new_edit[o + t] = spos[start[h] + t];
        }
        if (e == m - 1) {
            const uint32_t total = scan[e];
            *d_out_len = total < out_cap ? total : out_cap;
            if (d_required) *d_required = total;
        }
    }
    if (m == 0 && blockIdx.x == 0 && threadIdx.x == 0) {
        *d_out_len = 0u;
        if (d_required) *d_required = 0u;
    }
}

__global__ void k_le_append(uint32_t *dst, uint32_t *d_dst_len, const uint32_t *src, const uint32_t *d_src_len,
                            uint32_t stride, uint32_t dst_cap, uint32_t *d_base) {
    // one pass: every thread reads the old length; the last block's first thread
    // would race with the reads, so the new length is written by a second kernel
    const uint32_t n0 = *d_dst_len, m = *d_src_len;
    const uint32_t room = dst_cap > n0 ? dst_cap - n0 : 0u;
    const uint32_t k = m < room ? m : room;
    const uint64_t words = (uint64_t)k * stride;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < words; w += (uint64_t)gridDim.x * blockDim.x)
        dst[(uint64_t)n0 * stride + w] = src[w];
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_base = n0 + k;
}

__global__ void k_le_set_len(uint32_t *d_len, const uint32_t *v) { *d_len = *v; }

}  // namespace
}  // namespace apbf

using namespace apbf;

static apbf_status le_scratch(apbf_ctx *ctx, uint32_t need) {
    if (need > ctx->cfg.particle_capacity) {
        set_error("list services: lengths above the context's particle capacity");
        return APBF_ERR_INVALID_ARG;
    }
    if (!ctx->le_buf) {
        const size_t cap = ctx->cfg.particle_capacity + 1;
        APBF_CUDA(cudaMalloc(&ctx->le_buf, 6 * cap * sizeof(uint32_t)));
    }
    return APBF_OK;
}

extern "C" apbf_status apbf_list_apply_edit(const uint32_t *d_src, uint32_t stride_words, const uint32_t *d_edit,
                                            const uint32_t *d_edit_len, uint32_t max_edit, uint32_t *d_dst,
                                            void *stream) {
    if (!d_src || !d_edit || !d_dst || !stride_words || d_src == d_dst) return APBF_ERR_INVALID_ARG;
    if (!max_edit) return APBF_OK;
    const uint64_t words = (uint64_t)max_edit * stride_words;
    const int blocks = (int)std::min<uint64_t>((words + 255) / 256, 4096);
    k_le_apply<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_src, stride_words, d_edit, d_edit_len, max_edit, d_dst);
    APBF_CUDA(cudaGetLastError());
    return APBF_OK;
}

extern "C" apbf_status apbf_list_delete_edit(apbf_ctx *ctx, const uint32_t *d_deleted, const uint32_t *d_deleted_len,
                                             uint32_t max_deleted, uint32_t n_hidden, uint32_t *d_edit,
                                             uint32_t *d_edit_len, void *stream) {
    if (!ctx || !d_edit || !d_edit_len || (max_deleted && (!d_deleted || !d_deleted_len))) return APBF_ERR_INVALID_ARG;
    apbf_status r = le_scratch(ctx, n_hidden);
    if (r != APBF_OK) return r;
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t *flags = ctx->le_buf;
    uint32_t *len = ctx->le_buf + 5 * (size_t)(ctx->cfg.particle_capacity + 1);
    const int g = grid_for(ctx, n_hidden ? n_hidden : 1);
    k_le_fill<<<g, kBlock, 0, s>>>(flags, n_hidden, 1u);
    if (max_deleted) k_le_mark<<<grid_for(ctx, max_deleted), kBlock, 0, s>>>(d_deleted, d_deleted_len, max_deleted,
                                                                              n_hidden, flags);
    APBF_CUDA(cudaGetLastError());
    APBF_CUDA(cudaMemcpyAsync(len, &n_hidden, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    r = prefix_sum_device(ctx, flags, len, n_hidden, s);
    if (r != APBF_OK) return r;
    k_le_survivors<<<g, kBlock, 0, s>>>(flags, n_hidden, d_edit, d_edit_len);
    APBF_CUDA(cudaGetLastError());
    APBF_CUDA(cudaStreamSynchronize(s));  // `len` is a host value copied by the call
    return APBF_OK;
}

extern "C" apbf_status apbf_list_remap_index(apbf_ctx *ctx, const uint32_t *d_list, const uint32_t *d_list_len,
                                             uint32_t max_list, const uint32_t *d_edit, const uint32_t *d_edit_len,
                                             uint32_t max_edit, uint32_t n_hidden_old, uint32_t *d_out,
                                             uint32_t *d_new_edit, uint32_t out_cap, uint32_t *d_out_len,
                                             uint32_t *d_required, void *stream) {
    if (!ctx || !d_list || !d_list_len || !d_edit || !d_edit_len || !d_out || !d_out_len) return APBF_ERR_INVALID_ARG;
    apbf_status r = le_scratch(ctx, std::max(std::max(max_list, max_edit), n_hidden_old + 1));
    if (r != APBF_OK) return r;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t cap = ctx->cfg.particle_capacity + 1;
    uint32_t *keys = ctx->le_buf, *vals = keys + cap, *start = vals + cap, *end = start + cap, *cnt = end + cap;
    uint32_t *sk = ctx->list_a, *sv = ctx->list_b;  // sorted pairs (substep scratch, free between substeps)
    k_le_fill<<<grid_for(ctx, n_hidden_old + 1), kBlock, 0, s>>>(start, n_hidden_old + 1, 0u);
    k_le_fill<<<grid_for(ctx, n_hidden_old + 1), kBlock, 0, s>>>(end, n_hidden_old + 1, 0u);
    if (max_list) {
        k_le_keys<<<grid_for(ctx, max_list), kBlock, 0, s>>>(d_list, d_list_len, max_list, n_hidden_old, keys, vals);
        APBF_CUDA(cudaGetLastError());
        uint32_t bits = 1;
        while (bits < 32 && (1ull << bits) <= n_hidden_old) ++bits;
        r = sort_pairs_device(ctx, keys, vals, d_list_len, max_list, bits, sk, sv, s);
        if (r != APBF_OK) return r;
        k_le_ranges<<<grid_for(ctx, max_list), kBlock, 0, s>>>(sk, d_list_len, max_list, n_hidden_old, start, end);
    }
    if (max_edit) {
        k_le_counts<<<grid_for(ctx, max_edit), kBlock, 0, s>>>(d_edit, d_edit_len, max_edit, n_hidden_old, start, end,
                                                              cnt);
        APBF_CUDA(cudaGetLastError());
        r = prefix_sum_device(ctx, cnt, d_edit_len, max_edit, s);
        if (r != APBF_OK) return r;
    }
    k_le_emit<<<grid_for(ctx, max_edit ? max_edit : 1), kBlock, 0, s>>>(d_edit, d_edit_len, max_edit, n_hidden_old,
                                                                        start, cnt, sv, out_cap, d_out, d_new_edit,
                                                                        d_out_len, d_required);
    APBF_CUDA(cudaGetLastError());
    return APBF_OK;
}

extern "C" apbf_status apbf_list_append(uint32_t *d_dst, uint32_t *d_dst_len, uint32_t dst_cap, const uint32_t *d_src,
                                        const uint32_t *d_src_len, uint32_t max_src, uint32_t stride_words,
                                        uint32_t *d_scratch_word, void *stream) {
    if (!d_dst || !d_dst_len || !d_src || !d_src_len || !stride_words || !d_scratch_word) return APBF_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t words = (uint64_t)std::max(max_src, 1u) * stride_words;
    const int blocks = (int)std::min<uint64_t>((words + 255) / 256, 4096);
    k_le_append<<<blocks, 256, 0, s>>>(d_dst, d_dst_len, d_src, d_src_len, stride_words, dst_cap, d_scratch_word);
    k_le_set_len<<<1, 1, 0, s>>>(d_dst_len, d_scratch_word);
    APBF_CUDA(cudaGetLastError());
    return APBF_OK;
}
