// sort.cu -- parallel primitives: stable LSD radix sort of (key, value) pairs and
// inclusive prefix sum, both single-pass per digit / per scan with decoupled
// look-back between tiles.
//
// Replaces algorithms::sort (source/algorithms.cpp:59-91, 4-bit digits, three
// dispatches per digit plus a recursive scan) and algorithms::prefix_sum
// (source/algorithms.cpp:93-118, recursive three-kernel block scan).
//
// Radix sort: one histogram kernel counts the digits of every pass in one read of
// the keys; then one kernel per 8-bit digit ranks a tile of 4096 keys (8 warps x
// 16 keys per lane, warp-striped so loads coalesce), publishes the tile's digit
// counts, looks back over earlier tiles for its global offsets and scatters.
// Stability: inside a warp the keys are ranked in index order with
// __match_any_sync; warps are combined in index order; tiles in tile order.
// Every wait on another tile is bounded (kSpinLimit) and records
// APBF_FLAG_SPIN_LIMIT instead of hanging.
#include <algorithm>
#include <mutex>

#include "apbf_internal.cuh"

namespace apbf {
namespace {

constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagIncl = 2u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1u;

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) { return *(const volatile uint32_t *)p; }
__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v) { *(volatile uint32_t *)p = v; }

// Digit widths of the radix sort (bits per pass); the tuner picks one per context.
constexpr int kMaxSortPasses = 6;  // 32-bit keys at 6-bit digits

// Counts the BITS-bit digits of every pass.  hist: passes x 2^BITS.
template <int BITS>
__global__ void __launch_bounds__(256) k_sort_hist(const uint32_t *__restrict__ keys, const uint32_t *d_count,
                                                   uint32_t max_count, uint32_t key_mask, int passes,
                                                   uint32_t *__restrict__ hist) {
    constexpr uint32_t NB = 1u << BITS;
    constexpr int PM = (32 + BITS - 1) / BITS;
    __shared__ uint32_t sh[PM][NB];
    for (uint32_t q = threadIdx.x; q < PM * NB; q += blockDim.x) (&sh[0][0])[q] = 0u;
    __syncthreads();
    uint32_t n = min(*d_count, max_count);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t k = keys[i] & key_mask;
        for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][(k >> (BITS * p)) & (NB - 1u)], 1u);
    }
    __syncthreads();
    for (int p = 0; p < passes; ++p)
        for (uint32_t b = threadIdx.x; b < NB; b += blockDim.x)
            if (sh[p][b]) atomicAdd(&hist[p * NB + b], sh[p][b]);
}

// One BITS-bit digit pass.  tile_status: tiles x 2^BITS words (flag << 30 | count).
// Thread t < 2^BITS owns digit t.
template <int BITS>
__global__ void __launch_bounds__(256) k_onesweep(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                                                  uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                  const uint32_t *d_count, uint32_t max_count, uint32_t key_mask,
                                                  int shift, const uint32_t *__restrict__ hist,
                                                  uint32_t *tile_counter, uint32_t *tile_status, Status *st) {
    constexpr uint32_t NB = 1u << BITS;
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_cnt[kSortWarps][NB];
    __shared__ uint32_t s_base[NB];
    __shared__ uint32_t s_scan[NB];

    const int t = threadIdx.x, w = t >> 5, l = t & 31;
    const bool owner = (uint32_t)t < NB;
    if (t == 0) s_tile = atomicAdd(tile_counter, 1u);
    if (owner)
        for (int k = 0; k < kSortWarps; ++k) s_cnt[k][t] = 0u;
    // exclusive scan of the global digit histogram (same in every tile)
    const uint32_t hist_t = owner ? hist[t] : 0u;
    if (owner) s_scan[t] = hist_t;
    __syncthreads();
    for (uint32_t off = 1; off < NB; off <<= 1) {
        uint32_t v = (owner && (uint32_t)t >= off) ? s_scan[t - off] : 0u;
        __syncthreads();
        if (owner) s_scan[t] += v;
        __syncthreads();
    }
    const uint32_t digit_excl = owner ? s_scan[t] - hist_t : 0u;

    const uint32_t n = min(*d_count, max_count);
    const uint32_t ntiles = (n + kSortTile - 1) / kSortTile;
    const uint32_t tile = s_tile;
    if (tile >= ntiles) return;

    const uint32_t base = tile * kSortTile + (uint32_t)w * (32 * kSortItems);
    uint32_t keys[kSortItems], vals[kSortItems], rank[kSortItems];
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        uint32_t idx = base + k * 32 + l;
        bool valid = idx < n;
        keys[k] = valid ? kin[idx] : 0u;
        vals[k] = valid ? vin[idx] : 0u;
    }
    const uint32_t lt = (1u << l) - 1u;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        uint32_t idx = base + k * 32 + l;
        bool valid = idx < n;
        uint32_t d = valid ? ((keys[k] & key_mask) >> shift) & (NB - 1u) : NB + (uint32_t)l;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = valid ? s_cnt[w][d] : 0u;
        rank[k] = before + __popc(peers & lt);
        __syncwarp();
        if (valid && (__ffs(peers) - 1) == l) s_cnt[w][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // thread t owns digit t: warp exclusive offsets and the tile total
    uint32_t run = 0;
    if (owner) {
#pragma unroll
        for (int k = 0; k < kSortWarps; ++k) {
            uint32_t c = s_cnt[k][t];
            s_cnt[k][t] = run;
            run += c;
        }
    }
    uint32_t *my = tile_status + (size_t)tile * NB + t;
    uint32_t excl = 0;
    if (!owner) {
    } else if (tile == 0) {
        st_volatile(my, kFlagIncl | run);
    } else {
        st_volatile(my, kFlagAgg | run);
        int j = (int)tile - 1;
        uint32_t spins = 0;
        bool inject;
        const uint32_t limit = wait_limit(st, kSpinLimit, inject);
        while (j >= 0) {
            uint32_t v = ld_volatile(tile_status + (size_t)j * NB + t);
            uint32_t f = inject ? 0u : (v & ~kValMask);
            if (f == 0u) {
                if (++spins > limit) {
                    set_flag(st, APBF_FLAG_SPIN_LIMIT);
                    st->spin_where = 1u;
                    break;
                }
                __nanosleep(32);
                continue;
            }
            excl += v & kValMask;
            if (f == kFlagIncl) break;
            --j;
        }
        st_volatile(my, kFlagIncl | ((excl + run) & kValMask));
    }
    if (owner) s_base[t] = digit_excl + excl;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        uint32_t idx = base + k * 32 + l;
        if (idx < n) {
            uint32_t d = ((keys[k] & key_mask) >> shift) & (NB - 1u);
            uint32_t pos = s_base[d] + s_cnt[w][d] + rank[k];
            kout[pos] = keys[k];
            vout[pos] = vals[k];
        }
    }
}

// Single-pass inclusive scan with decoupled look-back; tile = 256 threads x 16.
constexpr int kScanItems = 16;
constexpr int kScanTile = 256 * kScanItems;

__global__ void __launch_bounds__(256) k_scan(uint32_t *data, const uint32_t *d_count, uint32_t max_count,
                                              uint32_t *tile_counter, uint32_t *tile_status, Status *st) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[8];
    __shared__ uint32_t s_excl;
    const int t = threadIdx.x, w = t >> 5, l = t & 31;
    if (t == 0) s_tile = atomicAdd(tile_counter, 1u);
    __syncthreads();
    const uint32_t n = min(*d_count, max_count);
    const uint32_t ntiles = (n + kScanTile - 1) / kScanTile;
    const uint32_t tile = s_tile;
    if (tile >= ntiles) return;
    // blocked arrangement: thread t owns items [t*16, t*16+16) of the tile
    const uint32_t base = tile * kScanTile + (uint32_t)t * kScanItems;
    uint32_t v[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        uint32_t idx = base + k;
        v[k] = idx < n ? data[idx] : 0u;
        sum += v[k];
        v[k] = sum;  // thread-local inclusive
    }
    // block exclusive scan of thread sums
    uint32_t x = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (l >= off) x += y;
    }
    if (l == 31) s_warp[w] = x;
    __syncthreads();
    if (t < 32) {
        uint32_t ws = t < 8 ? s_warp[t] : 0u;
        uint32_t wi = ws;
#pragma unroll
        for (int off = 1; off < 8; off <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, wi, off);
            if (t >= off) wi += y;
        }
        if (t < 8) s_warp[t] = wi - ws;  // exclusive warp offsets
        uint32_t total = __shfl_sync(0xffffffffu, wi, 7);
        if (t == 0) {
            uint32_t excl = 0;
            uint32_t *my = tile_status + tile;
            if (tile == 0) {
                st_volatile(my, kFlagIncl | (total & kValMask));
            } else {
                st_volatile(my, kFlagAgg | (total & kValMask));
                int j = (int)tile - 1;
                uint32_t spins = 0;
                bool inject;
                const uint32_t limit = wait_limit(st, kSpinLimit, inject);
                while (j >= 0) {
                    uint32_t s = ld_volatile(tile_status + j);
                    uint32_t f = inject ? 0u : (s & ~kValMask);
                    if (f == 0u) {
                        if (++spins > limit) {
                            set_flag(st, APBF_FLAG_SPIN_LIMIT);
                            st->spin_where = 2u;
                            break;
                        }
                        __nanosleep(32);
                        continue;
                    }
                    excl += s & kValMask;
                    if (f == kFlagIncl) break;
                    --j;
                }
                st_volatile(my, kFlagIncl | ((excl + total) & kValMask));
            }
            s_excl = excl;
        }
    }
    __syncthreads();
    const uint32_t off = s_excl + s_warp[w] + (x - sum);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        uint32_t idx = base + k;
        if (idx < n) data[idx] = v[k] + off;
    }
}

}  // namespace

// Stable sort by the low key_bits bits of the keys (rounded up to whole 4-bit
// digits exactly as the reference's pass loop, algorithms.cpp:73).
apbf_status sort_pairs_device(apbf_ctx *ctx, const uint32_t *keys_in, const uint32_t *vals_in, const uint32_t *d_count,
                              uint32_t max_count, uint32_t key_bits, uint32_t *keys_out, uint32_t *vals_out,
                              cudaStream_t s) {
    if (max_count == 0) return APBF_OK;
    if (max_count >= (1u << 30)) return APBF_ERR_INVALID_ARG;
    uint32_t nib = (key_bits + 3u) / 4u;  // 4-bit subkeys the reference would sort
    if (nib > 8u) nib = 8u;
    uint32_t bits = nib * 4u;
    uint32_t key_mask = bits >= 32u ? 0xffffffffu : ((1u << bits) - 1u);
    const uint32_t dbits = ctx->tuning.sort_digit_bits == 6u || ctx->tuning.sort_digit_bits == 7u
                               ? ctx->tuning.sort_digit_bits
                               : 8u;  // digit width: the tuner's choice, 8 by default
    const uint32_t nb = 1u << dbits;
    int passes = (int)((bits + dbits - 1u) / dbits);
    uint32_t tiles = (max_count + kSortTile - 1) / kSortTile;
    if (tiles > ctx->sort_tiles) return APBF_ERR_INVALID_ARG;
    if (passes == 0) {
        APBF_CUDA(cudaMemcpyAsync(keys_out, keys_in, (size_t)max_count * 4, cudaMemcpyDeviceToDevice, s));
        APBF_CUDA(cudaMemcpyAsync(vals_out, vals_in, (size_t)max_count * 4, cudaMemcpyDeviceToDevice, s));
        return APBF_OK;
    }
    // scratch: hist passes x nb <= 4 x 256 words, status passes x tiles x nb <= 4 x tiles x 256
    APBF_CUDA(cudaMemsetAsync(ctx->sort_hist, 0, (size_t)passes * nb * sizeof(uint32_t), s));
    APBF_CUDA(cudaMemsetAsync(ctx->sort_counters, 0, 8 * sizeof(uint32_t), s));
    APBF_CUDA(cudaMemsetAsync(ctx->sort_status, 0, (size_t)passes * tiles * nb * sizeof(uint32_t), s));
    APBF_BEFORE_LAUNCH(ctx, s, "k_sort_hist");
    const int hgrid = grid_for(ctx, max_count, 256, 4);
    if (dbits == 6u)
        k_sort_hist<6><<<hgrid, 256, 0, s>>>(keys_in, d_count, max_count, key_mask, passes, ctx->sort_hist);
    else if (dbits == 7u)
        k_sort_hist<7><<<hgrid, 256, 0, s>>>(keys_in, d_count, max_count, key_mask, passes, ctx->sort_hist);
    else
        k_sort_hist<8><<<hgrid, 256, 0, s>>>(keys_in, d_count, max_count, key_mask, passes, ctx->sort_hist);
    APBF_AFTER_LAUNCH(ctx, s, "k_sort_hist");
    // Ping-pong between the output (A) and scratch (B) so that the last pass lands
    // in the output: pass p writes A when (passes - 1 - p) is even.  An input that
    // aliases the output is first copied to a second scratch buffer.
    const uint32_t *src_k = keys_in, *src_v = vals_in;
    if (keys_in == keys_out || vals_in == vals_out || keys_in == vals_out || vals_in == keys_out) {
        APBF_CUDA(cudaMemcpyAsync(ctx->keys[0], keys_in, (size_t)max_count * 4, cudaMemcpyDeviceToDevice, s));
        APBF_CUDA(cudaMemcpyAsync(ctx->vals[0], vals_in, (size_t)max_count * 4, cudaMemcpyDeviceToDevice, s));
        src_k = ctx->keys[0];
        src_v = ctx->vals[0];
    }
    for (int p = 0; p < passes; ++p) {
        bool to_out = ((passes - 1 - p) & 1) == 0;
        uint32_t *dk = to_out ? keys_out : ctx->keys[1];
        uint32_t *dv = to_out ? vals_out : ctx->vals[1];
        APBF_BEFORE_LAUNCH(ctx, s, "k_onesweep");
        const int sh = (int)dbits * p;
        uint32_t *hp = ctx->sort_hist + p * nb, *tp = ctx->sort_status + (size_t)p * tiles * nb;
        if (dbits == 6u)
            k_onesweep<6><<<tiles, 256, 0, s>>>(src_k, src_v, dk, dv, d_count, max_count, key_mask, sh, hp,
                                                ctx->sort_counters + p, tp, ctx->status);
        else if (dbits == 7u)
            k_onesweep<7><<<tiles, 256, 0, s>>>(src_k, src_v, dk, dv, d_count, max_count, key_mask, sh, hp,
                                                ctx->sort_counters + p, tp, ctx->status);
        else
            k_onesweep<8><<<tiles, 256, 0, s>>>(src_k, src_v, dk, dv, d_count, max_count, key_mask, sh, hp,
                                                ctx->sort_counters + p, tp, ctx->status);
        APBF_AFTER_LAUNCH(ctx, s, "k_onesweep");
        src_k = dk;
        src_v = dv;
    }
    if (src_k != keys_out) {
        APBF_CUDA(cudaMemcpyAsync(keys_out, src_k, (size_t)max_count * 4, cudaMemcpyDeviceToDevice, s));
        APBF_CUDA(cudaMemcpyAsync(vals_out, src_v, (size_t)max_count * 4, cudaMemcpyDeviceToDevice, s));
    }
    return APBF_OK;
}

apbf_status prefix_sum_device(apbf_ctx *ctx, uint32_t *d_values, const uint32_t *d_count, uint32_t max_count,
                              cudaStream_t s) {
    if (max_count == 0) return APBF_OK;
    if (max_count >= (1u << 30)) return APBF_ERR_INVALID_ARG;
    uint32_t tiles = (max_count + kScanTile - 1) / kScanTile;
    if (tiles > ctx->sort_tiles * 256u) return APBF_ERR_INVALID_ARG;
    APBF_CUDA(cudaMemsetAsync(ctx->sort_counters + 7, 0, sizeof(uint32_t), s));
    APBF_CUDA(cudaMemsetAsync(ctx->sort_status, 0, (size_t)tiles * sizeof(uint32_t), s));
    APBF_BEFORE_LAUNCH(ctx, s, "k_scan");
    k_scan<<<tiles, 256, 0, s>>>(d_values, d_count, max_count, ctx->sort_counters + 7, ctx->sort_status, ctx->status);
    APBF_AFTER_LAUNCH(ctx, s, "k_scan");
    return APBF_OK;
}

}  // namespace apbf

// ---------------------------------------------------------------------------
// Allocation-free variant of the stable radix sort (apbf_sort_pairs_noalloc).
//
// Some callers cannot call cudaMalloc: a host whose device memory belongs to
// another allocator, or a per-frame path on which cudaMalloc / cudaFree would
// synchronise the device and stall the frame.  For them this entry point keeps
// its scratch (the second key/value buffer, digit histograms, tile counters and
// look-back words) in one file-scope device array of fixed size, so a call needs
// no context and allocates nothing.  Every device that loads the library holds
// the array (about 9 MB) until the process exits.
namespace apbf {
namespace {

constexpr uint32_t kNoAllocMax = 1u << 20;  // largest max_count accepted
constexpr uint32_t kNoAllocTiles = (kNoAllocMax + kSortTile - 1) / kSortTile;

struct NoAllocScratch {
    uint32_t keys[kNoAllocMax];
    uint32_t vals[kNoAllocMax];
    uint32_t hist[4 * 256];
    uint32_t counters[8];
    uint32_t tile_status[4 * kNoAllocTiles * 256];
    Status status;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

constexpr int kMaxDevices = 64;
NoAllocScratch *g_noalloc_addr[kMaxDevices] = {};
int g_noalloc_sms[kMaxDevices] = {};
std::mutex g_noalloc_mutex;

// Device address of the scratch array on the current device (looked up once per
// device; a host-side use of g_noalloc_scratch would name host memory).
apbf_status noalloc_scratch(int dev, NoAllocScratch **out, int *sms) {
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("apbf_sort_pairs_noalloc: device ordinal out of range");
        return APBF_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return cuda_check(e, "cudaDeviceGetAttribute");
        g_noalloc_addr[dev] = (NoAllocScratch *)p;
        g_noalloc_sms[dev] = n;
    }
    *out = g_noalloc_addr[dev];
    *sms = g_noalloc_sms[dev];
    return APBF_OK;
}

}  // namespace
}  // namespace apbf

extern "C" apbf_status apbf_sort_pairs_noalloc(const uint32_t *d_keys, const uint32_t *d_values,
                                               const uint32_t *d_count, uint32_t max_count,
                                               uint32_t value_upper_bound, uint32_t *d_out_keys,
                                               uint32_t *d_out_values, void *stream) {
    using namespace apbf;
    if (!d_keys || !d_values || !d_count || !d_out_keys || !d_out_values) {
        set_error("apbf_sort_pairs_noalloc: null pointer");
        return APBF_ERR_INVALID_ARG;
    }
    if (max_count > kNoAllocMax) {
        set_error("apbf_sort_pairs_noalloc: max_count above the fixed scratch size of 1048576 elements");
        return APBF_ERR_INVALID_ARG;
    }
    {  // each output range [p, p + 4 max_count) must overlap no other buffer's range
        const uintptr_t bytes = (uintptr_t)max_count * 4u;
        auto overlap = [bytes](const void *x, const void *y) {
            const uintptr_t a = (uintptr_t)x, b = (uintptr_t)y;
            return bytes != 0 && a < b + bytes && b < a + bytes;
        };
        if (overlap(d_out_keys, d_out_values) || overlap(d_out_keys, d_keys) || overlap(d_out_keys, d_values) ||
            overlap(d_out_values, d_keys) || overlap(d_out_values, d_values)) {
            set_error("apbf_sort_pairs_noalloc: an output overlaps an input or the other output");
            return APBF_ERR_INVALID_ARG;
        }
    }
    if (max_count == 0) return APBF_OK;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_check(e, "cudaGetDevice");
    NoAllocScratch *sc = nullptr;
    int sms = 0;
    apbf_status r = noalloc_scratch(dev, &sc, &sms);
    if (r != APBF_OK) return r;
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t bits = 0;
    for (uint32_t v = value_upper_bound; v; v >>= 1) ++bits;
    uint32_t nib = (bits + 3u) / 4u;
    if (nib > 8u) nib = 8u;
    bits = nib * 4u;
    const uint32_t key_mask = bits >= 32u ? 0xffffffffu : ((1u << bits) - 1u);
    const int passes = (int)((bits + 7u) / 8u);
    const uint32_t tiles = (max_count + kSortTile - 1) / kSortTile;
    if (passes == 0) {
        APBF_CUDA(cudaMemcpyAsync(d_out_keys, d_keys, (size_t)max_count * 4, cudaMemcpyDeviceToDevice, s));
        APBF_CUDA(cudaMemcpyAsync(d_out_values, d_values, (size_t)max_count * 4, cudaMemcpyDeviceToDevice, s));
        return APBF_OK;
    }
    // the array keeps the previous call's contents: clear what must start at zero
    APBF_CUDA(cudaMemsetAsync(sc->hist, 0, sizeof(sc->hist), s));
    APBF_CUDA(cudaMemsetAsync(sc->counters, 0, sizeof(sc->counters), s));
    APBF_CUDA(cudaMemsetAsync(sc->tile_status, 0, (size_t)passes * tiles * 256 * sizeof(uint32_t), s));
    APBF_CUDA(cudaMemsetAsync(&sc->status, 0, sizeof(Status), s));
    uint64_t need = ((uint64_t)max_count + 255) / 256;
    const int hist_grid = (int)std::min<uint64_t>(std::max<uint64_t>(need, 1), (uint64_t)sms * 4);
    k_sort_hist<8><<<hist_grid, 256, 0, s>>>(d_keys, d_count, max_count, key_mask, passes, sc->hist);
    APBF_CUDA(cudaGetLastError());
    const uint32_t *src_k = d_keys, *src_v = d_values;
    for (int p = 0; p < passes; ++p) {
        const bool to_out = ((passes - 1 - p) & 1) == 0;
        uint32_t *dk = to_out ? d_out_keys : sc->keys;
        uint32_t *dv = to_out ? d_out_values : sc->vals;
        k_onesweep<8><<<tiles, 256, 0, s>>>(src_k, src_v, dk, dv, d_count, max_count, key_mask, 8 * p,
                                         sc->hist + p * 256, sc->counters + p,
                                         sc->tile_status + (size_t)p * tiles * 256, &sc->status);
        APBF_CUDA(cudaGetLastError());
        src_k = dk;
        src_v = dv;
    }
    return APBF_OK;
}
