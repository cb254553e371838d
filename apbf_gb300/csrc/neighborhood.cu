// neighborhood.cu -- neighborhood_green::apply (source/neighborhood_green.cpp:27-77).
//
//  1. k_position_keys: Morton key of each particle's grid cell
//     (calculate_position_hash.comp:23-46; canonical integer cell mapping).
//  2. sort_pairs_device: stable sort of (key, particle id).
//  3. k_reorder: gather every particle attribute into the alternate buffer set and
//     swap (hidden_list().apply_edit + mParticles->sort(), neighborhood_green.cpp:54-56),
//     remap the transfer list (indexed_list.h:288-308).
//  4. k_cell_ranges: [start, end) of every occupied cell (find_value_ranges.comp).
//  5. k_build_rows: per particle, walk the cells overlapping [X - R, X + R] and keep
//     every other particle within R (neighborhood_green.comp:49-87), written
//     column-major so that consecutive particles' k-th entries are contiguous.
//     When the search radii differ it also writes correction rows into the
//     reverse-row arrays (the rare one-sided pairs), so that the position-update
//     pass gathers over the particle's own row plus its corrections instead of
//     scattering with atomics, and no transpose is needed.
//  6. k_reverse_rows (binary-search rows and pruned rows): the transpose.
#include <algorithm>

#include "apbf_internal.cuh"

namespace apbf {
namespace {

struct Bounds {
    long long lo[3];
    long long hi[3];
};

Bounds fixed_bounds(const float minp[3], const float maxp[3]) {
    Bounds b;
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = llround((double)minp[d] * 262144.0);
        b.hi[d] = llround((double)maxp[d] * 262144.0);
        if (b.hi[d] <= b.lo[d]) b.hi[d] = b.lo[d] + 1;
    }
    return b;
}

__global__ void k_position_keys(const int4 *__restrict__ pos, const uint32_t *d_len, Bounds b, uint32_t L,
                                uint32_t *__restrict__ keys, uint32_t *__restrict__ seq) {
    uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int4 p = pos[i];
        uint32_t cx = cell_coord(p.x, b.lo[0], b.hi[0], L);
        uint32_t cy = cell_coord(p.y, b.lo[1], b.hi[1], L);
        uint32_t cz = cell_coord(p.z, b.lo[2], b.hi[2], L);
        keys[i] = morton3(cx, cy, cz);
        seq[i] = i;
    }
}

// Gather of every attribute by the sort permutation (copy_scattered_read.comp).
// With srec non-null it also writes each particle's search record (position xyz,
// fixed-point search radius R = range_fixed(kw, scale) in w, -1 for a NaN or
// negative width) and reduces the radii's range into the status block, so that the
// row build knows before it starts whether every radius is equal.
__global__ void k_reorder(FluidBufs src, FluidBufs dst, const uint32_t *__restrict__ perm,
                          uint32_t *__restrict__ inv_perm, const uint32_t *d_len, int4 *__restrict__ srec,
                          float scale, Status *st) {
    uint32_t n = d_len[kLenParticles];
    long long rmin = 0x7fffffffffffffffll, rmax = -1;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        uint32_t o = perm[k];
        int4 p = src.pos[o];
        p.w = __float_as_int(1.0f / src.inv_mass[o]);  // the solver's per-particle mass (position.w is reserved)
        dst.pos[k] = p;
        dst.vel[k] = src.vel[o];
        dst.inv_mass[k] = src.inv_mass[o];
        dst.radius[k] = src.radius[o];
        dst.pos_backup[k] = src.pos_backup[o];
        dst.transferring[k] = src.transferring[o];
        dst.target_radius[k] = src.target_radius[o];
        dst.kernel_width[k] = src.kernel_width[o];
        dst.boundariness[k] = src.boundariness[o];
        dst.lambda_prev[k] = src.lambda_prev[o];
        dst.boundary_distance[k] = src.boundary_distance[o];
        inv_perm[o] = k;
        if (srec) {
            const long long R = range_fixed(src.kernel_width[o], scale);
            srec[k] = make_int4(p.x, p.y, p.z, (int)R);
            if (R >= 0) {
                rmin = R < rmin ? R : rmin;
                rmax = R > rmax ? R : rmax;
            }
        }
    }
    if (!srec) return;  // uniform over the grid
    for (int off = 16; off > 0; off >>= 1) {
        const long long a2 = __shfl_down_sync(0xffffffffu, rmin, off);
        const long long c2 = __shfl_down_sync(0xffffffffu, rmax, off);
        rmin = a2 < rmin ? a2 : rmin;
        rmax = c2 > rmax ? c2 : rmax;
    }
    if ((threadIdx.x & 31) == 0 && rmax >= 0) {
        atomicMin(&st->range_min, (unsigned long long)rmin);
        atomicMax(&st->range_max, (unsigned long long)rmax);
    }
}

__global__ void k_remap_transfers(TransferBufs t, const uint32_t *__restrict__ inv_perm, const uint32_t *d_len,
                                  Status *st) {
    const uint32_t nt = d_len[kLenTransfers], n = d_len[kLenParticles];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
        const uint32_t s = t.source[k], g = t.target[k];
        if (s >= n || g >= n) {  // a transfer naming a particle that does not exist
            set_flag(st, APBF_FLAG_NONFINITE);
            continue;
        }
        t.source[k] = inv_perm[s];
        t.target[k] = inv_perm[g];
    }
}

// find_value_ranges.comp:15-31 (cell arrays zeroed beforehand).
__global__ void k_cell_ranges(const uint32_t *__restrict__ skeys, const uint32_t *d_len, uint32_t *__restrict__ start,
                              uint32_t *__restrict__ end) {
    uint32_t n = d_len[kLenParticles];
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += gridDim.x * blockDim.x) {
        uint32_t cur = skeys[id];
        uint32_t prev = id == 0 ? cur : skeys[id - 1];
        if (id == 0 || cur != prev) start[cur] = id;
        if (id != 0 && cur != prev) end[prev] = id;
        if (id == n - 1) end[cur] = id + 1u;
    }
}

// Exact 32-bit form of `within` for particles that both lie inside the grid
// (coordinates differ by less than 2^31): the same predicate, half the
// instructions.  R2 = R * R.
__device__ __forceinline__ bool within32(int4 a, int4 b, uint32_t R, unsigned long long R2) {
    const uint32_t ax = (uint32_t)abs(b.x - a.x), ay = (uint32_t)abs(b.y - a.y), az = (uint32_t)abs(b.z - a.z);
    if (max(ax, max(ay, az)) > R) return false;
    const unsigned long long s = (unsigned long long)ax * ax + (unsigned long long)ay * ay + (unsigned long long)az * az;
    return s <= R2;
}

struct BuildArgs {
    const int4 *pos;
    int4 *pos_box;  // when non-null: receives box_collision(pos) (the first Jacobi iteration's box pass)
    const float *range;
    const float *radius;
    const float4 *bmin, *bmax, *rot;
    uint32_t nboxes;
    float scale;
    const uint32_t *d_len;
    Bounds b;
    uint32_t L;
    int fast_ok;  // the grid spans less than 2^31 units on every axis
    const uint32_t *cstart, *cend;
    uint32_t stride, maxn;
    uint32_t *count, *idx;
    unsigned long long *total;
    Status *st;
    const int4 *srec;         // per particle: position xyz and fixed-point search radius R (w)
    uint32_t *ucount, *uidx;  // correction rows (the reverse-row arrays), when the radii differ
    uint32_t *one_sided;      // per particle: one-sided pairs of its row (radii that differ)
    int corrections;          // 0: no correction rows (the caller transposes pruned rows next)
};

// Appends an entry to a correction row (the reverse-row arrays; their counts were
// zeroed before the walk, and any walk may append, so the slot is an atomic).
__device__ __forceinline__ void push_correction(const BuildArgs &a, uint32_t row, uint32_t entry) {
    const uint32_t slot = atomicAdd(&a.ucount[row], 1u);
    if (slot < a.maxn) {
        a.uidx[(size_t)slot * a.stride + row] = entry;
    } else {
        set_flag(a.st, APBF_FLAG_NEIGHBOR_OVERFLOW);
        atomicMax(&a.st->required_neighbors, slot + 1u);
    }
}

// Squared distance of two fixed-point positions when no axis differs by more than R
// (else ~0: the pair is beyond R whatever the other axes).  FAST: both lie inside
// the grid, so the 32-bit differences cannot wrap.
template <bool FAST>
__device__ __forceinline__ unsigned long long dist2_within(int4 a, int4 b, uint32_t R) {
    uint32_t ax, ay, az;
    if (FAST) {
        ax = (uint32_t)abs(b.x - a.x);
        ay = (uint32_t)abs(b.y - a.y);
        az = (uint32_t)abs(b.z - a.z);
    } else {
        long long dx = (long long)b.x - a.x, dy = (long long)b.y - a.y, dz = (long long)b.z - a.z;
        dx = dx < 0 ? -dx : dx;
        dy = dy < 0 ? -dy : dy;
        dz = dz < 0 ? -dz : dz;
        if (dx > (long long)R || dy > (long long)R || dz > (long long)R) return ~0ull;
        ax = (uint32_t)dx;
        ay = (uint32_t)dy;
        az = (uint32_t)dz;
    }
    if (max(ax, max(ay, az)) > R) return ~0ull;
    return (unsigned long long)ax * ax + (unsigned long long)ay * ay + (unsigned long long)az * az;
}

// Walks the cells [x0, x1] x [y0, y1] x [z0, z1] and appends every neighbour of
// particle i: j != i with |x_j - x_i| <= R_i (the neighbour predicate, C2).  The
// walk is a chain of dependent loads (cell range -> candidates), so the ranges of
// up to four cells of one (z, y) row are loaded together and candidates four at a
// time.
//
// Correction rows (UNI, when the search radii differ): the position update of
// particle i sums over the particles k whose rows hold i (|x_i - x_k| <= R_k),
// and its deferred boundariness filter tests i's own row.  It sums over i's own
// row and then over i's correction row: entries j of i's row whose radius does not
// reach i (flagged kNoDelta, their terms subtracted), and particles k whose rows
// hold i although i's radius does not reach them (added).  Both kinds are one-sided
// pairs, found here (one_sided counts them) and appended after the walk.
template <bool FAST>
__device__ __forceinline__ uint32_t walk_cells(const BuildArgs &a, uint32_t i, int4 p, long long R, uint32_t x0,
                                               uint32_t x1, uint32_t y0, uint32_t y1, uint32_t z0, uint32_t z1,
                                               bool uni, uint32_t &one_sided) {
    const uint32_t R32 = (uint32_t)R;
    const unsigned long long R2 = (unsigned long long)R32 * R32;
    uint32_t c = 0;
    for (uint32_t cz = z0; cz <= z1; ++cz)
        for (uint32_t cy = y0; cy <= y1; ++cy) {
            const uint32_t yz = (spread3(cy) << 1) | (spread3(cz) << 2);
            for (uint32_t cx0 = x0; cx0 <= x1; cx0 += 4) {
                uint32_t cs[4], ce[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const bool in = cx0 + v <= x1;
                    const uint32_t key = yz | spread3(cx0 + v);
                    cs[v] = in ? a.cstart[key] : 0u;
                    ce[v] = in ? a.cend[key] : 0u;
                }
#pragma unroll 1  // one copy of the candidate loop: the kernel is bound by its instruction cache
                for (int v = 0; v < 4; ++v) {
                    const uint32_t s = cs[v], e = ce[v];
                    for (uint32_t j0 = s; j0 < e; j0 += 4) {
                        int4 q[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) q[u] = j0 + u < e ? a.srec[j0 + u] : p;
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const uint32_t j = j0 + u;
                            if (j >= e || j == i) continue;
                            const unsigned long long d2 = dist2_within<FAST>(p, q[u], R32);
                            if (d2 > R2) continue;
                            if (uni) {
                                const unsigned long long Rj = (unsigned long long)(uint32_t)max(q[u].w, 0);
                                one_sided += (q[u].w >= 0 && d2 <= Rj * Rj) ? 0u : 1u;
                            }
                            if (c < a.maxn) a.idx[(size_t)c * a.stride + i] = j;
                            ++c;
                        }
                    }
                }
            }
        }
    return c;
}

// box_push as a call: the walk's kernel is bound by its instruction cache, and the
// box pass runs once per particle.
__device__ __noinline__ int4 box_push_call(int4 ip, float r, uint32_t id, const float4 *__restrict__ bmin,
                                           const float4 *__restrict__ bmax, const float4 *__restrict__ rot,
                                           uint32_t nb) {
    return box_push(ip, r, id, bmin, bmax, rot, nb);
}

// The one-sided pairs of the rows just built (radii that differ; particles whose
// walk counted some): found again on the particle's row, i's correction row
// subtracts j, j's adds i.  A kernel of its own, so that the walk holds no atomics.
__global__ void k_corrections(BuildArgs a) {
    if (!a.corrections || a.st->range_min == a.st->range_max) return;  // none wanted, or nothing one-sided
    const uint32_t n = a.d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!a.one_sided[i]) continue;
        const int4 p = a.srec[i];
        const uint32_t m = a.count[i];
        for (uint32_t k = 0; k < m; ++k) {
            const uint32_t j = a.idx[(size_t)k * a.stride + i];
            const int4 q = a.srec[j];
            const unsigned long long Rj = (unsigned long long)(uint32_t)max(q.w, 0);
            if (q.w >= 0 && dist2_within<false>(p, q, (uint32_t)Rj) <= Rj * Rj) continue;
            push_correction(a, i, j | kNoDelta);
            push_correction(a, j, i);
        }
    }
}

// neighborhood_green.comp:49-87 with the canonical predicate (C2), one thread per
// particle, candidates read from the search records.  A box that touches no edge
// cell of the grid only meets particles inside the grid (edge cells also hold the
// clamped outsiders), so it uses the 32-bit differences.
__global__ void __launch_bounds__(256, 4) k_build_rows(BuildArgs a) {
    const uint32_t n = a.d_len[kLenParticles];
    const uint32_t last = (1u << a.L) - 1u;
    const bool uni = a.corrections && a.st->range_min != a.st->range_max;  // the radii differ: correction rows
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st->union_rows = uni ? 1u : 0u;
    unsigned long long local = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 p = a.srec[i];
        const long long R = p.w;
        uint32_t c = 0;
        if (R < 0) {
            set_flag(a.st, APBF_FLAG_NONFINITE);  // NaN or negative kernel width: no neighbours
        } else {
            const Bounds &b = a.b;
            const uint32_t x0 = cell_coord((long long)p.x - R, b.lo[0], b.hi[0], a.L);
            const uint32_t x1 = cell_coord((long long)p.x + R, b.lo[0], b.hi[0], a.L);
            const uint32_t y0 = cell_coord((long long)p.y - R, b.lo[1], b.hi[1], a.L);
            const uint32_t y1 = cell_coord((long long)p.y + R, b.lo[1], b.hi[1], a.L);
            const uint32_t z0 = cell_coord((long long)p.z - R, b.lo[2], b.hi[2], a.L);
            const uint32_t z1 = cell_coord((long long)p.z + R, b.lo[2], b.hi[2], a.L);
            const bool fast = a.fast_ok && x0 > 0 && y0 > 0 && z0 > 0 && x1 < last && y1 < last && z1 < last;
            uint32_t one_sided = 0;
            c = fast ? walk_cells<true>(a, i, p, R, x0, x1, y0, y1, z0, z1, uni, one_sided)
                     : walk_cells<false>(a, i, p, R, x0, x1, y0, y1, z0, z1, uni, one_sided);
            if (uni) a.one_sided[i] = one_sided;  // k_corrections appends them
        }
        if (c > a.maxn) {
            set_flag(a.st, APBF_FLAG_NEIGHBOR_OVERFLOW);
            atomicMax(&a.st->required_neighbors, c);
        }
        a.count[i] = c < a.maxn ? c : a.maxn;
        local += c < a.maxn ? c : a.maxn;
        if (a.pos_box) a.pos_box[i] = box_push_call(a.pos[i], a.radius[i], i, a.bmin, a.bmax, a.rot, a.nboxes);
    }
    for (int off = 16; off > 0; off >>= 1) local += __shfl_down_sync(0xffffffffu, local, off);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(a.total, local);
}

__global__ void k_reverse_rows(const uint32_t *d_len, uint32_t stride, uint32_t maxn, const uint32_t *__restrict__ count,
                               const uint32_t *__restrict__ idx, uint32_t *__restrict__ rcount,
                               uint32_t *__restrict__ ridx, Status *st) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st->union_rows = 0u;
    if (st->range_min == st->range_max) return;  // symmetric rows: reverse = forward
    uint32_t n = d_len[kLenParticles];
    // four entries per batch: their slot atomics are in flight together (the slots'
    // order within a reverse row is arbitrary either way, and the position update's
    // integer sums do not depend on it)
    constexpr uint32_t U = 4;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t c = count[i];
        for (uint32_t k0 = 0; k0 < c; k0 += U) {
            uint32_t j[U], slot[U];
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) j[u] = k0 + u < c ? idx[(size_t)(k0 + u) * stride + i] : 0u;
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) slot[u] = k0 + u < c ? atomicAdd(&rcount[j[u]], 1u) : 0u;
#pragma unroll
            for (uint32_t u = 0; u < U; ++u) {
                if (k0 + u >= c) break;
                if (slot[u] < maxn) {
                    ridx[(size_t)slot[u] * stride + j[u]] = i;
                } else {
                    set_flag(st, APBF_FLAG_NEIGHBOR_OVERFLOW);
                    atomicMax(&st->required_neighbors, slot[u] + 1u);
                }
            }
        }
    }
}

__global__ void k_clamp_rev(const uint32_t *d_len, uint32_t maxn, uint32_t *rcount, Status *st) {
    if (st->range_min == st->range_max) return;
    uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (rcount[i] > maxn) rcount[i] = maxn;
}

__global__ void k_reset_search(Status *st, unsigned long long *total) {
    st->range_min = 0xffffffffffffffffull;
    st->range_max = 0ull;
    *total = 0ull;
}

// Pair export (the reference's uvec2 list): row-major order of the rows.
__global__ void k_export_pairs(const uint32_t *d_len, uint32_t stride, const uint32_t *__restrict__ count,
                               const uint32_t *__restrict__ idx, const uint32_t *__restrict__ offsets, uint32_t cap,
                               uint2 *__restrict__ out) {
    uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t c = count[i];
        uint32_t o = offsets[i] - c;  // inclusive scan -> row start
        for (uint32_t k = 0; k < c; ++k)
            if (o + k < cap) out[o + k] = make_uint2(i, idx[(size_t)k * stride + i]);
    }
}

__global__ void k_export_len(const uint32_t *d_len, const uint32_t *offsets, uint32_t *out_len) {
    uint32_t n = d_len[kLenParticles];
    *out_len = n ? offsets[n - 1] : 0u;
}

void swap_all(apbf_ctx *ctx) { ctx->fcur ^= 1; }

}  // namespace

// Gathers every particle attribute in the order ctx->perm gives (new id -> old id),
// remaps the transfer and glue lists, and makes the gathered set current.
// With `search` the gather also writes the search records (srec) for range scale
// `scale` and reduces the search radii's range into the status block.
apbf_status reorder_particles(apbf_ctx *ctx, cudaStream_t s, bool search, float scale) {
    const uint32_t cap = ctx->cfg.particle_capacity;
    FluidBufs &cur = ctx->fl[ctx->fcur];
    FluidBufs &alt = ctx->fl[ctx->fcur ^ 1];
    APBF_BEFORE_LAUNCH(ctx, s, "k_reorder");
    k_reorder<<<grid_for(ctx, cap), kBlock, 0, s>>>(cur, alt, ctx->perm, ctx->inv_perm, ctx->d_len,
                                                    search ? ctx->srec : nullptr, scale, ctx->status);
    APBF_AFTER_LAUNCH(ctx, s, "k_reorder");
    APBF_BEFORE_LAUNCH(ctx, s, "k_remap_transfers");
    k_remap_transfers<<<grid_for(ctx, ctx->cfg.transfer_capacity), kBlock, 0, s>>>(ctx->tr[ctx->tcur], ctx->inv_perm,
                                                                                    ctx->d_len, ctx->status);
    APBF_AFTER_LAUNCH(ctx, s, "k_remap_transfers");
    apbf_status r = glue_remap(ctx, s);
    if (r != APBF_OK) return r;
    swap_all(ctx);
    return APBF_OK;
}

apbf_status neighborhood_green(apbf_ctx *ctx, float range_scale, const float minp[3], const float maxp[3],
                               uint32_t L, cudaStream_t s, bool fuse_box, bool corrections) {
    if (L < 1 || L > ctx->cfg.max_log2res || L > 10) {
        set_error("neighborhood_green: log2res must be in [1, max_log2res of apbf_create]");
        return APBF_ERR_INVALID_ARG;
    }
    const uint32_t cap = ctx->cfg.particle_capacity;
    Bounds b = fixed_bounds(minp, maxp);
    FluidBufs &cur = ctx->fl[ctx->fcur];
    const int g = grid_for(ctx, cap);

    APBF_BEFORE_LAUNCH(ctx, s, "k_position_keys");
    k_position_keys<<<g, kBlock, 0, s>>>(cur.pos, ctx->d_len, b, L, ctx->keys[0], ctx->vals[0]);
    APBF_AFTER_LAUNCH(ctx, s, "k_position_keys");
    apbf_status r = sort_pairs_device(ctx, ctx->keys[0], ctx->vals[0], ctx->d_len + kLenParticles, cap, 3u * L,
                                      ctx->sorted_keys, ctx->perm, s);
    if (r != APBF_OK) return r;
    // the reorder reduces the search radii's range: reset it first
    APBF_BEFORE_LAUNCH(ctx, s, "k_reset_search");
    k_reset_search<<<1, 1, 0, s>>>(ctx->status, ctx->d_pairs);
    APBF_AFTER_LAUNCH(ctx, s, "k_reset_search");
    r = reorder_particles(ctx, s, true, range_scale);
    if (r != APBF_OK) return r;
    FluidBufs &f = ctx->fl[ctx->fcur];

    const size_t ncells = (size_t)1 << (3 * L);
    APBF_CUDA(cudaMemsetAsync(ctx->cell_start, 0, ncells * sizeof(uint32_t), s));
    APBF_CUDA(cudaMemsetAsync(ctx->cell_end, 0, ncells * sizeof(uint32_t), s));
    APBF_BEFORE_LAUNCH(ctx, s, "k_cell_ranges");
    k_cell_ranges<<<g, kBlock, 0, s>>>(ctx->sorted_keys, ctx->d_len, ctx->cell_start, ctx->cell_end);
    APBF_AFTER_LAUNCH(ctx, s, "k_cell_ranges");
    APBF_BEFORE_LAUNCH(ctx, s, "k_build_rows");
    BuildArgs ba;
    ba.pos = f.pos;
    FluidBufs &spare = ctx->fl[ctx->fcur ^ 1];
    ba.pos_box = fuse_box ? spare.pos : nullptr;
    ba.range = f.kernel_width;
    ba.radius = f.radius;
    ba.bmin = ctx->box_min;
    ba.bmax = ctx->box_max;
    ba.rot = ctx->box_rot;
    ba.nboxes = ctx->n_boxes;
    ba.scale = range_scale;
    ba.d_len = ctx->d_len;
    ba.b = b;
    ba.L = L;
    ba.fast_ok = 1;
    for (int d = 0; d < 3; ++d)
        if (b.hi[d] - b.lo[d] >= (1ll << 31)) ba.fast_ok = 0;
    ba.cstart = ctx->cell_start;
    ba.cend = ctx->cell_end;
    ba.stride = ctx->row_stride;
    ba.maxn = ctx->cfg.max_neighbors;
    ba.count = ctx->nb_count;
    ba.idx = ctx->nb_idx;
    ba.total = ctx->d_pairs;
    ba.st = ctx->status;
    ba.srec = ctx->srec;
    ba.ucount = ctx->rev_count;
    ba.uidx = ctx->rev_idx;
    ba.one_sided = ctx->flag_scan;  // scratch: not in use during the search
    ba.corrections = corrections ? 1 : 0;
    APBF_CUDA(cudaMemsetAsync(ctx->rev_count, 0, (size_t)cap * sizeof(uint32_t), s));  // correction rows
    k_build_rows<<<grid_for(ctx, cap, kBlock, 8), kBlock, 0, s>>>(ba);
    APBF_AFTER_LAUNCH(ctx, s, "k_build_rows");
    APBF_BEFORE_LAUNCH(ctx, s, "k_corrections");
    k_corrections<<<grid_for(ctx, cap), kBlock, 0, s>>>(ba);
    APBF_AFTER_LAUNCH(ctx, s, "k_corrections");
    if (fuse_box) {  // the box-collided positions are the current ones now
        int4 *t = f.pos;
        f.pos = spare.pos;
        spare.pos = t;
    }
    APBF_BEFORE_LAUNCH(ctx, s, "k_clamp_rev");
    k_clamp_rev<<<grid_for(ctx, cap), kBlock, 0, s>>>(ctx->d_len, ctx->cfg.max_neighbors, ctx->rev_count, ctx->status);
    APBF_AFTER_LAUNCH(ctx, s, "k_clamp_rev");
    return APBF_OK;
}

// Reverse rows by transposing the forward rows (the binary-search neighbourhood and
// the rows spread_kernel_width prunes): row j lists every i whose row holds j, with
// no forward prefix, so the boundariness filter stays in the density pass
// (status union_rows = 0).
apbf_status build_reverse_rows(apbf_ctx *ctx, cudaStream_t s) {
    const uint32_t cap = ctx->cfg.particle_capacity;
    APBF_CUDA(cudaMemsetAsync(ctx->rev_count, 0, (size_t)cap * sizeof(uint32_t), s));
    APBF_BEFORE_LAUNCH(ctx, s, "k_reverse_rows");
    k_reverse_rows<<<grid_for(ctx, cap), kBlock, 0, s>>>(ctx->d_len, ctx->row_stride, ctx->cfg.max_neighbors,
                                                         ctx->nb_count, ctx->nb_idx, ctx->rev_count, ctx->rev_idx,
                                                         ctx->status);
    APBF_AFTER_LAUNCH(ctx, s, "k_reverse_rows");
    APBF_BEFORE_LAUNCH(ctx, s, "k_clamp_rev");
    k_clamp_rev<<<grid_for(ctx, cap), kBlock, 0, s>>>(ctx->d_len, ctx->cfg.max_neighbors, ctx->rev_count, ctx->status);
    APBF_AFTER_LAUNCH(ctx, s, "k_clamp_rev");
    return APBF_OK;
}

apbf_status export_pairs(apbf_ctx *ctx, uint32_t *d_pairs, uint32_t cap_pairs, uint32_t *d_length, cudaStream_t s) {
    const uint32_t cap = ctx->cfg.particle_capacity;
    APBF_CUDA(cudaMemcpyAsync(ctx->scan_tmp, ctx->nb_count, (size_t)cap * 4, cudaMemcpyDeviceToDevice, s));
    apbf_status r = prefix_sum_device(ctx, ctx->scan_tmp, ctx->d_len + kLenParticles, cap, s);
    if (r != APBF_OK) return r;
    k_export_pairs<<<grid_for(ctx, cap), kBlock, 0, s>>>(ctx->d_len, ctx->row_stride, ctx->nb_count, ctx->nb_idx,
                                                         ctx->scan_tmp, cap_pairs, (uint2 *)d_pairs);
    APBF_AFTER_LAUNCH(ctx, s, "k_export_pairs");
    APBF_BEFORE_LAUNCH(ctx, s, "k_export_len");
    k_export_len<<<1, 1, 0, s>>>(ctx->d_len, ctx->scan_tmp, d_length);
    APBF_AFTER_LAUNCH(ctx, s, "k_export_len");
    return APBF_OK;
}

}  // namespace apbf
