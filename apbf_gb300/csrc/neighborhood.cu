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
//  6. k_reverse_rows (only when search radii differ): transpose the rows, so the
//     position-update pass can gather instead of scattering with atomics.
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
__global__ void k_reorder(FluidBufs src, FluidBufs dst, const uint32_t *__restrict__ perm,
                          uint32_t *__restrict__ inv_perm, const uint32_t *d_len) {
    uint32_t n = d_len[kLenParticles];
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

// Walks the cells [x0, x1] x [y0, y1] x [z0, z1] and appends every neighbour of
// particle i.  The walk is a chain of dependent loads (cell range -> candidates),
// so the ranges of up to four cells of one (z, y) row are loaded together and
// candidates four at a time.
template <bool FAST>
__device__ __forceinline__ uint32_t walk_cells(uint32_t i, int4 p, long long R, uint32_t x0, uint32_t x1, uint32_t y0,
                                               uint32_t y1, uint32_t z0, uint32_t z1,
                                               const int4 *__restrict__ pos, const uint32_t *__restrict__ cstart,
                                               const uint32_t *__restrict__ cend, uint32_t stride, uint32_t maxn,
                                               uint32_t *__restrict__ idx) {
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
                    cs[v] = in ? cstart[key] : 0u;
                    ce[v] = in ? cend[key] : 0u;
                }
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const uint32_t s = cs[v], e = ce[v];
                    for (uint32_t j0 = s; j0 < e; j0 += 4) {
                        int4 q[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) q[u] = j0 + u < e ? pos[j0 + u] : p;
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const uint32_t j = j0 + u;
                            if (j >= e || j == i) continue;
                            if (FAST ? !within32(p, q[u], R32, R2) : !within(p, q[u], R)) continue;
                            if (c < maxn) idx[(size_t)c * stride + i] = j;
                            ++c;
                        }
                    }
                }
            }
        }
    return c;
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
};

// neighborhood_green.comp:49-87 with the canonical predicate (C2), one thread per
// particle.  A box that touches no edge cell of the grid only meets particles
// inside the grid (edge cells also hold the clamped outsiders), so it uses the
// 32-bit predicate.
__global__ void __launch_bounds__(256, 4) k_build_rows(BuildArgs a) {
    const uint32_t n = a.d_len[kLenParticles];
    const uint32_t last = (1u << a.L) - 1u;
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
            const Bounds &b = a.b;
            const uint32_t x0 = cell_coord((long long)p.x - R, b.lo[0], b.hi[0], a.L);
            const uint32_t x1 = cell_coord((long long)p.x + R, b.lo[0], b.hi[0], a.L);
            const uint32_t y0 = cell_coord((long long)p.y - R, b.lo[1], b.hi[1], a.L);
            const uint32_t y1 = cell_coord((long long)p.y + R, b.lo[1], b.hi[1], a.L);
            const uint32_t z0 = cell_coord((long long)p.z - R, b.lo[2], b.hi[2], a.L);
            const uint32_t z1 = cell_coord((long long)p.z + R, b.lo[2], b.hi[2], a.L);
            const bool fast = a.fast_ok && x0 > 0 && y0 > 0 && z0 > 0 && x1 < last && y1 < last && z1 < last;
            if (fast)
                c = walk_cells<true>(i, p, R, x0, x1, y0, y1, z0, z1, a.pos, a.cstart, a.cend, a.stride, a.maxn, a.idx);
            else
                c = walk_cells<false>(i, p, R, x0, x1, y0, y1, z0, z1, a.pos, a.cstart, a.cend, a.stride, a.maxn,
                                      a.idx);
        }
        if (c > a.maxn) {
            set_flag(a.st, APBF_FLAG_NEIGHBOR_OVERFLOW);
            atomicMax(&a.st->required_neighbors, c);
        }
        a.count[i] = c < a.maxn ? c : a.maxn;
        local += c < a.maxn ? c : a.maxn;
        if (a.pos_box) a.pos_box[i] = box_push(p, a.radius[i], i, a.bmin, a.bmax, a.rot, a.nboxes);
    }
    // block reduction of the pair count and of the radius range
    for (int off = 16; off > 0; off >>= 1) {
        local += __shfl_down_sync(0xffffffffu, local, off);
        long long a2 = __shfl_down_sync(0xffffffffu, rmin, off);
        long long c2 = __shfl_down_sync(0xffffffffu, rmax, off);
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

// The same rows as k_build_rows, built by blocks of kTileP consecutive (Morton-
// sorted) particles that stage their candidates in shared memory: the block takes
// the union of its particles' cell boxes (at most kTileCells cells), loads the
// particles of those cells kTileBuf at a time with coalesced reads, and every
// thread tests its particle against each staged candidate whose cell lies in the
// particle's own box.  Candidates come in (z, y, x) cell order and index order
// within a cell, the order of walk_cells, so the rows are identical.  A block whose
// union is larger (a jump of the Morton curve inside the block) walks per thread.
constexpr int kTileP = 64;
constexpr int kTileCells = 216;
constexpr int kTileBuf = 512;

__global__ void __launch_bounds__(kTileP) k_build_rows_tiled(BuildArgs a) {
    __shared__ int4 s_pos[kTileBuf];
    __shared__ uint32_t s_idx[kTileBuf];
    __shared__ uint16_t s_cell[kTileBuf];        // region-relative cell of the candidate: x | y << 5 | z << 10
    __shared__ uint32_t s_start[kTileCells];
    __shared__ uint32_t s_pre[kTileCells + 1];  // exclusive prefix of the cells' particle counts
    __shared__ int s_box[6];
    const uint32_t n = a.d_len[kLenParticles];
    const uint32_t last = (1u << a.L) - 1u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long local = 0;
    long long rmin = 0x7fffffffffffffffll, rmax = -1;
    for (uint32_t base = blockIdx.x * kTileP; base < n; base += gridDim.x * kTileP) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        int4 p = make_int4(0, 0, 0, 0);
        long long R = -1;
        uint32_t x0 = 1, x1 = 0, y0 = 1, y1 = 0, z0 = 1, z1 = 0;
        if (valid) {
            p = a.pos[i];
            R = range_fixed(a.range[i], a.scale);
            if (R < 0) {
                set_flag(a.st, APBF_FLAG_NONFINITE);
            } else {
                rmin = R < rmin ? R : rmin;
                rmax = R > rmax ? R : rmax;
                const Bounds &b = a.b;
                x0 = cell_coord((long long)p.x - R, b.lo[0], b.hi[0], a.L);
                x1 = cell_coord((long long)p.x + R, b.lo[0], b.hi[0], a.L);
                y0 = cell_coord((long long)p.y - R, b.lo[1], b.hi[1], a.L);
                y1 = cell_coord((long long)p.y + R, b.lo[1], b.hi[1], a.L);
                z0 = cell_coord((long long)p.z - R, b.lo[2], b.hi[2], a.L);
                z1 = cell_coord((long long)p.z + R, b.lo[2], b.hi[2], a.L);
            }
        }
        const bool has = valid && R >= 0;
        if (threadIdx.x == 0) {
            s_box[0] = s_box[2] = s_box[4] = 0x7fffffff;
            s_box[1] = s_box[3] = s_box[5] = -1;
        }
        __syncthreads();
        if (has) {
            atomicMin(&s_box[0], (int)x0);
            atomicMax(&s_box[1], (int)x1);
            atomicMin(&s_box[2], (int)y0);
            atomicMax(&s_box[3], (int)y1);
            atomicMin(&s_box[4], (int)z0);
            atomicMax(&s_box[5], (int)z1);
        }
        __syncthreads();
        const int bx0 = s_box[0], by0 = s_box[2], bz0 = s_box[4];
        const int nx = s_box[1] - bx0 + 1, ny = s_box[3] - by0 + 1, nz = s_box[5] - bz0 + 1;
        const bool fast = has && a.fast_ok && x0 > 0 && y0 > 0 && z0 > 0 && x1 < last && y1 < last && z1 < last;
        uint32_t c = 0;
        if (s_box[1] < 0) {
            // no particle of the block searches
        } else if ((long long)nx * ny * nz > kTileCells || nx > 31 || ny > 31 || nz > 31) {
            if (has) {
                c = fast ? walk_cells<true>(i, p, R, x0, x1, y0, y1, z0, z1, a.pos, a.cstart, a.cend, a.stride,
                                            a.maxn, a.idx)
                         : walk_cells<false>(i, p, R, x0, x1, y0, y1, z0, z1, a.pos, a.cstart, a.cend, a.stride,
                                             a.maxn, a.idx);
            }
        } else {
            const int cells = nx * ny * nz;
            // cell ranges of the region in (z, y, x) order
            for (int k = threadIdx.x; k < cells; k += kTileP) {
                const uint32_t cx = bx0 + k % nx, cy = by0 + (k / nx) % ny, cz = bz0 + k / (nx * ny);
                const uint32_t key = spread3(cx) | (spread3(cy) << 1) | (spread3(cz) << 2);
                const uint32_t cs = a.cstart[key], ce = a.cend[key];
                s_start[k] = cs;
                s_pre[k + 1] = ce - cs;
            }
            __syncthreads();
            if (warp == 0) {  // exclusive prefix over the cells: 7 per lane, then a warp scan
                uint32_t v[7], sum = 0;
#pragma unroll
                for (int t = 0; t < 7; ++t) {
                    const int k = lane * 7 + t;
                    v[t] = k < cells ? s_pre[k + 1] : 0u;
                    sum += v[t];
                }
                uint32_t incl = sum;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const uint32_t o = __shfl_up_sync(0xffffffffu, incl, off);
                    if (lane >= off) incl += o;
                }
                uint32_t run = incl - sum;
#pragma unroll
                for (int t = 0; t < 7; ++t) {
                    const int k = lane * 7 + t;
                    if (k < cells) s_pre[k] = run;
                    run += v[t];
                }
                if (lane == 31) s_pre[cells] = incl;
            }
            __syncthreads();
            const uint32_t total = s_pre[cells];
            // this particle's own box relative to the region
            const int ox0 = (int)x0 - bx0, ox1 = (int)x1 - bx0, oy0 = (int)y0 - by0, oy1 = (int)y1 - by0,
                      oz0 = (int)z0 - bz0, oz1 = (int)z1 - bz0;
            const uint32_t R32 = (uint32_t)R;
            const unsigned long long R2 = (unsigned long long)R32 * R32;
            for (uint32_t b0 = 0; b0 < total; b0 += kTileBuf) {
                const uint32_t m = total - b0 < (uint32_t)kTileBuf ? total - b0 : (uint32_t)kTileBuf;
                for (uint32_t k = threadIdx.x; k < m; k += kTileP) {
                    const uint32_t g = b0 + k;
                    int lo = 0, hi = cells;  // largest cell with s_pre[cell] <= g
                    while (hi - lo > 1) {
                        const int mid = (lo + hi) >> 1;
                        if (s_pre[mid] <= g) lo = mid;
                        else hi = mid;
                    }
                    const uint32_t j = s_start[lo] + (g - s_pre[lo]);
                    s_pos[k] = a.pos[j];
                    s_idx[k] = j;
                    s_cell[k] = (uint16_t)((lo % nx) | (((lo / nx) % ny) << 5) | ((lo / (nx * ny)) << 10));
                }
                __syncthreads();
                if (has) {
                    for (uint32_t k = 0; k < m; ++k) {
                        const uint32_t rc = s_cell[k];
                        const int rx = rc & 31, ry = (rc >> 5) & 31, rz = rc >> 10;
                        if (rx < ox0 || rx > ox1 || ry < oy0 || ry > oy1 || rz < oz0 || rz > oz1) continue;
                        const uint32_t j = s_idx[k];
                        if (j == i) continue;
                        const int4 q = s_pos[k];
                        if (fast ? !within32(p, q, R32, R2) : !within(p, q, R)) continue;
                        if (c < a.maxn) a.idx[(size_t)c * a.stride + i] = j;
                        ++c;
                    }
                }
                __syncthreads();
            }
        }
        if (valid) {
            if (c > a.maxn) {
                set_flag(a.st, APBF_FLAG_NEIGHBOR_OVERFLOW);
                atomicMax(&a.st->required_neighbors, c);
            }
            a.count[i] = c < a.maxn ? c : a.maxn;
            local += c < a.maxn ? c : a.maxn;
            if (a.pos_box) a.pos_box[i] = box_push(p, a.radius[i], i, a.bmin, a.bmax, a.rot, a.nboxes);
        }
        __syncthreads();  // s_box is reused by the next chunk
    }
    for (int off = 16; off > 0; off >>= 1) {
        local += __shfl_down_sync(0xffffffffu, local, off);
        long long a2 = __shfl_down_sync(0xffffffffu, rmin, off);
        long long c2 = __shfl_down_sync(0xffffffffu, rmax, off);
        rmin = a2 < rmin ? a2 : rmin;
        rmax = c2 > rmax ? c2 : rmax;
    }
    if (lane == 0) {
        if (local) atomicAdd(a.total, local);
        if (rmax >= 0) {
            atomicMin(&a.st->range_min, (unsigned long long)rmin);
            atomicMax(&a.st->range_max, (unsigned long long)rmax);
        }
    }
}

// The same rows again, one warp per particle: lanes take 32 of the particle's
// cells at a time, a warp scan turns their particle counts into offsets, and each
// round the 32 lanes test 32 consecutive candidates (of whichever cells they fall
// in) and append the hits with a ballot, so the row keeps the walk's order (cells
// in (z, y, x) order, indices ascending within a cell) and the lanes stay busy
// whatever the particles' cell counts.
__global__ void __launch_bounds__(256) k_build_rows_warp(BuildArgs a) {
    const uint32_t n = a.d_len[kLenParticles];
    const uint32_t last = (1u << a.L) - 1u;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    unsigned long long local = 0;
    long long rmin = 0x7fffffffffffffffll, rmax = -1;
    for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {  // warp-uniform
        const int4 p = a.pos[i];
        const long long R = range_fixed(a.range[i], a.scale);
        uint32_t c = 0;
        if (R < 0) {
            if (lane == 0) set_flag(a.st, APBF_FLAG_NONFINITE);
        } else {
            rmin = R < rmin ? R : rmin;
            rmax = R > rmax ? R : rmax;
            const Bounds &b = a.b;
            const uint32_t x0 = cell_coord((long long)p.x - R, b.lo[0], b.hi[0], a.L);
            const uint32_t x1 = cell_coord((long long)p.x + R, b.lo[0], b.hi[0], a.L);
            const uint32_t y0 = cell_coord((long long)p.y - R, b.lo[1], b.hi[1], a.L);
            const uint32_t y1 = cell_coord((long long)p.y + R, b.lo[1], b.hi[1], a.L);
            const uint32_t z0 = cell_coord((long long)p.z - R, b.lo[2], b.hi[2], a.L);
            const uint32_t z1 = cell_coord((long long)p.z + R, b.lo[2], b.hi[2], a.L);
            const bool fast = a.fast_ok && x0 > 0 && y0 > 0 && z0 > 0 && x1 < last && y1 < last && z1 < last;
            const uint32_t nx = x1 - x0 + 1, ny = y1 - y0 + 1, nz = z1 - z0 + 1;
            const uint32_t ncells = nx * ny * nz;
            const uint32_t R32 = (uint32_t)R;
            const unsigned long long R2 = (unsigned long long)R32 * R32;
            for (uint32_t cb = 0; cb < ncells; cb += 32) {
                // this lane's cell and its particle range
                const uint32_t k = cb + lane;
                uint32_t cs = 0, cnt = 0;
                if (k < ncells) {
                    const uint32_t cx = x0 + k % nx, cy = y0 + (k / nx) % ny, cz = z0 + k / (nx * ny);
                    const uint32_t key = spread3(cx) | (spread3(cy) << 1) | (spread3(cz) << 2);
                    cs = a.cstart[key];
                    cnt = a.cend[key] - cs;
                }
                uint32_t incl = cnt;  // inclusive scan of the counts over the lanes
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const uint32_t o = __shfl_up_sync(0xffffffffu, incl, off);
                    if (lane >= (uint32_t)off) incl += o;
                }
                const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
                const uint32_t excl = incl - cnt;
                for (uint32_t t0 = 0; t0 < total; t0 += 32) {
                    const uint32_t g = t0 + lane;
                    // the lane whose cell holds candidate g: the last lane with excl <= g
                    uint32_t lo = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const uint32_t e = __shfl_sync(0xffffffffu, excl, lo + step);
                        if (e <= g) lo += step;
                    }
                    const uint32_t owner_cs = __shfl_sync(0xffffffffu, cs, lo);
                    const uint32_t owner_ex = __shfl_sync(0xffffffffu, excl, lo);
                    bool hit = false;
                    uint32_t j = 0;
                    if (g < total) {
                        j = owner_cs + (g - owner_ex);
                        if (j != i) {
                            const int4 q = a.pos[j];
                            hit = fast ? within32(p, q, R32, R2) : within(p, q, R);
                        }
                    }
                    const uint32_t mask = __ballot_sync(0xffffffffu, hit);
                    if (hit) {
                        const uint32_t slot = c + __popc(mask & ((1u << lane) - 1u));
                        if (slot < a.maxn) a.idx[(size_t)slot * a.stride + i] = j;
                    }
                    c += __popc(mask);
                }
            }
        }
        if (lane == 0) {
            if (c > a.maxn) {
                set_flag(a.st, APBF_FLAG_NEIGHBOR_OVERFLOW);
                atomicMax(&a.st->required_neighbors, c);
            }
            a.count[i] = c < a.maxn ? c : a.maxn;
            local += c < a.maxn ? c : a.maxn;
            if (a.pos_box) a.pos_box[i] = box_push(p, a.radius[i], i, a.bmin, a.bmax, a.rot, a.nboxes);
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        local += __shfl_down_sync(0xffffffffu, local, off);
        long long a2 = __shfl_down_sync(0xffffffffu, rmin, off);
        long long c2 = __shfl_down_sync(0xffffffffu, rmax, off);
        rmin = a2 < rmin ? a2 : rmin;
        rmax = c2 > rmax ? c2 : rmax;
    }
    if (lane == 0) {
        if (local) atomicAdd(a.total, local);
        if (rmax >= 0) {
            atomicMin(&a.st->range_min, (unsigned long long)rmin);
            atomicMax(&a.st->range_max, (unsigned long long)rmax);
        }
    }
}

__global__ void k_reverse_rows(const uint32_t *d_len, uint32_t stride, uint32_t maxn, const uint32_t *__restrict__ count,
                               const uint32_t *__restrict__ idx, uint32_t *__restrict__ rcount,
                               uint32_t *__restrict__ ridx, Status *st) {
    if (st->range_min == st->range_max) return;  // symmetric rows: reverse = forward
    uint32_t n = d_len[kLenParticles];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t c = count[i];
        for (uint32_t k = 0; k < c; ++k) {
            uint32_t j = idx[(size_t)k * stride + i];
            uint32_t slot = atomicAdd(&rcount[j], 1u);
            if (slot < maxn) {
                ridx[(size_t)slot * stride + j] = i;
            } else {
                set_flag(st, APBF_FLAG_NEIGHBOR_OVERFLOW);
                atomicMax(&st->required_neighbors, slot + 1u);
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
apbf_status reorder_particles(apbf_ctx *ctx, cudaStream_t s) {
    const uint32_t cap = ctx->cfg.particle_capacity;
    FluidBufs &cur = ctx->fl[ctx->fcur];
    FluidBufs &alt = ctx->fl[ctx->fcur ^ 1];
    APBF_BEFORE_LAUNCH(ctx, s, "k_reorder");
    k_reorder<<<grid_for(ctx, cap), kBlock, 0, s>>>(cur, alt, ctx->perm, ctx->inv_perm, ctx->d_len);
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
                               uint32_t L, cudaStream_t s, bool fuse_box) {
    if (L < 1 || L > ctx->cfg.max_log2res || L > 10) {
        set_error("neighborhood_green: log2res must be in [1, max_log2res of apbf_create]");
        return APBF_ERR_INVALID_ARG;
    }
    const uint32_t cap = ctx->cfg.particle_capacity;
    Bounds b = fixed_bounds(minp, maxp);
    FluidBufs &cur = ctx->fl[ctx->fcur];
    FluidBufs &alt = ctx->fl[ctx->fcur ^ 1];
    const int g = grid_for(ctx, cap);

    APBF_BEFORE_LAUNCH(ctx, s, "k_position_keys");
    k_position_keys<<<g, kBlock, 0, s>>>(cur.pos, ctx->d_len, b, L, ctx->keys[0], ctx->vals[0]);
    APBF_AFTER_LAUNCH(ctx, s, "k_position_keys");
    apbf_status r = sort_pairs_device(ctx, ctx->keys[0], ctx->vals[0], ctx->d_len + kLenParticles, cap, 3u * L,
                                      ctx->sorted_keys, ctx->perm, s);
    if (r != APBF_OK) return r;
    r = reorder_particles(ctx, s);
    if (r != APBF_OK) return r;
    FluidBufs &f = ctx->fl[ctx->fcur];

    const size_t ncells = (size_t)1 << (3 * L);
    APBF_CUDA(cudaMemsetAsync(ctx->cell_start, 0, ncells * sizeof(uint32_t), s));
    APBF_CUDA(cudaMemsetAsync(ctx->cell_end, 0, ncells * sizeof(uint32_t), s));
    APBF_BEFORE_LAUNCH(ctx, s, "k_cell_ranges");
    k_cell_ranges<<<g, kBlock, 0, s>>>(ctx->sorted_keys, ctx->d_len, ctx->cell_start, ctx->cell_end);
    APBF_AFTER_LAUNCH(ctx, s, "k_cell_ranges");
    APBF_BEFORE_LAUNCH(ctx, s, "k_reset_search");
    k_reset_search<<<1, 1, 0, s>>>(ctx->status, ctx->d_pairs);
    APBF_AFTER_LAUNCH(ctx, s, "k_reset_search");
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
    if (ctx->tuning.build_tiled == 1)
        k_build_rows_tiled<<<grid_for(ctx, cap, kTileP, 24), kTileP, 0, s>>>(ba);
    else if (ctx->tuning.build_tiled == 2)
        k_build_rows_warp<<<grid_for(ctx, (uint32_t)std::min<uint64_t>((uint64_t)cap * 32u, 0xffffffffu), kBlock, 8),
                            kBlock, 0, s>>>(ba);
    else
        k_build_rows<<<grid_for(ctx, cap, kBlock, 8), kBlock, 0, s>>>(ba);
    APBF_AFTER_LAUNCH(ctx, s, "k_build_rows");
    if (fuse_box) {  // the box-collided positions are the current ones now
        int4 *t = f.pos;
        f.pos = spare.pos;
        spare.pos = t;
    }
    return build_reverse_rows(ctx, s);
}

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
